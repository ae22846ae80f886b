// gbmd.cc -- the "gbmd" LPMD integrator plugin: whole timesteps of the chosen integrator
// through libgbmd, with the configuration's own (host) cell manager and potentials recreated on
// the device from their names and arguments.  Built by the Makefile beside it against an lpmd2
// checkout's liblpmd headers (make LPMD=<checkout>); loaded by the lpmd program like any other
// plugin.  The GPU plugins under LPMD's own names (plugins.cc) need no control-file edit; this
// one takes `integrator gbmd` in place of the integrator and leaves the rest as it is.
#include <lpmd/error.h>
#include <lpmd/integrator.h>
#include <lpmd/plugin.h>
#include <lpmd/simulation.h>

#include <cstdlib>
#include <string>

#include "gbmd_session.h"

using namespace lpmd;

class GBMDIntegrator : public Integrator, public Plugin {
 public:
  explicit GBMDIntegrator(std::string args) : Plugin("gbmd", "1.0") {
    DefineKeyword("dt", "1.0");
    DefineKeyword("precision", "mixed");  // fp64 | mixed
    DefineKeyword("device", "0");
    // host atoms brought up to date every n steps (1: after every step, which the per-step tags
    // of SetSimulationTags need; a FixedSizeParticleSet is copied in bulk, not atom by atom)
    DefineKeyword("sync-each", "1");
    // the integrator run on the GPU: velocityverlet | euler | leapfrog | verlet | beeman |
    // nosehoover (the last with fmass and t, as the nosehoover plugin takes them)
    DefineKeyword("scheme", "velocityverlet");
    DefineKeyword("fmass", "0");
    DefineKeyword("t", "300.0");
    ProcessArguments(args);
    dt = std::atof(std::string((*this)["dt"]).c_str());
    gbmd_lpmd::plugin_born();
  }
  ~GBMDIntegrator() { gbmd_lpmd::plugin_died(); }

  // One Simulation::DoStep on the GPU: the chosen integrator's force evaluations and updates.
  void Advance(Simulation& s, Potential&) override {
    const std::string device = (*this)["device"];
    setenv("GBMD_DEVICE", device.c_str(), 0);
    const std::string scheme = (*this)["scheme"];
    std::string iargs = "dt " + std::string((*this)["dt"]);
    if (scheme == "nosehoover") iargs += " fmass " + std::string((*this)["fmass"]) + " t " + std::string((*this)["t"]);
    const std::string precision = (*this)["precision"];
    gbmd_lpmd::advance(s, scheme, iargs, precision == "fp64" ? "fp64" : "mixed",
                       std::atoi(std::string((*this)["sync-each"]).c_str()));
  }
};

extern "C" Plugin* create(std::string args) { return new GBMDIntegrator(args); }
extern "C" void destroy(Plugin* m) { delete m; }

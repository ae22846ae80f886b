// plugins.cc -- GPU plugins under the names of LPMD's own: placed ahead of the reference's
// plugin directory on LPMD_PATH (liblpmd/plugins/pluginmanager.cc:74-84), a control file that
// names lennardjones / suttonchen / finnissinclair / finnissinclair-ext / gupta / fastlj,
// linkedcell / verletlist / minimumimage / lcbinary and velocityverlet runs them without an
// edit.  Compiled once per plugin by the Makefile beside it:
//
//   -DGBMD_LPMD_NAME='"lennardjones"' -DGBMD_LPMD_VERSION='"2.0"' -DGBMD_LPMD_KIND=1
//
// kind 1: pair potential    lpmd::PairPotential + lpmd::Plugin   (plugins/lennardjones.h:11)
// kind 2: metal potential   lpmd::MetalPotential + lpmd::Plugin  (plugins/suttonchen.h:12)
// kind 3: cell manager      lpmd::CellManager + lpmd::Plugin     (plugins/linkedcell.h:14)
// kind 4: integrator        lpmd::Integrator + lpmd::Plugin      (plugins/velocityverlet.h:12)
//
// Each keeps the reference plugin's keywords and defaults.  The device work goes through the
// shared session of gbmd_session.h; the scalar functionals host consumers call (pairEnergy,
// pairForce, rhoij, F, PairForce, ManyBodies: atomenergy and similar properties) are libgbmd's
// FP64 host evaluations, in the reference's formulas.  Extra keywords: `precision fp64|mixed`
// on a potential (default $GBMD_PRECISION, else fp64) and `sync-each n` on the integrator.
#include <lpmd/cellmanager.h>
#include <lpmd/configuration.h>
#include <lpmd/error.h>
#include <lpmd/integrator.h>
#include <lpmd/metalpotential.h>
#include <lpmd/pairpotential.h>
#include <lpmd/plugin.h>
#include <lpmd/simulation.h>
#include <lpmd/vector.h>

#include <cstdlib>
#include <string>

#include "gbmd_session.h"

#ifndef GBMD_LPMD_NAME
#error "compile with -DGBMD_LPMD_NAME=... -DGBMD_LPMD_VERSION=... -DGBMD_LPMD_KIND=..."
#endif

using namespace lpmd;

namespace {

// The plugin's libgbmd handle for the host functionals and the cutoff.  An argument error is
// kept and raised at first use: create() itself must not throw.
class HostHandle {
 public:
  void open(const Module& m) {
    gbmd_status rc = gbmd_plugin_create(m.Name().c_str(), gbmd_lpmd::module_args(m).c_str(), &h_);
    if (rc != GBMD_OK) {
      rc_ = rc;
      msg_ = gbmd_last_error();
      h_ = nullptr;
    }
  }
  ~HostHandle() {
    if (h_) gbmd_plugin_destroy(h_);
  }
  const gbmd_plugin* get() const {
    if (!h_) {
      if (rc_ == GBMD_ERR_SYNTAX) throw SyntaxError(msg_);
      throw PluginError(GBMD_LPMD_NAME, msg_);
    }
    return h_;
  }
  double cutoff() const {
    double c = 0.0;
    if (h_) gbmd_plugin_cutoff(h_, &c);
    return c;
  }
  double eval1(int what, const double* args) const {
    double out[3] = {0.0, 0.0, 0.0};
    gbmd_lpmd::check(gbmd_potential_eval(get(), what, args, out));
    return out[0];
  }
  Vector eval3(int what, const double* args) const {
    double out[3] = {0.0, 0.0, 0.0};
    gbmd_lpmd::check(gbmd_potential_eval(get(), what, args, out));
    return Vector(out[0], out[1], out[2]);
  }

 private:
  gbmd_plugin* h_ = nullptr;
  gbmd_status rc_ = GBMD_OK;
  std::string msg_;
};

void define_keywords(Module& m, bool potential) {
  gbmd_lpmd::define_reference_keywords(m, GBMD_LPMD_NAME);
  if (potential) {
    const char* p = std::getenv("GBMD_PRECISION");
    m.DefineKeyword("precision", p ? p : "fp64");
  }
}

}  // namespace

#if GBMD_LPMD_KIND == 1

class GpuPairPotential : public PairPotential, public Plugin, public gbmd_lpmd::DevicePlugin {
 public:
  explicit GpuPairPotential(std::string args) : Plugin(GBMD_LPMD_NAME, GBMD_LPMD_VERSION) {
    define_keywords(*this, true);
    ProcessArguments(args);
    host_.open(*this);
    SetCutoff(host_.cutoff());
    gbmd_lpmd::plugin_born();
  }
  ~GpuPairPotential() { gbmd_lpmd::plugin_died(); }

  double pairEnergy(const double& r) const override {
    const double a[1] = {r};
    return host_.eval1(0, a);
  }
  Vector pairForce(const Vector& r) const override {
    const double a[3] = {r[0], r[1], r[2]};
    return host_.eval3(1, a);
  }
  void UpdateForces(Configuration& conf) override {
    host_.get();
    gbmd_lpmd::update_forces(conf, *this, energycache);
  }
  double energy(Configuration& conf) override { return gbmd_lpmd::energy_of(conf, *this); }

 private:
  HostHandle host_;
};

extern "C" Plugin* create(std::string args) { return new GpuPairPotential(args); }

#elif GBMD_LPMD_KIND == 2

class GpuMetalPotential : public MetalPotential, public Plugin, public gbmd_lpmd::DevicePlugin {
 public:
  explicit GpuMetalPotential(std::string args) : Plugin(GBMD_LPMD_NAME, GBMD_LPMD_VERSION) {
    define_keywords(*this, true);
    ProcessArguments(args);
    host_.open(*this);
    SetCutoff(host_.cutoff());
    gbmd_lpmd::plugin_born();
  }
  ~GpuMetalPotential() { gbmd_lpmd::plugin_died(); }

  double pairEnergy(const double& r) const override {
    const double a[1] = {r};
    return host_.eval1(0, a);
  }
  double rhoij(const double& r) const override {
    const double a[1] = {r};
    return host_.eval1(2, a);
  }
  double F(const double& rho) const override {
    const double a[1] = {rho};
    return host_.eval1(3, a);
  }
  Vector PairForce(const Vector& normr, const double& mod) const override {
    const double a[4] = {normr[0], normr[1], normr[2], mod};
    return host_.eval3(5, a);
  }
  Vector ManyBodies(const Vector& normr, const double& rhoi, const double& rhoj, const double& mod) const override {
    const double a[6] = {normr[0], normr[1], normr[2], rhoi, rhoj, mod};
    return host_.eval3(6, a);
  }
  // The reference computes these once, prints them and drops them (metalpotential.cc:62-180);
  // nothing uses them, so the GPU plugin returns zero.
  Vector UpdateCorrections(const double&, const int&, const double&) const override { return Vector(0.0, 0.0, 0.0); }
  void UpdateForces(Configuration& conf) override {
    host_.get();
    gbmd_lpmd::update_forces(conf, *this, energycache);
  }
  double energy(Configuration& conf) override { return gbmd_lpmd::energy_of(conf, *this); }

 private:
  HostHandle host_;
};

extern "C" Plugin* create(std::string args) { return new GpuMetalPotential(args); }

#elif GBMD_LPMD_KIND == 3

class GpuCellManager : public CellManager, public Plugin, public gbmd_lpmd::DevicePlugin {
 public:
  explicit GpuCellManager(std::string args) : Plugin(GBMD_LPMD_NAME, GBMD_LPMD_VERSION) {
    define_keywords(*this, false);
    ProcessArguments(args);
    cutoff_ = std::atof(std::string((*this)["cutoff"]).c_str());
    gbmd_lpmd::plugin_born();
  }
  ~GpuCellManager() { gbmd_lpmd::plugin_died(); }

  double Cutoff() const override { return cutoff_; }
  void Reset() override {}
  // The device re-bins and rebuilds its lists itself at every force evaluation or step that
  // needs them; on the host side UpdateCell only retires the exported neighbour sets.
  void UpdateCell(Configuration& conf) override { gbmd_lpmd::cells_changed(conf); }
  void UpdateAtom(Configuration& conf, long) override { gbmd_lpmd::cells_changed(conf); }
  void BuildNeighborList(Configuration& conf, long i, NeighborList& nlist, bool full, double rcut) override {
    gbmd_lpmd::build_neighbor_list(conf, i, nlist, full, rcut);
  }

 private:
  double cutoff_ = 0.0;
};

extern "C" Plugin* create(std::string args) { return new GpuCellManager(args); }

#elif GBMD_LPMD_KIND == 4

class GpuVelocityVerlet : public Integrator, public Plugin, public gbmd_lpmd::DevicePlugin {
 public:
  explicit GpuVelocityVerlet(std::string args) : Plugin(GBMD_LPMD_NAME, GBMD_LPMD_VERSION) {
    define_keywords(*this, false);
    DefineKeyword("sync-each", "1");  // host atoms brought up to date every n steps
    ProcessArguments(args);
    dt = std::atof(std::string((*this)["dt"]).c_str());
    gbmd_lpmd::plugin_born();
  }
  ~GpuVelocityVerlet() { gbmd_lpmd::plugin_died(); }

  // VelocityVerlet::Initialize backs up the configuration (plugins/velocityverlet.cc:55-58);
  // the device integrator keeps its own history, and accounts for that UpdateCell call itself.
  void Initialize(Simulation& sim, Potential& p) override { Integrator::Initialize(sim, p); }
  void Advance(Simulation& sim, Potential&) override {
    gbmd_lpmd::advance(sim, "velocityverlet", gbmd_lpmd::module_args(*this), nullptr,
                       std::atoi(std::string((*this)["sync-each"]).c_str()));
  }
};

extern "C" Plugin* create(std::string args) { return new GpuVelocityVerlet(args); }

#endif

extern "C" void destroy(Plugin* m) { delete m; }

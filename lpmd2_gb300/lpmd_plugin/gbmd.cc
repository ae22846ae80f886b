// gbmd.cc -- LPMD integrator plugin running the whole timestep through libgbmd.
// Built by the Makefile beside it against an lpmd2 checkout's liblpmd headers
// (make LPMD=<checkout>); loaded by the lpmd program like any other plugin.
#include <lpmd/cellmanager.h>
#include <lpmd/combinedpotential.h>
#include <lpmd/error.h>
#include <lpmd/integrator.h>
#include <lpmd/plugin.h>
#include <lpmd/simulation.h>
#include <lpmd/util.h>

#include <vector>

#include "gbmd.h"

using namespace lpmd;

namespace {

void check(gbmd_status rc) {
  switch (rc) {
    case GBMD_OK: return;
    case GBMD_ERR_SYNTAX: throw SyntaxError(gbmd_last_error());
    case GBMD_ERR_PLUGIN: throw PluginError("gbmd", gbmd_last_error());
    case GBMD_ERR_MISSING: throw MissingComponent(gbmd_last_error());
    default: throw RuntimeError(gbmd_last_error());
  }
}

// "keyword value ..." of a loaded module: the argument string its create() was given.
std::string module_args(const Module& m) {
  std::string out;
  Array<std::string> kw = StringSplit(m.Keywords());
  for (long k = 0; k < kw.Size(); ++k) out += kw[k] + " " + m[kw[k]] + " ";
  return out;
}

// Potential::SetValidSpecies stores s1 + s2 only; recover a pair with the same sum.
void species_of(const Potential& p, int& s1, int& s2) {
  s1 = s2 = -1;                                   // wildcard
  if (p.AppliesTo(-1000, -1000)) return;
  for (int z = 0; z <= 2 * 118; ++z)
    if (p.AppliesTo(z, 0)) { s1 = z; s2 = 0; return; }
}

}  // namespace

class GBMDIntegrator : public Integrator, public Plugin {
 public:
  explicit GBMDIntegrator(std::string args) : Plugin("gbmd", "1.0") {
    DefineKeyword("dt", "1.0");
    DefineKeyword("precision", "mixed");   // fp64 | mixed
    DefineKeyword("device", "0");
    DefineKeyword("sync-each", "1");       // copy the state back every n steps
    // the integrator run on the GPU: velocityverlet | euler | leapfrog | verlet | beeman |
    // nosehoover (the last with fmass and t, as the nosehoover plugin takes them)
    DefineKeyword("scheme", "velocityverlet");
    DefineKeyword("fmass", "0");
    DefineKeyword("t", "300.0");
    ProcessArguments(args);
  }
  ~GBMDIntegrator() { if (sim) gbmd_sim_destroy(sim); }

  void Initialize(Simulation& s, Potential& p) override {
    Integrator::Initialize(s, p);
    BasicParticleSet& atoms = s.Atoms();
    n = atoms.Size();
    double L[3] = {s.Cell()[0].Module(), s.Cell()[1].Module(), s.Cell()[2].Module()};
    check(gbmd_sim_create(int((*this)["device"]), n, L, &sim));
    std::vector<double> pos(3 * n), vel(3 * n), acc(3 * n), mass(n);
    std::vector<int32_t> Z(n);
    std::vector<uint8_t> flags(n, 0);
    for (long i = 0; i < n; ++i) {
      for (int q = 0; q < 3; ++q) {
        pos[3 * i + q] = atoms[i].Position()[q];
        vel[3 * i + q] = atoms[i].Velocity()[q];
        acc[3 * i + q] = atoms[i].Acceleration()[q];
      }
      Z[i] = atoms[i].Z();
      mass[i] = atoms[i].Mass();
      if (atoms.Have(atoms[i], Tag("fixedvel"))) flags[i] |= GBMD_FLAG_FIXEDVEL;
      if (atoms.Have(atoms[i], Tag("fixedpos")) && atoms.GetTag(atoms[i], Tag("fixedpos")) == "true")
        flags[i] |= GBMD_FLAG_FIXEDPOS;
    }
    check(gbmd_sim_set_atoms(sim, pos.data(), vel.data(), acc.data(), Z.data(), mass.data()));
    check(gbmd_sim_set_flags(sim, flags.data()));

    gbmd_plugin* h = nullptr;
    const Module& cm = dynamic_cast<const Module&>(s.GetCellManager());
    check(gbmd_plugin_create(cm.Name().c_str(), module_args(cm).c_str(), &h));
    check(gbmd_sim_set_cell_manager(sim, h));
    gbmd_plugin_destroy(h);
    CombinedPotential& pots = s.Potentials();
    for (int k = 0; k < pots.Size(); ++k) {
      const Module& pm = dynamic_cast<const Module&>(pots[k]);
      int s1, s2;
      species_of(pots[k], s1, s2);
      check(gbmd_plugin_create(pm.Name().c_str(), module_args(pm).c_str(), &h));
      check(gbmd_sim_add_potential(sim, h, s1, s2));
      gbmd_plugin_destroy(h);
    }
    const std::string scheme = (*this)["scheme"];
    std::string iargs = "dt " + (*this)["dt"];
    if (scheme == "nosehoover") iargs += " fmass " + (*this)["fmass"] + " t " + (*this)["t"];
    check(gbmd_plugin_create(scheme.c_str(), iargs.c_str(), &h));
    check(gbmd_sim_set_integrator(sim, h));
    gbmd_plugin_destroy(h);
    check(gbmd_sim_set_precision(sim, (*this)["precision"] == "fp64" ? GBMD_PRECISION_FP64
                                                                       : GBMD_PRECISION_MIXED));
    check(gbmd_sim_update_forces(sim));
    pull(s);
  }

  // One Simulation::DoStep on the GPU: the chosen integrator's force evaluations and updates.
  void Advance(Simulation& s, Potential&) override {
    check(gbmd_sim_do_steps(sim, 1));
    if (++since_sync >= int((*this)["sync-each"])) { pull(s); since_sync = 0; }
  }

 private:
  // What the host side reads after DoStep: atoms, virial, stress and the
  // "potential-energy" tag that SetSimulationTags turns into the energy tags.
  void pull(Simulation& s) {
    std::vector<double> pos(3 * n), vel(3 * n), acc(3 * n);
    check(gbmd_sim_get_atoms(sim, pos.data(), vel.data(), acc.data()));
    BasicParticleSet& atoms = s.Atoms();
    for (long i = 0; i < n; ++i) {
      atoms[i].Position() = Vector(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      atoms[i].Velocity() = Vector(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
      atoms[i].Acceleration() = Vector(acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]);
    }
    gbmd_thermo th;
    check(gbmd_sim_thermo(sim, &th));
    s.Virial() = th.virial;
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) s.StressTensor().Set(p, q, th.stress[3 * p + q]);
    s.SetTag(s, Tag("potential-energy"), th.potential_energy);
  }

  gbmd_sim* sim = nullptr;
  long n = 0;
  int since_sync = 0;
};

extern "C" Plugin* create(std::string args) { return new GBMDIntegrator(args); }
extern "C" void destroy(Plugin* m) { delete m; }

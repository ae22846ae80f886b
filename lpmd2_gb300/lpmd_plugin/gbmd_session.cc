// gbmd_session.cc -- libgbmd_lpmd.so: the device simulation the GPU plugins of one host
// configuration share (see gbmd_session.h for the protocol).
#include "gbmd_session.h"

#include <lpmd/basicparticleset.h>
#include <lpmd/cellmanager.h>
#include <lpmd/combinedpotential.h>
#include <lpmd/error.h>
#include <lpmd/simulation.h>
#include <lpmd/util.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <utility>

using namespace lpmd;

namespace gbmd_lpmd {

static_assert(sizeof(Vector) == 3 * sizeof(double), "an lpmd::Vector is three contiguous doubles");

DevicePlugin::~DevicePlugin() {}

void check(gbmd_status rc) {
  switch (rc) {
    case GBMD_OK: return;
    case GBMD_ERR_SYNTAX: throw SyntaxError(gbmd_last_error());
    case GBMD_ERR_PLUGIN: throw PluginError("gbmd", gbmd_last_error());
    case GBMD_ERR_MISSING: throw MissingComponent(gbmd_last_error());
    default: throw RuntimeError(gbmd_last_error());
  }
}

std::string module_args(const Module& m) {
  std::string out;
  Array<std::string> kw = StringSplit(m.Keywords());
  for (long k = 0; k < kw.Size(); ++k) {
    std::string v;
    try {
      v = std::string(m[kw[k]]);
    } catch (Error&) {
      continue;  // a keyword without a value (and without a default) is left out
    }
    if (!v.empty()) out += kw[k] + " " + v + " ";
  }
  return out;
}

namespace {

struct Keyword {
  const char* name;
  const char* def;  // nullptr: no default (the reference's DefineKeyword(kw))
};
struct Spec {
  const char* name;
  std::vector<Keyword> kw;
};

// The keyword sets and defaults of the reference plugins: plugins/lennardjones.cc:14-16,
// fastlj.cc:14-17, suttonchen.cc:14-20, finnissinclair.cc:12-18, finnissinclair-ext.cc:13-21,
// gupta.cc:13-18, linkedcell.cc:19-24, verletlist.cc:15-18, minimumimage.cc:15, lcbinary.cc:11-15,
// velocityverlet.cc:14-15.
const std::vector<Spec>& specs() {
  static const std::vector<Spec> s = {
      {"lennardjones", {{"sigma", nullptr}, {"epsilon", nullptr}, {"cutoff", nullptr}}},
      {"fastlj", {{"sigma", nullptr}, {"epsilon", nullptr}, {"cutoff", nullptr}, {"bins", "500"}}},
      {"suttonchen",
       {{"e", nullptr}, {"a", nullptr}, {"n", nullptr}, {"m", nullptr}, {"c", nullptr}, {"cutoff", nullptr},
        {"corrections", "false"}}},
      {"finnissinclair",
       {{"c0", nullptr}, {"c1", nullptr}, {"c2", nullptr}, {"A", nullptr}, {"B", nullptr}, {"c", nullptr},
        {"d", nullptr}}},
      {"finnissinclair-ext",
       {{"c0", nullptr}, {"c1", nullptr}, {"c2", nullptr}, {"c3", nullptr}, {"c4", nullptr}, {"A", nullptr},
        {"B", nullptr}, {"c", nullptr}, {"d", nullptr}}},
      {"gupta", {{"A", nullptr}, {"r0", nullptr}, {"p", nullptr}, {"B", nullptr}, {"q", nullptr}, {"cutoff", nullptr}}},
      {"linkedcell",
       {{"cutoff", "7.0"}, {"nx", "0"}, {"ny", "0"}, {"nz", "0"}, {"mode", "noauto"}, {"warn-outside", "true"}}},
      {"verletlist", {{"cutoff", "0.0"}, {"extcutoff", "0.0"}, {"maxneighbors", "80"}, {"each", "5"}}},
      {"minimumimage", {{"cutoff", "0.0"}}},
      {"lcbinary", {{"cutoff", "7.0"}, {"nx", "0"}, {"ny", "0"}, {"nz", "0"}, {"mode", "noauto"}}},
      {"velocityverlet", {{"dt", "1.0"}, {"start", "1"}}},
  };
  return s;
}

}  // namespace

bool define_reference_keywords(Module& m, const std::string& name) {
  for (const Spec& s : specs()) {
    if (name != s.name) continue;
    for (const Keyword& k : s.kw) {
      if (k.def)
        m.DefineKeyword(k.name, k.def);
      else
        m.DefineKeyword(k.name);
    }
    return true;
  }
  return false;
}

gbmd_plugin* make_handle(const Module& m) {
  gbmd_plugin* h = nullptr;
  check(gbmd_plugin_create(m.Name().c_str(), module_args(m).c_str(), &h));
  return h;
}

namespace {

// One device simulation and the host state it was last given or returned.
struct Session {
  gbmd_sim* sim = nullptr;
  long n = 0;
  double L[3] = {0.0, 0.0, 0.0};
  bool integ_set = false;
  std::string precision = "fp64";
  const Potential* evaluator = nullptr;  // the GPU potential that runs the device evaluation
  double epot = 0.0;                     // device potential energy of the last evaluation or step
  long since_sync = 0;
  bool host_stale = false;               // the device is ahead of the host (sync_each > 1)
  std::vector<double> shadow_pos, shadow_vel, pos, vel, acc;
  bool nb_valid = false;
  int nb_full = -1;
  double nb_rcut = -1.0;
  std::vector<int64_t> nb_counts, nb_offs, nb_idx;
  ~Session() {
    if (sim) gbmd_sim_destroy(sim);
  }
};

using Key = std::pair<const void*, const void*>;  // (configuration, potential or nullptr)
std::map<Key, std::unique_ptr<Session>> g_sessions;
long g_plugins = 0;

int env_device() {
  const char* d = std::getenv("GBMD_DEVICE");
  return d ? std::atoi(d) : 0;
}

// Positions, velocities and accelerations as contiguous double[3n] blocks where the particle
// set stores them that way (FixedSizeParticleSet, liblpmd/lpmd/fixedsizeparticleset.h:33-43),
// else null pointers and the per-atom accessors are used.
bool contiguous(BasicParticleSet& atoms, double** p, double** v, double** a) {
  const long n = atoms.Size();
  if (n == 0) return false;
  double* p0 = &atoms[0].Position()[0];
  double* v0 = &atoms[0].Velocity()[0];
  double* a0 = &atoms[0].Acceleration()[0];
  if (&atoms[n - 1].Position()[0] != p0 + 3 * (n - 1)) return false;
  if (&atoms[n - 1].Velocity()[0] != v0 + 3 * (n - 1)) return false;
  if (&atoms[n - 1].Acceleration()[0] != a0 + 3 * (n - 1)) return false;
  *p = p0;
  *v = v0;
  *a = a0;
  return true;
}

void read_host(Configuration& conf, Session& s) {
  BasicParticleSet& atoms = conf.Atoms();
  const long n = s.n;
  s.pos.resize(3 * n);
  s.vel.resize(3 * n);
  s.acc.resize(3 * n);
  double *p, *v, *a;
  if (contiguous(atoms, &p, &v, &a)) {
    std::memcpy(s.pos.data(), p, sizeof(double) * 3 * n);
    std::memcpy(s.vel.data(), v, sizeof(double) * 3 * n);
    std::memcpy(s.acc.data(), a, sizeof(double) * 3 * n);
    return;
  }
  for (long i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) {
      s.pos[3 * i + q] = atoms[i].Position()[q];
      s.vel[3 * i + q] = atoms[i].Velocity()[q];
      s.acc[3 * i + q] = atoms[i].Acceleration()[q];
    }
}

// Host atoms <- s.pos / s.vel / s.acc (add_acc: accumulate the accelerations instead).
void write_host(Configuration& conf, Session& s, bool positions, bool add_acc) {
  BasicParticleSet& atoms = conf.Atoms();
  const long n = s.n;
  double *p, *v, *a;
  if (contiguous(atoms, &p, &v, &a)) {
    if (positions) {
      std::memcpy(p, s.pos.data(), sizeof(double) * 3 * n);
      std::memcpy(v, s.vel.data(), sizeof(double) * 3 * n);
    }
    if (add_acc)
      for (long k = 0; k < 3 * n; ++k) a[k] += s.acc[k];
    else
      std::memcpy(a, s.acc.data(), sizeof(double) * 3 * n);
    return;
  }
  for (long i = 0; i < n; ++i) {
    if (positions) {
      atoms[i].Position() = Vector(s.pos[3 * i], s.pos[3 * i + 1], s.pos[3 * i + 2]);
      atoms[i].Velocity() = Vector(s.vel[3 * i], s.vel[3 * i + 1], s.vel[3 * i + 2]);
    }
    const Vector ai(s.acc[3 * i], s.acc[3 * i + 1], s.acc[3 * i + 2]);
    if (add_acc)
      atoms[i].Acceleration() += ai;
    else
      atoms[i].Acceleration() = ai;
  }
}

// Potential::SetValidSpecies keeps s1 + s2 only; a pair with the same sum for the device.
void species_of(const Potential& p, int& s1, int& s2) {
  s1 = s2 = -1;
  if (p.AppliesTo(-1000, -1000)) return;  // wildcard
  for (int z = 0; z <= 2 * 118; ++z)
    if (p.AppliesTo(z, 0)) {
      s1 = z;
      s2 = 0;
      return;
    }
}

const char* env_precision() {
  const char* p = std::getenv("GBMD_PRECISION");
  return p ? p : "fp64";
}

// The potentials the device evaluates for this configuration: every potential of a
// Simulation's CombinedPotential, recreated on the device from its name and arguments (host
// plugins included: a device step or a neighbour export never calls them), or `self` alone on
// any other configuration.
std::vector<const Potential*> device_potentials(Configuration& conf, const Potential* self) {
  std::vector<const Potential*> out;
  Simulation* sim = dynamic_cast<Simulation*>(&conf);
  if (!sim) {
    if (self) out.push_back(self);
    return out;
  }
  CombinedPotential& pots = sim->Potentials();
  for (int k = 0; k < pots.Size(); ++k) out.push_back(&pots[k]);
  return out;
}

// Creates (or re-creates, when the atom count or the box changed) the session of `key`.
// precision: "fp64" / "mixed" for the device, or null for the potentials' `precision` keyword
// (any "mixed" wins), else $GBMD_PRECISION, else fp64.
Session& ensure(Configuration& conf, const void* owner, const std::vector<const Potential*>& pots,
                const char* precision_override = nullptr) {
  BasicParticleSet& atoms = conf.Atoms();
  const long n = atoms.Size();
  double L[3];
  for (int q = 0; q < 3; ++q) L[q] = conf.Cell()[q].Module();
  std::unique_ptr<Session>& slot = g_sessions[Key(&conf, owner)];
  if (slot && slot->n == n && slot->L[0] == L[0] && slot->L[1] == L[1] && slot->L[2] == L[2]) {
    if (precision_override && slot->precision != precision_override) {
      check(gbmd_sim_set_precision(slot->sim, std::string(precision_override) == "mixed" ? GBMD_PRECISION_MIXED
                                                                                         : GBMD_PRECISION_FP64));
      slot->precision = precision_override;
    }
    return *slot;
  }
  // built aside and registered only once complete: a failed set-up leaves no half session
  std::unique_ptr<Session> fresh(new Session);
  Session& s = *fresh;
  s.n = n;
  for (int q = 0; q < 3; ++q) s.L[q] = L[q];
  check(gbmd_sim_create(env_device(), n, L, &s.sim));
  std::vector<int32_t> Z(n);
  std::vector<double> mass(n);
  std::vector<uint8_t> flags(n, 0);
  bool any_flag = false;
  for (long i = 0; i < n; ++i) {
    Z[i] = atoms[i].Z();
    mass[i] = atoms[i].Mass();
    if (atoms.Have(atoms[i], Tag("fixedvel"))) flags[i] |= GBMD_FLAG_FIXEDVEL;
    if (atoms.Have(atoms[i], Tag("fixedpos")) && atoms.GetTag(atoms[i], Tag("fixedpos")) == "true")
      flags[i] |= GBMD_FLAG_FIXEDPOS;
    any_flag = any_flag || flags[i];
  }
  read_host(conf, s);
  check(gbmd_sim_set_atoms(s.sim, s.pos.data(), s.vel.data(), s.acc.data(), Z.data(), mass.data()));
  if (any_flag) check(gbmd_sim_set_flags(s.sim, flags.data()));
  s.shadow_pos = s.pos;
  s.shadow_vel = s.vel;
  gbmd_plugin* h = nullptr;
  const Module& cm = dynamic_cast<const Module&>(conf.GetCellManager());
  check(gbmd_plugin_create(cm.Name().c_str(), module_args(cm).c_str(), &h));
  gbmd_status rc = gbmd_sim_set_cell_manager(s.sim, h);
  gbmd_plugin_destroy(h);
  check(rc);
  std::string precision = env_precision();
  for (const Potential* p : pots) {
    const Module& pm = dynamic_cast<const Module&>(*p);
    int s1, s2;
    species_of(*p, s1, s2);
    check(gbmd_plugin_create(pm.Name().c_str(), module_args(pm).c_str(), &h));
    rc = gbmd_sim_add_potential(s.sim, h, s1, s2);
    gbmd_plugin_destroy(h);
    check(rc);
    try {
      if (std::string(pm["precision"]) == "mixed") precision = "mixed";
    } catch (Error&) {
    }
  }
  if (precision_override) precision = precision_override;
  check(gbmd_sim_set_precision(s.sim, precision == "mixed" ? GBMD_PRECISION_MIXED : GBMD_PRECISION_FP64));
  s.precision = precision;
  for (const Potential* p : pots)
    if (dynamic_cast<const DevicePlugin*>(p)) {
      s.evaluator = p;
      break;
    }
  slot = std::move(fresh);
  return *slot;
}

// Uploads the host atoms when they differ from what the device holds (a modifier between
// steps, a host-side integrator, an input plugin).
void push_if_changed(Configuration& conf, Session& s) {
  if (s.host_stale) return;  // the host has not been brought up to date: nothing of it is newer
  read_host(conf, s);
  if (s.pos == s.shadow_pos && s.vel == s.shadow_vel) return;
  check(gbmd_sim_set_atoms(s.sim, s.pos.data(), s.vel.data(), s.acc.data(), nullptr, nullptr));
  s.shadow_pos = s.pos;
  s.shadow_vel = s.vel;
  s.nb_valid = false;
}

void pull_thermo(Configuration& conf, Session& s, bool add) {
  gbmd_thermo th;
  check(gbmd_sim_thermo(s.sim, &th));
  s.epot = th.potential_energy;
  conf.Virial() = (add ? conf.Virial() : 0.0) + th.virial;
  for (int p = 0; p < 3; ++p)
    for (int q = 0; q < 3; ++q)
      conf.StressTensor().Set(p, q, (add ? conf.StressTensor().Get(p, q) : 0.0) + th.stress[3 * p + q]);
}

}  // namespace

void plugin_born() { ++g_plugins; }

void plugin_died() {
  if (--g_plugins == 0) g_sessions.clear();
}

void update_forces(Configuration& conf, const Potential& self, double& energy) {
  const bool is_sim = dynamic_cast<Simulation*>(&conf) != nullptr;
  const void* owner = is_sim ? nullptr : &self;
  std::vector<const Potential*> pots = device_potentials(conf, &self);
  // the device evaluates every potential of the configuration at once; a host potential beside
  // it would add its forces a second time
  for (const Potential* p : pots)
    if (!dynamic_cast<const DevicePlugin*>(p))
      throw PluginError(dynamic_cast<const Module&>(self).Name(),
                        "GPU and host potentials cannot be combined in one configuration (host potential \"" +
                            dynamic_cast<const Module&>(*p).Name() + "\")");
  Session& s = ensure(conf, owner, pots);
  if (s.evaluator != &self) {  // another GPU potential of this configuration evaluated them all
    energy = 0.0;
    return;
  }
  push_if_changed(conf, s);
  check(gbmd_sim_update_forces(s.sim));
  check(gbmd_sim_get_atoms(s.sim, nullptr, nullptr, s.acc.data()));
  // CombinedPotential::UpdateForces zeroed the accelerations, virial and stress before the
  // potentials run (liblpmd/lpmd/combinedpotential.h:39-52): the GPU part is added to them
  write_host(conf, s, false, true);
  pull_thermo(conf, s, true);
  energy = s.epot;
  s.nb_valid = false;
}

void advance(Configuration& conf, const std::string& scheme, const std::string& args, const char* precision,
             int sync_each) {
  Simulation* sim = dynamic_cast<Simulation*>(&conf);
  if (!sim) throw RuntimeError("gbmd: a device integrator needs a Simulation");
  Session& s = ensure(conf, nullptr, device_potentials(conf, nullptr), precision);
  if (!s.integ_set) {
    gbmd_plugin* h = nullptr;
    check(gbmd_plugin_create(scheme.c_str(), args.c_str(), &h));
    gbmd_status rc = gbmd_sim_set_integrator(s.sim, h);
    gbmd_plugin_destroy(h);
    check(rc);
    s.integ_set = true;
  }
  push_if_changed(conf, s);
  check(gbmd_sim_do_steps(s.sim, 1));
  s.nb_valid = false;
  if (++s.since_sync >= (sync_each < 1 ? 1 : sync_each)) {
    check(gbmd_sim_get_atoms(s.sim, s.pos.data(), s.vel.data(), s.acc.data()));
    write_host(conf, s, true, false);
    s.shadow_pos = s.pos;
    s.shadow_vel = s.vel;
    s.since_sync = 0;
    s.host_stale = false;
  } else {
    s.host_stale = true;
  }
  // DoStep zeroed the virial and stress before Advance (simulationbuilder.cc:126-136);
  // SetSimulationTags reads them and the "potential-energy" tag after it
  pull_thermo(conf, s, false);
  conf.SetTag(conf, Tag("potential-energy"), s.epot);
}

double energy_of(Configuration& conf, const Potential& self) {
  const bool is_sim = dynamic_cast<Simulation*>(&conf) != nullptr;
  auto it = g_sessions.find(Key(&conf, is_sim ? nullptr : &self));
  if (it == g_sessions.end() || it->second->evaluator != &self) return 0.0;
  return it->second->epot;
}

void cells_changed(Configuration& conf) {
  for (auto& kv : g_sessions)
    if (kv.first.first == &conf) kv.second->nb_valid = false;
}

void build_neighbor_list(Configuration& conf, long i, NeighborList& nlist, bool full, double rcut) {
  nlist.Clear();
  const bool is_sim = dynamic_cast<Simulation*>(&conf) != nullptr;
  Session* sp = nullptr;
  if (is_sim) {
    sp = &ensure(conf, nullptr, device_potentials(conf, nullptr));
  } else {
    // a backed-up configuration: the session of the potential that evaluates it, if any
    for (auto& kv : g_sessions)
      if (kv.first.first == &conf) {
        sp = kv.second.get();
        break;
      }
    if (!sp) throw RuntimeError("gbmd cell manager: no GPU potential evaluates this configuration");
  }
  Session& s = *sp;
  const int f = full ? 1 : 0;
  if (!s.nb_valid || s.nb_full != f || s.nb_rcut != rcut) {
    // once per export (UpdateCell invalidates it), not once per atom
    push_if_changed(conf, s);
    int64_t total = 0;
    s.nb_counts.assign(s.n, 0);
    check(gbmd_sim_neighbors(s.sim, f, rcut, s.nb_counts.data(), nullptr, 0, &total));
    s.nb_idx.assign(total > 0 ? total : 1, 0);
    check(gbmd_sim_neighbors(s.sim, f, rcut, s.nb_counts.data(), s.nb_idx.data(), total, &total));
    s.nb_offs.assign(s.n + 1, 0);
    for (long k = 0; k < s.n; ++k) s.nb_offs[k + 1] = s.nb_offs[k] + s.nb_counts[k];
    s.nb_valid = true;
    s.nb_full = f;
    s.nb_rcut = rcut;
  }
  if (i < 0 || i >= s.n) return;
  BasicParticleSet& atoms = conf.Atoms();
  BasicCell& cell = conf.Cell();
  AtomPair nn;
  nn.i = &atoms[i];
  nn.i_index = i;
  for (int64_t k = s.nb_offs[i]; k < s.nb_offs[i + 1]; ++k) {
    const long j = (long)s.nb_idx[k];
    nn.j = &atoms[j];
    nn.j_index = j;
    nn.rij = cell.Displacement(nn.i->Position(), nn.j->Position());
    nn.r2 = nn.rij.SquareModule();
    nlist.Append(nn);
  }
}

}  // namespace gbmd_lpmd

// engine.h -- host-side runtime of libgbmd: device state of an ensemble of independent MD
// systems and the step pipeline that drives the sm_103a kernels in engine.cu.
//
// Reference correspondence (jperaltac/lpmd2):
//   Engine::update_forces   CombinedPotential::UpdateForces   liblpmd/lpmd/combinedpotential.h:39-52
//   Engine::do_steps        SimulationEngine::DoStep + TwoStepIntegrator::Advance
//                           liblpmd/simulation/simulationbuilder.cc:126-136,
//                           liblpmd/simulation/twostepintegrator.cc:12-68
//   CellManagerCfg          LinkedCell / VerletListCellManager / MinimumImage / LCBinary plugins
//   PotParams               LennardJones / FastLJ / SuttonChen / FinnisSinclair(-Ext) / Gupta plugins
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace gbmd {

// Error carrying a gbmd_status code; converted at the C ABI.
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

enum PotKind { POT_LJ = 1, POT_SC = 2, POT_FS = 3, POT_FSEXT = 4, POT_GUPTA = 5, POT_FASTLJ = 6 };
enum CmKind { CM_LINKEDCELL = 1, CM_VERLETLIST = 2, CM_MINIMUMIMAGE = 3, CM_LCBINARY = 4 };
enum NbMode { NB_ALLPAIRS = 0, NB_CELLS = 1, NB_LIST = 2 };
enum Rebuild { REBUILD_SKIN = 0, REBUILD_EACH = 1, REBUILD_BOTH = 2 };
enum Precision { PREC_FP64 = 0, PREC_MIXED = 1 };

// Potential parameters, shared by host and device code (plain data).
struct PotParams {
  int kind;
  int spc_sum;        // Potential::SetValidSpecies: s1 + s2; negative = wildcard
  double cutoff;      // Potential::GetCutoff
  double rc2;         // cutoff * cutoff, rounded as the reference computes it
  double p[10];       // plugin parameters in the plugin's keyword order
  double an, am;      // Sutton-Chen pow(a, n), pow(a, m)
  int int_n, int_m;   // integral Sutton-Chen exponents (or -1: general pow)
  float f[16];        // FP32 constants of the mixed path
  const double* tab;  // fastlj: device tables etable[bins], fftable[bins] (set by add_potential)
};

struct CellManagerCfg {
  int kind = CM_LINKEDCELL;
  double cutoff = 7.0;
  int nx = 0, ny = 0, nz = 0;
  bool mode_auto = false;
  double skin = -1.0;           // < 0: default for the plugin
  int64_t maxneighbors = 80;    // verletlist
  int64_t each = 5;             // verletlist rebuild period in UpdateCell calls
  int rebuild = REBUILD_BOTH;   // verletlist policy
  bool compat = false;          // force the reference stencil traversal (linkedcell)
};

struct IntegratorCfg {
  int kind = 0;         // INT_* of integrators.cuh: 0 velocityverlet, 1 euler, 2 leapfrog, 3 verlet,
                        // 4 beeman, 5 nosehoover
  double dt = 1.0;
  int64_t start = 1;
  double fmass = 0.0;   // nosehoover: thermostat mass Q
  double t = 300.0;     // nosehoover: target temperature
};

struct Thermo {
  double v[22];
};

struct Stats {
  int64_t steps = 0, force_evaluations = 0, list_rebuilds = 0, kernel_launches = 0;
  int64_t max_neighbors = 0, list_capacity = 0, neighbor_mode = 0;
  int64_t cell_grid[3] = {0, 0, 0};
  double list_radius = 0.0;
  int64_t device_bytes = 0;
  int64_t fp_guard_rechecks = 0;
  double force_ms = 0.0, drift_ms = 0.0, rebuild_ms = 0.0;
  int64_t force_launches = 0, drift_launches = 0, rebuild_launches = 0;
};

class Engine {
 public:
  Engine(int device, const std::vector<int64_t>& natoms, const std::vector<std::array<double, 3>>& cells);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  int nsys() const { return (int)natoms_.size(); }
  int64_t natoms(int s) const { return natoms_[s]; }

  void set_atoms(int sys, const double* pos, const double* vel, const double* acc, const int32_t* Z,
                 const double* mass);
  void set_flags(int sys, const uint8_t* flags);
  void get_atoms(int sys, double* pos, double* vel, double* acc);
  // Inactive systems are skipped by every kernel; their state is left as it was.
  void set_active(int sys, bool on);
  // Velocity rescaling between steps (mode 0: set temperature, 1: Berendsen); sys < 0: all.
  void scale_velocities(int sys, int mode, double target, double dt_over_tau);
  // Lossless snapshot of the whole engine state; load needs an identically configured engine.
  size_t checkpoint_size();
  void checkpoint_save(void* buf, size_t bytes);
  void checkpoint_load(const void* buf, size_t bytes);

  void set_cell_manager(const CellManagerCfg& cfg);
  void add_potential(const PotParams& p);
  void set_integrator(const IntegratorCfg& cfg);
  void set_precision(int precision);
  void set_option(const std::string& key, const std::string& value);

  void update_forces();
  void do_steps(int64_t nsteps);
  void synchronize();

  void thermo(int sys, double* out22);
  int64_t thermo_log(int sys, double* out, int64_t cap);
  Stats stats();
  void* stream() const;

  void neighbors(int sys, int full, double rcut, int64_t* counts, int64_t* idx, int64_t cap, int64_t* total);
  void cell_sort(int sys, const int32_t n[3], int64_t* cell, int64_t* order);

  struct Impl;

 private:
  std::vector<int64_t> natoms_;
  Impl* d_;
};

// Plugin argument parsing (Module::ProcessArguments, liblpmd/plugins/module.cc:77-103).
struct PluginSpec {
  std::string name;
  int kind = 0;  // GBMD_KIND_*
  std::vector<std::pair<std::string, std::string>> params;
  CellManagerCfg cm;
  PotParams pot{};
  IntegratorCfg integ;
  int precision = -1;  // "precision" keyword on a potential, -1 = not given
  std::string get(const std::string& key) const;
};

// Guard band of the mixed path's FP32 cutoff test: a pair with FP32 r^2 below band_lo(rc2) is
// inside, at or above band_hi(rc2) outside, in between it is decided by the reference's exact
// FP64 r^2.  The band is >= 5x the worst FP32 error of r^2 on cell-relative offsets.
inline float band_lo(double rc2) { return (float)(rc2 * (1.0 - 8e-6)); }
inline float band_hi(double rc2) { return (float)(rc2 * (1.0 + 8e-6)); }

PluginSpec make_plugin(const std::string& name, const std::string& args);
void potential_eval(const PotParams& p, int what, const double* args, double* out);
// Runs the bounded-wait failure path once (a wait nothing completes); returns 1 if it gave up.
int wait_selftest(int device, long long polls);
// Pair forces of one small system with no device allocation (static_forces.cu); stream is a
// cudaStream_t.
void pair_forces_static(const PotParams& P, const double* pos, int n, const double* box, double* force, double* out,
                        void* stream);
PotParams finalize_potential(int kind, const double* params, int s1, int s2);

}  // namespace gbmd

/*
 * gbmd.h -- C ABI of libgbmd, the GB300 (sm_103a) short-range MD timestep behind LPMD's
 * plugin interfaces.
 *
 * Conventions: every entry point returns a gbmd_status (0 = success) and never throws;
 * gbmd_last_error() gives the message of the last failure on the calling thread.  Host
 * buffers are owned by the caller; device buffers are owned by the library.  Vector
 * quantities are xyz-interleaved double[3n] arrays indexed by the caller's atom index
 * (the layout of LPMD's FixedSizeParticleSet, liblpmd/lpmd/fixedsizeparticleset.h:33-43);
 * the device keeps its own cell-sorted copy.  Units are LPMD's: angstrom, fs, amu, eV.
 *
 * Each entry point names the reference interface it replaces (file:line in jperaltac/lpmd2).
 */
#ifndef GBMD_H
#define GBMD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int gbmd_status;

/* Status codes, standing in for LPMD's exception hierarchy (liblpmd/lpmd/error.h:13-76). */
#define GBMD_OK 0
#define GBMD_ERR_INVALID 1     /* InvalidRequest / bad argument                        */
#define GBMD_ERR_SYNTAX 2      /* SyntaxError while parsing plugin arguments            */
#define GBMD_ERR_PLUGIN 3      /* PluginError (unknown plugin, "maxneighbors is too small!") */
#define GBMD_ERR_MISSING 4     /* MissingComponent (no cell manager / potential / integrator) */
#define GBMD_ERR_CUDA 5        /* a CUDA runtime call failed, or no usable GPU           */
#define GBMD_ERR_NOMEM 6       /* device or host allocation failed / over the memory budget */
#define GBMD_ERR_OVERFLOW 7    /* device-side capacity or fixed-point range exceeded     */
#define GBMD_ERR_RUNTIME 8     /* RuntimeError (e.g. atom far outside the box)           */
#define GBMD_ERR_CAPACITY 9    /* caller's output buffer too small                       */

/* Arithmetic of the force path. */
#define GBMD_PRECISION_FP64 0  /* FP64 pair maths and accumulation (the reference's)        */
#define GBMD_PRECISION_MIXED 1 /* FP32 pair maths, int64 fixed-point force/density/energy/
                                  virial sums, FP64 integration, embedding and global
                                  reductions                                                */

/* Per-atom flags: the "fixedvel" and "fixedpos" atom tags honoured by
 * TwoStepIntegrator::Advance (liblpmd/simulation/twostepintegrator.cc:20-41). */
#define GBMD_FLAG_FIXEDVEL 1
#define GBMD_FLAG_FIXEDPOS 2

/* Plugin kinds (the dynamic_cast targets of CastModule<T>, liblpmd/lpmd/pluginmanager.h:24-30). */
#define GBMD_KIND_CELLMANAGER 1
#define GBMD_KIND_POTENTIAL 2
#define GBMD_KIND_INTEGRATOR 3

/* Thermodynamic record: the numeric content of SetSimulationTags
 * (liblpmd/simulation/simulationbuilder.cc:84-124) at full FP64 precision. */
typedef struct gbmd_thermo {
  double step;
  double potential_energy;   /* eV, CombinedPotential::energy                          */
  double kinetic_energy;     /* eV, KineticEnergy (liblpmd/lpmd/properties.h:22-37)     */
  double total_energy;
  double temperature;        /* K, Temperature (liblpmd/lpmd/properties.h:39-53)        */
  double virial;             /* eV, Configuration::Virial                              */
  double momentum[3];        /* amu A/fs, Momentum (liblpmd/lpmd/properties.h:64-81)    */
  double volume;             /* A^3                                                    */
  double virial_pressure;    /* MPa                                                    */
  double kinetic_pressure;   /* MPa                                                    */
  double pressure;           /* MPa                                                    */
  double stress[9];          /* eV, Configuration::StressTensor, row-major [q][p]      */
} gbmd_thermo;

/* Counters of the device work done so far. */
typedef struct gbmd_stats {
  int64_t steps;             /* MD steps advanced                                      */
  int64_t force_evaluations;
  int64_t list_rebuilds;     /* neighbour-list rebuilds summed over systems            */
  int64_t kernel_launches;   /* kernels launched by the library (graph nodes included) */
  int64_t max_neighbors;     /* largest per-atom list length seen at the last rebuild  */
  int64_t list_capacity;     /* current per-atom list capacity                         */
  int64_t neighbor_mode;     /* 0 all-pairs, 1 reference linked cells, 2 Verlet list   */
  int64_t cell_grid[3];      /* grid of the last rebuild (first system)                */
  double list_radius;        /* cutoff + skin of the Verlet list (first system)        */
  int64_t device_bytes;      /* device memory held                                     */
  int64_t fp_guard_rechecks; /* pairs whose cutoff test was re-done in FP64 (mixed)    */
  /* Device time per kernel class, from CUDA events recorded on the simulation's stream
   * around each launch; only with option "time_kernels" 1 and direct launches
   * ("graph_mode" 0). */
  double force_ms;           /* force passes (density + force + kick) summed          */
  int64_t force_launches;    /* force evaluations timed                                */
  double drift_ms;
  int64_t drift_launches;
  double rebuild_ms;         /* cell sort + list build (only evaluations that rebuilt) */
  int64_t rebuild_launches;
} gbmd_stats;

/* ---------------------------------------------------------------------------------------- */
/* Library                                                                                  */
/* ---------------------------------------------------------------------------------------- */

/* Message of the last failed call on this thread ("" if none). */
const char* gbmd_last_error(void);
/* ABI version of this header (increases on incompatible changes). */
int gbmd_abi_version(void);
/* Number of usable CUDA devices (0 without a GPU; never fails). */
gbmd_status gbmd_device_count(int* count);

/* ---------------------------------------------------------------------------------------- */
/* Plugins                                                                                  */
/* ---------------------------------------------------------------------------------------- */

typedef struct gbmd_plugin gbmd_plugin;

/* Creates a plugin from its LPMD name and argument string, as
 * PluginManager::LoadPlugin(name, id, args) + extern "C" create(std::string args) do
 * (liblpmd/plugins/pluginmanager.cc:123-143, liblpmd/lpmd/plugin.h:45-46).  Names:
 * "linkedcell", "verletlist", "minimumimage", "lcbinary", "lennardjones", "fastlj", "suttonchen", "gupta",
 * "finnissinclair", "finnissinclair-ext", "velocityverlet", "euler", "leapfrog", "verlet",
 * "beeman", "nosehoover".  Arguments are parsed as
 * Module::ProcessArguments does (liblpmd/plugins/module.cc:77-103): whitespace-separated
 * keyword/value pairs, a trailing keyword without a value is GBMD_ERR_SYNTAX. */
gbmd_status gbmd_plugin_create(const char* name, const char* args, gbmd_plugin** out);
/* extern "C" destroy(Plugin*) (liblpmd/lpmd/plugin.h:46). */
void gbmd_plugin_destroy(gbmd_plugin* plugin);
/* GBMD_KIND_* of a plugin. */
gbmd_status gbmd_plugin_kind(const gbmd_plugin* plugin, int* kind);
/* ParamList::operator[] (liblpmd/core/paramlist.cc:38): the parameter's value as text. */
gbmd_status gbmd_plugin_param(const gbmd_plugin* plugin, const char* key, char* buf, size_t len);
/* Potential::GetCutoff (liblpmd/lpmd/potential.h:22) or CellManager::Cutoff
 * (liblpmd/lpmd/cellmanager.h:26). */
gbmd_status gbmd_plugin_cutoff(const gbmd_plugin* plugin, double* cutoff);

/* Host FP64 evaluation of a potential's functionals, for host consumers such as the
 * atomenergy/localpressure properties:
 *   what 0: pairEnergy(r)                         args {r}                 out {E}
 *   what 1: pairForce(rij) (pair) / PairForce(r^, r) (metal, out = scalar*r^)
 *                                                 args {rx, ry, rz}        out {Fx, Fy, Fz}
 *   what 2: rhoij(r)  (metal)                     args {r}                 out {rho}
 *   what 3: F(rho)    (metal)                     args {rho}               out {F}
 *   what 4: ManyBodies(r^, rhoi, rhoj, r) (metal) args {rx,ry,rz,rhoi,rhoj} out {Fx,Fy,Fz}
 *   what 5: PairForce(normrij, rmod)  (metal)     args {nx,ny,nz,rmod}     out {Fx,Fy,Fz}
 *   what 6: ManyBodies(normrij, rhoi, rhoj, rmod) args {nx,ny,nz,rhoi,rhoj,rmod} out {Fx,Fy,Fz}
 *           (5 and 6 take the unit vector and modulus as the reference's virtuals receive them,
 *           so their results are the reference's bit for bit)
 * PairPotential (liblpmd/lpmd/pairpotential.h:23-25), MetalPotential
 * (liblpmd/lpmd/metalpotential.h:26-35). */
gbmd_status gbmd_potential_eval(const gbmd_plugin* plugin, int what, const double* args, double* out);

/* ---------------------------------------------------------------------------------------- */
/* Simulation (one system)                                                                  */
/* ---------------------------------------------------------------------------------------- */

typedef struct gbmd_sim gbmd_sim;

/* SimulationBuilder::CreateFixedOrthogonal (liblpmd/simulation/simulationbuilder.cc:321-326)
 * with Cell()[q] = cell[q] * e_q, all axes periodic, on CUDA device `device`. */
gbmd_status gbmd_sim_create(int device, int64_t natoms, const double cell[3], gbmd_sim** out);
void gbmd_sim_destroy(gbmd_sim* sim);

/* Atoms()[i].Position()/Velocity()/Acceleration()/Z()/Mass() for every atom
 * (liblpmd/lpmd/basicatom.h:27-55).  vel/acc may be NULL (zero). */
gbmd_status gbmd_sim_set_atoms(gbmd_sim* sim, const double* pos, const double* vel,
                               const double* acc, const int32_t* Z, const double* mass);
gbmd_status gbmd_sim_set_flags(gbmd_sim* sim, const uint8_t* flags);
/* Copies the current state back in the caller's atom order; any pointer may be NULL. */
gbmd_status gbmd_sim_get_atoms(gbmd_sim* sim, double* pos, double* vel, double* acc);

/* Configuration::SetCellManager (liblpmd/lpmd/configuration.h:54-57). */
gbmd_status gbmd_sim_set_cell_manager(gbmd_sim* sim, const gbmd_plugin* cellmanager);
/* CombinedPotential append + Potential::SetValidSpecies(s1, s2)
 * (lpmd/application.cc:369-391, liblpmd/simulation/potential.cc:22-27). */
gbmd_status gbmd_sim_add_potential(gbmd_sim* sim, const gbmd_plugin* potential, int s1, int s2);
/* Simulation::SetIntegrator (liblpmd/lpmd/simulation.h:37). */
gbmd_status gbmd_sim_set_integrator(gbmd_sim* sim, const gbmd_plugin* integrator);
gbmd_status gbmd_sim_set_precision(gbmd_sim* sim, int precision);
/* Tuning/behaviour options as text key/value pairs.  Unknown keys are GBMD_ERR_INVALID.
 *   "skin"             Verlet skin in A (overrides the cell manager's)
 *   "cell_scale"       1: list-build cells >= cutoff+skin (27-cell stencil), 2: half that (125)
 *   "graph_block"      steps per captured CUDA graph (default 10)
 *   "graph_mode"       0 direct launches, 1 graphs, 2 graphs with a device-decided rebuild (default)
 *   "maxneighbors_cap" verletlist maxneighbors (PluginError when reached)
 *   "time_kernels"     1: CUDA-event timing of every kernel class (graph_mode 0), see gbmd_stats
 *   "stream_priority"  1: the highest stream priority, 0: the lowest (default); replaces the
 *                      stream, so read gbmd_*_stream afterwards
 *   "lanes_per_atom"   mixed Lennard-Jones force pass: 1 (default), 2, 4, 8, 16 or 32 lanes
 *                      share an atom's neighbour list, i.e. 32 to 1 atoms per warp (same
 *                      forces bit for bit; for small systems)
 *   "list_feed"        how the mixed passes read their Verlet-list rows: 0 auto (default:
 *                      registers for a single EAM system, a shared-memory ring of bulk copies
 *                      otherwise), 1 registers, 2 ring (the same results either way) */
gbmd_status gbmd_sim_set_option(gbmd_sim* sim, const char* key, const char* value);

/* CombinedPotential::UpdateForces (liblpmd/lpmd/combinedpotential.h:39-52): zeroes
 * accelerations, virial and stress, updates the cells and evaluates every potential. */
gbmd_status gbmd_sim_update_forces(gbmd_sim* sim);
/* Simulation::DoSteps (liblpmd/simulation/simulationbuilder.cc:126-136): nsteps
 * velocity-Verlet steps (TwoStepIntegrator::Advance, twostepintegrator.cc:12-68).  The
 * second force evaluation of each reference step is the only one made: the first one of
 * the next step sees identical positions. */
gbmd_status gbmd_sim_do_steps(gbmd_sim* sim, int64_t nsteps);
/* Waits for the device work queued on the simulation's stream. */
gbmd_status gbmd_sim_synchronize(gbmd_sim* sim);

/* Thermo record of the last force evaluation / step. */
gbmd_status gbmd_sim_thermo(gbmd_sim* sim, gbmd_thermo* out);
/* Per-step thermo records kept on the device since the last call (oldest first). */
gbmd_status gbmd_sim_thermo_log(gbmd_sim* sim, gbmd_thermo* out, int64_t cap, int64_t* count);
gbmd_status gbmd_sim_stats(gbmd_sim* sim, gbmd_stats* out);
/* The cudaStream_t the simulation's kernels run on. */
gbmd_status gbmd_sim_stream(gbmd_sim* sim, void** stream);

/* Thermostats applied between steps (LPMD's modifiers, which run after DoStep).  The
 * temperature is measured from the current velocities, as the modifiers measure it; the thermo
 * record of the step stays as the step reported it (LPMD's monitor prints those tags):
 *   GBMD_SCALE_SET_TEMPERATURE  T over the atoms without fixedvel/fixedpos, v *= sqrt(target / T)
 *       for those atoms: SimulationBuilder::SetTemperature
 *       (liblpmd/simulation/simulationbuilder.cc:53-72), used by the tempscaling and temperature
 *       modifiers (plugins/tempscaling.cc:66-71, plugins/temperature.cc:58-62)
 *   GBMD_SCALE_BERENDSEN        T over all atoms, v *= sqrt(1 + dt_over_tau * (target / T - 1))
 *       for every atom: BerendsenModifier::Apply (plugins/berendsen.cc:72-99)
 * A system at T = 0 is left unchanged.  The next step's position update is redone with the new
 * velocities. */
#define GBMD_SCALE_SET_TEMPERATURE 0
#define GBMD_SCALE_BERENDSEN 1
gbmd_status gbmd_sim_scale_velocities(gbmd_sim* sim, int mode, double target, double dt_over_tau);

/* Checkpoint / restore, replacing Simulation::Dump / Restore
 * (liblpmd/simulation/simulationbuilder.cc:195-293), which write 6-significant-digit text:
 * a binary snapshot of the complete state (atoms in device order, lists, counters, thermo
 * log).  Load it into a simulation created and configured the same way (same atoms count and
 * cell, cell manager, potentials, integrator, precision and options): it then continues bit
 * for bit as the saved one would have.  A different configuration is GBMD_ERR_INVALID; a
 * buffer smaller than gbmd_sim_checkpoint_size is GBMD_ERR_CAPACITY. */
gbmd_status gbmd_sim_checkpoint_size(gbmd_sim* sim, size_t* bytes);
gbmd_status gbmd_sim_checkpoint_save(gbmd_sim* sim, void* buf, size_t bytes);
gbmd_status gbmd_sim_checkpoint_load(gbmd_sim* sim, const void* buf, size_t bytes);

/* CellManager::BuildNeighborList(conf, i, nlist, full, rcut) for every atom
 * (liblpmd/lpmd/cellmanager.h:25): the j indices with r^2 < rcut^2 as the force kernels
 * see them, per atom in the caller's order (neighbour order within an atom unspecified).
 * counts[natoms]; idx receives sum(counts) indices (cap entries). */
gbmd_status gbmd_sim_neighbors(gbmd_sim* sim, int full, double rcut, int64_t* counts,
                               int64_t* idx, int64_t cap, int64_t* total);
/* LinkedCell binning (plugins/linkedcell.cc:244-266) on an n[0] x n[1] x n[2] grid:
 * cell[i] = WrapAround(floor(n*x/L)) linear index, and order = the atoms sorted by
 * (cell, index), i.e. the reference's head/next traversal order. */
gbmd_status gbmd_sim_cell_sort(gbmd_sim* sim, const int32_t n[3], int64_t* cell, int64_t* order);

/* ---------------------------------------------------------------------------------------- */
/* Batched ensemble: many independent systems advanced by the same kernels                 */
/* ---------------------------------------------------------------------------------------- */

typedef struct gbmd_batch gbmd_batch;

/* nsys systems with natoms[s] atoms and cubic/orthogonal cells cells[3*s..3*s+2]. */
gbmd_status gbmd_batch_create(int device, int nsys, const int64_t* natoms, const double* cells,
                              gbmd_batch** out);
void gbmd_batch_destroy(gbmd_batch* batch);
gbmd_status gbmd_batch_set_atoms(gbmd_batch* batch, int sys, const double* pos, const double* vel,
                                 const int32_t* Z, const double* mass);
gbmd_status gbmd_batch_get_atoms(gbmd_batch* batch, int sys, double* pos, double* vel, double* acc);
/* Takes a system out of (active = 0) or back into (1) the work of later calls: every kernel
 * skips an inactive system and its positions, velocities and counters stay as they were.
 * Serving retires finished jobs this way while the rest of the batch runs on.  No
 * counterpart in the reference (one LPMD process runs one system). */
gbmd_status gbmd_batch_set_active(gbmd_batch* batch, int sys, int active);
/* The same cell manager / potential / integrator plugins apply to every system. */
gbmd_status gbmd_batch_set_cell_manager(gbmd_batch* batch, const gbmd_plugin* cellmanager);
gbmd_status gbmd_batch_add_potential(gbmd_batch* batch, const gbmd_plugin* potential, int s1, int s2);
gbmd_status gbmd_batch_set_integrator(gbmd_batch* batch, const gbmd_plugin* integrator);
gbmd_status gbmd_batch_set_precision(gbmd_batch* batch, int precision);
gbmd_status gbmd_batch_set_option(gbmd_batch* batch, const char* key, const char* value);
gbmd_status gbmd_batch_update_forces(gbmd_batch* batch);
gbmd_status gbmd_batch_do_steps(gbmd_batch* batch, int64_t nsteps);
gbmd_status gbmd_batch_synchronize(gbmd_batch* batch);
gbmd_status gbmd_batch_thermo(gbmd_batch* batch, int sys, gbmd_thermo* out);
gbmd_status gbmd_batch_stats(gbmd_batch* batch, gbmd_stats* out);
gbmd_status gbmd_batch_stream(gbmd_batch* batch, void** stream);
/* gbmd_sim_neighbors for system sys of the batch (CellManager::BuildNeighborList,
 * liblpmd/lpmd/cellmanager.h:25), indices local to the system. */
gbmd_status gbmd_batch_neighbors(gbmd_batch* batch, int sys, int full, double rcut, int64_t* counts,
                                 int64_t* idx, int64_t cap, int64_t* total);
/* gbmd_sim_scale_velocities for system `sys` of a batch (-1: every active system). */
gbmd_status gbmd_batch_scale_velocities(gbmd_batch* batch, int sys, int mode, double target, double dt_over_tau);
/* gbmd_sim_checkpoint_* for a whole batch. */
gbmd_status gbmd_batch_checkpoint_size(gbmd_batch* batch, size_t* bytes);
gbmd_status gbmd_batch_checkpoint_save(gbmd_batch* batch, void* buf, size_t bytes);
gbmd_status gbmd_batch_checkpoint_load(gbmd_batch* batch, const void* buf, size_t bytes);

/* Self-test of the failure path of the kernels' bounded waits (no counterpart in the
 * reference): one warp waits, with the force kernel's wait routine, on an asynchronous-copy
 * barrier that nothing completes, gives up after `polls` polls (1..2^22) and returns;
 * *gave_up = 1 means the wait ended by its bound, the status was reported and the device
 * stays usable.  Nothing faults, traps or hangs. */
gbmd_status gbmd_selftest_bounded_wait(int device, int64_t polls, int* gave_up);

/* ---------------------------------------------------------------------------------------- */
/* Pair forces without device allocation                                                    */
/* ---------------------------------------------------------------------------------------- */

/* Largest system gbmd_pair_forces_static accepts (atoms). */
#define GBMD_STATIC_MAX_ATOMS 16384

/* FP64 pair forces, energy, virial and stress of ONE periodic orthorhombic system whose
 * positions are already in device memory, computed without allocating any device memory.
 * No counterpart in the reference: it packages the minimum-image pair-force evaluation
 * (PairPotential::UpdateForces over MinimumImageCellManager, liblpmd/simulation/
 * pairpotential.cc:35-75, plugins/minimumimage.cc:68-100) for callers that cannot allocate
 * at call time -- host code that hands the whole device memory budget to its own pool, or a
 * latency-bound loop that must not pay for cudaMalloc/cudaFree -- and that bring their own
 * device buffers.  The gbmd_sim_* path allocates its pools in gbmd_sim_create instead.
 *
 *   plugin  a "lennardjones" potential plugin; its cutoff applies, its species
 *           restriction does not (every pair interacts, as with gbmd_sim_add_potential
 *           and s1 = s2 = -1)
 *   pos     device, 3*n doubles (x0 y0 z0 x1 ...), minimum-image displacements as the
 *           reference's Displacement (one wrap of each component)
 *   n       1..GBMD_STATIC_MAX_ATOMS; anything else is GBMD_ERR_INVALID with a message
 *   box     host, 3 doubles: the cell's edge lengths
 *   force   device, 3*n doubles, written: forces in eV/A (no forcefactor/mass scaling)
 *   out     device, 11 doubles, written: pair energy (eV), virial, stress xx xy xz yx yy yz
 *           zx zy zz -- the values gbmd_sim_thermo reports for the same system
 *   stream  cudaStream_t the two kernels are queued on (NULL: the default stream); the call
 *           returns without waiting for them
 *
 * Scratch: the per-block partial sums live in a fixed 11 KB device array inside the
 * library, overwritten by every call; the caller's output buffers need not start at zero.
 * The first call on a device (with that device current) looks the array up, which may load
 * the module: make that first call before anything that must not see module loading, such
 * as stream capture.  The address is kept for the life of the process, so do not call this
 * entry point on a device after cudaDeviceReset on it.  Calls that overlap in time on one
 * device (other host threads, other streams) share the array and race: serialise them. */
gbmd_status gbmd_pair_forces_static(const gbmd_plugin* plugin, const double* pos, int n, const double* box,
                                    double* force, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif

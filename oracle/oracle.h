/*
 * oracle.h -- CPU restatement of LPMD's short-range MD timestep.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the oracle for the GPU library: it is
 * loaded by the tests, by __graft_entry__.smoke() and by the CPU-baseline leg of
 * bench.py, and by nothing else.  The product path (libgbmd) never links or calls it.
 *
 * It restates, loop for loop and in the same floating-point operation order, the
 * reference plugins and drivers of jperaltac/lpmd2:
 *   - OrthogonalCell::Displacement / FittedInside   liblpmd/lpmd/orthogonalcell.h:90-149
 *   - LinkedCell::UpdateCell / BuildNeighborList     plugins/linkedcell.cc:9-15,112-267,293-360
 *   - VerletListCellManager                          plugins/verletlist.cc:12-29,67-167
 *   - MinimumImage cell manager                      plugins/minimumimage.cc:55-100
 *   - PairPotential::UpdateForces                    liblpmd/simulation/pairpotential.cc:35-84
 *   - LennardJones::pairEnergy / pairForce           plugins/lennardjones.cc:53-67
 *   - MetalPotential::UpdateForces                   liblpmd/simulation/metalpotential.cc:62-180
 *   - SuttonChen functionals                         plugins/suttonchen.cc:73-95
 *   - FinnisSinclair / FinnisSinclairExt             plugins/finnissinclair.cc:75-113,
 *                                                    plugins/finnissinclair-ext.cc:85-128
 *   - Gupta functionals                              plugins/gupta.cc:52-75
 *   - FastLJ tables and lookups                      plugins/fastlj.cc:38-73
 *   - LCBinary grid, growth and neighbour lists      plugins/lcbinary.cc:50-254
 *   - Euler, Leapfrog, Verlet, Beeman, NoseHoover    plugins/euler.cc, leapfrog.cc, verlet.cc,
 *                                                    beeman.cc, nosehoover.cc
 *   - CombinedPotential::UpdateForces                liblpmd/lpmd/combinedpotential.h:39-52
 *   - TwoStepIntegrator::Advance + VelocityVerlet    liblpmd/simulation/twostepintegrator.cc:12-68,
 *                                                    plugins/velocityverlet.cc:55-75,
 *                                                    liblpmd/simulation/integrator.cc:16-22
 *   - SimulationEngine::DoStep / SetSimulationTags   liblpmd/simulation/simulationbuilder.cc:84-136
 *   - KineticEnergy / Temperature / Momentum         liblpmd/lpmd/properties.h:22-81
 *
 * Pinning: tests/test_oracle_golden.py checks this restatement against golden
 * vectors produced by the reference itself (tests/golden/make_golden.py drives
 * the reference sources compiled by oracle/Makefile into oracle/_ref/), against the
 * reference unit-test vectors for the cell geometry (liblpmd/tests/orthogonalcelltest.unit)
 * and against the 108-atom neighbour known-answer program (liblpmd/demos/linkedcell.cc).
 *
 * Build with -ffp-contract=off so that no multiply-add is fused on any host (the
 * reference is built for x86-64 without FMA, so its products and sums round separately).
 */
#ifndef LPMD_ORACLE_H
#define LPMD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_OK = 0,
  ORC_ERR_INVALID = 1,      /* bad argument (the reference would divide by zero or crash) */
  ORC_ERR_MAXNEIGHBORS = 2, /* PluginError("verletlist", "maxneighbors is too small!") */
  ORC_ERR_NOMEM = 3,
  ORC_ERR_MISSING = 4,      /* MissingComponent: no cell manager / integrator */
  ORC_ERR_CAPACITY = 5      /* caller buffer too small */
};

enum { ORC_CM_LINKEDCELL = 1, ORC_CM_VERLETLIST = 2, ORC_CM_MINIMUMIMAGE = 3, ORC_CM_LCBINARY = 4 };

enum { ORC_POT_LJ = 1, ORC_POT_SC = 2, ORC_POT_FS = 3, ORC_POT_FSEXT = 4, ORC_POT_GUPTA = 5, ORC_POT_FASTLJ = 6 };

/* Per-atom flag bits, standing in for the "fixedvel" / "fixedpos" atom tags
 * (liblpmd/simulation/twostepintegrator.cc:20-41). */
enum { ORC_FIXEDVEL = 1, ORC_FIXEDPOS = 2 };

/* Layout of the thermo record (doubles), mirroring SetSimulationTags
 * (liblpmd/simulation/simulationbuilder.cc:84-124) at full precision. */
enum {
  ORC_T_STEP = 0,
  ORC_T_EPOT = 1,
  ORC_T_EKIN = 2,
  ORC_T_ETOT = 3,
  ORC_T_TEMP = 4,
  ORC_T_VIRIAL = 5,
  ORC_T_PX = 6,
  ORC_T_PY = 7,
  ORC_T_PZ = 8,
  ORC_T_VOLUME = 9,
  ORC_T_VIRIAL_PRESSURE = 10,
  ORC_T_KINETIC_PRESSURE = 11,
  ORC_T_PRESSURE = 12,
  ORC_T_STRESS = 13, /* 9 values: stress[q][p] raw (eV), row-major */
  ORC_THERMO_LEN = 22
};

typedef struct orc_sim orc_sim;

/* SimulationBuilder::CreateFixedOrthogonal + setting Cell()[q] = L[q]*e_q. */
orc_sim* orc_sim_create(int64_t n, const double L[3]);
void orc_sim_destroy(orc_sim* s);

/* Writes positions/velocities/accelerations (xyz interleaved, 3n doubles each),
 * atomic numbers and masses.  vel/acc may be NULL (zero). */
int orc_sim_set_atoms(orc_sim* s, const double* pos, const double* vel, const double* acc,
                      const int32_t* Z, const double* mass);
int orc_sim_set_flags(orc_sim* s, const uint8_t* flags);
int orc_sim_get_atoms(const orc_sim* s, double* pos, double* vel, double* acc);

/* Cell managers.  Mirrors SetCellManager: the manager is created and UpdateCell is
 * called once on the current positions (liblpmd/lpmd/configuration.h:54-57). */
int orc_sim_set_linkedcell(orc_sim* s, double cutoff, int nx, int ny, int nz, int mode_auto);
int orc_sim_set_verletlist(orc_sim* s, double cutoff, int64_t maxneighbors, int64_t each);
int orc_sim_set_minimumimage(orc_sim* s, double cutoff);
int orc_sim_set_lcbinary(orc_sim* s, double cutoff, int nx, int ny, int nz, int mode_auto);

/* Appends a potential to the CombinedPotential with SetValidSpecies(s1, s2).
 * params: LJ {sigma, epsilon, cutoff}; SC {e, a, n, m, c, cutoff};
 *         FS {c0, c1, c2, A, B, c, d}; FSEXT {c0, c1, c2, c3, c4, A, B, c, d}. */
int orc_sim_add_potential(orc_sim* s, int kind, const double* params, int nparams, int s1, int s2);

int orc_sim_set_velocityverlet(orc_sim* s, double dt);
enum { ORC_INT_VV = 0, ORC_INT_EULER = 1, ORC_INT_LEAPFROG = 2, ORC_INT_VERLET = 3, ORC_INT_BEEMAN = 4,
       ORC_INT_NOSEHOOVER = 5 };
/* velocityverlet, euler, leapfrog, verlet, beeman, nosehoover (fmass, t: nosehoover only) */
int orc_sim_set_integrator(orc_sim* s, int kind, double dt, double fmass, double t);

/* CombinedPotential::UpdateForces: zero acc/virial/stress, UpdateCell, every potential. */
int orc_sim_update_forces(orc_sim* s);

/* DoStep x nsteps; if thermo is non-NULL it receives nsteps records of ORC_THERMO_LEN. */
int orc_sim_do_steps(orc_sim* s, int64_t nsteps, double* thermo);

/* Current thermo record (uses the last force evaluation's energy/virial/stress). */
int orc_sim_thermo(const orc_sim* s, double* out);

/* Potential energy of the last UpdateForces (CombinedPotential::energy). */
double orc_sim_energy(const orc_sim* s);
double orc_sim_virial(const orc_sim* s);
void orc_sim_stress(const orc_sim* s, double out[9]);

/* CellManager::BuildNeighborList for every atom, after the last UpdateCell.
 * counts[n]; idx receives the j indices concatenated in list order (cap entries). */
int orc_sim_neighbors(orc_sim* s, int full, double rcut, int64_t* counts, int64_t* idx,
                      int64_t cap, int64_t* total);

/* Number of UpdateCell calls made so far (the verletlist rebuild clock). */
int64_t orc_sim_update_cell_calls(const orc_sim* s);

/* Geometry primitives (OrthogonalCell, all axes periodic). */
void orc_displacement(const double L[3], const double a[3], const double b[3], double out[3]);
void orc_fitted_inside(const double L[3], const double a[3], double out[3]);

/* LinkedCell stencil as the reference builds it: side and number of stencil cells. */
int orc_linkedcell_geometry(const double L[3], double cutoff, int nx, int ny, int nz, int mode_auto,
                            int* out_n /*3*/, int* out_side, int* out_cells_inside);

#ifdef __cplusplus
}
#endif

#endif

// gbmd_session.h -- what the GPU plugins named like LPMD's own share: one libgbmd simulation per host
// configuration, kept in step with the host atoms, plus the helpers every plugin needs.
//
// LPMD loads every plugin as its own .so (liblpmd/plugins/pluginmanager.cc:74-84,123-143) and
// hands each one the host Configuration.  The GPU plugins (lennardjones.so, suttonchen.so,
// linkedcell.so, velocityverlet.so, ... built from plugins.cc) all link libgbmd_lpmd.so, whose
// registry gives them the same device simulation for the same configuration, so a control file
// that names them runs its whole timestep on the GPU:
//
//   Potential::UpdateForces (liblpmd/lpmd/potential.h:27)   the first GPU potential of the
//       configuration's CombinedPotential evaluates every GPU potential of it on the device
//       (gbmd_sim_update_forces) and adds their forces, virial and stress to the host; the
//       others find the evaluation done.  A configuration that is not a Simulation (the backed-up
//       copy some integrators evaluate, liblpmd/simulation/integrator.cc:16-22) gets a session
//       per potential instead.
//   Integrator::Advance (liblpmd/lpmd/integrator.h:32)      one whole velocity-Verlet step on the
//       device (gbmd_sim_do_steps), then the host atoms, virial, stress and the
//       "potential-energy" tag are brought up to date.
//   CellManager::BuildNeighborList (liblpmd/lpmd/cellmanager.h:25)  the device's neighbour sets
//       (gbmd_sim_neighbors), exported once per UpdateCell, for host consumers.
//
// The device holds the state between calls.  Before each device call the host atoms are compared
// with the copy the device was last given or returned (positions, velocities), and uploaded when
// they differ -- a modifier such as tempscaling rescales velocities on the host between steps.
// Errors come back as the reference's exception classes (liblpmd/lpmd/error.h:13-76).
#pragma once

#include <lpmd/atompair.h>
#include <lpmd/configuration.h>
#include <lpmd/module.h>
#include <lpmd/potential.h>

#include <string>
#include <vector>

#include "gbmd.h"

namespace gbmd_lpmd {

// Marks the GPU plugins (a common base reachable by dynamic_cast from any LPMD interface).
class DevicePlugin {
 public:
  virtual ~DevicePlugin();
};

// Status of a libgbmd call to LPMD's exception classes.
void check(gbmd_status rc);

// "keyword value ..." of a loaded module: the argument string that recreates it.
std::string module_args(const lpmd::Module& m);

// The reference plugin's keywords and defaults (name -> list of {keyword, default or null}),
// defined on `m`; returns false for a name that has no GPU implementation.
bool define_reference_keywords(lpmd::Module& m, const std::string& name);

// A libgbmd plugin handle with the module's name and arguments (host functionals, cutoff).
gbmd_plugin* make_handle(const lpmd::Module& m);

// Registration of the GPU plugin objects alive in the process: the last one to go releases the
// device simulations.
void plugin_born();
void plugin_died();

// Potential::UpdateForces of a GPU potential (see above).  `energy` receives its part of the
// potential energy (the whole GPU part for the potential that evaluated, zero for the others).
void update_forces(lpmd::Configuration& conf, const lpmd::Potential& self, double& energy);

// Potential::energy of a GPU potential: the device's potential energy for the potential that
// evaluates the configuration, zero for the others (their sum is the CombinedPotential's).
double energy_of(lpmd::Configuration& conf, const lpmd::Potential& self);

// Integrator::Advance of a device integrator: one step of `sim` on the device with libgbmd's
// integrator `scheme` ("velocityverlet", "beeman", ...; `args` its keywords), the host atoms
// brought up to date every `sync_each` steps.  precision: "fp64", "mixed" or null (see
// gbmd_session.cc::ensure).  Every potential of the simulation is recreated on the device from
// its name and arguments, so host potentials are fine here.
void advance(lpmd::Configuration& sim, const std::string& scheme, const std::string& args, const char* precision,
             int sync_each);

// CellManager::UpdateCell / UpdateAtom of a GPU cell manager: the exported neighbour sets of the
// configuration are stale from here on.
void cells_changed(lpmd::Configuration& conf);

// CellManager::BuildNeighborList of a GPU cell manager.
void build_neighbor_list(lpmd::Configuration& conf, long i, lpmd::NeighborList& nlist, bool full, double rcut);

}  // namespace gbmd_lpmd

// ref_driver.cpp -- drives the reference LPMD sources (compiled by oracle/Makefile into
// oracle/_ref/) on caller-supplied inputs, for pinning the C restatement in oracle.c.
//
// TEST INFRASTRUCTURE ONLY.  Built only where the reference sources are present; the
// product never links it.  It follows the harness pattern of liblpmd/demos/simplemd.cc:47-80
// and does not use the lpmd CLI (whose plugin keyword probe crashes in this checkout):
//   SimulationBuilder::CreateFixedOrthogonal -> Cell()[q] -> positions/velocities
//   -> SetCellManager(plugin) -> Potentials().Append(plugin with SetValidSpecies)
//   -> SetIntegrator(velocityverlet) -> Potentials().UpdateForces -> DoStep() x n.
// Plugins are constructed directly from their classes; every plugin translation unit is
// compiled with its create/destroy entry points renamed so they can share one library.
#include <lpmd/atom.h>
#include <lpmd/cellmanager.h>
#include <lpmd/combinedpotential.h>
#include <lpmd/integrator.h>
#include <lpmd/potential.h>
#include <lpmd/properties.h>
#include <lpmd/simulationbuilder.h>
#include <runtime/runtime_context.h>

#include "finnissinclair-ext.h"
#include "lpmd.h"
#include "xyz.h"
#include "fastlj.h"
#include "finnissinclair.h"
#include "gupta.h"
#include "lcbinary.h"
#include "lennardjones.h"
#include "linkedcell.h"
#include "minimumimage.h"
#include "suttonchen.h"
#include "beeman.h"
#include "euler.h"
#include "leapfrog.h"
#include "nosehoover.h"
#include "velocityverlet.h"
#include "verlet.h"
#include "verletlist.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <fstream>
#include <string>

using namespace lpmd;

namespace {

enum { T_STEP = 0, T_EPOT, T_EKIN, T_ETOT, T_TEMP, T_VIRIAL, T_PX, T_PY, T_PZ, T_VOLUME,
       T_VIRIAL_PRESSURE, T_KINETIC_PRESSURE, T_PRESSURE, T_STRESS, THERMO_LEN = 22 };

char g_error[512];
std::string g_integ_name = "velocityverlet", g_integ_args;  // integrator of the next ref_run
bool g_supply_context = false;  // give the backed-up configuration the runtime context

Integrator* make_integ(const std::string& name, const std::string& args) {
  if (name == "velocityverlet") return new VelocityVerlet(args);
  if (name == "euler") return new Euler(args);
  if (name == "leapfrog") return new Leapfrog(args);
  if (name == "verlet") return new Verlet(args);
  if (name == "beeman") return new Beeman(args);
  if (name == "nosehoover") return new NoseHoover(args);
  return nullptr;
}

CellManager* make_cm(const std::string& name, const std::string& args) {
  if (name == "linkedcell") return new LinkedCell(args);
  if (name == "verletlist") return new VerletListCellManager(args);
  if (name == "minimumimage") return new MinimumImageCellManager(args);
  if (name == "lcbinary") return new LCBinary(args);
  return nullptr;
}

Potential* make_pot(const std::string& name, const std::string& args) {
  if (name == "lennardjones") return new LennardJones(args);
  if (name == "suttonchen") return new SuttonChen(args);
  if (name == "finnissinclair") return new FinnisSinclair(args);
  if (name == "finnissinclair-ext") return new FinnisSinclairExt(args);
  if (name == "gupta") return new Gupta(args);
  if (name == "fastlj") return new FastLJ(args);
  return nullptr;
}

void thermo(Simulation& md, double* out) {
  BasicParticleSet& atoms = md.Atoms();
  const double pressfactor = double(md.Context().session()["pressfactor"]);
  const double v = md.Cell().Volume();
  const Vector P = Momentum(atoms, false);
  const double kin = KineticEnergy(atoms, false);
  const double epot = md.Potentials().energy(md);
  std::memset(out, 0, sizeof(double) * THERMO_LEN);
  out[T_STEP] = double(md.CurrentStep());
  out[T_EPOT] = epot;
  out[T_EKIN] = kin;
  out[T_ETOT] = epot + kin;
  out[T_TEMP] = Temperature(atoms, false);
  out[T_VIRIAL] = md.Virial();
  out[T_PX] = P[0];
  out[T_PY] = P[1];
  out[T_PZ] = P[2];
  out[T_VOLUME] = v;
  out[T_VIRIAL_PRESSURE] = (pressfactor / v) * (1.0 / 3.0) * md.Virial();
  out[T_KINETIC_PRESSURE] = (pressfactor / v) * (2.0 / 3.0) * kin;
  out[T_PRESSURE] = (pressfactor / v) * ((2.0 / 3.0) * kin + (1.0 / 3.0) * md.Virial());
  const Matrix& s = md.StressTensor();
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) out[T_STRESS + 3 * a + b] = s.Get(a, b);
}

void neighbors(Simulation& md, int full, double rcut, int64_t* counts, int64_t* idx, int64_t cap,
               int64_t* total) {
  BasicParticleSet& atoms = md.Atoms();
  int64_t t = 0;
  for (long i = 0; i < atoms.Size(); ++i) {
    NeighborList& nl = md.Neighbors(i, full != 0, rcut);
    if (counts) counts[i] = nl.Size();
    for (long k = 0; k < nl.Size(); ++k) {
      if (idx && t < cap) idx[t] = nl[k].j_index;
      ++t;
    }
  }
  if (total) *total = t;
}

}  // namespace

extern "C" const char* ref_last_error() { return g_error; }

// Selects the integrator plugin (and its arguments, "dt" appended by ref_run) of the next
// ref_run call, velocityverlet afterwards; supply_context: see ref_run.
extern "C" void ref_set_integrator(const char* name, const char* args, int supply_context) {
  g_integ_name = name ? name : "velocityverlet";
  g_integ_args = args ? args : "";
  g_supply_context = supply_context != 0;
}

// Runs one reference simulation.  Inputs are xyz-interleaved.  Outputs (each may be NULL):
//   out_mass[n]                     masses the reference assigned from `symbol`
//   out_acc0[3n], out_thermo0[22]   after the initial Potentials().UpdateForces(md)
//   neigh_*                         BuildNeighborList for every atom right after that call
//   out_thermo[nsteps*22]           after every DoStep
//   out_pos/out_vel/out_acc[3n]     final state
// Returns 0 on success, 1 on a reference exception (message in ref_last_error()).
extern "C" int ref_run(int64_t n, const double* L, const char* symbol, const double* pos,
                       const double* vel, const char* cm_name, const char* cm_args, int npot,
                       const char* const* pot_names, const char* const* pot_args,
                       const int32_t* spc, double dt, int64_t nsteps, double* out_mass,
                       double* out_acc0, double* out_thermo0, int neigh_full, double neigh_rcut,
                       int64_t* neigh_counts, int64_t* neigh_idx, int64_t neigh_cap,
                       int64_t* neigh_total, double* out_thermo, double* out_pos, double* out_vel,
                       double* out_acc) {
  g_error[0] = 0;
  try {
    static RuntimeContext context;
    Simulation& md = SimulationBuilder::CreateFixedOrthogonal(context, long(n), Atom(symbol));
    BasicCell& cell = md.Cell();
    cell[0] = L[0] * e1;
    cell[1] = L[1] * e2;
    cell[2] = L[2] * e3;
    BasicParticleSet& atoms = md.Atoms();
    for (long i = 0; i < atoms.Size(); ++i) {
      atoms[i].Position() = Vector(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      atoms[i].Velocity() =
          vel ? Vector(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]) : Vector(0.0, 0.0, 0.0);
      atoms[i].Acceleration() = Vector(0.0, 0.0, 0.0);
      if (out_mass) out_mass[i] = atoms[i].Mass();
    }
    CellManager* cm = make_cm(cm_name, cm_args);
    if (!cm) {
      std::snprintf(g_error, sizeof g_error, "unknown cell manager %s", cm_name);
      return 1;
    }
    md.SetCellManager(*cm);
    for (int p = 0; p < npot; ++p) {
      Potential* pot = make_pot(pot_names[p], pot_args[p]);
      if (!pot) {
        std::snprintf(g_error, sizeof g_error, "unknown potential %s", pot_names[p]);
        return 1;
      }
      pot->SetValidSpecies(spc[2 * p], spc[2 * p + 1]);
      md.Potentials().Append(*pot);
    }
    Integrator* vv = nullptr;
    if (nsteps > 0) {
      char dtarg[64];
      std::snprintf(dtarg, sizeof dtarg, "dt %.17g", dt);
      vv = make_integ(g_integ_name, std::string(dtarg) + (g_integ_args.empty() ? "" : " " + g_integ_args));
      g_integ_name = "velocityverlet";
      g_integ_args.clear();
      if (!vv) {
        std::snprintf(g_error, sizeof g_error, "unknown integrator");
        return 1;
      }
      md.SetIntegrator(*vv);
    }
    md.Potentials().Initialize(md);
    md.Potentials().UpdateForces(md);
    if (out_acc0)
      for (long i = 0; i < atoms.Size(); ++i)
        for (int q = 0; q < 3; ++q) out_acc0[3 * i + q] = atoms[i].Acceleration()[q];
    if (out_thermo0) thermo(md, out_thermo0);
    if (neigh_counts || neigh_idx || neigh_total)
      neighbors(md, neigh_full, neigh_rcut, neigh_counts, neigh_idx, neigh_cap, neigh_total);
    if (vv && g_supply_context) {
      // leapfrog / beeman / nosehoover: Initialize evaluates forces on the configuration
      // UseOldConfig backs up, which never receives the runtime context, so the unmodified
      // reference throws MissingComponent("runtime_context") at its first step.  The backup is
      // made here, where Initialize would make it, and given the context; Initialize then
      // finds it and runs the reference's own code unchanged.
      vv->UseOldConfig(md);
      vv->OldConfig().SetRuntimeContext(context);
    }
    g_supply_context = false;
    for (int64_t k = 0; k < nsteps; ++k) {
      md.DoStep();
      if (out_thermo) thermo(md, out_thermo + k * THERMO_LEN);
    }
    for (long i = 0; i < atoms.Size(); ++i)
      for (int q = 0; q < 3; ++q) {
        if (out_pos) out_pos[3 * i + q] = atoms[i].Position()[q];
        if (out_vel) out_vel[3 * i + q] = atoms[i].Velocity()[q];
        if (out_acc) out_acc[3 * i + q] = atoms[i].Acceleration()[q];
      }
    return 0;
  } catch (std::exception& e) {
    std::snprintf(g_error, sizeof g_error, "%s", e.what());
    return 1;
  }
}

// Writes nframes configurations of n atoms through the reference's own output plugin (`module`
// "lpmd" or "xyz", constructed with `args`, which name the file): CellWriter::WriteHeader once,
// then WriteCell per frame (the calls Application::OpenOutputStreams and
// SaveCurrentConfiguration make, lpmd/application.cc:537-578).  Frames are [nframes][n][3];
// vel/acc may be NULL (zeros).  Returns 0, or 1 with the message in ref_last_error().
extern "C" int ref_write_frames(int64_t n, const double* L, const int32_t* Z, int64_t nframes,
                                const double* pos, const double* vel, const double* acc,
                                const char* module, const char* args, const char* path) {
  g_error[0] = 0;
  try {
    static RuntimeContext context;
    Simulation& md = SimulationBuilder::CreateFixedOrthogonal(context, long(n), Atom("H"));
    BasicCell& cell = md.Cell();
    cell[0] = L[0] * e1;
    cell[1] = L[1] * e2;
    cell[2] = L[2] * e3;
    BasicParticleSet& atoms = md.Atoms();
    LPMDFormat* lp = nullptr;
    XYZFormat* xy = nullptr;
    CellWriter* w = nullptr;
    if (std::string(module) == "lpmd")
      w = lp = new LPMDFormat(args);
    else if (std::string(module) == "xyz")
      w = xy = new XYZFormat(args);
    else {
      std::snprintf(g_error, sizeof g_error, "unknown output module %s", module);
      return 1;
    }
    {
      std::ofstream os(path, std::ios::binary);
      w->WriteHeader(os, nullptr);
      for (int64_t f = 0; f < nframes; ++f) {
        const int64_t b = f * n * 3;
        for (long i = 0; i < atoms.Size(); ++i) {
          atoms[i].Z() = Z[i];
          atoms[i].Position() = Vector(pos[b + 3 * i], pos[b + 3 * i + 1], pos[b + 3 * i + 2]);
          atoms[i].Velocity() =
              vel ? Vector(vel[b + 3 * i], vel[b + 3 * i + 1], vel[b + 3 * i + 2]) : Vector(0.0, 0.0, 0.0);
          atoms[i].Acceleration() =
              acc ? Vector(acc[b + 3 * i], acc[b + 3 * i + 1], acc[b + 3 * i + 2]) : Vector(0.0, 0.0, 0.0);
        }
        w->WriteCell(os, md);
      }
    }
    delete lp;
    delete xy;
    return 0;
  } catch (std::exception& e) {
    std::snprintf(g_error, sizeof g_error, "%s", e.what());
    return 1;
  }
}

// Simulation::Dump (liblpmd/simulation/simulationbuilder.cc:195-238) of n atoms at step 0:
// Z, positions, velocities, accelerations; flags[i] & 1 tags the atom fixedvel, & 2 fixedpos.
extern "C" int ref_dump(int64_t n, const double* L, const int32_t* Z, const double* pos, const double* vel,
                        const double* acc, const uint8_t* flags, const char* path) {
  g_error[0] = 0;
  try {
    static RuntimeContext context;
    Simulation& md = SimulationBuilder::CreateFixedOrthogonal(context, long(n), Atom("H"));
    BasicCell& cell = md.Cell();
    cell[0] = L[0] * e1;
    cell[1] = L[1] * e2;
    cell[2] = L[2] * e3;
    BasicParticleSet& atoms = md.Atoms();
    for (long i = 0; i < atoms.Size(); ++i) {
      atoms[i].Z() = Z[i];
      atoms[i].Position() = Vector(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      atoms[i].Velocity() = Vector(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
      atoms[i].Acceleration() = Vector(acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]);
      if (flags && (flags[i] & 1)) atoms.SetTag(atoms[i], Tag("fixedvel"), "true");
      if (flags && (flags[i] & 2)) atoms.SetTag(atoms[i], Tag("fixedpos"), "true");
    }
    md.Dump(path);
    return 0;
  } catch (std::exception& e) {
    std::snprintf(g_error, sizeof g_error, "%s", e.what());
    return 1;
  }
}

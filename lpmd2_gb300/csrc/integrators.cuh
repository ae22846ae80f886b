// integrators.cuh -- the integrators other than velocityverlet, as per-atom kernels around a
// plain force evaluation (EPI_FORCES).  velocityverlet keeps its fused kick/drift epilogue in
// forces.cuh; these run at HBM speed on their own (a few doubles per atom per step).
//
// Reference correspondence (jperaltac/lpmd2):
//   OneStepIntegrator::Advance   liblpmd/simulation/onestepintegrator.cc:13-40 (force
//                                evaluation, fixedvel accelerations zeroed, Advance(i) for
//                                every atom without fixedpos)
//   TwoStepIntegrator::Advance   liblpmd/simulation/twostepintegrator.cc:12-68
//   Integrator::UseOldConfig / GoBack   liblpmd/simulation/integrator.cc:16-42
//   euler       plugins/euler.cc:37-43
//   leapfrog    plugins/leapfrog.cc:36-57
//   verlet      plugins/verlet.cc:35-55
//   beeman      plugins/beeman.cc:37-70
//   nosehoover  plugins/nosehoover.cc:43-83
// Every formula keeps the reference's operation order in FP64 (in both precisions: the
// mixed path differs only in its forces).
#pragma once

#include "forces.cuh"

namespace gbmd {

enum IntegKind { INT_VV = 0, INT_EULER = 1, INT_LEAPFROG = 2, INT_VERLET = 3, INT_BEEMAN = 4, INT_NOSEHOOVER = 5 };

__device__ __forceinline__ double& ist_at(const Dev& D, int slot, long long i) { return D.ist[slot * D.N + i]; }

// Writes the new position of atom i (FittedInside unless `keep`) into the output buffer and its
// gather copies; returns the squared displacement since the last list build.
__device__ __forceinline__ float commit_position(const Dev& D, const SysDev& S, long long i, double nx, double ny,
                                                 double nz, bool keep) {
  if (!keep) {
    nx = ref_fitted(nx, S.L[0]);
    ny = ref_fitted(ny, S.L[1]);
    nz = ref_fitted(nz, S.L[2]);
  }
  D.xo[i] = nx;
  D.yo[i] = ny;
  D.zo[i] = nz;
  float4 g = write_gather(D, S, i, nx, ny, nz, D.type[i], D.g64o, D.g32o);
  return S.mode == NB_LIST ? displacement2(D, i, g) : 0.0f;
}

__device__ __forceinline__ bool fixed_position(const Dev& D, long long i) {
  return D.has_flags && (D.flags[i] & FLAG_FIXEDPOS);
}

// One-step integrators, after the force evaluation at x(t) (accelerations a(t), fixedvel
// atoms' zeroed): new positions into the output buffer, velocities and history in place.
//   euler     x' = Fit(x + v dt), v' = v + a dt
//   leapfrog  vh = v_old + a dt, x' = Fit(x + vh dt), v' = 0.5 (vh + v_old), v_old = vh
//   verlet    x' = Fit((2 x - x_old) + a dt dt), v' = Displacement(x_old, x') / (2 dt), x_old = x
template <int KIND>
__global__ void __launch_bounds__(TILE) k_onestep(Dev D, double dt) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) {
    hold_tile(D, S, tile, false);
    return;
  }
  const long long i = D.tile_first[tile] + threadIdx.x;
  float d2 = 0.0f;
  if ((int)threadIdx.x < D.tile_count[tile]) {
    const double x = D.x[i], y = D.y[i], z = D.z[i];
    if (fixed_position(D, i)) {
      d2 = commit_position(D, S, i, x, y, z, true);
    } else {
      const double vx = D.vx[i], vy = D.vy[i], vz = D.vz[i];
      const double ax = D.ax[i], ay = D.ay[i], az = D.az[i];
      if (KIND == INT_EULER) {
        d2 = commit_position(D, S, i, dadd(x, dmul(vx, dt)), dadd(y, dmul(vy, dt)), dadd(z, dmul(vz, dt)), false);
        D.vx[i] = dadd(vx, dmul(ax, dt));
        D.vy[i] = dadd(vy, dmul(ay, dt));
        D.vz[i] = dadd(vz, dmul(az, dt));
      } else if (KIND == INT_LEAPFROG) {
        const double ox = ist_at(D, IS_OLD, i), oy = ist_at(D, IS_OLD + 1, i), oz = ist_at(D, IS_OLD + 2, i);
        const double hx = dadd(ox, dmul(ax, dt)), hy = dadd(oy, dmul(ay, dt)), hz = dadd(oz, dmul(az, dt));
        d2 = commit_position(D, S, i, dadd(x, dmul(hx, dt)), dadd(y, dmul(hy, dt)), dadd(z, dmul(hz, dt)), false);
        D.vx[i] = dmul(0.5, dadd(hx, ox));
        D.vy[i] = dmul(0.5, dadd(hy, oy));
        D.vz[i] = dmul(0.5, dadd(hz, oz));
        ist_at(D, IS_OLD, i) = hx;
        ist_at(D, IS_OLD + 1, i) = hy;
        ist_at(D, IS_OLD + 2, i) = hz;
      } else {  // INT_VERLET
        const double px = ist_at(D, IS_OLD, i), py = ist_at(D, IS_OLD + 1, i), pz = ist_at(D, IS_OLD + 2, i);
        const double nx = ref_fitted(dadd(dsub(dmul(2.0, x), px), dmul(dmul(ax, dt), dt)), S.L[0]);
        const double ny = ref_fitted(dadd(dsub(dmul(2.0, y), py), dmul(dmul(ay, dt), dt)), S.L[1]);
        const double nz = ref_fitted(dadd(dsub(dmul(2.0, z), pz), dmul(dmul(az, dt), dt)), S.L[2]);
        ist_at(D, IS_OLD, i) = x;
        ist_at(D, IS_OLD + 1, i) = y;
        ist_at(D, IS_OLD + 2, i) = z;
        d2 = commit_position(D, S, i, nx, ny, nz, true);
        const double two_dt = dmul(2.0, dt);
        D.vx[i] = ddiv(ref_wrap(dsub(nx, px), S.L[0], S.Lh[0]), two_dt);
        D.vy[i] = ddiv(ref_wrap(dsub(ny, py), S.L[1], S.Lh[1]), two_dt);
        D.vz[i] = ddiv(ref_wrap(dsub(nz, pz), S.L[2], S.Lh[2]), two_dt);
      }
    }
  }
  track_displacement_warp(D, s, d2);
}

// Beeman / Nose-Hoover AdvancePosition with a(t) from the last evaluation:
//   beeman      aux = a_old, x' = Fit(((x + v dt) + (2/3) a dt dt) - (1/6) a_old dt dt), a_old = a
//   nosehoover  the same with a replaced by a - v f_i, where the friction f_i grows by
//               (3N/Q) k_B (T - T0) dt for every moving atom up to and including atom i (in the
//               reference's atom order; f_i = f_before + rank_i * increment here)
template <int KIND>
__global__ void __launch_bounds__(TILE) k_twostep_position(Dev D, double dt) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) {
    hold_tile(D, S, tile, false);
    return;
  }
  const long long i = D.tile_first[tile] + threadIdx.x;
  float d2 = 0.0f;
  if ((int)threadIdx.x < D.tile_count[tile]) {
    const double x = D.x[i], y = D.y[i], z = D.z[i];
    if (fixed_position(D, i)) {
      d2 = commit_position(D, S, i, x, y, z, true);
    } else {
      const double vx = D.vx[i], vy = D.vy[i], vz = D.vz[i];
      double ax = D.ax[i], ay = D.ay[i], az = D.az[i];
      if (KIND == INT_NOSEHOOVER) {
        const double* nh = D.nh + (long long)s * NH_LEN;
        const double f = dadd(nh[NH_F0], dmul(ist_at(D, IS_RANK, i), nh[NH_D]));
        ax = dsub(ax, dmul(vx, f));
        ay = dsub(ay, dmul(vy, f));
        az = dsub(az, dmul(vz, f));
      }
      const double ox = ist_at(D, IS_OLD, i), oy = ist_at(D, IS_OLD + 1, i), oz = ist_at(D, IS_OLD + 2, i);
      const double c23 = 2.0 / 3.0, c16 = 1.0 / 6.0;
      const double nx = dsub(dadd(dadd(x, dmul(vx, dt)), dmul(dmul(dmul(ax, c23), dt), dt)), dmul(dmul(dmul(ox, c16), dt), dt));
      const double ny = dsub(dadd(dadd(y, dmul(vy, dt)), dmul(dmul(dmul(ay, c23), dt), dt)), dmul(dmul(dmul(oy, c16), dt), dt));
      const double nz = dsub(dadd(dadd(z, dmul(vz, dt)), dmul(dmul(dmul(az, c23), dt), dt)), dmul(dmul(dmul(oz, c16), dt), dt));
      ist_at(D, IS_AUX, i) = ox;
      ist_at(D, IS_AUX + 1, i) = oy;
      ist_at(D, IS_AUX + 2, i) = oz;
      ist_at(D, IS_OLD, i) = ax;
      ist_at(D, IS_OLD + 1, i) = ay;
      ist_at(D, IS_OLD + 2, i) = az;
      d2 = commit_position(D, S, i, nx, ny, nz, false);
    }
  }
  track_displacement_warp(D, s, d2);
}

// Beeman / Nose-Hoover AdvanceVelocity after the evaluation at x' (a' = accelerations there):
// v' = ((v + (1/3) a' dt) + (5/6) a_old dt) - (1/6) aux dt.
__global__ void __launch_bounds__(TILE) k_twostep_velocity(Dev D, double dt) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  if (!D.sysd[s].active) return;
  const long long i = D.tile_first[tile] + threadIdx.x;
  if ((int)threadIdx.x >= D.tile_count[tile] || fixed_position(D, i)) return;
  const double c13 = 1.0 / 3.0, c56 = 5.0 / 6.0, c16 = 1.0 / 6.0;
  double* v[3] = {D.vx, D.vy, D.vz};
  const double* a[3] = {D.ax, D.ay, D.az};
  for (int q = 0; q < 3; ++q) {
    const double o = ist_at(D, IS_OLD + q, i), u = ist_at(D, IS_AUX + q, i);
    v[q][i] = dsub(dadd(dadd(v[q][i], dmul(dmul(a[q][i], c13), dt)), dmul(dmul(o, c56), dt)), dmul(dmul(u, c16), dt));
  }
}

// Nose-Hoover friction increment of this step from the kinetic energy of all atoms (int64 sum
// in the system's kinetic slot, filled by k_scale_kinetic with mode 1): lpmd::Temperature with
// tag false (liblpmd/lpmd/properties.h:40-53), then (((3 N) / Q) k_B (T - T0)) dt per moving atom
// with the session's k_B, which the reference stores as text with 8 decimals
// (liblpmd/runtime/session.cc:17-32): 0.00008617.
__global__ void k_nh_friction(Dev D, double dt, double q, double t0) {
  for (int s = threadIdx.x; s < D.nsys; s += blockDim.x) {
    const SysDev& S = D.sysd[s];
    if (!S.active) continue;
    const double KIN2EV = 103.64269, KBOLTZMANN = 8.6173422E-05;  // liblpmd/lpmd/properties.h:10-11
    const double ke = (double)(long long)__ldcg(D.sys_acc + (long long)s * SA_LEN + SA_KE) * (1.0 / FIX_KE);
    const double T = S.natoms == 0 ? 0.0 : ddiv(dmul(2.0 / 3.0, dmul(ke, KIN2EV)), dmul(KBOLTZMANN, (double)S.natoms));
    double* nh = D.nh + (long long)s * NH_LEN;
    const double KB_SESSION = 0.00008617;
    const double inc = dmul(dmul(dmul(ddiv(dmul(3.0, (double)S.natoms), q), KB_SESSION), dsub(T, t0)), dt);
    nh[NH_F0] = nh[NH_F];
    nh[NH_D] = inc;
    nh[NH_F] = dadd(nh[NH_F], dmul(nh[NH_NMOVE], inc));
  }
}

// Initialize, part 1 (UseOldConfig -> GoBack on the backed-up configuration): puts the
// current positions and accelerations aside and writes the backed-up positions
// Fit(x - v dt) into the current buffer (a force evaluation there follows, with a re-sort);
// leapfrog keeps v - a dt as its old velocity, verlet the backed-up position as its old one
// (verlet evaluates no forces there, so its current positions stay).
template <int KIND>
__global__ void k_init_backup(Dev D, double dt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  const SysDev& S = D.sysd[D.sysid[i]];
  if (!S.active) return;
  double* p[3] = {D.x, D.y, D.z};
  const double* v[3] = {D.vx, D.vy, D.vz};
  const double* a[3] = {D.ax, D.ay, D.az};
  for (int q = 0; q < 3; ++q) {
    const double back = ref_fitted(dsub(p[q][i], dmul(v[q][i], dt)), S.L[q]);
    if (KIND == INT_VERLET) {
      ist_at(D, IS_OLD + q, i) = back;
      continue;
    }
    ist_at(D, IS_SAVEX + q, i) = p[q][i];
    ist_at(D, IS_SAVEA + q, i) = a[q][i];
    if (KIND == INT_LEAPFROG) ist_at(D, IS_OLD + q, i) = dsub(v[q][i], dmul(a[q][i], dt));
    p[q][i] = back;
  }
}

// Initialize, part 2, after the force evaluation at the backed-up positions (accelerations a_b,
// fixedvel atoms' not zeroed, as a bare UpdateForces leaves them): leapfrog v_old += a_b 0.5 dt;
// beeman / nosehoover a_old = a_b, aux = 0.  Then the current positions and accelerations come
// back (the caller forces a re-sort before the next evaluation).
template <int KIND>
__global__ void k_init_restore(Dev D, double dt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  const SysDev& S = D.sysd[D.sysid[i]];
  if (!S.active) return;
  double* p[3] = {D.x, D.y, D.z};
  double* a[3] = {D.ax, D.ay, D.az};
  for (int q = 0; q < 3; ++q) {
    if (KIND == INT_LEAPFROG) {
      ist_at(D, IS_OLD + q, i) = dadd(ist_at(D, IS_OLD + q, i), dmul(dmul(a[q][i], 0.5), dt));
    } else {
      ist_at(D, IS_OLD + q, i) = a[q][i];
      ist_at(D, IS_AUX + q, i) = 0.0;
    }
    p[q][i] = ist_at(D, IS_SAVEX + q, i);
    a[q][i] = ist_at(D, IS_SAVEA + q, i);
  }
  refresh_gather(D, S, i, true);
}

// Kinetic sums of the velocities after an integrator step, as the last force pass of a
// velocity-Verlet step makes them (finish_atom with kinetic sums and the same reductions):
// FP64 tile sums for k_thermo (MIXED 0) or the int64 system accumulators for k_tail (MIXED 1,
// KE and momentum slots cleared by k_kinetic_slots_clear first).
__global__ void k_kinetic_slots_clear(Dev D) {
  for (int s = threadIdx.x; s < D.nsys; s += blockDim.x) {
    if (!D.sysd[s].active) continue;
    unsigned long long* acc = D.sys_acc + (long long)s * SA_LEN;
    acc[SA_KE] = 0ull;
    for (int k = 0; k < 3; ++k) acc[SA_P + k] = 0ull;
  }
}

template <int MIXED>
__global__ void __launch_bounds__(TILE) k_step_kinetic(Dev D) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  if (!D.sysd[s].active) return;
  const long long i = D.tile_first[tile] + threadIdx.x;
  double ke = 0.0, px = 0.0, py = 0.0, pz = 0.0;
  if ((int)threadIdx.x < D.tile_count[tile]) {
    const unsigned char fl = D.has_flags ? D.flags[i] : 0;
    if (!(fl & (FLAG_FIXEDVEL | FLAG_FIXEDPOS))) {
      const double m = D.mass[i], vx = D.vx[i], vy = D.vy[i], vz = D.vz[i];
      ke = MIXED ? (0.5 * m) * fma(vx, vx, fma(vy, vy, vz * vz)) : dmul(dmul(0.5, m), ref_sq(vx, vy, vz));
      px = dmul(vx, m);
      py = dmul(vy, m);
      pz = dmul(vz, m);
    }
  }
  if (MIXED) {
    const double kw = warp_sum(ke);
    long long k4[4] = {(threadIdx.x & 31) == 0 ? __double2ll_rn(kw * FIX_KE) : 0ll, __double2ll_rn(px * FIX_KE),
                       __double2ll_rn(py * FIX_KE), __double2ll_rn(pz * FIX_KE)};
    long long kt[4];
    block_sum<long long, 4>(k4, kt);
    if (threadIdx.x == 0) {
      unsigned long long* acc = D.sys_acc + (long long)s * SA_LEN;
      atomicAdd(acc + SA_KE, (unsigned long long)kt[0]);
      for (int k = 0; k < 3; ++k) atomicAdd(acc + SA_P + k, (unsigned long long)kt[1 + k]);
    }
  } else {
    double k4[4] = {ke, px, py, pz};
    double kt[4];
    block_sum<double, 4>(k4, kt);
    if (threadIdx.x == 0) {
      double* t = D.tile_d + (long long)tile * PART_D;
      t[PD_KE] = kt[0];
      for (int k = 0; k < 3; ++k) t[PD_PX + k] = kt[1 + k];
    }
  }
}

// Marks every active system for a re-sort at the next rebuild decision.
__global__ void k_force_rebuild(Dev D) {
  for (int s = threadIdx.x; s < D.nsys; s += blockDim.x)
    if (D.sysd[s].active) D.sst[s].force_rebuild = 1;
}

// Scatters the Nose-Hoover ranks (by original atom index) into the history slot.
__global__ void k_set_rank(Dev D, const double* rank_by_tag) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  ist_at(D, IS_RANK, i) = rank_by_tag[D.sysd[D.sysid[i]].atom_base + D.tag[i]];
}

}  // namespace gbmd

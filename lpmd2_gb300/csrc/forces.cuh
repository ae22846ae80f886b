// forces.cuh -- force, density and thermo kernels (one thread per atom, one block per tile of
// 128 atoms of one system; every atom gathers over its full neighbour list, so no atomics and
// every sum has a fixed order).
#pragma once

#include "kernels.cuh"

namespace gbmd {

enum PotClass { PC_PAIR = 0, PC_EAM = 1 };


// Visits the candidate neighbours j of atom i under neighbour mode NB (compile-time).
template <int NB, class F>
__device__ __forceinline__ void for_each_candidate(const Dev& D, const SysDev& S, long long i, F&& f) {
  if (NB == NB_LIST) {
    const int na = S.natoms;
    const uint4* L = list_group(D, S, (int)(i - S.atom_base), 0);
    const int cnt = D.ncount[i];
    for (int k = 0; k < cnt; k += 4) {
      const uint4 e4 = __ldg(L);
      L += na;
      const unsigned e[4] = {e4.x, e4.y, e4.z, e4.w};
      for (int u = 0; u < 4 && k + u < cnt; ++u) f(S.atom_base + (long long)(e[u] & LOCAL_MASK), e[u] >> CODE_SHIFT);
    }
  } else if (NB == NB_CELLS) {
    // The reference stencil of LinkedCell (plugins/linkedcell.cc:221-240), duplicates included.
    const int h = D.home[i] - S.cell_base;
    const int cx = h % S.n[0], cy = (h / S.n[0]) % S.n[1], cz = h / (S.n[0] * S.n[1]);
    const int sd = S.lc_side;
    for (int dz = -sd; dz <= sd; ++dz) {
      int zc = wrap_around(cz + dz, S.n[2]);
      for (int dy = -sd; dy <= sd; ++dy) {
        int yc = wrap_around(cy + dy, S.n[1]);
        for (int dx = -sd; dx <= sd; ++dx) {
          int xc = wrap_around(cx + dx, S.n[0]);
          int g = S.cell_base + (zc * S.n[1] + yc) * S.n[0] + xc;
          int b = D.cstart[g], e = b + D.ccnt[g];
          for (int j = b; j < e; ++j)
            if (j != i) f((long long)j, 0u);
        }
      }
    }
  } else {
    for (long long j = S.atom_base; j < S.atom_base + S.natoms; ++j)
      if (j != i) f(j, 0u);
  }
}

// Exact FP64 reference cutoff test of pair (i, j) from the master positions.
__device__ __forceinline__ bool exact_inside(const Dev& D, const SysDev& S, long long i, long long j, double rc2) {
  double dx = ref_wrap(dsub(D.x[j], D.x[i]), S.L[0], S.Lh[0]);
  double dy = ref_wrap(dsub(D.y[j], D.y[i]), S.L[1], S.Lh[1]);
  double dz = ref_wrap(dsub(D.z[j], D.z[i]), S.L[2], S.Lh[2]);
  return ref_sq(dx, dy, dz) < rc2;
}

// Out-of-line copy for the hot loops: the guard-band recheck is rare (a few pairs per thousand
// atoms), and keeping its FP64 code out of the loop body keeps the body small.
__device__ __noinline__ bool exact_inside_cold(const Dev* D, const SysDev* S, long long i, long long j, double rc2) {
  return exact_inside(*D, *S, i, j, rc2);
}

// Loads the cell-shift table (k * cell edge, k in -2..2 per axis) of system S into shared memory.
__device__ __forceinline__ void load_shifts(const SysDev& S, float4* sh) {
  for (int c = threadIdx.x; c < 125; c += blockDim.x) {
    int kx = c % 5 - 2, ky = (c / 5) % 5 - 2, kz = c / 25 - 2;
    sh[c] = make_float4((float)kx * S.df[0], (float)ky * S.df[1], (float)kz * S.df[2], 0.0f);
  }
  __syncthreads();
}

// The cell-shift table of the mixed force and density passes: the block's own copy in shared
// memory, or (GBMD_SHIFTS_GLOBAL) the system's copy in global memory, read through L1 and
// leaving the shared-memory carve-out to L1 (the host writes the same values, D.shift_tab).
#ifndef GBMD_SHIFTS_GLOBAL
#define GBMD_SHIFTS_GLOBAL 0
#endif
#if GBMD_SHIFTS_GLOBAL
#define SHIFT_TABLE(name) const float4* __restrict__ name = D.shift_tab + (long long)s * 128
#else
#define SHIFT_TABLE(name)   \
  __shared__ float4 name[125]; \
  load_shifts(S, name)
#endif

// Epilogue shared by the force kernels: turns the total force on atom i into its acceleration
// (a = F * forcefactor/m, liblpmd/simulation/pairpotential.cc:62), applies fixedvel, and unless
// EPI_FORCES advances the velocity: v = v + (0.5*dt) * (a_old + a) (plugins/velocityverlet.cc:73-74).
// EPI_KICK_DRIFT then also advances the position for the next step (AdvancePosition) into the
// output position buffer.  Returns the kinetic terms of the updated velocity and the squared
// displacement since the last list build.
template <int MIXED>
__device__ __forceinline__ float finish_atom(const Dev& D, const SysDev& S, long long i, double Fx, double Fy,
                                             double Fz, const StepParams& sp, double& ke, double& px, double& py,
                                             double& pz) {
  // mixed: F arrives in 2^-32 eV/A units; scaling fm by the power of two is exact and gives
  // the same products as scaling F
  const double fm = MIXED ? D.fm[i] * (1.0 / FIX_F) : D.fm[i];
  double ax = dmul(Fx, fm), ay = dmul(Fy, fm), az = dmul(Fz, fm);
  unsigned char fl = D.has_flags ? D.flags[i] : 0;
  if ((fl & FLAG_FIXEDVEL) && !sp.raw_acc) ax = ay = az = 0.0;
  double vx = D.vx[i], vy = D.vy[i], vz = D.vz[i];
  if (sp.epi != EPI_FORCES && !(fl & FLAG_FIXEDPOS)) {
    if (MIXED) {
      vx = fma(sp.half_dt, D.ax[i] + ax, vx);
      vy = fma(sp.half_dt, D.ay[i] + ay, vy);
      vz = fma(sp.half_dt, D.az[i] + az, vz);
    } else {
      vx = dadd(vx, dmul(sp.half_dt, dadd(D.ax[i], ax)));
      vy = dadd(vy, dmul(sp.half_dt, dadd(D.ay[i], ay)));
      vz = dadd(vz, dmul(sp.half_dt, dadd(D.az[i], az)));
    }
    D.vx[i] = vx;
    D.vy[i] = vy;
    D.vz[i] = vz;
  }
  D.ax[i] = ax;
  D.ay[i] = ay;
  D.az[i] = az;
  ke = 0.0;
  px = py = pz = 0.0;
  // KineticEnergy/Momentum skip tagged atoms (liblpmd/lpmd/properties.h:22-37,64-81)
  if (sp.kinetic && !(fl & (FLAG_FIXEDVEL | FLAG_FIXEDPOS))) {
    const double m = D.mass[i];
    ke = MIXED ? (0.5 * m) * fma(vx, vx, fma(vy, vy, vz * vz)) : dmul(dmul(0.5, m), ref_sq(vx, vy, vz));
    px = dmul(vx, m);
    py = dmul(vy, m);
    pz = dmul(vz, m);
  }
  if (sp.epi == EPI_KICK_DRIFT) return drift_atom<MIXED>(D, S, i, sp.dt, sp.half_dt2, vx, vy, vz, ax, ay, az);
  return 0.0f;
}

// Kinetic energy and momentum of the calling warp's atoms as int64 fixed point (2^-44 units):
// FP64 warp sums in a fixed shuffle order, rounded once, on lane 0 (zeros elsewhere).  A warp
// never spans two systems (tiles start at a system's first atom), so the sums are the same in a
// batch and alone.
__device__ __forceinline__ void warp_kinetic_fix(double ke, double px, double py, double pz, long long (&k4)[4]) {
  const double s[4] = {warp_sum(ke), warp_sum(px), warp_sum(py), warp_sum(pz)};
  const bool lead = (threadIdx.x & 31) == 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) k4[k] = lead ? __double2ll_rn(s[k] * FIX_KE) : 0ll;
}

// Writes the tile's FP64 partials (slots [lo, hi) of the 16) with overwrite or accumulate.
__device__ __forceinline__ void store_tile_d(const Dev& D, int tile, const double* v, int lo, int hi, bool first) {
  double* t = D.tile_d + (long long)tile * PART_D;
  for (int k = lo; k < hi; ++k) t[k] = first ? v[k] : t[k] + v[k];
}

// ------------------------------------------------------------------------------------------
// FP64 force pass: pair (LJ) or EAM force.
// ------------------------------------------------------------------------------------------

template <int NB, int PC>
__global__ void __launch_bounds__(TILE) k_force64(Dev D, PotParams P, StepParams sp) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) {  // whole block: one tile belongs to one system
    if (sp.epi == EPI_KICK_DRIFT && sp.last) hold_tile(D, S, tile, true);
    return;
  }
  const long long i = D.tile_first[tile] + threadIdx.x;
  const bool active = (int)threadIdx.x < D.tile_count[tile];
  double fx = 0.0, fy = 0.0, fz = 0.0, ep = 0.0, vir = 0.0;
  double sxx = 0.0, sxy = 0.0, sxz = 0.0, syy = 0.0, syz = 0.0, szz = 0.0;
  if (active) {
    const double4_32a pi = D.g64[i];
    const int ti = (int)pi.w;
    const double phi_i = (PC == PC_EAM) ? D.phi[i] : 0.0;
    for_each_candidate<NB>(D, S, i, [&](long long j, unsigned) {
      const double4_32a pj = D.g64[j];
      double dx = ref_wrap(dsub(pj.x, pi.x), S.L[0], S.Lh[0]);
      double dy = ref_wrap(dsub(pj.y, pi.y), S.L[1], S.Lh[1]);
      double dz = ref_wrap(dsub(pj.z, pi.z), S.L[2], S.Lh[2]);
      double r2 = ref_sq(dx, dy, dz);
      if (r2 < P.rc2 && applies_to(P.spc_sum, ti, (int)pj.w)) {
        double g, e;
        if (PC == PC_PAIR) {
          if (P.kind == POT_FASTLJ)
            fastlj_pair64(P, r2, g, e);
          else
            lj_pair64(P, r2, g, e);
        } else {
          double r = sqrt(r2);
          double sc;
          eam_pair64(P, r, phi_i, D.phi[j], sc, e);
          g = ddiv(sc, r);
        }
        fx += g * dx;
        fy += g * dy;
        fz += g * dz;
        ep += e;
        vir -= g * r2;
        sxx -= g * dx * dx;
        sxy -= g * dx * dy;
        sxz -= g * dx * dz;
        syy -= g * dy * dy;
        syz -= g * dy * dz;
        szz -= g * dz * dz;
      }
    });
  }
  double ke = 0.0, px = 0.0, py = 0.0, pz = 0.0;
  float d2 = 0.0f;
  if (active) {
    long long N = D.N;
    if (!sp.first) {
      fx += D.dacc[i];
      fy += D.dacc[N + i];
      fz += D.dacc[2 * N + i];
    }
    if (sp.last) {
      d2 = finish_atom<0>(D, S, i, fx, fy, fz, sp, ke, px, py, pz);
    } else {
      D.dacc[i] = fx;
      D.dacc[N + i] = fy;
      D.dacc[2 * N + i] = fz;
    }
  }
  track_displacement_warp(D, s, d2);
  // the full list counts each pair twice: halve energy, virial and stress
  double v[13] = {0.5 * ep, 0.5 * vir, 0.5 * sxx, 0.5 * sxy, 0.5 * sxz, 0.5 * sxy, 0.5 * syy,
                  0.5 * syz, 0.5 * sxz, 0.5 * syz, 0.5 * szz, ke, 0.0};
  double tot[13];
  block_sum<double, 13>(v, tot);
  if (threadIdx.x == 0) {
    double out[PART_D] = {0};
    out[PD_EPAIR] = tot[0];
    out[PD_VIR] = tot[1];
    for (int k = 0; k < 9; ++k) out[PD_STRESS + k] = tot[2 + k];
    store_tile_d(D, tile, out, PD_EPAIR, PD_EPAIR + 1, sp.first);
    store_tile_d(D, tile, out, PD_VIR, PD_STRESS + 9, sp.first);
  }
  if (sp.last) {
    double k4[4] = {ke, px, py, pz};
    double kt[4];
    block_sum<double, 4>(k4, kt);
    if (threadIdx.x == 0) {
      double* t = D.tile_d + (long long)tile * PART_D;
      t[PD_KE] = kt[0];
      t[PD_PX] = kt[1];
      t[PD_PX + 1] = kt[2];
      t[PD_PX + 2] = kt[3];
    }
  }
}

// ------------------------------------------------------------------------------------------
// Mixed force pass: FP32 pair maths, int64 fixed-point force sums, FP64 cutoff test inside a
// guard band around rc^2 so the set of interacting pairs is the FP64 reference's.
// ------------------------------------------------------------------------------------------

// Thermo record of system s (one thread): SetSimulationTags' quantities from the FP64 tile
// sums `tot` (FP64 path) or, with tot == nullptr, from the system's int64 accumulators.
__device__ __forceinline__ void thermo_record(const Dev& D, int s, const double* tot_in, int count_step) {
  const SysDev& S = D.sysd[s];
  SysState& st = D.sst[s];
  double tot[PART_D];
  for (int k = 0; k < PART_D; ++k) tot[k] = tot_in ? tot_in[k] : 0.0;
  double epair = tot[PD_EPAIR], vir = tot[PD_VIR];
  double stress[9];
  for (int k = 0; k < 9; ++k) stress[k] = tot[PD_STRESS + k];
  if (!tot_in) {
    const long long* acc = (const long long*)D.sys_acc + (long long)s * SA_LEN;
    const double inv = 1.0 / FIX_E, invk = 1.0 / FIX_KE;
    epair = (double)__ldcg(acc + SA_EPAIR) * inv;
    vir = (double)__ldcg(acc + SA_VIR) * inv;
    for (int k = 0; k < 9; ++k) stress[k] = (double)__ldcg(acc + SA_STRESS + k) * inv;
    tot[PD_EEMBED] = (double)__ldcg(acc + SA_EEMBED) * inv;
    tot[PD_KE] = (double)__ldcg(acc + SA_KE) * invk;
    for (int k = 0; k < 3; ++k) tot[PD_PX + k] = (double)__ldcg(acc + SA_P + k) * invk;
  }
  if (count_step) st.step += 1;
  const double KIN2EV = 103.64269;  // liblpmd/lpmd/properties.h:10
  double epot = epair + tot[PD_EEMBED];
  double kin = dmul(tot[PD_KE], KIN2EV);
  double temp = (S.natoms == 0) ? 0.0 : ddiv(dmul(2.0 / 3.0, kin), S.kbn);
  const double vol = S.vol, pv = S.pv;  // volume and pressfactor/volume, computed on the host
  double r[THERMO_LEN];
  r[0] = (double)st.step;
  r[1] = epot;
  r[2] = kin;
  r[3] = epot + kin;
  r[4] = temp;
  r[5] = vir;
  r[6] = tot[PD_PX];
  r[7] = tot[PD_PX + 1];
  r[8] = tot[PD_PX + 2];
  r[9] = vol;
  r[10] = dmul(dmul(pv, 1.0 / 3.0), vir);
  r[11] = dmul(dmul(pv, 2.0 / 3.0), kin);
  r[12] = dmul(pv, dadd(dmul(2.0 / 3.0, kin), dmul(1.0 / 3.0, vir)));
  for (int k = 0; k < 9; ++k) r[13 + k] = stress[k];
  double* last = D.thermo_last + (long long)s * THERMO_LEN;
  double* log = D.thermo_log + ((long long)s * D.log_cap + (st.step % D.log_cap)) * THERMO_LEN;
  for (int k = 0; k < THERMO_LEN; ++k) {
    last[k] = r[k];
    if (count_step) log[k] = r[k];
  }
}

// Tail of a mixed force evaluation, one thread per system: the thermo records from the int64
// accumulators and, inside a step sequence, the next step's rebuild decision and graph
// conditional -- one launch instead of a k_thermo and a k_decide.  The conditional starts every
// graph launch at 0 (cudaGraphCondAssignDefault), so a block raises it only when one of its
// systems rebuilds and no block ever lowers it.
constexpr int TAIL_THREADS = 128;
__global__ void __launch_bounds__(TAIL_THREADS) k_tail(Dev D, int count_step, int decide_next,
                                                       unsigned long long cond_next) {
  const int s = blockIdx.x * TAIL_THREADS + threadIdx.x;
  int need = 0;
  if (s < D.nsys) {
    if (D.sysd[s].active) thermo_record(D, s, nullptr, count_step);
    if (decide_next) need = decide_system(D, s, 2, 0);
  }
  if (__syncthreads_or(need) && threadIdx.x == 0 && cond_next)
    cudaGraphSetConditional((cudaGraphConditionalHandle)cond_next, 1u);
}

// Resident blocks per SM the register allocation of the mixed force kernel is sized for.
#ifndef GBMD_FORCE_MIN_BLOCKS
#define GBMD_FORCE_MIN_BLOCKS 8
#endif
// Packed displacement arithmetic in the EAM force pass as well (the pair force pass always
// uses it when GBMD_F32X2 is on).
#ifndef GBMD_F32X2_EAM_FORCE
#define GBMD_F32X2_EAM_FORCE 1
#endif
// Pair functions of two list entries at a time in packed pairs (LJ; folded Sutton-Chen).
#ifndef GBMD_F32X2_PAIRMATH_LJ
#define GBMD_F32X2_PAIRMATH_LJ 1
#endif
#ifndef GBMD_F32X2_PAIRMATH_EAM
#define GBMD_F32X2_PAIRMATH_EAM 1
#endif

// The same for the mixed EAM density pass (0: no minimum, the compiler's own choice).
#ifndef GBMD_DENSITY_MIN_BLOCKS
#define GBMD_DENSITY_MIN_BLOCKS 0
#endif
#if GBMD_DENSITY_MIN_BLOCKS > 0
#define GBMD_DENSITY_BOUNDS __launch_bounds__(TILE, GBMD_DENSITY_MIN_BLOCKS)
#else
#define GBMD_DENSITY_BOUNDS __launch_bounds__(TILE)
#endif

// List groups per ring iteration of the pair and the EAM force passes (1 or 2).
#ifndef GBMD_EAM_RING_GROUPS
#define GBMD_EAM_RING_GROUPS 2
#endif
#ifndef GBMD_PAIR_RING_GROUPS
#define GBMD_PAIR_RING_GROUPS 2
#endif

// After a bounded wait gave up at group q no further copies are issued; lane 0 then waits (again
// bounded) for the copies already in flight -- groups q .. q+RING-1 below ngw, one per stage --
// so the warp never leaves while the copy engine still writes into its stages.
__device__ __forceinline__ void ring_drain(unsigned long long* bar, int q, int ngw) {
  if ((threadIdx.x & 31) == 0)
    for (int g = q; g < q + RING && g < ngw; ++g) mbar_wait_bounded(&bar[g & (RING - 1)], (unsigned)((g / RING) & 1));
  __syncwarp();
}

// Streams the list groups of the calling warp's 32 atoms (32 x 16 bytes, contiguous for a
// fixed group index) through the warp's RING-stage shared-memory ring with bulk asynchronous
// copies, calling body(group q, this lane's uint4 of that group) for q < ngw, the warp's
// largest group count.  Lane 0 issues the copies; every wait is bounded.  Returns false if a
// wait gave up: the warp then stops (uniformly), drains its copies in flight and skips the
// remaining groups.
template <class F>
__device__ __forceinline__ bool warp_list_ring(const Dev& D, const SysDev& S, int wfirst, int wcount, int ngw,
                                               uint4 (*ring)[32], unsigned long long* bar, F&& body) {
  const int lane = threadIdx.x & 31;
  const uint4* src0 = list_group(D, S, wfirst, 0);
  const unsigned bytes = (unsigned)wcount * 16u;
  const int na = S.natoms;
  if (lane == 0 && ngw > 0) {
    for (int r = 0; r < RING; ++r) mbar_init(&bar[r], 1);
    mbar_init_fence();
    for (int r = 0; r < RING && r < ngw; ++r) {
      mbar_expect_tx(&bar[r], bytes);
      bulk_g2s(ring[r], src0 + (long long)r * na, bytes, &bar[r]);
    }
  }
  __syncwarp();
  for (int q = 0; q < ngw; ++q) {
    const int r = q & (RING - 1);
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(&bar[r], (unsigned)((q / RING) & 1)))) {
      ring_drain(bar, q, ngw);
      return false;
    }
    const uint4 cur = ring[r][lane];
    __syncwarp();  // every lane has its entry: the stage can be refilled
    if (lane == 0 && q + RING < ngw) {
      fence_proxy_async_shared();
      mbar_expect_tx(&bar[r], bytes);
      bulk_g2s(ring[r], src0 + (long long)(q + RING) * na, bytes, &bar[r]);
    }
    body(q, cur);
  }
  return true;
}

// As warp_list_ring, two groups per iteration: both stages are read before either body runs,
// so the two groups' neighbour gathers can be in flight together (for latency-bound bodies).
template <class F>
__device__ __forceinline__ bool warp_list_ring2(const Dev& D, const SysDev& S, int wfirst, int wcount, int ngw,
                                                uint4 (*ring)[32], unsigned long long* bar, F&& body) {
  const int lane = threadIdx.x & 31;
  const uint4* src0 = list_group(D, S, wfirst, 0);
  const unsigned bytes = (unsigned)wcount * 16u;
  const int na = S.natoms;
  if (lane == 0 && ngw > 0) {
    for (int r = 0; r < RING; ++r) mbar_init(&bar[r], 1);
    mbar_init_fence();
    for (int r = 0; r < RING && r < ngw; ++r) {
      mbar_expect_tx(&bar[r], bytes);
      bulk_g2s(ring[r], src0 + (long long)r * na, bytes, &bar[r]);
    }
  }
  __syncwarp();
  for (int q = 0; q < ngw; q += 2) {
    const bool two = q + 1 < ngw;
    const int r0 = q & (RING - 1), r1 = (q + 1) & (RING - 1);
    bool ok = mbar_wait_bounded(&bar[r0], (unsigned)((q / RING) & 1));
    if (two && ok) ok = mbar_wait_bounded(&bar[r1], (unsigned)(((q + 1) / RING) & 1));
    if (!__all_sync(0xffffffffu, ok)) {
      ring_drain(bar, q, ngw);
      return false;
    }
    const uint4 c0 = ring[r0][lane];
    const uint4 c1 = two ? ring[r1][lane] : make_uint4(0u, 0u, 0u, 0u);
    __syncwarp();  // every lane has its entries: the stages can be refilled
    if (lane == 0) {
      fence_proxy_async_shared();
      if (q + RING < ngw) {
        mbar_expect_tx(&bar[r0], bytes);
        bulk_g2s(ring[r0], src0 + (long long)(q + RING) * na, bytes, &bar[r0]);
      }
      if (two && q + 1 + RING < ngw) {
        mbar_expect_tx(&bar[r1], bytes);
        bulk_g2s(ring[r1], src0 + (long long)(q + 1 + RING) * na, bytes, &bar[r1]);
      }
    }
    body(q, c0);
    if (two) body(q + 1, c1);
  }
  return true;
}

// Streaming 16-byte load that does not allocate in L1 (the list is read once per launch; L1 is
// left to the neighbour gathers).
__device__ __forceinline__ uint4 ld_stream(const uint4* p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

// As warp_list_ring2 with the list rows in registers instead of shared memory: each lane loads
// its own 16-byte entry of rows q + 2 and q + 3 while rows q and q + 1 are evaluated.  Lanes
// without an atom (has = false) load nothing; rows up to the warp's largest group count lie
// inside every atom's list capacity.
template <class F>
__device__ __forceinline__ void warp_list_prefetch2(const Dev& D, const SysDev& S, int li, bool has, int ngw, F&& body) {
  const uint4* src = list_group(D, S, li, 0);
  const long long row = S.natoms;
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  uint4 n0 = (has && ngw > 0) ? ld_stream(src) : zero;
  uint4 n1 = (has && ngw > 1) ? ld_stream(src + row) : zero;
  for (int q = 0; q < ngw; q += 2) {
    const uint4 c0 = n0, c1 = n1;
    if (has && q + 2 < ngw) n0 = ld_stream(src + (long long)(q + 2) * row);
    if (has && q + 3 < ngw) n1 = ld_stream(src + (long long)(q + 3) * row);
    body(q, c0);
    if (q + 1 < ngw) body(q + 1, c1);
  }
}

// How the mixed force and density passes read their list rows (template parameter FEED, chosen
// per launch): FEED_REGS, each lane loads its own entries into registers with L1-bypassing loads;
// FEED_RING, bulk asynchronous copies into a per-warp shared-memory ring.  Results are bitwise
// the same.  Measured on the GB300: the single 495k copper system runs 1.5 % faster with
// registers (without the ring's shared memory the L1 that serves the neighbour gathers is 32 KB
// larger per SM), the single 256k LJ liquid 0.4 % and the 512-system LJ ensemble 2.6 % faster
// with the ring.
constexpr int FEED_REGS = 0, FEED_RING = 1;

// Tile of a block of the mixed force and density passes: blockIdx.x, or with GBMD_SM_TILES=1 a
// tile claimed from a contiguous range per SM (a block takes the next tile of the range of the
// SM it runs on, of the next SM's once that range is used up), so that the blocks resident on an
// SM at the same time work on neighbouring cells and share their neighbours' positions in L1.
// Every block gets exactly one tile: a launch has as many blocks as tiles, each block claims at
// most one, and a block that scanned every range without success would mean that the other
// blocks had claimed all tiles.  The last block of a launch to finish zeroes the counters.
// Measured on the GB300 (results bitwise equal): LJ force pass 150 us against 93 us with
// blockIdx.x, copper density + force 0.590 against 0.480 ms, so the claim is off by default.
#ifndef GBMD_SM_TILES
#define GBMD_SM_TILES 0
#endif
__device__ __forceinline__ int claim_tile(const Dev& D) {
#if GBMD_SM_TILES
  __shared__ int s_tile;
  if (threadIdx.x == 0) {
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    const int P = D.claim_slots, T = (int)gridDim.x;
    int k = (int)(smid % (unsigned)P), tile = -1;
    for (int probe = 0; probe < P && tile < 0; ++probe) {
      const int lo = (int)((long long)T * k / P), n = (int)((long long)T * (k + 1) / P) - lo;
      if (n > 0 && (int)__ldcg(D.tile_claim + k) < n) {
        const int idx = (int)atomicAdd(D.tile_claim + k, 1u);
        if (idx < n) tile = lo + idx;
      }
      k = (k + 1 == P) ? 0 : k + 1;
    }
    s_tile = tile;
  }
  __syncthreads();
  return s_tile;
#else
  return (int)blockIdx.x;
#endif
}
__device__ __forceinline__ void release_tile(const Dev& D) {
#if GBMD_SM_TILES
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(D.tile_claim + D.claim_slots, 1u) == gridDim.x - 1) {
      for (int k = 0; k <= D.claim_slots; ++k) D.tile_claim[k] = 0u;
      __threadfence();
    }
  }
#endif
}

template <int PC, int SPECIES, int SCN, int SCM, int FEED>
__device__ __forceinline__ void force32_tile(const Dev& D, const PotParams& P, const StepParams& sp, const int tile) {
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) {  // whole block: one tile belongs to one system
    if (sp.epi == EPI_KICK_DRIFT && sp.last) hold_tile(D, S, tile, true);
    return;
  }
  SHIFT_TABLE(shifts);
  const ShiftCorr corr = shift_corr(S);
  const int li = D.tile_first[tile] - (int)S.atom_base + (int)threadIdx.x;  // index within the system
  const long long i = S.atom_base + li;
  const bool active = (int)threadIdx.x < D.tile_count[tile];
  const float4* __restrict__ g32 = D.g32 + S.atom_base;
  // EAM without a species filter gathers the density pass's copy, whose w holds the
  // neighbour's embedding factor (one 16-byte gather per pair instead of 16 + 4 bytes)
  constexpr bool PHI_IN_W = PC == PC_EAM && !SPECIES;
  const float4* __restrict__ gsrc = PHI_IN_W ? D.g32e + S.atom_base : g32;
  // force, energy and virial: each group of four list entries is summed in FP32 and the group
  // sum rounded into int64 fixed point (forces 2^-32 eV/A; energy and virial 2^-26 eV, scaled
  // to the system accumulators' 2^-32 by an exact integer shift); stress components are summed
  // in FP32 per atom (sab = sum of f_a * r_b with f = g * r; stress_ab = -sab/2), rounded once
  Fix fqx, fqy, fqz, fqe, fqv;
  float sxx = 0.f, sxy = 0.f, sxz = 0.f, syy = 0.f, syz = 0.f, szz = 0.f;
  const float rc2_lo = P.f[12], rc2_hi = P.f[13];
  unsigned rechecks = 0;
  bool bad = false;
  // Each warp streams its 32 atoms' list groups (32 x 16 bytes, contiguous for a fixed group
  // index), with FEED_RING through its own ring of shared-memory stages filled by bulk
  // asynchronous copies (TMA engine) that run RING groups ahead of the force evaluation, with
  // FEED_REGS through registers loaded two groups ahead.  Warps never wait on each other
  // inside the loop.
  __shared__ __align__(16) uint4 ring[TILE / 32][RING][32];
  __shared__ __align__(8) unsigned long long bar[TILE / 32][RING];
  {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float4 gi = active ? g32[li] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int ti = __float_as_int(gi.w);
    // the embedding factor as the loop uses it: the density pass's copy (f[14] x 1/sqrt(rho),
    // f[14] = the Sutton-Chen many-body prefactor in the folded form, else 1) where gathered
    const float phi_i = (PC == PC_EAM && active) ? (PHI_IN_W ? gsrc[li].w : D.phif[i]) : 0.f;
    constexpr bool FOLDED = PHI_IN_W && SCN > 0;
    constexpr bool PACKED_R2 = GBMD_F32X2 && (PC == PC_PAIR || GBMD_F32X2_EAM_FORCE);
    const int na = S.natoms;
    const int cnt = active ? D.ncount[i] : 0;
    const int ng = (cnt + 3) >> 2;
    // Guard-band entries (a few per thousand atoms) are only noted in the loop and decided in
    // FP64 afterwards; their forces then go straight into the fixed-point sums.
    constexpr unsigned NO_BAND = 0xffffffffu;
    unsigned band_e = NO_BAND;
    bool band_more = false;
    float ge = 0.f, gv = 0.f;  // the current group's energy and sum of g r^2
    // Branch-free body: every candidate is evaluated and out-of-range pairs are masked to
    // zero, so lanes never diverge on the cutoff test (70% of Verlet-list entries are inside).
    // Returns g with f = g * d; the caller sums a group's four forces in FP32 and adds the
    // group sum to the int64 fixed-point accumulators.
    auto pair = [&](unsigned e, bool valid, float& dx, float& dy, float& dz) -> float {
      const int j = (int)(e & LOCAL_MASK);
      const float4 gj = gsrc[j];
      const float r2 = entry_r2<PACKED_R2>(gi, gj, shifts[e >> CODE_SHIFT], corr, dx, dy, dz);
      bool in = valid && r2 < rc2_lo;
      if (valid && r2 >= rc2_lo && r2 < rc2_hi) {  // guard band: decided in FP64 after the loop
        if (band_e == NO_BAND)
          band_e = e;
        else
          band_more = true;
      }
      if (SPECIES) in = in && applies_to(P.spc_sum, ti, __float_as_int(gj.w));
      float g, en;
      if (PC == PC_PAIR) {
        lj_pair32(P, rcp_approx(r2), g, en);
      } else if constexpr (FOLDED) {
        eam_sc_pair32_q<SCN, SCM>(P, r2, phi_i, gj.w, g, en);
      } else {
        eam_pair32_t<SCN, SCM>(P, r2, phi_i, PHI_IN_W ? gj.w : D.phif[S.atom_base + j], g, en);
      }
      g = in ? g : 0.0f;
      ge += in ? en : 0.0f;
      gv = fmaf(g, r2, gv);
      const float fx = g * dx, fy = g * dy, fz = g * dz;
      sxx = fmaf(fx, dx, sxx);
      sxy = fmaf(fx, dy, sxy);
      sxz = fmaf(fx, dz, sxz);
      syy = fmaf(fy, dy, syy);
      syz = fmaf(fy, dz, syz);
      szz = fmaf(fz, dz, szz);
      return g;
    };
    // The same two entries at a time, with the pair functions' products of variables as packed
    // FP32 pairs (LJ and folded Sutton-Chen; bitwise the values of `pair`).
    auto geom = [&](unsigned e, bool valid, float& dx, float& dy, float& dz, bool& in, float& qj) -> float {
      const int j = (int)(e & LOCAL_MASK);
      const float4 gj = gsrc[j];
      const float r2 = entry_r2<PACKED_R2>(gi, gj, shifts[e >> CODE_SHIFT], corr, dx, dy, dz);
      in = valid && r2 < rc2_lo;
      if (valid && r2 >= rc2_lo && r2 < rc2_hi) {
        if (band_e == NO_BAND)
          band_e = e;
        else
          band_more = true;
      }
      if (SPECIES) in = in && applies_to(P.spc_sum, ti, __float_as_int(gj.w));
      qj = gj.w;
      return r2;
    };
    auto accum = [&](float g, float en, bool in, float r2, float dx, float dy, float dz) -> float {
      g = in ? g : 0.0f;
      ge += in ? en : 0.0f;
      gv = fmaf(g, r2, gv);
      const float fx = g * dx, fy = g * dy, fz = g * dz;
      sxx = fmaf(fx, dx, sxx);
      sxy = fmaf(fx, dy, sxy);
      sxz = fmaf(fx, dz, sxz);
      syy = fmaf(fy, dy, syy);
      syz = fmaf(fy, dz, syz);
      szz = fmaf(fz, dz, szz);
      return g;
    };
    auto two = [&](unsigned ea, unsigned eb, bool va, bool vb, float& ax, float& ay, float& az, float& bx,
                   float& by, float& bz, float& ga, float& gb) {
      bool ina, inb;
      float qa, qb;
      const float r2a = geom(ea, va, ax, ay, az, ina, qa);
      const float r2b = geom(eb, vb, bx, by, bz, inb, qb);
      float sa, sb, ena, enb;
      if constexpr (PC == PC_PAIR) {
        lj_pair32_x2(P, rcp_approx(r2a), rcp_approx(r2b), sa, sb, ena, enb);
      } else if constexpr (FOLDED) {
        eam_sc_pair32_q_x2<SCN, SCM>(P, r2a, r2b, phi_i, qa, qb, sa, sb, ena, enb);
      } else {
        sa = sb = ena = enb = 0.0f;  // not reached: `two` serves the LJ and folded forms only
      }
      ga = accum(sa, ena, ina, r2a, ax, ay, az);
      gb = accum(sb, enb, inb, r2b, bx, by, bz);
    };
    constexpr bool PAIRED =
        GBMD_F32X2 && ((PC == PC_PAIR && GBMD_F32X2_PAIRMATH_LJ) || (FOLDED && GBMD_F32X2_PAIRMATH_EAM));
    // One group of four entries (rem = entries left in the atom's list from this group on).
    auto group = [&](const uint4& cur, int rem) {
      ge = 0.f;
      gv = 0.f;
      float ax, ay, az, bx, by, bz;
      float g0, g1;
      if constexpr (PAIRED) {
        two(cur.x, cur.y, true, rem > 1, ax, ay, az, bx, by, bz, g0, g1);
      } else {
        g0 = pair(cur.x, true, ax, ay, az);
        g1 = pair(cur.y, rem > 1, bx, by, bz);
      }
      float gx = fmaf(g1, bx, g0 * ax), gy = fmaf(g1, by, g0 * ay), gz = fmaf(g1, bz, g0 * az);
      if constexpr (PAIRED) {
        two(cur.z, cur.w, rem > 2, rem > 3, ax, ay, az, bx, by, bz, g0, g1);
      } else {
        g0 = pair(cur.z, rem > 2, ax, ay, az);
        g1 = pair(cur.w, rem > 3, bx, by, bz);
      }
      gx = fmaf(g1, bx, fmaf(g0, ax, gx));
      gy = fmaf(g1, by, fmaf(g0, ay, gy));
      gz = fmaf(g1, bz, fmaf(g0, az, gz));
      fqx.add_scaled32(gx);
      fqy.add_scaled32(gy);
      fqz.add_scaled32(gz);
      // halved: the full list counts each pair twice; virial = -sum g r^2 / 2
      fqe.add_scaled26(0.5f * ge);
      fqv.add_scaled26(-0.5f * gv);
      // |group force| < 4096 eV/A keeps the force split exact
      bad |= fmaxf(fabsf(gx), fmaxf(fabsf(gy), fabsf(gz))) > 4000.0f;
    };
    const int ngw = __reduce_max_sync(0xffffffffu, (unsigned)ng);
    const int wfirst = D.tile_first[tile] - (int)S.atom_base + 32 * w;
    const int wcount = min(32, max(0, D.tile_count[tile] - 32 * w));
    bool waited = true;
    if constexpr (FEED == FEED_REGS &&
                  ((PC == PC_PAIR && GBMD_PAIR_RING_GROUPS == 2) || (PC == PC_EAM && GBMD_EAM_RING_GROUPS == 2))) {
      warp_list_prefetch2(D, S, li, lane < wcount, ngw, [&](int q, const uint4& cur) {
        if (q < ng) group(cur, cnt - 4 * q);
      });
    } else if constexpr ((PC == PC_PAIR && GBMD_PAIR_RING_GROUPS == 2) || (PC == PC_EAM && GBMD_EAM_RING_GROUPS == 2)) {
      // two list groups per iteration: eight neighbour gathers in flight per lane
      waited = warp_list_ring2(D, S, wfirst, wcount, ngw, ring[w], bar[w], [&](int q, const uint4& cur) {
        if (q < ng) group(cur, cnt - 4 * q);
      });
    } else {
      // one group per iteration, written out here: through the helper the EAM body spills more
      const uint4* src0 = list_group(D, S, wfirst, 0);
      const unsigned bytes = (unsigned)wcount * 16u;
      unsigned long long* wbar = bar[w];
      if (lane == 0 && ngw > 0) {
        for (int r = 0; r < RING; ++r) mbar_init(&wbar[r], 1);
        mbar_init_fence();
        for (int r = 0; r < RING && r < ngw; ++r) {
          mbar_expect_tx(&wbar[r], bytes);
          bulk_g2s(ring[w][r], src0 + (long long)r * na, bytes, &wbar[r]);
        }
      }
      __syncwarp();
      for (int q = 0; q < ngw; ++q) {
        const int r = q & (RING - 1);
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(&wbar[r], (unsigned)((q / RING) & 1)))) {
          ring_drain(wbar, q, ngw);  // stop issuing, wait for the copies in flight, skip the rest
          waited = false;
          break;
        }
        const uint4 cur = ring[w][r][lane];
        __syncwarp();  // every lane has its entry: the stage can be refilled
        if (lane == 0 && q + RING < ngw) {
          fence_proxy_async_shared();
          mbar_expect_tx(&wbar[r], bytes);
          bulk_g2s(ring[w][r], src0 + (long long)(q + RING) * na, bytes, &wbar[r]);
        }
        if (q < ng) group(cur, cnt - 4 * q);
      }
    }
    if (!waited) atomicOr(&D.sst[s].error, ERR_WAIT);
    if (band_e != NO_BAND) {
      // exact FP64 cutoff decision (the reference's Displacement and r^2) for the guard-band
      // entries; one noted entry per atom, else a rescan of the atom's list
      auto settle = [&](unsigned e) {
        const int j = (int)(e & LOCAL_MASK);
        const float4 gj = g32[j];
        float dx, dy, dz;
        const float r2 = entry_r2(gi, gj, shifts[e >> CODE_SHIFT], corr, dx, dy, dz);
        if (!(r2 >= rc2_lo && r2 < rc2_hi)) return;
        ++rechecks;
        if (!exact_inside_cold(&D, &S, i, S.atom_base + j, P.rc2)) return;
        if (SPECIES && !applies_to(P.spc_sum, ti, __float_as_int(gj.w))) return;
        float g, en;
        if (PC == PC_PAIR) {
          lj_pair32(P, rcp_approx(r2), g, en);
        } else {
          // the unscaled embedding factors of both atoms (rare path)
          eam_pair32_t<SCN, SCM>(P, r2, D.phif[i], D.phif[S.atom_base + j], g, en);
        }
        const float fx = g * dx, fy = g * dy, fz = g * dz;
        fqx.add_scaled32(fx);
        fqy.add_scaled32(fy);
        fqz.add_scaled32(fz);
        fqe.add_scaled26(0.5f * en);
        fqv.add_scaled26(-0.5f * (g * r2));
        bad |= fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) > 4000.0f;
        sxx = fmaf(fx, dx, sxx);
        sxy = fmaf(fx, dy, sxy);
        sxz = fmaf(fx, dz, sxz);
        syy = fmaf(fy, dy, syy);
        syz = fmaf(fy, dz, syz);
        szz = fmaf(fz, dz, szz);
      };
      if (!band_more) {
        settle(band_e);
      } else {
        const uint4* L = list_group(D, S, li, 0);
        for (int q = 0; q < ng; ++q) {
          const uint4 e4 = __ldg(L + (long long)q * na);
          const int rem = cnt - 4 * q;
          settle(e4.x);
          if (rem > 1) settle(e4.y);
          if (rem > 2) settle(e4.z);
          if (rem > 3) settle(e4.w);
        }
      }
    }
  }
  double ke = 0.0, px = 0.0, py = 0.0, pz = 0.0;
  float d2 = 0.0f;
  if (active) {
    const long long N = D.N;
    long long qx = fqx.value(), qy = fqy.value(), qz = fqz.value();
    if (!sp.first) {
      qx += D.facc[i];
      qy += D.facc[N + i];
      qz += D.facc[2 * N + i];
    }
    if (sp.last) {
      d2 = finish_atom<1>(D, S, i, (double)qx, (double)qy, (double)qz, sp, ke, px, py, pz);
    } else {
      D.facc[i] = qx;
      D.facc[N + i] = qy;
      D.facc[2 * N + i] = qz;
    }
    if (rechecks) atomicAdd(&D.sst[s].rechecks, (unsigned long long)rechecks);
    if (bad) atomicOr(&D.sst[s].error, ERR_FIXED);
  }
  track_displacement_warp(D, s, d2);
  // energy and virial already in fixed point; per-atom stress (halved: full list) rounded to
  // int64 once; exact block sums and one integer atomic per quantity into the system's slots
  const float ms = (float)(-0.5 * FIX_E);
  long long v[11] = {fqe.value() * 64, fqv.value() * 64, fix64(sxx * ms), fix64(sxy * ms), fix64(sxz * ms),
                     fix64(sxy * ms), fix64(syy * ms), fix64(syz * ms), fix64(sxz * ms), fix64(syz * ms),
                     fix64(szz * ms)};
  long long tot[11];
  block_sum<long long, 11>(v, tot);
  if (threadIdx.x == 0) {
    unsigned long long* acc = D.sys_acc + (long long)s * SA_LEN;
    for (int k = 0; k < 11; ++k) atomicAdd(acc + k, (unsigned long long)tot[k]);
  }
  if (sp.last) {
    // kinetic energy and momentum: FP64 warp sums in a fixed order, rounded once per warp to
    // int64 (2^-44 units); exact int64 sums from there on
    long long k4[4];
    warp_kinetic_fix(ke, px, py, pz, k4);
    long long kt[4];
    block_sum<long long, 4>(k4, kt);
    if (threadIdx.x == 0) {
      unsigned long long* acc = D.sys_acc + (long long)s * SA_LEN;
      atomicAdd(acc + SA_KE, (unsigned long long)kt[0]);
      for (int k = 0; k < 3; ++k) atomicAdd(acc + SA_P + k, (unsigned long long)kt[1 + k]);
    }
  }
}


template <int PC, int SPECIES, int SCN = 0, int SCM = 0, int FEED = FEED_REGS>
__global__ void __launch_bounds__(TILE, GBMD_FORCE_MIN_BLOCKS) k_force32(Dev D, PotParams P, StepParams sp) {
  const int tile = claim_tile(D);
  if (tile >= 0) force32_tile<PC, SPECIES, SCN, SCM, FEED>(D, P, sp, tile);
  release_tile(D);
}

// ------------------------------------------------------------------------------------------
// Mixed LJ force pass with LANES lanes per atom (LANES = 2, 4, 8: 16, 8 or 4 atoms per warp),
// for systems too small to fill the GPU one lane per atom.  The atom's list groups go
// round-robin to its lanes (plain cached loads instead of the bulk-copy ring); each group is
// evaluated and summed exactly as in k_force32, and the lanes' fixed-point partials are
// combined with integer shuffles, so the forces are bitwise those of k_force32.  Energy and
// stress partials are rounded to fixed point per lane (a 2^-32 eV-scale difference).  A tile
// of 128 atoms is spread over LANES blocks of 128 threads.
// ------------------------------------------------------------------------------------------

template <int SPECIES, int LANES>
__global__ void __launch_bounds__(TILE, GBMD_FORCE_MIN_BLOCKS) k_force32_lanes(Dev D, PotParams P, StepParams sp) {
  __shared__ float4 shifts[125];
  constexpr int APB = TILE / LANES;  // atoms per block
  const int tile = blockIdx.x / LANES, part = blockIdx.x % LANES;
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) {  // whole block: one tile belongs to one system
    if (part == 0 && sp.epi == EPI_KICK_DRIFT && sp.last) hold_tile(D, S, tile, true);
    return;
  }
  load_shifts(S, shifts);
  const ShiftCorr corr = shift_corr(S);
  const int sub = threadIdx.x % LANES;
  const int slot = part * APB + (int)threadIdx.x / LANES;  // atom within the tile
  const int li = D.tile_first[tile] - (int)S.atom_base + slot;
  const long long i = S.atom_base + li;
  const bool active = slot < D.tile_count[tile];
  const float4* __restrict__ g32 = D.g32 + S.atom_base;
  Fix fqx, fqy, fqz, fqe, fqv;
  float sxx = 0.f, sxy = 0.f, sxz = 0.f, syy = 0.f, syz = 0.f, szz = 0.f;
  const float rc2_lo = P.f[12], rc2_hi = P.f[13];
  unsigned rechecks = 0;
  bool bad = false;
  const float4 gi = active ? g32[li] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int ti = __float_as_int(gi.w);
  const int na = S.natoms;
  const int cnt = active ? D.ncount[i] : 0;
  const int ng = (cnt + 3) >> 2;
  constexpr unsigned NO_BAND = 0xffffffffu;
  unsigned band_e = NO_BAND;
  bool band_more = false;
  float ge = 0.f, gv = 0.f;
  auto pair = [&](unsigned e, bool valid, float& dx, float& dy, float& dz) -> float {
    const int j = (int)(e & LOCAL_MASK);
    const float4 gj = g32[j];
    const float r2 = entry_r2(gi, gj, shifts[e >> CODE_SHIFT], corr, dx, dy, dz);
    bool in = valid && r2 < rc2_lo;
    if (valid && r2 >= rc2_lo && r2 < rc2_hi) {
      if (band_e == NO_BAND)
        band_e = e;
      else
        band_more = true;
    }
    if (SPECIES) in = in && applies_to(P.spc_sum, ti, __float_as_int(gj.w));
    float g, en;
    lj_pair32(P, rcp_approx(r2), g, en);
    g = in ? g : 0.0f;
    ge += in ? en : 0.0f;
    gv = fmaf(g, r2, gv);
    const float fx = g * dx, fy = g * dy, fz = g * dz;
    sxx = fmaf(fx, dx, sxx);
    sxy = fmaf(fx, dy, sxy);
    sxz = fmaf(fx, dz, sxz);
    syy = fmaf(fy, dy, syy);
    syz = fmaf(fy, dz, syz);
    szz = fmaf(fz, dz, szz);
    return g;
  };
  const uint4* L = active ? list_group(D, S, li, 0) : nullptr;
  for (int q = sub; q < ng; q += LANES) {
    const uint4 cur = __ldg(L + (long long)q * na);
    const int rem = cnt - 4 * q;
    ge = 0.f;
    gv = 0.f;
    float ax, ay, az, bx, by, bz;
    float g0 = pair(cur.x, true, ax, ay, az);
    float g1 = pair(cur.y, rem > 1, bx, by, bz);
    float gx = fmaf(g1, bx, g0 * ax), gy = fmaf(g1, by, g0 * ay), gz = fmaf(g1, bz, g0 * az);
    g0 = pair(cur.z, rem > 2, ax, ay, az);
    g1 = pair(cur.w, rem > 3, bx, by, bz);
    gx = fmaf(g1, bx, fmaf(g0, ax, gx));
    gy = fmaf(g1, by, fmaf(g0, ay, gy));
    gz = fmaf(g1, bz, fmaf(g0, az, gz));
    fqx.add_scaled32(gx);
    fqy.add_scaled32(gy);
    fqz.add_scaled32(gz);
    fqe.add_scaled26(0.5f * ge);
    fqv.add_scaled26(-0.5f * gv);
    bad |= fmaxf(fabsf(gx), fmaxf(fabsf(gy), fabsf(gz))) > 4000.0f;
  }
  if (band_e != NO_BAND) {
    auto settle = [&](unsigned e) {
      const int j = (int)(e & LOCAL_MASK);
      const float4 gj = g32[j];
      float dx, dy, dz;
      const float r2 = entry_r2(gi, gj, shifts[e >> CODE_SHIFT], corr, dx, dy, dz);
      if (!(r2 >= rc2_lo && r2 < rc2_hi)) return;
      ++rechecks;
      if (!exact_inside_cold(&D, &S, i, S.atom_base + j, P.rc2)) return;
      if (SPECIES && !applies_to(P.spc_sum, ti, __float_as_int(gj.w))) return;
      float g, en;
      lj_pair32(P, rcp_approx(r2), g, en);
      const float fx = g * dx, fy = g * dy, fz = g * dz;
      fqx.add_scaled32(fx);
      fqy.add_scaled32(fy);
      fqz.add_scaled32(fz);
      fqe.add_scaled26(0.5f * en);
      fqv.add_scaled26(-0.5f * (g * r2));
      bad |= fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) > 4000.0f;
      sxx = fmaf(fx, dx, sxx);
      sxy = fmaf(fx, dy, sxy);
      sxz = fmaf(fx, dz, sxz);
      syy = fmaf(fy, dy, syy);
      syz = fmaf(fy, dz, syz);
      szz = fmaf(fz, dz, szz);
    };
    if (!band_more) {
      settle(band_e);
    } else {
      for (int q = sub; q < ng; q += LANES) {
        const uint4 e4 = __ldg(L + (long long)q * na);
        const int rem = cnt - 4 * q;
        settle(e4.x);
        if (rem > 1) settle(e4.y);
        if (rem > 2) settle(e4.z);
        if (rem > 3) settle(e4.w);
      }
    }
  }
  // the atom's lanes are adjacent: exact integer sums of the fixed-point partials
#pragma unroll
  for (int m = 1; m < LANES; m <<= 1) {
    fqx.hi += __shfl_xor_sync(0xffffffffu, fqx.hi, m);
    fqx.lo += __shfl_xor_sync(0xffffffffu, fqx.lo, m);
    fqy.hi += __shfl_xor_sync(0xffffffffu, fqy.hi, m);
    fqy.lo += __shfl_xor_sync(0xffffffffu, fqy.lo, m);
    fqz.hi += __shfl_xor_sync(0xffffffffu, fqz.hi, m);
    fqz.lo += __shfl_xor_sync(0xffffffffu, fqz.lo, m);
  }
  double ke = 0.0, px = 0.0, py = 0.0, pz = 0.0;
  float d2 = 0.0f;
  if (active && sub == 0) {
    const long long N = D.N;
    long long qx = fqx.value(), qy = fqy.value(), qz = fqz.value();
    if (!sp.first) {
      qx += D.facc[i];
      qy += D.facc[N + i];
      qz += D.facc[2 * N + i];
    }
    if (sp.last) {
      d2 = finish_atom<1>(D, S, i, (double)qx, (double)qy, (double)qz, sp, ke, px, py, pz);
    } else {
      D.facc[i] = qx;
      D.facc[N + i] = qy;
      D.facc[2 * N + i] = qz;
    }
  }
  if (active) {
    if (rechecks) atomicAdd(&D.sst[s].rechecks, (unsigned long long)rechecks);
    if (bad) atomicOr(&D.sst[s].error, ERR_FIXED);
  }
  track_displacement_warp(D, s, d2);
  // energy and virial: every lane's own fixed-point partial (exact integer block sums), so they
  // do not depend on the lane count; stress rounded per lane
  const float ms = (float)(-0.5 * FIX_E);
  long long v[11] = {fqe.value() * 64, fqv.value() * 64, fix64(sxx * ms), fix64(sxy * ms), fix64(sxz * ms),
                     fix64(sxy * ms), fix64(syy * ms), fix64(syz * ms), fix64(sxz * ms), fix64(syz * ms),
                     fix64(szz * ms)};
  long long tot[11];
  block_sum<long long, 11>(v, tot);
  if (threadIdx.x == 0) {
    unsigned long long* acc = D.sys_acc + (long long)s * SA_LEN;
    for (int k = 0; k < 11; ++k) atomicAdd(acc + k, (unsigned long long)tot[k]);
  }
  if (sp.last) {
    long long k4[4];
    warp_kinetic_fix(ke, px, py, pz, k4);
    long long kt[4];
    block_sum<long long, 4>(k4, kt);
    if (threadIdx.x == 0) {
      unsigned long long* acc = D.sys_acc + (long long)s * SA_LEN;
      atomicAdd(acc + SA_KE, (unsigned long long)kt[0]);
      for (int k = 0; k < 3; ++k) atomicAdd(acc + SA_P + k, (unsigned long long)kt[1 + k]);
    }
  }
}

// ------------------------------------------------------------------------------------------
// EAM density pass + embedding (FP64 embedding in both precisions).
// ------------------------------------------------------------------------------------------

// Mixed density pass over the Verlet list: FP32 rho_ij of each group of four entries
// (branch-free, out-of-range entries masked), the group sum added to the int64 fixed-point
// density; cutoff decisions in the guard band re-done in FP64 as in the force kernel.
template <int SCM, int FEED>
__device__ __forceinline__ void density32_tile(const Dev& D, const PotParams& P, const int tile) {
  __shared__ __align__(16) uint4 ring_s[TILE / 32][RING][32];
  __shared__ __align__(8) unsigned long long bar_s[TILE / 32][RING];
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) return;  // whole block: one tile belongs to one system
  SHIFT_TABLE(shifts);
  const ShiftCorr corr = shift_corr(S);
  const int li = D.tile_first[tile] - (int)S.atom_base + (int)threadIdx.x;
  const long long i = S.atom_base + li;
  const bool active = (int)threadIdx.x < D.tile_count[tile];
  const float4* __restrict__ g32 = D.g32 + S.atom_base;
  const float4 gi = active ? g32[li] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float rc2_lo = P.f[12], rc2_hi = P.f[13];
  const int cnt = active ? D.ncount[i] : 0;
  const int ng = (cnt + 3) >> 2;
  Fix q;
  unsigned rechecks = 0;
  // guard-band entries are noted in the loop and decided in FP64 afterwards (as in k_force32)
  constexpr unsigned NO_BAND = 0xffffffffu;
  unsigned band_e = NO_BAND;
  bool band_more = false;
  auto term = [&](unsigned e, bool valid) -> float {
    const int j = (int)(e & LOCAL_MASK);
    float dx, dy, dz;
    const float r2 = entry_r2(gi, g32[j], shifts[e >> CODE_SHIFT], corr, dx, dy, dz);
    const bool in = valid && r2 < rc2_lo;
    if (valid && r2 >= rc2_lo && r2 < rc2_hi) {
      if (band_e == NO_BAND)
        band_e = e;
      else
        band_more = true;
    }
    const float v = eam_rho32_t<SCM>(P, r2);
    return in ? v : 0.0f;
  };
  const float scale = (float)FIX_RHO;
  // every lane of the warp takes part in the ring (lanes without an atom have no groups)
  const int w = threadIdx.x >> 5;
  const int wfirst = D.tile_first[tile] - (int)S.atom_base + 32 * w;
  const int wcount = min(32, max(0, D.tile_count[tile] - 32 * w));
  const int ngw = __reduce_max_sync(0xffffffffu, (unsigned)ng);
  auto row = [&](int g, const uint4& e4) {
    if (g < ng) {
      const int rem = cnt - 4 * g;
      const float part = ((term(e4.x, true) + term(e4.y, rem > 1)) + term(e4.z, rem > 2)) + term(e4.w, rem > 3);
      q.add(part * scale);
    }
  };
  bool waited = true;
  if constexpr (FEED == FEED_RING)
    waited = warp_list_ring2(D, S, wfirst, wcount, ngw, ring_s[w], bar_s[w], row);
  else
    warp_list_prefetch2(D, S, li, active, ngw, row);
  if (!waited) atomicOr(&D.sst[s].error, ERR_WAIT);
  if (band_e != NO_BAND) {
    auto settle = [&](unsigned e) {
      const int j = (int)(e & LOCAL_MASK);
      float dx, dy, dz;
      const float r2 = entry_r2(gi, g32[j], shifts[e >> CODE_SHIFT], corr, dx, dy, dz);
      if (!(r2 >= rc2_lo && r2 < rc2_hi)) return;
      ++rechecks;
      if (exact_inside_cold(&D, &S, i, S.atom_base + j, P.rc2)) q.add(eam_rho32_t<SCM>(P, r2) * scale);
    };
    if (!band_more) {
      settle(band_e);
    } else {
      const uint4* L = list_group(D, S, li, 0);
      for (int g = 0; g < ng; ++g) {
        const uint4 e4 = __ldg(L + (long long)g * S.natoms);
        const int rem = cnt - 4 * g;
        settle(e4.x);
        if (rem > 1) settle(e4.y);
        if (rem > 2) settle(e4.z);
        if (rem > 3) settle(e4.w);
      }
    }
  }
  if (rechecks) atomicAdd(&D.sst[s].rechecks, (unsigned long long)rechecks);
  double F = 0.0;
  if (active) {
    const double rho = (double)q.value() * (1.0 / FIX_RHO);
    double phi;
    eam_embed64(P, rho, F, phi);
    D.rho[i] = rho;
    D.phi[i] = phi;
    D.phif[i] = (float)phi;
    D.g32e[i] = make_float4(gi.x, gi.y, gi.z, (float)((double)P.f[14] * phi));
  }
  // FP64 embedding energies summed exactly as int64 fixed point (2^-32 eV per atom)
  long long v[1] = {active ? __double2ll_rn(F * FIX_E) : 0ll};
  long long t[1];
  block_sum<long long, 1>(v, t);
  if (threadIdx.x == 0) atomicAdd(D.sys_acc + (long long)s * SA_LEN + SA_EEMBED, (unsigned long long)t[0]);
}


template <int SCM, int FEED = FEED_REGS>
__global__ void GBMD_DENSITY_BOUNDS k_eam_density32(Dev D, PotParams P) {
  const int tile = claim_tile(D);
  if (tile >= 0) density32_tile<SCM, FEED>(D, P, tile);
  release_tile(D);
}

// FP64 density pass (the plain path, any neighbour mode): reference r and rhoij, FP64
// embedding, per-tile FP64 partial of the embedding energy.
template <int NB>
__global__ void __launch_bounds__(TILE) k_eam_density(Dev D, PotParams P, int first) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) return;  // whole block: one tile belongs to one system
  const long long i = D.tile_first[tile] + threadIdx.x;
  const bool active = (int)threadIdx.x < D.tile_count[tile];
  double F = 0.0;
  if (active) {
    double rho = 0.0;
    const double4_32a pi = D.g64[i];
    for_each_candidate<NB>(D, S, i, [&](long long j, unsigned) {
      const double4_32a pj = D.g64[j];
      double dx = ref_wrap(dsub(pj.x, pi.x), S.L[0], S.Lh[0]);
      double dy = ref_wrap(dsub(pj.y, pi.y), S.L[1], S.Lh[1]);
      double dz = ref_wrap(dsub(pj.z, pi.z), S.L[2], S.Lh[2]);
      double r2 = ref_sq(dx, dy, dz);
      if (r2 < P.rc2) rho += eam_rho64(P, sqrt(r2));
    });
    double phi;
    eam_embed64(P, rho, F, phi);
    D.rho[i] = rho;
    D.phi[i] = phi;
    D.phif[i] = (float)phi;
  }
  double v[1] = {F};
  double t[1];
  block_sum<double, 1>(v, t);
  if (threadIdx.x == 0) {
    double* td = D.tile_d + (long long)tile * PART_D;
    td[PD_EEMBED] = first ? t[0] : td[PD_EEMBED] + t[0];
  }
}

// ------------------------------------------------------------------------------------------
// Thermo record per system of the FP64 path (one block per system; fixed-order tile sums).
// ------------------------------------------------------------------------------------------

__global__ void __launch_bounds__(TILE) k_thermo(Dev D, int count_step) {
  const int s = blockIdx.x;
  const SysDev& S = D.sysd[s];
  if (!S.active) return;
  double v[PART_D];
  for (int k = 0; k < PART_D; ++k) v[k] = 0.0;
  for (int t = threadIdx.x; t < S.ntiles; t += blockDim.x) {
    const double* td = D.tile_d + (long long)(S.tile_base + t) * PART_D;
    for (int k = 0; k < PART_D; ++k) v[k] += td[k];
  }
  double tot[PART_D];
  block_sum<double, PART_D>(v, tot);
  if (threadIdx.x == 0) thermo_record(D, s, tot, count_step);
}

}  // namespace gbmd

// kernels.cuh -- the sm_103a kernels of the MD timestep.
//
//   k_decide       per system: does this force evaluation need a cell/list rebuild?
//                  (LinkedCell rebuilds at every UpdateCell, plugins/linkedcell.cc:112-267;
//                   the Verlet list on displacement > skin/2 and/or every `each` UpdateCell
//                   calls, plugins/verletlist.cc:124-131)
//   k_bin          FP64 cell index of every atom (plugins/linkedcell.cc:249-253) + histogram
//   k_scan         per-system exclusive scan of the cell histogram
//   k_scatter      counting-sort scatter into cells
//   k_cellsort     orders each cell by original atom index (the reference's linked-list order)
//   k_permute      gathers every per-atom field into the new cell-sorted order (scratch)
//   k_copyback     writes the sorted fields back, refreshes gather copies and home cells
//   k_buildlist    Verlet list from the 27/125-cell stencil with per-pair cell-shift codes
//   k_drift        VelocityVerlet::AdvancePosition (plugins/velocityverlet.cc:60-68) + wrap,
//                  gather copies, displacement tracking
//   k_pair_force   PairPotential::UpdateForces (liblpmd/simulation/pairpotential.cc:35-84)
//                  as a full-list gather, fused with VelocityVerlet::AdvanceVelocity
//                  (plugins/velocityverlet.cc:70-75) and the per-tile thermo sums
//   k_eam_density  MetalPotential rho pass + embedding (liblpmd/simulation/metalpotential.cc:118-132,168)
//   k_eam_force    MetalPotential force pass (liblpmd/simulation/metalpotential.cc:137-169)
//   k_thermo       per-system reduction of the tile sums into the thermo record
//                  (SetSimulationTags, liblpmd/simulation/simulationbuilder.cc:84-124)
#pragma once

#include "device.cuh"
#include "potentials.cuh"

namespace gbmd {

enum EpiMode { EPI_FORCES = 0, EPI_KICK = 1, EPI_KICK_DRIFT = 2 };

struct StepParams {
  double dt;
  double half_dt;       // 0.5 * dt, as AdvanceVelocity computes it
  double half_dt2;      // 0.5 * dt * dt (mixed drift)
  int epi;              // EpiMode of the final force pass
  int first;            // first potential pass of this evaluation (overwrite partials)
  int last;             // last potential pass (write accelerations)
  int count_step;       // k_thermo advances the step counter
  int kinetic;          // compute kinetic sums in the epilogue
  int raw_acc;          // keep fixedvel atoms' accelerations (a bare UpdateForces, no integrator)
};

// ---------------------------------------------------------------------------------------------
// Rebuild decision
// ---------------------------------------------------------------------------------------------

// ucall_inc: how many emulated UpdateCell calls this evaluation stands for (verletlist "each").
// Rebuild decision of one system for the next force evaluation (one thread): clears the
// system's fixed-point accumulators and returns whether its cells/list are rebuilt.
__device__ __forceinline__ int decide_system(const Dev& D, int s, int ucall_inc, int force_all) {
  const SysDev& S = D.sysd[s];
  SysState& st = D.sst[s];
  if (!S.active) {
    st.need_rebuild = 0;
    return 0;
  }
  int need = force_all | st.force_rebuild;
  if (S.mode == NB_CELLS) need = 1;
  if (S.mode == NB_LIST) {
    float md2 = __int_as_float((int)__ldcg(&st.maxdisp2));  // atomics of the previous launch
    if ((S.rebuild_policy == REBUILD_SKIN || S.rebuild_policy == REBUILD_BOTH) && (double)md2 > S.thresh2)
      need = 1;
    if (S.rebuild_policy == REBUILD_EACH || S.rebuild_policy == REBUILD_BOTH) {
      for (int k = 0; k < ucall_inc; ++k)
        if (((st.ucalls + k) % S.each) == 0) need = 1;
    }
  }
  st.ucalls += ucall_inc;
  if (S.mode == NB_ALLPAIRS) need = 0;
  for (int k = 0; k < SA_LEN; ++k) D.sys_acc[(long long)s * SA_LEN + k] = 0ull;
  st.need_rebuild = need;
  st.force_rebuild = 0;
  if (need) {
    st.maxdisp2 = 0u;
    st.rebuilds += (S.mode == NB_LIST) ? 1 : 0;
  }
  return need;
}

// One thread per system.  Inside a graph the conditional of the step starts at 0 at every graph
// launch (cudaGraphCondAssignDefault): a block raises it when one of its systems rebuilds.
constexpr int DECIDE_THREADS = 128;
__global__ void __launch_bounds__(DECIDE_THREADS) k_decide(Dev D, int nsys, int ucall_inc, int force_all,
                                                           unsigned long long cond_handle, int use_cond) {
  const int s = blockIdx.x * DECIDE_THREADS + threadIdx.x;
  const int need = s < nsys ? decide_system(D, s, ucall_inc, force_all) : 0;
  if (__syncthreads_or(need) && use_cond && threadIdx.x == 0)
    cudaGraphSetConditional((cudaGraphConditionalHandle)cond_handle, 1u);
}

// ---------------------------------------------------------------------------------------------
// Binning and counting sort
// ---------------------------------------------------------------------------------------------

// Sort-chain options: warp-aggregated cell atomics in k_bin / k_scatter (one atomic per cell
// and warp instead of one per atom), several cells per thread in k_scan.
#ifndef GBMD_SORT_AGGREGATE
#define GBMD_SORT_AGGREGATE 1
#endif
#ifndef GBMD_SCAN_CELLS
#define GBMD_SCAN_CELLS 4
#endif

__global__ void k_bin(Dev D) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  int s = D.sysid[i];
  if (!D.sst[s].need_rebuild) return;
  const SysDev& S = D.sysd[s];
  bool ok = true;
  int cx, cy, cz;
  if (S.mode == NB_LIST) {
    // Verlet-list grid: cells are wider than the list radius by a margin, so the binning may
    // round differently from LinkedCell's; one multiply instead of a division per axis
    cx = list_cell_coord(D.x[i] * S.ninv[0], S.n[0], ok);
    cy = list_cell_coord(D.y[i] * S.ninv[1], S.n[1], ok);
    cz = list_cell_coord(D.z[i] * S.ninv[2], S.n[2], ok);
  } else {
    cx = ref_cell_coord(D.x[i], S.L[0], S.n[0], ok);
    cy = ref_cell_coord(D.y[i], S.L[1], S.n[1], ok);
    cz = ref_cell_coord(D.z[i], S.L[2], S.n[2], ok);
  }
  if (!ok) {
    atomicOr(&D.sst[s].error, ERR_OUTSIDE);
    cx = cy = cz = 0;
  }
  int c = S.cell_base + (cz * S.n[1] + cy) * S.n[0] + cx;
  D.acell[i] = c;
#if GBMD_SORT_AGGREGATE
  // consecutive atoms mostly share a cell (the arrays are in the previous cell order): one
  // atomic per cell and warp
  const unsigned peers = __match_any_sync(__activemask(), c);
  if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&D.ccount[c], __popc(peers));
#else
  atomicAdd(&D.ccount[c], 1);
#endif
}

// One block per system: exclusive scan of the cell counts, GBMD_SCAN_CELLS consecutive cells
// per thread; resets counts and cursors.
__global__ void k_scan(Dev D) {
  const int s = blockIdx.x;
  if (!D.sst[s].need_rebuild) return;
  const SysDev& S = D.sysd[s];
  const int nc = S.ncells, cb = S.cell_base;
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < nc; base += blockDim.x * GBMD_SCAN_CELLS) {
    const int c0 = base + threadIdx.x * GBMD_SCAN_CELLS;
    int v[GBMD_SCAN_CELLS];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < GBMD_SCAN_CELLS; ++k) {
      v[k] = (c0 + k < nc) ? D.ccount[cb + c0 + k] : 0;
      sum += v[k];
    }
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = (lane < nw) ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    int excl = x - sum + (w > 0 ? warp_tot[w - 1] : 0) + carry;
#pragma unroll
    for (int k = 0; k < GBMD_SCAN_CELLS; ++k) {
      if (c0 + k < nc) {
        D.cstart[cb + c0 + k] = (int)(S.atom_base) + excl;  // global slot
        D.ccnt[cb + c0 + k] = v[k];
        D.ccount[cb + c0 + k] = 0;
        D.ccursor[cb + c0 + k] = 0;
      }
      excl += v[k];
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl;  // the block's running total
    __syncthreads();
  }
}

// LCBinary::UpdateCell keeps at most one atom per sub-cell (plugins/lcbinary.cc:162-193): flags
// the systems whose re-sort put two atoms into one cell (their grid then grows by 2 per axis).
__global__ void k_binary_collide(Dev D) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= D.total_cells) return;
  const int s = D.cell_sys[g];
  if (!D.sysd[s].active || !D.sst[s].need_rebuild) return;
  if (D.ccnt[g] > 1) atomicOr(&D.sst[s].collide, 1);
}

__global__ void k_binary_clear(Dev D) {
  for (int s = threadIdx.x; s < D.nsys; s += blockDim.x) D.sst[s].collide = 0;
}

__global__ void k_scatter(Dev D) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  int s = D.sysid[i];
  if (!D.sst[s].need_rebuild) return;
  int c = D.acell[i];
#if GBMD_SORT_AGGREGATE
  // the warp's atoms of one cell take consecutive slots from one atomic (their order inside
  // the cell is set by k_cellsort either way)
  const unsigned peers = __match_any_sync(__activemask(), c);
  const int lane = threadIdx.x & 31, lead = __ffs(peers) - 1;
  int first = 0;
  if (lane == lead) first = atomicAdd(&D.ccursor[c], __popc(peers));
  first = __shfl_sync(peers, first, lead);
  int p = D.cstart[c] + first + __popc(peers & ((1u << lane) - 1u));
#else
  int p = D.cstart[c] + atomicAdd(&D.ccursor[c], 1);
#endif
  D.perm[p] = (int)i;
}

// One warp per cell over the cells of every system (flat index g; cell_sys maps it back):
// orders the cell's slots by original index, the order in which LinkedCell's head/next lists
// visit them.  Each atom's rank is the number of smaller tags in its cell: up to 32 atoms the
// lanes compare through shuffles, up to SORT_STAGE atoms (dense cells of a liquid, coarse
// LinkedCell grids) through a copy of the cell's tags in shared memory, and beyond that through
// global scratch (n^2/32 compares per lane).
constexpr int SORT_WARPS = 4;    // cells per block
constexpr int SORT_STAGE = 256;  // atoms per cell ranked in shared memory
__global__ void __launch_bounds__(32 * SORT_WARPS) k_cellsort(Dev D) {
  __shared__ int s_tag[SORT_WARPS][SORT_STAGE];
  __shared__ int s_idx[SORT_WARPS][SORT_STAGE];
  const int w = threadIdx.x >> 5;
  const int g = blockIdx.x * SORT_WARPS + w;
  if (g >= D.total_cells) return;
  const int s = D.cell_sys[g];
  if (!D.sst[s].need_rebuild) return;
  const int lane = threadIdx.x & 31;
  const int b = D.cstart[g], n = D.ccnt[g];
  if (n <= 32) {
    int v = lane < n ? D.perm[b + lane] : 0;
    int tv = lane < n ? D.tag[v] : 0x7fffffff;
    int rank = 0;
    for (int k = 0; k < n; ++k) {
      int tk = __shfl_sync(0xffffffffu, tv, k);
      rank += (tk < tv) ? 1 : 0;
    }
    __syncwarp();
    if (lane < n) D.perm[b + rank] = v;
    return;
  }
  if (n <= SORT_STAGE) {
    int* tg = s_tag[w];
    int* ix = s_idx[w];
    for (int k = lane; k < n; k += 32) {
      const int v = D.perm[b + k];
      ix[k] = v;
      tg[k] = D.tag[v];
    }
    __syncwarp();  // every slot is read before any is rewritten
    for (int k = lane; k < n; k += 32) {
      const int t = tg[k];
      int rank = 0;
      for (int m = 0; m < n; ++m) rank += (tg[m] < t) ? 1 : 0;
      D.perm[b + rank] = ix[k];
    }
    return;
  }
  // larger cells: the same ranks through global scratch, the cell's own slots [b, b + n) of the
  // permutation staging (free until k_permute fills it)
  int* const tags = D.sint;
  int* const sorted = D.sint + D.N;
  for (int k = lane; k < n; k += 32) tags[b + k] = D.tag[D.perm[b + k]];
  __syncwarp();
  for (int k = lane; k < n; k += 32) {
    const int t = tags[b + k];
    int rank = 0;
    for (int m = 0; m < n; ++m) rank += (tags[b + m] < t) ? 1 : 0;
    sorted[b + rank] = D.perm[b + k];
  }
  __syncwarp();
  for (int k = lane; k < n; k += 32) D.perm[b + k] = sorted[b + k];
}

__global__ void k_permute(Dev D) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= D.N) return;
  int s = D.sysid[p];
  if (!D.sst[s].need_rebuild) return;
  const long long N = D.N;
  int o = D.perm[p];
  double* sd = D.sdbl;
  sd[0 * N + p] = D.x[o];
  sd[1 * N + p] = D.y[o];
  sd[2 * N + p] = D.z[o];
  sd[3 * N + p] = D.vx[o];
  sd[4 * N + p] = D.vy[o];
  sd[5 * N + p] = D.vz[o];
  sd[6 * N + p] = D.ax[o];
  sd[7 * N + p] = D.ay[o];
  sd[8 * N + p] = D.az[o];
  sd[9 * N + p] = D.mass[o];
  sd[10 * N + p] = D.fm[o];
  int* si = D.sint;
  si[0 * N + p] = D.type[o];
  si[1 * N + p] = D.tag[o];
  si[2 * N + p] = D.acell[o];
  if (D.has_flags) D.sflags[p] = D.flags[o];
  if (D.ist)
    for (int k = 0; k < IST_K; ++k) D.ist_alt[k * N + p] = D.ist[k * N + o];
}

// Offset of x from the centre xc of its home cell, wrapped into [-L/2, L/2).  Two FP64-pipe
// operations on the common path (the FP64 unit is GB300's scarcest); the wrap is only taken
// for atoms far from their home cell (outside the box in the input).
__device__ __forceinline__ float home_offset(double x, double xc, double L, double Lh) {
  double o = x - xc;
  float of = (float)o;
  if (fabsf(of) >= 0.999f * (float)Lh) {
    if (o >= Lh) o = dsub(o, L);
    if (o < -Lh) o = dadd(o, L);
    of = (float)o;
  }
  return of;
}

// Gather copies of atom p at position (xx, yy, zz): the FP64 double4 (not by the mixed path's
// fused drift, WRITE64 = 0: no mixed kernel reads it, and a change of precision re-sorts, which
// rewrites it) and, for Verlet lists, the FP32 offset from the home-cell centre (returned, for
// displacement tracking).
template <int WRITE64 = 1>
__device__ __forceinline__ float4 write_gather(const Dev& D, const SysDev& S, long long p, double xx, double yy,
                                               double zz, int t, double4_32a* g64, float4* g32) {
  if (WRITE64) g64[p] = make_double4_32a(xx, yy, zz, (double)t);
  float4 g = make_float4(0.f, 0.f, 0.f, __int_as_float(t));
  if (S.mode == NB_LIST) {
    const double* c = D.ccentre + 3 * (long long)D.home[p];
    g = make_float4(home_offset(xx, c[0], S.L[0], S.Lh[0]), home_offset(yy, c[1], S.L[1], S.Lh[1]),
                    home_offset(zz, c[2], S.L[2], S.Lh[2]), __int_as_float(t));
    g32[p] = g;
  }
  return g;
}

__device__ __forceinline__ void refresh_gather(const Dev& D, const SysDev& S, long long p, bool set_ref) {
  float4 g = write_gather(D, S, p, D.x[p], D.y[p], D.z[p], D.type[p], D.g64, D.g32);
  if (set_ref && S.mode == NB_LIST) D.ref[p] = g;
}

// Squared displacement since the last list build (FP32 offsets, home cell unchanged).
__device__ __forceinline__ float displacement2(const Dev& D, long long p, float4 g) {
  float4 r = D.ref[p];
  float dx = g.x - r.x, dy = g.y - r.y, dz = g.z - r.z;
  return dx * dx + dy * dy + dz * dz;
}

// Largest displacement^2 of a warp whose lanes all belong to system s (whole tiles/blocks).
__device__ __forceinline__ void track_displacement_warp(const Dev& D, int s, float d2) {
  unsigned m = __reduce_max_sync(0xffffffffu, (unsigned)__float_as_int(d2));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(&D.sst[s].maxdisp2, m);
}

__global__ void k_copyback(Dev D) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= D.N) return;
  int s = D.sysid[p];
  if (!D.sst[s].need_rebuild) return;
  const long long N = D.N;
  const double* sd = D.sdbl;
  D.x[p] = sd[0 * N + p];
  D.y[p] = sd[1 * N + p];
  D.z[p] = sd[2 * N + p];
  D.vx[p] = sd[3 * N + p];
  D.vy[p] = sd[4 * N + p];
  D.vz[p] = sd[5 * N + p];
  D.ax[p] = sd[6 * N + p];
  D.ay[p] = sd[7 * N + p];
  D.az[p] = sd[8 * N + p];
  D.mass[p] = sd[9 * N + p];
  D.fm[p] = sd[10 * N + p];
  const int* si = D.sint;
  D.type[p] = si[0 * N + p];
  D.tag[p] = si[1 * N + p];
  D.home[p] = si[2 * N + p];
  if (D.has_flags) D.flags[p] = D.sflags[p];
  if (D.ist)
    for (int k = 0; k < IST_K; ++k) D.ist[k * N + p] = D.ist_alt[k * N + p];
  refresh_gather(D, D.sysd[s], p, true);
}

// ---------------------------------------------------------------------------------------------
// Verlet list with cell-shift codes
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ int shift_code(int kx, int ky, int kz) { return (kx + 2) + 5 * ((ky + 2) + 5 * (kz + 2)); }

// One warp per home cell (per-block table of system and cells): the lanes hold up to 32 atoms
// of the cell, and the atoms of each stencil cell are staged through shared memory 32 at a
// time; every lane then tests the staged candidate against its own atom (broadcast reads, no
// divergence between lanes, since all atoms of a cell share the stencil and its cell-shift
// codes), and appends its hits in candidate order through a bit mask.
constexpr int LIST_WARPS = 4;
// Candidate tests four at a time over a sentinel-padded stage, appends through a running write
// position (1); or one candidate per iteration with the entry address recomputed per append (0).
#ifndef GBMD_LIST_UNROLL4
#define GBMD_LIST_UNROLL4 1
#endif
// Resident blocks per SM the register allocation of the list build is sized for.
#ifndef GBMD_LIST_MIN_BLOCKS
#define GBMD_LIST_MIN_BLOCKS 4
#endif

__global__ void __launch_bounds__(32 * LIST_WARPS, GBMD_LIST_MIN_BLOCKS) k_buildlist(Dev D) {
#if GBMD_LIST_UNROLL4 && GBMD_F32X2
  // coordinates staged as three arrays, so that one 16-byte shared load gives the x (y, z)
  // of four consecutive candidates: two packed pairs
  __shared__ __align__(16) float stage[LIST_WARPS][3][32];
#else
  __shared__ float4 stage[LIST_WARPS][32];
#endif
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // every block covers LIST_WARPS cells of one system (a per-block table), so the system
  // index is the same for the whole block and the grid holds no block of an empty range
  const int s = D.lblk_sys[blockIdx.x];
  const int g0 = D.lblk_cell[blockIdx.x] + w;
  if (g0 >= D.sysd[s].cell_base + D.sysd[s].ncells) return;
  if (!D.sst[s].need_rebuild) return;
  // the system's grid in registers: the list stores below may alias any global memory, so
  // fields read through the SysDev reference would be re-read after every store
  const SysDev& S = D.sysd[s];
  if (S.mode != NB_LIST) return;
  const int nx = S.n[0], ny = S.n[1], nz = S.n[2];
  const float dfx = S.df[0], dfy = S.df[1], dfz = S.df[2];
  const int cell_base = S.cell_base;
  const long long atom_base = S.atom_base;
  const float rlist2 = S.rlist2f;
  const int R = S.stencil_r;
  const int na = S.natoms;
  unsigned* const nl = D.nl + S.nl_base;
  const int* __restrict__ cstart = D.cstart;
  const int* __restrict__ ccnt = D.ccnt;
  const float4* __restrict__ g32 = D.g32;
  const int maxnb = D.maxnb;
  const int c = g0 - cell_base;
  const int b0 = cstart[g0], n0 = ccnt[g0];
  const int cx = c % nx, cy = (c / nx) % ny, cz = c / (nx * ny);
#if GBMD_LIST_UNROLL4 && GBMD_F32X2
  float* const stx = stage[w][0];
  float* const sty = stage[w][1];
  float* const stz = stage[w][2];
#else
  float4* st = stage[w];
#endif
  for (int base = 0; base < n0; base += 32) {
    const bool has = base + lane < n0;
    const long long i = (long long)b0 + base + lane;
    const int li = (int)(i - atom_base);
    const float4 gi = has ? g32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rl2 = has ? rlist2 : -1.0f;  // lanes without an atom never match
    unsigned* out = nl + (long long)li * 4;
    const long long gstride = (long long)na * 4;  // words between consecutive groups of four
    int cnt = 0;
#if GBMD_LIST_UNROLL4
    unsigned* wp = out;
#endif
    for (int dz = -R; dz <= R; ++dz) {
      const int zc = wrap_around(cz + dz, nz);
      const float sz = (float)dz * dfz;
      for (int dy = -R; dy <= R; ++dy) {
        const int yc = wrap_around(cy + dy, ny);
        const float sy = (float)dy * dfy;
        for (int dx = -R; dx <= R; ++dx) {
          const int xc = wrap_around(cx + dx, nx);
          const float sx = (float)dx * dfx;
          const int g = cell_base + (zc * ny + yc) * nx + xc;
          const int b = cstart[g], n = ccnt[g];
          const unsigned code = (unsigned)shift_code(dx, dy, dz) << CODE_SHIFT;
          const float ox = sx - gi.x, oy = sy - gi.y, oz = sz - gi.z;
#if GBMD_LIST_UNROLL4 && GBMD_F32X2
          const f32x2 ox2 = f2_pack(ox, ox), oy2 = f2_pack(oy, oy), oz2 = f2_pack(oz, oz);
#endif
          for (int jb = 0; jb < n; jb += 32) {
            __syncwarp();
#if GBMD_LIST_UNROLL4 && GBMD_F32X2
            {
              const float4 gj = jb + lane < n ? g32[b + jb + lane] : make_float4(1e18f, 1e18f, 1e18f, 0.f);
              stx[lane] = gj.x;
              sty[lane] = gj.y;
              stz[lane] = gj.z;
            }
#elif GBMD_LIST_UNROLL4
            // every stage slot is written: past the cell's atoms a far-away sentinel, so the test
            // loop runs in whole quads of candidates (the sentinel never hits: r^2 ~ 3e36)
            st[lane] = jb + lane < n ? g32[b + jb + lane] : make_float4(1e18f, 1e18f, 1e18f, 0.f);
#else
            if (jb + lane < n) st[lane] = g32[b + jb + lane];
#endif
            __syncwarp();
            const int m = min(32, n - jb);
            const int jl0 = b + jb - (int)atom_base;
            // pass 1: a bit per staged candidate inside the list radius (branch-free)
            unsigned hits = 0u;
#if GBMD_LIST_UNROLL4 && GBMD_F32X2
            for (int k = 0; k < m; k += 4) {
              // candidates k..k+3 as two packed pairs, in the scalar form's operation order
              const float4 X = *reinterpret_cast<const float4*>(stx + k);
              const float4 Y = *reinterpret_cast<const float4*>(sty + k);
              const float4 Z = *reinterpret_cast<const float4*>(stz + k);
              const f32x2 rx01 = f2_add(ox2, f2_pack(X.x, X.y)), rx23 = f2_add(ox2, f2_pack(X.z, X.w));
              const f32x2 ry01 = f2_add(oy2, f2_pack(Y.x, Y.y)), ry23 = f2_add(oy2, f2_pack(Y.z, Y.w));
              const f32x2 rz01 = f2_add(oz2, f2_pack(Z.x, Z.y)), rz23 = f2_add(oz2, f2_pack(Z.z, Z.w));
              const f32x2 q01 = f2_fma(rx01, rx01, f2_fma(ry01, ry01, f2_mul(rz01, rz01)));
              const f32x2 q23 = f2_fma(rx23, rx23, f2_fma(ry23, ry23, f2_mul(rz23, rz23)));
              float r0, r1, r2, r3;
              f2_unpack(q01, r0, r1);
              f2_unpack(q23, r2, r3);
              const unsigned nib = (r0 < rl2 ? 1u : 0u) | (r1 < rl2 ? 2u : 0u) | (r2 < rl2 ? 4u : 0u) |
                                   (r3 < rl2 ? 8u : 0u);
              hits |= nib << k;
            }
#elif GBMD_LIST_UNROLL4
            for (int k = 0; k < m; k += 4) {
              unsigned nib = 0u;
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const float4 gj = st[k + u];
                const float rx = ox + gj.x, ry = oy + gj.y, rz = oz + gj.z;
                const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                nib |= (r2 < rl2 ? 1u : 0u) << u;
              }
              hits |= nib << k;
            }
#else
            for (int k = 0; k < m; ++k) {
              const float4 gj = st[k];
              const float rx = ox + gj.x, ry = oy + gj.y, rz = oz + gj.z;
              const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
              hits |= (r2 < rl2 ? 1u : 0u) << k;
            }
#endif
            const int self = li - jl0;  // drop the atom itself
            if (self >= 0 && self < 32) hits &= ~(1u << self);
            // pass 2: append the hits in candidate order
            while (hits) {
              const int k = __ffs(hits) - 1;
              hits &= hits - 1u;
#if GBMD_LIST_UNROLL4
              // running write position: entry cnt of the atom lives at group cnt/4, slot cnt%4
              if (cnt < maxnb) *wp = code | (unsigned)(jl0 + k);
              wp += (cnt & 3) == 3 ? gstride - 3 : 1;
#else
              if (cnt < maxnb) out[(cnt >> 2) * gstride + (cnt & 3)] = code | (unsigned)(jl0 + k);
#endif
              ++cnt;
            }
          }
        }
      }
    }
    if (has) {
      D.ncount[i] = cnt < maxnb ? cnt : maxnb;
      atomicMax(&D.sst[s].max_count, cnt);
      if (cnt > maxnb) atomicOr(&D.sst[s].error, ERR_LIST);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Integration: drift half of velocity Verlet
// ---------------------------------------------------------------------------------------------

// Velocity rescaling between steps.  The temperature is measured afresh, as the modifiers do:
// k_kinetic_clear + k_scale_kinetic sum the kinetic energy of the current velocities into the
// system's int64 kinetic slot (2^-44 units; each warp's FP64 sum rounded once, so the total is
// order-independent), then k_scale_velocities scales.
//   mode 0, SimulationBuilder::SetTemperature (liblpmd/simulation/simulationbuilder.cc:53-72,
//     called by plugins/tempscaling.cc:66-71 and plugins/temperature.cc:58-62 with tag = "any
//     atom has fixedvel/fixedpos"): T over the untagged atoms, tagged atoms keep their velocity,
//     v *= sqrt(target / T);
//   mode 1, BerendsenModifier::Apply (plugins/berendsen.cc:72-99): T over all atoms
//     (lpmd::Temperature with tag false, liblpmd/lpmd/properties.h:40-53), every atom scaled by
//     sqrt(1 + dt/tau * (target / T - 1)).
// The kinetic slot is free between steps: the next force evaluation's decision clears it.
// A system at T = 0 is left as it is (the reference would divide by zero).
__global__ void k_kinetic_clear(Dev D) {
  for (int s = threadIdx.x; s < D.nsys; s += blockDim.x) D.sys_acc[(long long)s * SA_LEN + SA_KE] = 0ull;
}

__global__ void __launch_bounds__(TILE) k_scale_kinetic(Dev D, int sys, int mode) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  if ((sys >= 0 && s != sys) || !D.sysd[s].active) return;  // whole block: one tile, one system
  const long long i = D.tile_first[tile] + threadIdx.x;
  double ke = 0.0;
  if ((int)threadIdx.x < D.tile_count[tile] &&
      !(mode == 0 && D.has_flags && (D.flags[i] & (FLAG_FIXEDVEL | FLAG_FIXEDPOS)))) {
    const double vx = D.vx[i], vy = D.vy[i], vz = D.vz[i];
    ke = dmul(dmul(0.5, D.mass[i]), ref_sq(vx, vy, vz));
  }
  const double kw = warp_sum(ke);
  __shared__ long long part[TILE / 32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = __double2ll_rn(kw * FIX_KE);
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
    for (int w = 0; w < TILE / 32; ++w) t += part[w];
    atomicAdd(D.sys_acc + (long long)s * SA_LEN + SA_KE, (unsigned long long)t);
  }
}

__global__ void k_scale_velocities(Dev D, int sys, int mode, double target, double dt_over_tau) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  const int s = D.sysid[i];
  const SysDev& S = D.sysd[s];
  if ((sys >= 0 && s != sys) || !S.active) return;
  const double KIN2EV = 103.64269, KBOLTZMANN = 8.6173422E-05;  // liblpmd/lpmd/properties.h:10-11
  const double ke = (double)(long long)__ldcg(D.sys_acc + (long long)s * SA_LEN + SA_KE) * (1.0 / FIX_KE);
  const double kbn = mode == 0 ? S.kbn : dmul(KBOLTZMANN, (double)S.natoms);
  const double T = ddiv(dmul(2.0 / 3.0, dmul(ke, KIN2EV)), kbn);
  if (!(T > 0.0)) return;
  if (mode == 0 && D.has_flags && (D.flags[i] & (FLAG_FIXEDVEL | FLAG_FIXEDPOS))) return;
  const double f = mode == 0 ? sqrt(ddiv(target, T)) : sqrt(dadd(1.0, dmul(dt_over_tau, dsub(ddiv(target, T), 1.0))));
  D.vx[i] = dmul(D.vx[i], f);
  D.vy[i] = dmul(D.vy[i], f);
  D.vz[i] = dmul(D.vz[i], f);
}

// Centre of every Verlet-list cell: ((c + 1/2) * d) per axis, FP64.
__global__ void k_cell_centres(Dev D) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= D.total_cells) return;
  const SysDev& S = D.sysd[D.cell_sys[g]];
  const int c = g - S.cell_base;
  const int cx = c % S.n[0], cy = (c / S.n[0]) % S.n[1], cz = c / (S.n[0] * S.n[1]);
  D.ccentre[3 * (long long)g] = fma((double)cx, S.d[0], 0.5 * S.d[0]);
  D.ccentre[3 * (long long)g + 1] = fma((double)cy, S.d[1], 0.5 * S.d[1]);
  D.ccentre[3 * (long long)g + 2] = fma((double)cz, S.d[2], 0.5 * S.d[2]);
}

// VelocityVerlet::AdvancePosition of atom i from the evaluation buffer into the output buffer:
// newpos = x + v*dt + 0.5*a*dt*dt, then FittedInside.  The FP64 path rounds every product and
// sum separately as the reference does; the mixed path uses two FP64 fused multiply-adds per
// coordinate.  Returns the squared displacement since the last list build.
template <int MIXED>
__device__ __forceinline__ float drift_atom(const Dev& D, const SysDev& S, long long i, double dt, double h2,
                                            double vx, double vy, double vz, double ax, double ay, double az) {
  double nx = D.x[i], ny = D.y[i], nz = D.z[i];
  if (!(D.has_flags && (D.flags[i] & FLAG_FIXEDPOS))) {
    if (MIXED) {  // h2 = 0.5 * dt * dt
      nx = fma(h2, ax, fma(dt, vx, nx));
      ny = fma(h2, ay, fma(dt, vy, ny));
      nz = fma(h2, az, fma(dt, vz, nz));
    } else {
      nx = dadd(dadd(nx, dmul(vx, dt)), dmul(dmul(dmul(0.5, ax), dt), dt));
      ny = dadd(dadd(ny, dmul(vy, dt)), dmul(dmul(dmul(0.5, ay), dt), dt));
      nz = dadd(dadd(nz, dmul(vz, dt)), dmul(dmul(dmul(0.5, az), dt), dt));
    }
    nx = ref_fitted(nx, S.L[0]);
    ny = ref_fitted(ny, S.L[1]);
    nz = ref_fitted(nz, S.L[2]);
  }
  D.xo[i] = nx;
  D.yo[i] = ny;
  D.zo[i] = nz;
  float4 g = write_gather<!MIXED>(D, S, i, nx, ny, nz, D.type[i], D.g64o, D.g32o);
  return S.mode == NB_LIST ? displacement2(D, i, g) : 0.0f;
}

// Keeps an inactive system's committed positions in place across a launch that writes the
// other position buffer.  A fused force+drift launch reads the pending buffer (x) and writes
// the committed one (xo), after which the buffers swap roles: copy xo -> x (to_read = true).
// A stand-alone drift reads the committed buffer (x) and writes the pending one (xo): copy
// x -> xo (to_read = false).
__device__ __forceinline__ void hold_tile(const Dev& D, const SysDev& S, int tile, bool to_read) {
  if ((int)threadIdx.x >= D.tile_count[tile]) return;
  const long long i = D.tile_first[tile] + threadIdx.x;
  if (to_read) {
    D.x[i] = D.xo[i];
    D.y[i] = D.yo[i];
    D.z[i] = D.zo[i];
    D.g64[i] = D.g64o[i];
    if (S.mode == NB_LIST) D.g32[i] = D.g32o[i];
  } else {
    D.xo[i] = D.x[i];
    D.yo[i] = D.y[i];
    D.zo[i] = D.z[i];
    D.g64o[i] = D.g64[i];
    if (S.mode == NB_LIST) D.g32o[i] = D.g32[i];
  }
}

// Stand-alone drift (the first step of a run, before any fused force/drift launch).
template <int MIXED>
__global__ void __launch_bounds__(TILE) k_drift(Dev D, double dt, double h2) {
  const int tile = blockIdx.x;
  const int s = D.tile_sys[tile];
  const SysDev& S = D.sysd[s];
  if (!S.active) {
    hold_tile(D, S, tile, false);
    return;
  }
  const long long i = D.tile_first[tile] + threadIdx.x;
  float d2 = 0.0f;
  if ((int)threadIdx.x < D.tile_count[tile])
    d2 = drift_atom<MIXED>(D, S, i, dt, h2, D.vx[i], D.vy[i], D.vz[i], D.ax[i], D.ay[i], D.az[i]);
  track_displacement_warp(D, s, d2);
}

}  // namespace gbmd

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

enum EpiMode { EPI_FORCES = 0, EPI_KICK = 1 };

struct StepParams {
  double dt;
  double half_dt;       // 0.5 * dt, as AdvanceVelocity computes it
  int epi;              // EpiMode of the final force pass
  int first;            // first potential pass of this evaluation (overwrite partials)
  int last;             // last potential pass (write accelerations)
  int count_step;       // k_thermo advances the step counter
  int kinetic;          // compute kinetic sums in the epilogue
};

// ---------------------------------------------------------------------------------------------
// Rebuild decision
// ---------------------------------------------------------------------------------------------

// ucall_inc: how many emulated UpdateCell calls this evaluation stands for (verletlist "each").
__global__ void k_decide(Dev D, int nsys, int ucall_inc, int force_all, unsigned long long cond_handle,
                         int use_cond) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < nsys; s += blockDim.x) {
    const SysDev& S = D.sysd[s];
    SysState& st = D.sst[s];
    int need = force_all | st.force_rebuild;
    if (S.mode == NB_CELLS) need = 1;
    if (S.mode == NB_LIST) {
      float md2 = __int_as_float((int)st.maxdisp2);
      if ((S.rebuild_policy == REBUILD_SKIN || S.rebuild_policy == REBUILD_BOTH) && (double)md2 > S.thresh2)
        need = 1;
      if (S.rebuild_policy == REBUILD_EACH || S.rebuild_policy == REBUILD_BOTH) {
        for (int k = 0; k < ucall_inc; ++k)
          if (((st.ucalls + k) % S.each) == 0) need = 1;
      }
    }
    st.ucalls += ucall_inc;
    if (S.mode == NB_ALLPAIRS) need = 0;
    st.need_rebuild = need;
    st.force_rebuild = 0;
    if (need) {
      st.maxdisp2 = 0u;
      st.rebuilds += (S.mode == NB_LIST) ? 1 : 0;
      atomicOr(&any, 1);
    }
  }
  __syncthreads();
  if (use_cond && threadIdx.x == 0) cudaGraphSetConditional((cudaGraphConditionalHandle)cond_handle, any ? 1u : 0u);
}

// ---------------------------------------------------------------------------------------------
// Binning and counting sort
// ---------------------------------------------------------------------------------------------

__global__ void k_bin(Dev D) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  int s = D.sysid[i];
  if (!D.sst[s].need_rebuild) return;
  const SysDev& S = D.sysd[s];
  bool ok = true;
  int cx = ref_cell_coord(D.x[i], S.L[0], S.n[0], ok);
  int cy = ref_cell_coord(D.y[i], S.L[1], S.n[1], ok);
  int cz = ref_cell_coord(D.z[i], S.L[2], S.n[2], ok);
  if (!ok) {
    atomicOr(&D.sst[s].error, ERR_OUTSIDE);
    cx = cy = cz = 0;
  }
  int c = S.cell_base + (cz * S.n[1] + cy) * S.n[0] + cx;
  D.acell[i] = c;
  atomicAdd(&D.ccount[c], 1);
}

// One block per system: exclusive scan of the cell counts; resets counts and cursors.
__global__ void k_scan(Dev D) {
  const int s = blockIdx.x;
  if (!D.sst[s].need_rebuild) return;
  const SysDev& S = D.sysd[s];
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < S.ncells; base += blockDim.x) {
    int c = base + threadIdx.x;
    int v = (c < S.ncells) ? D.ccount[S.cell_base + c] : 0;
    int x = v;
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
    int excl = x - v + (w > 0 ? warp_tot[w - 1] : 0) + carry;
    if (c < S.ncells) {
      D.cstart[S.cell_base + c] = (int)(S.atom_base) + excl;  // global slot
      D.ccnt[S.cell_base + c] = v;
      D.ccount[S.cell_base + c] = 0;
      D.ccursor[S.cell_base + c] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
}

__global__ void k_scatter(Dev D) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  int s = D.sysid[i];
  if (!D.sst[s].need_rebuild) return;
  int c = D.acell[i];
  int p = D.cstart[c] + atomicAdd(&D.ccursor[c], 1);
  D.perm[p] = (int)i;
}

// One thread per cell (grid.y = system): insertion sort of the cell's slots by original index.
__global__ void k_cellsort(Dev D) {
  const int s = blockIdx.y;
  if (!D.sst[s].need_rebuild) return;
  const SysDev& S = D.sysd[s];
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S.ncells) return;
  int g = S.cell_base + c;
  int b = D.cstart[g], n = D.ccnt[g];
  for (int k = 1; k < n; ++k) {
    int v = D.perm[b + k];
    int tv = D.tag[v];
    int q = k - 1;
    while (q >= 0 && D.tag[D.perm[b + q]] > tv) {
      D.perm[b + q + 1] = D.perm[b + q];
      --q;
    }
    D.perm[b + q + 1] = v;
  }
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
}

// Offset of x from the centre of cell coordinate c (edge d), wrapped into [-L/2, L/2).
__device__ __forceinline__ float home_offset(double x, int c, double d, double L, double Lh) {
  double o = dsub(x, dmul(dadd((double)c, 0.5), d));
  if (o >= Lh) o = dsub(o, L);
  if (o < -Lh) o = dadd(o, L);
  return (float)o;
}

__device__ __forceinline__ void refresh_gather(const Dev& D, const SysDev& S, long long p, bool set_ref) {
  double xx = D.x[p], yy = D.y[p], zz = D.z[p];
  int t = D.type[p];
  D.g64[p] = make_double4_32a(xx, yy, zz, (double)t);
  if (S.mode == NB_LIST) {
    int h = D.home[p] - S.cell_base;
    int cx = h % S.n[0], cy = (h / S.n[0]) % S.n[1], cz = h / (S.n[0] * S.n[1]);
    float4 g = make_float4(home_offset(xx, cx, S.d[0], S.L[0], S.Lh[0]), home_offset(yy, cy, S.d[1], S.L[1], S.Lh[1]),
                           home_offset(zz, cz, S.d[2], S.L[2], S.Lh[2]), __int_as_float(t));
    D.g32[p] = g;
    if (set_ref) D.ref[p] = g;
  }
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
  refresh_gather(D, D.sysd[s], p, true);
}

// ---------------------------------------------------------------------------------------------
// Verlet list with cell-shift codes
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ int shift_code(int kx, int ky, int kz) { return (kx + 2) + 5 * ((ky + 2) + 5 * (kz + 2)); }

__global__ void k_buildlist(Dev D) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  int s = D.sysid[i];
  if (!D.sst[s].need_rebuild) return;
  const SysDev& S = D.sysd[s];
  if (S.mode != NB_LIST) return;
  const float4 gi = D.g32[i];
  const int h = D.home[i] - S.cell_base;
  const int cx = h % S.n[0], cy = (h / S.n[0]) % S.n[1], cz = h / (S.n[0] * S.n[1]);
  const int R = S.stencil_r;
  const long long li = i - S.atom_base;
  unsigned* out = D.nl + S.nl_base + li;
  const int na = S.natoms;
  int cnt = 0;
  for (int dz = -R; dz <= R; ++dz) {
    int zc = wrap_around(cz + dz, S.n[2]);
    float sz = (float)dz * S.df[2];
    for (int dy = -R; dy <= R; ++dy) {
      int yc = wrap_around(cy + dy, S.n[1]);
      float sy = (float)dy * S.df[1];
      for (int dx = -R; dx <= R; ++dx) {
        int xc = wrap_around(cx + dx, S.n[0]);
        float sx = (float)dx * S.df[0];
        int g = S.cell_base + (zc * S.n[1] + yc) * S.n[0] + xc;
        int b = D.cstart[g], e = b + D.ccnt[g];
        unsigned code = (unsigned)shift_code(dx, dy, dz) << CODE_SHIFT;
        for (int j = b; j < e; ++j) {
          if (j == i) continue;
          float4 gj = D.g32[j];
          float rx = (sx + gj.x) - gi.x, ry = (sy + gj.y) - gi.y, rz = (sz + gj.z) - gi.z;
          float r2 = rx * rx + ry * ry + rz * rz;
          if (r2 < S.rlist2f) {
            if (cnt < D.maxnb) out[(long long)cnt * na] = code | (unsigned)(j - S.atom_base);
            ++cnt;
          }
        }
      }
    }
  }
  D.ncount[i] = cnt < D.maxnb ? cnt : D.maxnb;
  atomicMax(&D.sst[s].max_count, cnt);
  if (cnt > D.maxnb) atomicOr(&D.sst[s].error, ERR_LIST);
}

// ---------------------------------------------------------------------------------------------
// Integration: drift half of velocity Verlet
// ---------------------------------------------------------------------------------------------

__global__ void k_drift(Dev D, double dt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  int s = D.sysid[i];
  const SysDev& S = D.sysd[s];
  bool fixed = D.has_flags && (D.flags[i] & FLAG_FIXEDPOS);
  if (!fixed) {
    // newpos = x + v*dt + 0.5*a*dt*dt, then FittedInside
    double nx = dadd(dadd(D.x[i], dmul(D.vx[i], dt)), dmul(dmul(dmul(0.5, D.ax[i]), dt), dt));
    double ny = dadd(dadd(D.y[i], dmul(D.vy[i], dt)), dmul(dmul(dmul(0.5, D.ay[i]), dt), dt));
    double nz = dadd(dadd(D.z[i], dmul(D.vz[i], dt)), dmul(dmul(dmul(0.5, D.az[i]), dt), dt));
    D.x[i] = ref_fitted(nx, S.L[0]);
    D.y[i] = ref_fitted(ny, S.L[1]);
    D.z[i] = ref_fitted(nz, S.L[2]);
  }
  refresh_gather(D, S, i, false);
  if (S.mode == NB_LIST) {
    float4 g = D.g32[i], r = D.ref[i];
    float dx = g.x - r.x, dy = g.y - r.y, dz = g.z - r.z;
    float d2 = dx * dx + dy * dy + dz * dz;
    unsigned bits = (unsigned)__float_as_int(d2);
    // aggregate the maximum over the lanes of the same system before the global atomic
    unsigned same = __match_any_sync(__activemask(), s);
    unsigned m = __reduce_max_sync(same, bits);
    if ((int)(threadIdx.x & 31) == __ffs(same) - 1) atomicMax(&D.sst[s].maxdisp2, m);
  }
}

}  // namespace gbmd

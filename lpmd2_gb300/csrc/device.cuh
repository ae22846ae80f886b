// device.cuh -- device-side data layout and helpers shared by the libgbmd kernels.
//
// Layout in HBM (one ensemble = one or many independent systems, atoms of a system
// contiguous, each system cell-sorted):
//   x,y,z / vx,vy,vz / ax,ay,az   FP64 structure-of-arrays master state, slot order
//   g64 (double4_32a)                 FP64 gather copy (x, y, z, type) for the FP64 force path
//   g32 (float4)                  position relative to the centre of the atom's home cell
//                                 (FP32) + type bits: the coalesced 16-byte gather of the
//                                 mixed path; differences of these offsets plus a per-pair
//                                 cell shift give r_ij without FP32 absolute-position loss
//   nl (uint32)                   Verlet list, column-major per system: entry k of local atom
//                                 i at nl_base + k*natoms + i; low 25 bits = local j, high 7
//                                 bits = cell-shift code (kx,ky,kz in -2..2)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace gbmd {

constexpr int TILE = 128;          // atoms per tile = threads per block of the per-atom kernels
constexpr int THERMO_LEN = 22;
constexpr int PART_D = 16;         // FP64 per-tile partial sums
constexpr int CODE_SHIFT = 25;
constexpr unsigned LOCAL_MASK = (1u << CODE_SHIFT) - 1u;
constexpr int MAX_SYSTEM_ATOMS = (1 << CODE_SHIFT);
constexpr double FIX_F = 4294967296.0;      // 2^32: force fixed-point scale (eV/A)
constexpr double FIX_E = 4294967296.0;      // 2^32: energy/virial/stress fixed-point scale (eV)
constexpr double FIX_RHO = 4294967296.0;    // 2^32: EAM density fixed-point scale

// Per-atom flag bits (GBMD_FLAG_FIXEDVEL / GBMD_FLAG_FIXEDPOS of gbmd.h)
constexpr unsigned char FLAG_FIXEDVEL = 1;
constexpr unsigned char FLAG_FIXEDPOS = 2;

// Error bits in SysState::error
constexpr int ERR_OUTSIDE = 1;     // atom far outside the box / NaN position
constexpr int ERR_LIST = 2;        // neighbour list capacity exceeded
constexpr int ERR_FIXED = 4;       // fixed-point range exceeded
constexpr int ERR_CELL = 8;        // cell occupancy beyond the sort capacity
constexpr int ERR_WAIT = 16;       // a bounded wait on an asynchronous copy gave up
// Shared-memory stages of the list ring (a power of two).  Two stages with two list groups per
// iteration keep the next iteration's rows in flight; every stage more takes shared memory from
// the L1 that serves the neighbour gathers (measured: 2 stages beat 4 by 3 % on the LJ force
// pass and 1.4 % on the copper passes, 8 stages lose 3 %).
#ifndef GBMD_RING
#define GBMD_RING 2
#endif
constexpr int RING = GBMD_RING;
static_assert((RING & (RING - 1)) == 0 && RING >= 2, "the list ring needs a power-of-two stage count");

// Per-tile partial-sum slots (FP64)
enum { PD_EPAIR = 0, PD_EEMBED = 1, PD_VIR = 2, PD_STRESS = 3, PD_KE = 12, PD_PX = 13 };
// Per-system int64 fixed-point accumulators of the mixed path (atomics from every block)
enum { SA_EPAIR = 0, SA_VIR = 1, SA_STRESS = 2, SA_KE = 11, SA_P = 12, SA_EEMBED = 15, SA_LEN = 16 };
// Integrator history slots (each N doubles): the old position / velocity / acceleration an
// integrator keeps (3), the previous old acceleration (3), the Nose-Hoover rank of the atom
// among the atoms that move (1), and the positions and accelerations put aside while the
// forces of the backed-up configuration are evaluated (3 + 3).
enum { IS_OLD = 0, IS_AUX = 3, IS_RANK = 6, IS_SAVEX = 7, IS_SAVEA = 10, IST_K = 13 };
// Nose-Hoover per-system record: friction after the last step, its increment per atom this
// step, friction before this step, number of atoms that move.
enum { NH_F = 0, NH_D = 1, NH_F0 = 2, NH_NMOVE = 3, NH_LEN = 4 };
constexpr double FIX_KE = 17592186044416.0;  // 2^44: kinetic energy (amu A^2/fs^2) and momentum

struct SysDev {
  long long atom_base;
  int natoms;
  int tile_base, ntiles;
  int mode;             // NbMode
  double L[3], Lh[3];   // box, 0.5*box
  // binning grid (list grid for NB_LIST, the reference grid for NB_CELLS)
  int n[3];
  int cell_base, ncells;
  int stencil_r;        // list stencil radius in cells (1 or 2)
  int lc_side;          // reference stencil side (NB_CELLS)
  double d[3];          // cell edge
  float df[3];
  float dfc[3];         // (d - df) / df: relative rounding of the FP32 cell edge (shift correction)
  float rlist2f;        // (cutoff + skin)^2 with a conservative margin
  double thresh2;       // rebuild when a displacement^2 exceeds this
  long long nl_base;
  int rebuild_policy;
  int each;
  int kind_cm;          // CmKind
  int nfree;            // atoms without fixedvel/fixedpos (Temperature's denominator)
  double vol;           // L0*L1*L2 (OrthogonalCell::Volume)
  double pv;            // pressfactor / volume
  double kbn;           // KBOLTZMANN * nfree
  double ninv[3];       // n / L: binning multiplier of the Verlet-list grid
  int active;           // 0: every kernel skips the system (its state is left as it was)
};

struct SysState {
  unsigned int maxdisp2;   // float bits of the largest displacement^2 since the last rebuild
  int need_rebuild;
  int force_rebuild;
  int max_count;
  int error;
  int collide;             // lcbinary: a sub-cell of the last re-sort holds two atoms
  long long rebuilds;
  long long ucalls;        // emulated UpdateCell calls (verletlist "each")
  long long step;
  unsigned long long rechecks;
};

struct Dev {
  long long N;
  // positions are double-buffered: (x, y, z, g32, g64) are the positions a launch evaluates
  // forces at; the fused drift writes the next step's positions into (xo, yo, zo, g32o, g64o)
  double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az;
  double *xo, *yo, *zo;
  float4* g32o;
  double4_32a* g64o;
  double *mass, *fm;
  int *type, *tag, *sysid;
  unsigned char* flags;
  double4_32a* g64;
  float4* g32;
  int* home;
  float4* ref;
  unsigned* nl;
  int* ncount;
  int maxnb;
  int *cstart, *ccnt, *ccount, *ccursor, *acell, *perm;
  int* cell_sys;     // system of each cell (flat cell index over every system)
  double* ccentre;   // cell centres (x, y, z per flat cell index) of Verlet-list grids
  int total_cells;
  int* lblk_sys;     // list-build blocks: system and first flat cell of each block
  int* lblk_cell;
  int list_blocks;
  // permutation scratch
  double* sdbl;   // 11*N doubles
  // integrator history of the integrators other than velocityverlet (IST_K*N doubles, moved
  // with the atoms when they are re-sorted; nullptr for velocityverlet), its re-sort scratch,
  // and the Nose-Hoover friction per system (NH_LEN doubles each)
  double* ist;
  double* ist_alt;
  double* nh;
  int* sint;      // 4*N ints
  unsigned char* sflags;
  // EAM
  double *rho, *phi;
  float* phif;
  float4* g32e;      // mixed density pass output: g32's offsets with the FP32 embedding factor
                     // 1/sqrt(rho) in w, gathered by the force pass of single-species systems
  // multi-potential accumulation
  long long* facc;   // 3*N fixed point
  double* dacc;      // 3*N FP64
  // SM-local tile claims of the mixed force and density passes: one counter per SM slot and a
  // completion counter (claim_slots + 1 entries, zero between launches)
  unsigned* tile_claim;
  int claim_slots;
  // per-system cell-shift tables (128 float4 per system, entries 0..124 used) for the mixed
  // passes that read them from global memory instead of shared memory (GBMD_SHIFTS_GLOBAL)
  float4* shift_tab;
  // reductions
  double* tile_d;
  unsigned long long* sys_acc;  // nsys * SA_LEN
  const SysDev* sysd;
  SysState* sst;
  const int* tile_sys;
  const int* tile_first;
  const int* tile_count;
  double* thermo_last;
  double* thermo_log;
  int log_cap;
  int has_flags;
  int nsys;
};

// Verlet-list layout: entries are stored in groups of four (16 bytes).  Group q of the local
// atom li of system S sits at uint4 index nl_base/4 + q*natoms + li, so a warp of consecutive
// atoms loads 512 contiguous bytes per group and each lane gets four entries per load.
__device__ __forceinline__ const uint4* list_group(const Dev& D, const SysDev& S, int li, int q) {
  return reinterpret_cast<const uint4*>(D.nl + S.nl_base) + (long long)q * S.natoms + li;
}
__device__ __forceinline__ unsigned* list_slot(const Dev& D, const SysDev& S, int li, int k) {
  return D.nl + S.nl_base + ((long long)(k >> 2) * S.natoms + li) * 4 + (k & 3);
}

// ---------------------------------------------------------------------------------------------
// FP64 helpers in the reference's rounding (no fused multiply-add anywhere)
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// One axis of OrthogonalCell::Displacement (liblpmd/lpmd/orthogonalcell.h:131-149).
__device__ __forceinline__ double ref_wrap(double d, double L, double Lh) {
  if (d >= Lh) return dsub(d, L);
  if (d < -Lh) return dadd(d, L);
  return d;
}

// Vector::SquareModule (liblpmd/lpmd/vector.h:107): (x*x + y*y) + z*z.
__device__ __forceinline__ double ref_sq(double x, double y, double z) {
  return dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z));
}

// One axis of OrthogonalCell::FittedInside (liblpmd/lpmd/orthogonalcell.h:102-114).
// The test (v < 0.0 || v > L) is decided on the bit patterns with integer compares instead of
// two compares on GB300's scarce FP64 pipe: v < 0 <=> sign bit set and v is not -0.0; for
// v >= +0, v > L <=> bits(v) > bits(L).  (A NaN is wrapped here and not in the reference; it
// stays NaN either way.)
__device__ __forceinline__ double ref_fitted(double v, double L) {
  const long long b = __double_as_longlong(v);
  if ((b < 0 && b != (long long)0x8000000000000000ULL) || b > __double_as_longlong(L))
    v = dsub(v, dmul(L, floor(ddiv(v, L))));
  return v;
}

// WrapAround (plugins/linkedcell.cc:9-15).
__device__ __forceinline__ int wrap_around(int i, int n) {
  if (i < 0)
    i += ((-i / n) + 1) * n;
  else if (i > n - 1)
    i -= (i / n) * n;
  return i;
}

// Cell coordinate of LinkedCell::UpdateCell (plugins/linkedcell.cc:249-253):
// WrapAround(int(floor(n * (x / L))), n).  ok=false for NaN / absurdly far positions.
__device__ __forceinline__ int ref_cell_coord(double x, double L, int n, bool& ok) {
  double t = floor(dmul((double)n, ddiv(x, L)));
  if (!(t > -1.0e9 && t < 1.0e9)) {
    ok = false;
    return 0;
  }
  return wrap_around((int)t, n);
}

// ---------------------------------------------------------------------------------------------
// Bulk asynchronous copies (TMA engine, non-tensor form) with mbarrier completion.
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Global -> shared bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Orders shared-memory reads made through ordinary loads (by this thread, or by threads that a
// preceding barrier synchronised with it) before this thread's next bulk copy into that memory.
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Waits for phase `phase` of the barrier with a bounded number of polls (each poll may suspend
// the thread for a hardware-defined interval).  Returns false if the bound was hit.
constexpr long long WAIT_POLLS = 1ll << 22;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned phase,
                                                  long long polls = WAIT_POLLS) {
  for (long long it = 0; it < polls; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

__device__ __forceinline__ int list_cell_coord(double t, int n, bool& ok) {
  double f = floor(t);
  if (!(f > -1.0e9 && f < 1.0e9)) {
    ok = false;
    return 0;
  }
  return wrap_around((int)f, n);
}

// ---------------------------------------------------------------------------------------------
// Reductions
// ---------------------------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum of NV values per thread; thread 0 gets the totals in out[].
template <typename T, int NV>
__device__ __forceinline__ void block_sum(T (&v)[NV], T* out) {
  __shared__ T sh[TILE / 32][NV];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    T s = warp_sum(v[k]);
    if (lane == 0) sh[w][k] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      T s = sh[0][k];
      for (int q = 1; q < TILE / 32; ++q) s += sh[q][k];
      out[k] = s;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------------------------
// Fixed-point accumulation on the FP32/INT pipes.
//
// GB300's FP64 unit (2 instructions/clock/SM) also executes every conversion to or from a
// 64-bit type, so __float2ll_rn per pair would make the force kernel FP64-bound.  Instead a
// scaled FP32 value y (|y| < 2^44) is split exactly as y = h*2^22 + l with integer h
// (|h| < 2^22) and |l| <= 2^21, and both parts are rounded to integers with the classic
// "add 1.5*2^23" trick (the integer lands in the low mantissa bits).  round(y) = h*2^22 +
// round(l) exactly, with round-half-even, so the int64 sums are exact and order-independent.
// ---------------------------------------------------------------------------------------------

constexpr float MAGIC = 12582912.0f;  // 1.5 * 2^23
constexpr int MAGIC_BITS = 0x4B400000;
constexpr float SPLIT = 4194304.0f;            // 2^22
constexpr float INV_SPLIT = 2.384185791015625e-07f;  // 2^-22

struct Fix {
  int hi = 0, lo = 0;
  __device__ __forceinline__ void add(float y) {
    float t = fmaf(y, INV_SPLIT, MAGIC);  // MAGIC + round(y / 2^22)
    float h = t - MAGIC;                  // exact
    float l = fmaf(-h, SPLIT, y);         // exact, |l| <= 2^21
    float u = l + MAGIC;                  // MAGIC + round(l)
    hi += __float_as_int(t) - MAGIC_BITS;
    lo += __float_as_int(u) - MAGIC_BITS;
  }
  // add(f * 2^32) for |f| < 2^12, with the scaling folded into the split (6 FP32/INT ops):
  // t = M + round(f*2^10); the remainder f - h*2^-10 is exact and |.| <= 2^-11.
  __device__ __forceinline__ void add_scaled32(float f) {
    float t = fmaf(f, 1024.0f, MAGIC);
    float h = t - MAGIC;
    float r = fmaf(-h, 9.765625e-04f, f);
    float u = fmaf(r, 4294967296.0f, MAGIC);
    hi += __float_as_int(t) - MAGIC_BITS;
    lo += __float_as_int(u) - MAGIC_BITS;
  }
  // add(f * 2^26) for |f| < 2^18: the energies and virials of a list group, whose range then
  // needs no check (a group beyond 2^18 eV implies forces far beyond the checked 4096 eV/A)
  __device__ __forceinline__ void add_scaled26(float f) {
    float t = fmaf(f, 16.0f, MAGIC);
    float h = t - MAGIC;
    float r = fmaf(-h, 0.0625f, f);
    float u = fmaf(r, 67108864.0f, MAGIC);
    hi += __float_as_int(t) - MAGIC_BITS;
    lo += __float_as_int(u) - MAGIC_BITS;
  }
  __device__ __forceinline__ long long value() const { return ((long long)hi << 22) + (long long)lo; }
};

// round(y) as int64 for one FP32 value (|y| < 2^44), FP32/INT pipes only.
__device__ __forceinline__ long long fix64(float y) {
  Fix f;
  f.add(y);
  return f.value();
}

// Approximate reciprocal (MUFU.RCP, <= 1 ulp).
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The hardware approximations above may err with a consistent sign, and raised to the high
// powers of the EAM functionals (r^-11, r^-8) a bias of 1e-7 becomes a systematic ~1e-6
// relative error of every pair term.  In the virial, where pair repulsion and many-body
// attraction cancel to a few percent, that showed up as a 1e-5 error.  One Newton step
// (y' = y + y (1 - x y^2) / 2, resp. y' = y + y (1 - x y)) leaves only the rounding of the
// step itself, which is unbiased.
__device__ __forceinline__ float rsqrt_nr(float x) {
  const float y = rsqrtf(x);
  const float e = fmaf(-x * y, y, 1.0f);
  return fmaf(0.5f * y, e, y);
}
__device__ __forceinline__ float rcp_nr(float x) {
  const float y = rcp_approx(x);
  return fmaf(y, fmaf(-x, y, 1.0f), y);
}

// Two FP32 values in one 64-bit register pair, operated on by the packed .f32x2 instructions
// (sm_100 and later): one instruction issue for two IEEE round-to-nearest results, each half
// rounded exactly as the scalar instruction rounds it, so a packed computation that keeps the
// scalar operation order gives bit-identical values.  GBMD_F32X2=0 selects the scalar forms.
#ifndef GBMD_F32X2
#define GBMD_F32X2 1
#endif
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(f32x2 v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// FP32 displacement and squared distance of a Verlet-list entry: cell shift of the entry's
// code plus the difference of the cell-relative offsets.  The force, density and neighbour
// export kernels all decide cutoffs on this value, so their pair sets agree bit for bit.
// The shift table holds k * (FP32 cell edge); the edge's rounding is the same for every pair
// that crosses a cell boundary, i.e. a uniform strain of the box of up to 6e-8, which the
// virial (stiff: pair repulsion and attraction cancel) amplifies.  With GBMD_SHIFT_CORR the
// exact edge is restored by one FMA per axis: dx + sh * (d - df) / df.
#ifndef GBMD_SHIFT_CORR
#define GBMD_SHIFT_CORR 1
#endif
struct ShiftCorr {
  float x, y, z;
};
__device__ __forceinline__ ShiftCorr shift_corr(const SysDev& S) {
  return ShiftCorr{S.dfc[0], S.dfc[1], S.dfc[2]};
}
template <bool PACKED = (GBMD_F32X2 != 0)>
__device__ __forceinline__ float entry_r2(const float4& gi, const float4& gj, const float4& sh, const ShiftCorr& c,
                                          float& dx, float& dy, float& dz) {
  if constexpr (PACKED) {
    // x and y as one packed pair (each float4's x, y sit in an aligned register pair)
    const f32x2 shxy = f2_pack(sh.x, sh.y);
    f32x2 dxy = f2_sub(f2_add(shxy, f2_pack(gj.x, gj.y)), f2_pack(gi.x, gi.y));
#if GBMD_SHIFT_CORR
    dxy = f2_fma(shxy, f2_pack(c.x, c.y), dxy);
#endif
    f2_unpack(dxy, dx, dy);
    dz = (sh.z + gj.z) - gi.z;
#if GBMD_SHIFT_CORR
    dz = fmaf(sh.z, c.z, dz);
#endif
  } else {
    dx = (sh.x + gj.x) - gi.x;
    dy = (sh.y + gj.y) - gi.y;
    dz = (sh.z + gj.z) - gi.z;
#if GBMD_SHIFT_CORR
    dx = fmaf(sh.x, c.x, dx);
    dy = fmaf(sh.y, c.y, dy);
    dz = fmaf(sh.z, c.z, dz);
#endif
  }
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

}  // namespace gbmd

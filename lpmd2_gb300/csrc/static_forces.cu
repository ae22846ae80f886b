// Pair forces of one small periodic system without any device allocation.
//
// The FP64 all-pairs pair-force pass (the minimum-image path of the force kernels in
// forces.cuh) rewritten so that its only scratch -- the per-block partial sums of energy,
// virial and stress -- lives in a fixed file-scope device array instead of the engine's
// allocated pools.  The caller brings the positions and receives forces and sums in device
// buffers it owns; this file allocates nothing, at set-up or per call.
//
// Set-up: the first call on a device (with that device current) looks up the array's device
// address with cudaGetSymbolAddress, which may load the module; the address is cached per
// device for the life of the process.  cudaDeviceReset unloads the module and invalidates the
// cached address, so a process that resets a device must not call this entry point on that
// device afterwards.  Calls from several host threads or streams share the one array per device
// and therefore must not overlap in time on the same device.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/gbmd.h"
#include "device.cuh"
#include "engine.h"
#include "potentials.cuh"

namespace gbmd {

namespace {

constexpr int ST_THREADS = 128;
constexpr int ST_MAX_ATOMS = GBMD_STATIC_MAX_ATOMS;
constexpr int ST_MAX_BLOCKS = (ST_MAX_ATOMS + ST_THREADS - 1) / ST_THREADS;
constexpr int ST_PART = 11;  // pair energy, virial, stress (9)
constexpr int ST_MAX_DEVICES = 64;
// block_sum (device.cuh) reduces one value per thread of a TILE-thread block
static_assert(ST_THREADS == TILE, "k_pair_forces_static launches TILE threads per block");

// Per-block partial sums (128 blocks x 11 doubles = 11 KB).  Each call's force launch writes
// the slots of every block it runs before the reduction launch reads them, so nothing in the
// array has to start at zero and nothing is carried from one call to the next.
static __device__ __align__(256) double g_static_scratch[ST_MAX_BLOCKS * ST_PART];

double* g_scratch_ptr[ST_MAX_DEVICES] = {};
std::mutex g_scratch_mu;

double* scratch_for_current_device() {
  int dev = 0;
  cudaError_t rc = cudaGetDevice(&dev);
  if (rc != cudaSuccess) throw Error(GBMD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(rc));
  if (dev < 0 || dev >= ST_MAX_DEVICES) throw Error(GBMD_ERR_CUDA, "device ordinal beyond the supported range");
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    double* p = nullptr;
    rc = cudaGetSymbolAddress((void**)&p, g_static_scratch);
    if (rc != cudaSuccess)
      throw Error(GBMD_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(rc));
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

// One thread per atom i; j runs over every other atom in index order.  The reference visits
// each pair once (j > i, plugins/minimumimage.cc:91) and applies the pair force to both atoms
// (liblpmd/simulation/pairpotential.cc:50-75); here each pair is seen from both ends, so the
// energy, virial and stress sums are halved.
__global__ void __launch_bounds__(ST_THREADS)
    k_pair_forces_static(PotParams P, const double* __restrict__ pos, int n, double Lx, double Ly, double Lz,
                         double* __restrict__ force, double* __restrict__ part) {
  const int i = blockIdx.x * ST_THREADS + threadIdx.x;
  const double Lhx = 0.5 * Lx, Lhy = 0.5 * Ly, Lhz = 0.5 * Lz;
  double v[ST_PART];
  for (int k = 0; k < ST_PART; ++k) v[k] = 0.0;
  if (i < n) {
    const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
    double fx = 0.0, fy = 0.0, fz = 0.0, ep = 0.0, vir = 0.0;
    double sxx = 0.0, sxy = 0.0, sxz = 0.0, syy = 0.0, syz = 0.0, szz = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const double dx = ref_wrap(dsub(pos[3 * j], xi), Lx, Lhx);
      const double dy = ref_wrap(dsub(pos[3 * j + 1], yi), Ly, Lhy);
      const double dz = ref_wrap(dsub(pos[3 * j + 2], zi), Lz, Lhz);
      const double r2 = ref_sq(dx, dy, dz);
      if (r2 < P.rc2) {
        double g, e;
        lj_pair64(P, r2, g, e);
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
    }
    force[3 * i] = fx;
    force[3 * i + 1] = fy;
    force[3 * i + 2] = fz;
    const double w[ST_PART] = {ep, vir, sxx, sxy, sxz, sxy, syy, syz, sxz, syz, szz};
    for (int k = 0; k < ST_PART; ++k) v[k] = 0.5 * w[k];
  }
  double tot[ST_PART];
  block_sum<double, ST_PART>(v, tot);
  if (threadIdx.x == 0)
    for (int k = 0; k < ST_PART; ++k) part[blockIdx.x * ST_PART + k] = tot[k];
}

// Sums the blocks' partials in block order (one thread per output value).
__global__ void k_pair_sums_static(const double* __restrict__ part, int nblocks, double* __restrict__ out) {
  const int k = threadIdx.x;
  if (k >= ST_PART) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += part[b * ST_PART + k];
  out[k] = s;
}

}  // namespace

void pair_forces_static(const PotParams& P, const double* pos, int n, const double* box, double* force, double* out,
                        void* stream_handle) {
  cudaStream_t stream = (cudaStream_t)stream_handle;
  if (n < 1 || n > ST_MAX_ATOMS)
    throw Error(GBMD_ERR_INVALID, "gbmd_pair_forces_static: n = " + std::to_string(n) +
                                      " atoms is outside 1.." + std::to_string(ST_MAX_ATOMS) +
                                      ", the capacity of its fixed scratch array");
  if (P.kind != POT_LJ)
    throw Error(GBMD_ERR_INVALID, "gbmd_pair_forces_static: only pair potentials (lennardjones) are supported");
  for (int a = 0; a < 3; ++a)
    if (!(box[a] > 0.0)) throw Error(GBMD_ERR_INVALID, "gbmd_pair_forces_static: box lengths must be positive");
  double* part = scratch_for_current_device();
  const int nblocks = (n + ST_THREADS - 1) / ST_THREADS;
  k_pair_forces_static<<<nblocks, ST_THREADS, 0, stream>>>(P, pos, n, box[0], box[1], box[2], force, part);
  k_pair_sums_static<<<1, 32, 0, stream>>>(part, nblocks, out);
  cudaError_t rc = cudaGetLastError();
  if (rc != cudaSuccess)
    throw Error(GBMD_ERR_CUDA, std::string("gbmd_pair_forces_static launch: ") + cudaGetErrorString(rc));
}

}  // namespace gbmd

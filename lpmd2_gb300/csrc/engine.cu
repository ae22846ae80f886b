// engine.cu -- host runtime of libgbmd: device memory of an ensemble of independent systems,
// configuration of the neighbour machinery, and the step pipeline (direct launches or CUDA
// graphs whose list rebuild sits behind a device-decided conditional node).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>

#include <nvtx3/nvToolsExt.h>

#include "forces.cuh"
#include "integrators.cuh"

namespace gbmd {

namespace {

// Device allocations and frees may synchronise the device, which must not happen while
// another thread's engine captures a CUDA graph; this process-wide lock keeps the two apart
// (engines driven from several host threads, as the job server does).
std::recursive_mutex g_dev_mu;

template <class T>
cudaError_t dev_malloc(T** p, size_t bytes) {
  std::lock_guard<std::recursive_mutex> lk(g_dev_mu);
  return cudaMalloc((void**)p, bytes);
}

void dev_free(void* p) {
  if (!p) return;
  std::lock_guard<std::recursive_mutex> lk(g_dev_mu);
  cudaFree(p);
}

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(5, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

#define CK(x) ck((x), #x)

// Automatic subdivision of LinkedCell, plugins/linkedcell.cc:146-204 (one axis).
// LCBinary's automatic grid (plugins/lcbinary.cc:52-107): sub-cells near cutoff/5 wide, the
// count rounded up to even.
int lcb_auto_n(double len, double cutoff) {
  double fnn = cutoff / 5.0;
  int n = 1;
  for (;;) {
    double previo = std::fabs(len / n - fnn);
    n++;
    double actual = std::fabs(len / n - fnn);
    if (actual < 1E-3) break;
    if (actual > previo) {
      n--;
      break;
    }
  }
  if ((n % 2) != 0) n++;
  return n;
}

int lc_auto_n(double len, double cutoff) {
  double fnn = (cutoff / 2.5);
  int n = 1;
  for (;;) {
    double previo = std::fabs(len / n - fnn);
    n++;
    double actual = std::fabs(len / n - fnn);
    if (actual < 1E-3) break;
    if (actual > previo) {
      n--;
      break;
    }
  }
  if ((n % 2) != 0) n--;
  return n;
}

inline unsigned nblocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// NVTX range over a host call (visible in Nsight Systems / ncu timelines; a no-op without a
// tool attached).
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};

}  // namespace

// ------------------------------------------------------------------------------------------
// Layout kernels
// ------------------------------------------------------------------------------------------

__global__ void k_init_layout(Dev D, int s, long long base, int n, int cell_base) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  long long i = base + k;
  D.sysid[i] = s;
  D.tag[i] = k;
  D.home[i] = cell_base;
}

// Writes caller-order (tag-indexed) interleaved host data into the slot-ordered SoA arrays.
__global__ void k_set_atoms(Dev D, long long base, int n, const double* pos, const double* vel,
                            const double* acc, const int* Z, const double* mass) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  long long i = base + k;
  int t = D.tag[i];
  if (pos) {
    D.x[i] = pos[3 * t];
    D.y[i] = pos[3 * t + 1];
    D.z[i] = pos[3 * t + 2];
  }
  if (vel) {
    D.vx[i] = vel[3 * t];
    D.vy[i] = vel[3 * t + 1];
    D.vz[i] = vel[3 * t + 2];
  }
  if (acc) {
    D.ax[i] = acc[3 * t];
    D.ay[i] = acc[3 * t + 1];
    D.az[i] = acc[3 * t + 2];
  }
  if (Z) D.type[i] = Z[t];
  if (mass) {
    D.mass[i] = mass[t];
    D.fm[i] = ddiv(0.00964853, mass[t]);  // forcefactor / Mass(), pairpotential.cc:62
  }
  D.g64[i] = make_double4_32a(D.x[i], D.y[i], D.z[i], (double)D.type[i]);
}

__global__ void k_set_flags(Dev D, long long base, int n, const unsigned char* flags) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  long long i = base + k;
  D.flags[i] = flags ? flags[D.tag[i]] : 0;
}

__global__ void k_get_atoms(Dev D, long long base, int n, double* pos, double* vel, double* acc) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  long long i = base + k;
  int t = D.tag[i];
  if (pos) {
    pos[3 * t] = D.x[i];
    pos[3 * t + 1] = D.y[i];
    pos[3 * t + 2] = D.z[i];
  }
  if (vel) {
    vel[3 * t] = D.vx[i];
    vel[3 * t + 1] = D.vy[i];
    vel[3 * t + 2] = D.vz[i];
  }
  if (acc) {
    acc[3 * t] = D.ax[i];
    acc[3 * t + 1] = D.ay[i];
    acc[3 * t + 2] = D.az[i];
  }
}

// Neighbour export: the pairs the force kernels would use, by original index.
// half: 0 full, 1 keep j < i (LinkedCell), 2 keep j > i (VerletList / MinimumImage).
template <int NB, int MIXED>
__global__ void k_export(Dev D, int s, double rc2, float rc2_lo, float rc2_hi, int half, long long* counts,
                         const long long* offsets, long long* idx) {
  __shared__ float4 shifts[125];
  const SysDev& S = D.sysd[s];
  if (MIXED) load_shifts(S, shifts);
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.natoms) return;
  long long i = S.atom_base + k;
  const int ti = D.tag[i];
  long long cnt = 0;
  long long o = offsets ? offsets[ti] : 0;
  const float4 gi = D.g32[i];
  const double4_32a pi = D.g64[i];
  for_each_candidate<NB>(D, S, i, [&](long long j, unsigned code) {
    bool in;
    if (MIXED) {
      // the force and density kernels' own decision: entry_r2, inside below rc2_lo, the exact
      // FP64 test in the guard band [rc2_lo, rc2_hi)
      float dx, dy, dz;
      const float r2 = entry_r2(gi, D.g32[j], shifts[code], shift_corr(S), dx, dy, dz);
      in = r2 < rc2_lo || (r2 < rc2_hi && exact_inside(D, S, i, j, rc2));
    } else {
      const double4_32a pj = D.g64[j];
      double dx = ref_wrap(dsub(pj.x, pi.x), S.L[0], S.Lh[0]);
      double dy = ref_wrap(dsub(pj.y, pi.y), S.L[1], S.Lh[1]);
      double dz = ref_wrap(dsub(pj.z, pi.z), S.L[2], S.Lh[2]);
      in = ref_sq(dx, dy, dz) < rc2;
    }
    const int tj = D.tag[j];
    if (half == 1 && tj > ti) in = false;
    if (half == 2 && tj < ti) in = false;
    if (in) {
      if (idx) idx[o + cnt] = tj;
      ++cnt;
    }
  });
  if (counts) counts[ti] = cnt;
}

__global__ void k_cells_out(Dev D, int s, long long* cell, long long* order) {
  const SysDev& S = D.sysd[s];
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.natoms) return;
  long long i = S.atom_base + k;
  cell[D.tag[i]] = D.home[i] - S.cell_base;
  order[k] = D.tag[i];
}

// Failure path of the bounded waits: one warp waits, with the force kernel's mbar_wait_bounded,
// on an mbarrier phase that nothing completes (no arrival, no copy in flight); after `polls`
// polls it gives up, records that in *gave_up and returns.
__global__ void k_wait_selftest(long long polls, int* gave_up) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncwarp();
  const bool done = mbar_wait_bounded(&bar, 0u, polls);
  if (threadIdx.x == 0) *gave_up = done ? 0 : 1;
}

__global__ void k_clear_state(Dev D, int nsys) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  D.sst[s].force_rebuild = 1;
  D.sst[s].maxdisp2 = 0u;
  D.sst[s].max_count = 0;
  D.sst[s].error = 0;
}

// ------------------------------------------------------------------------------------------
// Engine implementation
// ------------------------------------------------------------------------------------------

// Pair potentials (LennardJones, FastLJ) run the pair kernels; the rest are metal potentials.
inline bool pair_kind(int k) { return k == POT_LJ || k == POT_FASTLJ; }

// FastLJ::Tabulate (plugins/fastlj.cc:38-54): LJ at the lower edge r = cutoff i / bins of every
// bin, energies then force factors.
static std::vector<double> fastlj_table(double sigma, double epsilon, double cutoff, long bins) {
  std::vector<double> t(2 * (size_t)bins);
  for (long i = 0; i < bins; ++i) {
    double r = cutoff * double(i) / double(bins);
    double r6 = std::pow(sigma / r, 6.0e0);
    double r12 = r6 * r6;
    t[i] = 4.0e0 * epsilon * (r12 - r6);
    t[bins + i] = -48.0e0 * (epsilon / (r * r)) * (r12 - 0.50e0 * r6);
  }
  return t;
}

struct Engine::Impl {
  int device = 0;
  cudaStream_t stream = nullptr, stream2 = nullptr;
  int nsys = 0;
  std::vector<int64_t> natoms;
  std::vector<std::array<double, 3>> cells;
  std::vector<long long> atom_base;
  long long N = 0;

  CellManagerCfg cm;
  bool have_cm = false;
  std::vector<PotParams> pots;
  IntegratorCfg integ;
  bool have_integ = false;
  int precision = 0;

  // options
  double opt_skin = -1.0;
  int graph_block = 10;
  int graph_mode = 2;  // 0 direct, 1 captured, 2 captured with conditional rebuild
  int lanes = 1;       // lanes per atom of the mixed LJ force pass
  int list_feed = 0;   // list rows of the mixed passes: 0 auto, 1 registers, 2 ring
  int stencil_r = 1;
  int log_cap = 1024;

  std::vector<SysDev> sysd;
  std::vector<int> tile_sys, tile_first, tile_count;
  int ntiles = 0;
  int total_cells = 0;
  bool any_list = false;
  std::vector<std::array<int, 3>> lcb_n;  // lcbinary grids per system (they only grow)

  // LCBinary's stencil half-width: ceil(cutoff / d - 0.5) with d the narrowest sub-cell edge
  // (plugins/lcbinary.cc:113-119).
  static int lcb_side(const double* L, const int* n, double cutoff) {
    double d = L[0] / double(n[0]);
    if (L[1] / double(n[1]) < d) d = L[1] / double(n[1]);
    if (L[2] / double(n[2]) < d) d = L[2] / double(n[2]);
    int side = int(std::ceil((cutoff / d) - 0.5));
    return side < 0 ? 0 : side;
  }
  bool lcb_exact() const { return cm.kind == CM_LCBINARY && precision == PREC_FP64; }

  // After a re-sort on lcbinary grids: while some sub-cell holds two atoms, grow that system's
  // grid by 2 per axis and re-sort (LCBinary::UpdateCell, plugins/lcbinary.cc:176-193).
  void lcb_grow_until_single(cudaStream_t s) {
    for (int round = 0; round < 64; ++round) {
      k_binary_collide<<<nblocks(D.total_cells, 256), 256, 0, s>>>(D);
      launched();
      std::vector<SysState> hs(nsys);
      CK(cudaMemcpyAsync(hs.data(), d_sst, sizeof(SysState) * nsys, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      bool any = false;
      for (int q = 0; q < nsys; ++q)
        if (hs[q].collide) {
          any = true;
          for (int a = 0; a < 3; ++a) lcb_n[q][a] += 2;
        }
      if (!any) return;
      k_binary_clear<<<1, 256, 0, s>>>(D);
      launched();
      lcb_apply_grids(s);
      launch_rebuild_kernels(s);
    }
    throw Error(7, "lcbinary: no collision-free grid after 64 enlargements");
  }

  // New geometry for every system from lcb_n (cell bases move) and a fresh cell pool.
  void lcb_apply_grids(cudaStream_t s) {
    total_cells = 0;
    for (int q = 0; q < nsys; ++q) {
      SysDev& S = sysd[q];
      for (int a = 0; a < 3; ++a) S.n[a] = lcb_n[q][a];
      S.lc_side = lcb_side(S.L, S.n, cm.cutoff);
      for (int a = 0; a < 3; ++a) {
        S.d[a] = S.L[a] / (double)S.n[a];
        S.df[a] = (float)S.d[a];
        S.dfc[a] = (float)((S.d[a] - (double)S.df[a]) / (double)S.df[a]);
        S.ninv[a] = (double)S.n[a] / S.L[a];
      }
      S.ncells = S.n[0] * S.n[1] * S.n[2];
      S.cell_base = total_cells;
      total_cells += S.ncells;
    }
    for (int a = 0; a < 3; ++a) st.cell_grid[a] = sysd[0].n[a];
    free_cells();
    alloc_cells(total_cells);
    alloc_list(0);
    upload_sysd();
    k_cell_centres<<<nblocks(total_cells, 256), 256, 0, s>>>(D);
    launched();
  }

  Dev D{};
  SysDev* d_sysd = nullptr;
  SysState* d_sst = nullptr;
  int *d_tile_sys = nullptr, *d_tile_first = nullptr, *d_tile_count = nullptr;
  std::vector<std::pair<void*, size_t>> allocs;       // set-up pool: (pointer, bytes)
  std::vector<std::pair<void*, size_t>> cell_allocs;  // grid pool (cells, then the list last)
  size_t bytes = 0, cell_bytes = 0;
  bool configured = false, forces_valid = false, initialized = false, flags_any = false;
  Stats st;

  // double-buffered positions: cbuf holds the committed positions of the last completed step;
  // when pend is set, the other buffer already holds the drifted positions of the next step
  double* Pbuf[2] = {nullptr, nullptr};
  double4_32a* G64buf[2] = {nullptr, nullptr};
  float4* G32buf[2] = {nullptr, nullptr};
  int cbuf = 0;
  bool pend = false;

  // Points the launch descriptor at buffer `in` (evaluation) and 1-in (drift output).
  void set_buffers(int in) {
    const size_t n = (size_t)N;
    D.x = Pbuf[in];
    D.y = Pbuf[in] + n;
    D.z = Pbuf[in] + 2 * n;
    D.g64 = G64buf[in];
    D.g32 = G32buf[in];
    D.xo = Pbuf[1 - in];
    D.yo = Pbuf[1 - in] + n;
    D.zo = Pbuf[1 - in] + 2 * n;
    D.g64o = G64buf[1 - in];
    D.g32o = G32buf[1 - in];
  }

  cudaGraphExec_t gexec = nullptr;
  cudaGraph_t graph = nullptr;
  int gsteps = 0;
  int gparity = -1;  // cbuf the graph was captured for
  std::map<int, long long> read_from;  // next thermo-log step to hand out, per system
  int pending_ucalls = 0;              // UpdateCell calls owed to SetCellManager

  // kernel timing with CUDA events on the simulation's stream (direct launches only)
  enum { T_FORCE = 0, T_DRIFT = 1, T_REBUILD = 2 };
  int time_kernels = 0;
  bool capturing = false;
  struct Mark {
    cudaEvent_t a, b;
    int cls;
  };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t open_event[3] = {nullptr, nullptr, nullptr};

  bool timing() const { return time_kernels && !capturing; }
  cudaEvent_t get_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    return e;
  }
  void mark_begin(cudaStream_t s, int cls) {
    if (!timing()) return;
    open_event[cls] = get_event();
    CK(cudaEventRecord(open_event[cls], s));
  }
  void mark_end(cudaStream_t s, int cls) {
    if (!timing() || !open_event[cls]) return;
    cudaEvent_t e = get_event();
    CK(cudaEventRecord(e, s));
    marks.push_back({open_event[cls], e, cls});
    open_event[cls] = nullptr;
  }
  // Called after the stream was synchronised.
  void collect_marks() {
    for (const auto& m : marks) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) {
        if (m.cls == T_FORCE) {
          st.force_ms += ms;
          st.force_launches++;
        } else if (m.cls == T_DRIFT) {
          st.drift_ms += ms;
          st.drift_launches++;
        } else {
          st.rebuild_ms += ms;
          st.rebuild_launches++;
        }
      }
      cudaGetLastError();
      event_pool.push_back(m.a);
      event_pool.push_back(m.b);
    }
    marks.clear();
  }

  template <class T>
  T* alloc(size_t n, bool cellpool = false) {
    void* p = nullptr;
    size_t b = sizeof(T) * (n ? n : 1);
    cudaError_t e = dev_malloc(&p, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw Error(6, "device allocation of " + std::to_string(b) + " bytes failed: " + cudaGetErrorString(e));
    }
    CK(cudaMemsetAsync(p, 0, b, stream));
    (cellpool ? cell_allocs : allocs).emplace_back(p, b);
    (cellpool ? cell_bytes : bytes) += b;
    return (T*)p;
  }

  void free_cells() {
    for (auto& a : cell_allocs) dev_free(a.first);
    cell_allocs.clear();
    cell_bytes = 0;
  }

  void drop_graph() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr;
    graph = nullptr;
    gsteps = 0;
    gparity = -1;
  }

  void launched(int n = 1) { st.kernel_launches += n; }

  void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(5, std::string("kernel launch (") + what + "): " + cudaGetErrorString(e));
  }

  // --------------------------------------------------------------------------------------
  void setup(int dev, const std::vector<int64_t>& na, const std::vector<std::array<double, 3>>& cl) {
    device = dev;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
      cudaGetLastError();
      throw Error(5, "no CUDA device available: libgbmd runs only on the GPU");
    }
    if (dev < 0 || dev >= count) throw Error(1, "device index out of range");
    CK(cudaSetDevice(dev));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    natoms = na;
    cells = cl;
    nsys = (int)na.size();
    if (nsys <= 0) throw Error(1, "at least one system is required");
    atom_base.resize(nsys);
    long long b = 0;
    for (int s = 0; s < nsys; ++s) {
      if (na[s] < 0 || na[s] >= MAX_SYSTEM_ATOMS)
        throw Error(1, "atoms per system must be in [0, " + std::to_string(MAX_SYSTEM_ATOMS) + ")");
      for (int q = 0; q < 3; ++q)
        if (!(cl[s][q] > 0.0)) throw Error(1, "cell lengths must be positive");
      atom_base[s] = b;
      b += na[s];
    }
    N = b;
    // tiles
    for (int s = 0; s < nsys; ++s) {
      for (long long k = 0; k < na[s]; k += TILE) {
        tile_sys.push_back(s);
        tile_first.push_back((int)(atom_base[s] + k));
        tile_count.push_back((int)std::min<long long>(TILE, na[s] - k));
      }
    }
    ntiles = (int)tile_sys.size();
    sysd.resize(nsys);
    int tb = 0;
    for (int s = 0; s < nsys; ++s) {
      SysDev& S = sysd[s];
      std::memset(&S, 0, sizeof(S));
      S.atom_base = atom_base[s];
      S.natoms = (int)na[s];
      S.tile_base = tb;
      S.ntiles = (int)((na[s] + TILE - 1) / TILE);
      tb += S.ntiles;
      for (int q = 0; q < 3; ++q) {
        S.L[q] = cl[s][q];
        S.Lh[q] = 0.5 * cl[s][q];
      }
      S.n[0] = S.n[1] = S.n[2] = 1;
      S.ncells = 1;
      S.nfree = S.natoms;
      S.vol = (cl[s][0] * cl[s][1]) * cl[s][2];
      S.pv = 160217.65 / S.vol;  // pressfactor / Cell().Volume() (simulationbuilder.cc:86,112)
      S.kbn = 8.6173422E-05 * (double)S.nfree;
      S.each = 1;
      S.active = 1;
    }
    // per-atom arrays
    const size_t n = (size_t)N;
    D.N = N;
    double* st6 = alloc<double>(6 * n);
    D.vx = st6;
    D.vy = st6 + n;
    D.vz = st6 + 2 * n;
    D.ax = st6 + 3 * n;
    D.ay = st6 + 4 * n;
    D.az = st6 + 5 * n;
    for (int b = 0; b < 2; ++b) {
      Pbuf[b] = alloc<double>(3 * n);
      G64buf[b] = alloc<double4_32a>(n);
      G32buf[b] = alloc<float4>(n);
    }
    set_buffers(0);
    D.mass = alloc<double>(n);
    D.fm = alloc<double>(n);
    D.type = alloc<int>(n);
    D.tag = alloc<int>(n);
    D.sysid = alloc<int>(n);
    D.flags = alloc<unsigned char>(n);
    D.home = alloc<int>(n);
    D.ref = alloc<float4>(n);
    D.acell = alloc<int>(n);
    D.perm = alloc<int>(n);
    D.sdbl = alloc<double>(11 * n);
    D.sint = alloc<int>(4 * n);
    D.sflags = alloc<unsigned char>(n);
    D.ncount = alloc<int>(n);
    D.rho = alloc<double>(n);
    D.phi = alloc<double>(n);
    D.phif = alloc<float>(n);
    D.facc = alloc<long long>(3 * n);
    D.dacc = alloc<double>(3 * n);
    D.tile_d = alloc<double>((size_t)ntiles * PART_D);
    {
      int nsm = 0;
      CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
      D.claim_slots = nsm > 0 ? nsm : 1;
      D.tile_claim = alloc<unsigned>((size_t)D.claim_slots + 1);  // zeroed
    }
    D.shift_tab = alloc<float4>((size_t)nsys * 128);
    D.sys_acc = alloc<unsigned long long>((size_t)nsys * SA_LEN);
    D.thermo_last = alloc<double>((size_t)nsys * THERMO_LEN);
    D.log_cap = log_cap;
    D.nsys = nsys;
    D.thermo_log = alloc<double>((size_t)nsys * log_cap * THERMO_LEN);
    d_sysd = alloc<SysDev>(nsys);
    d_sst = alloc<SysState>(nsys);
    d_tile_sys = alloc<int>(ntiles);
    d_tile_first = alloc<int>(ntiles);
    d_tile_count = alloc<int>(ntiles);
    CK(cudaMemcpyAsync(d_tile_sys, tile_sys.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tile_first, tile_first.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tile_count, tile_count.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, stream));
    D.sysd = d_sysd;
    D.sst = d_sst;
    D.tile_sys = d_tile_sys;
    D.tile_first = d_tile_first;
    D.tile_count = d_tile_count;
    upload_sysd();
    for (int s = 0; s < nsys; ++s)
      if (na[s] > 0) {
        k_init_layout<<<nblocks(na[s], 256), 256, 0, stream>>>(D, s, atom_base[s], (int)na[s], 0);
        launched();
      }
    check_launch("init");
    CK(cudaStreamSynchronize(stream));
  }

  // Re-creates the two streams at the device's highest (high = 1) or lowest (0) priority:
  // when SM slots free up, blocks of high-priority streams are scheduled first, so a small
  // batch sharing the GPU with a large one keeps a short step latency.  Graph executables
  // are not bound to a stream and survive.
  void set_priority(int high) {
    CK(cudaSetDevice(device));
    CK(cudaStreamSynchronize(stream));
    CK(cudaStreamSynchronize(stream2));
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = high ? greatest : least;
    cudaStream_t a = nullptr, b = nullptr;
    CK(cudaStreamCreateWithPriority(&a, cudaStreamNonBlocking, prio));
    cudaError_t e = cudaStreamCreateWithPriority(&b, cudaStreamNonBlocking, prio);
    if (e != cudaSuccess) {
      cudaStreamDestroy(a);
      ck(e, "cudaStreamCreateWithPriority");
    }
    cudaStreamDestroy(stream);
    cudaStreamDestroy(stream2);
    stream = a;
    stream2 = b;
  }

  void upload_sysd() {
    CK(cudaMemcpyAsync(d_sysd, sysd.data(), sizeof(SysDev) * nsys, cudaMemcpyHostToDevice, stream));
    if (D.shift_tab) {
      // k * (FP32 cell edge) per axis, k in -2..2, as load_shifts computes it on the device
      // (a product with 0, +-1 or +-2 is exact, so host and device agree bit for bit)
      shift_host.assign((size_t)nsys * 128, make_float4(0.f, 0.f, 0.f, 0.f));
      for (int s = 0; s < nsys; ++s)
        for (int c = 0; c < 125; ++c) {
          const int kx = c % 5 - 2, ky = (c / 5) % 5 - 2, kz = c / 25 - 2;
          shift_host[(size_t)s * 128 + c] = make_float4((float)kx * sysd[s].df[0], (float)ky * sysd[s].df[1],
                                                        (float)kz * sysd[s].df[2], 0.0f);
        }
      CK(cudaMemcpyAsync(D.shift_tab, shift_host.data(), sizeof(float4) * shift_host.size(), cudaMemcpyHostToDevice,
                         stream));
    }
  }
  std::vector<float4> shift_host;  // pageable: the copy has taken the data when it returns

  ~Impl() {
    if (device >= 0) cudaSetDevice(device);
    drop_graph();
    if (stream) cudaStreamSynchronize(stream);
    for (const auto& m : marks) {
      cudaEventDestroy(m.a);
      cudaEventDestroy(m.b);
    }
    for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
    for (auto& a : allocs) dev_free(a.first);
    free_cells();
    if (stream) cudaStreamDestroy(stream);
    if (stream2) cudaStreamDestroy(stream2);
  }

  // --------------------------------------------------------------------------------------
  // Configuration of the neighbour machinery
  // --------------------------------------------------------------------------------------

  double max_cutoff() const {
    double rc = 0.0;
    for (const auto& p : pots) rc = std::max(rc, p.cutoff);
    return rc;
  }

  void configure() {
    if (!have_cm) throw Error(4, "MissingComponent: cellmanager");
    if (pots.empty()) throw Error(4, "MissingComponent: potential");
    drop_graph();
    const double rc = max_cutoff();
    total_cells = 0;
    any_list = false;
    double max_expect = 0.0;
    for (int s = 0; s < nsys; ++s) {
      SysDev& S = sysd[s];
      const double* L = S.L;
      S.kind_cm = cm.kind;
      S.rebuild_policy = REBUILD_SKIN;
      S.each = 1;
      S.stencil_r = stencil_r;
      S.lc_side = 1;
      int mode = NB_LIST;
      double rl = 0.0;
      if (cm.kind == CM_MINIMUMIMAGE) {
        mode = NB_ALLPAIRS;
      } else if (cm.kind == CM_LINKEDCELL) {
        int n[3] = {cm.nx, cm.ny, cm.nz};
        if (cm.mode_auto)
          for (int q = 0; q < 3; ++q) n[q] = lc_auto_n(L[q], cm.cutoff);
        if (n[0] <= 0 || n[1] <= 0 || n[2] <= 0)
          throw Error(1, "linkedcell: nx, ny and nz must be positive (or mode auto)");
        double d = L[0] / (double)n[0];
        if (L[1] / (double)n[1] < d) d = L[1] / (double)n[1];
        if (L[2] / (double)n[2] < d) d = L[2] / (double)n[2];
        int side = (int)std::ceil((cm.cutoff / d) - 0.5);
        bool complete = side >= 1;
        for (int q = 0; q < 3; ++q) {
          if (n[q] < 2 * side + 1) complete = false;
          if ((double)side * (L[q] / (double)n[q]) < rc) complete = false;
        }
        double skin = opt_skin >= 0 ? opt_skin : (cm.skin >= 0 ? cm.skin : 0.1 * rc);
        rl = rc + skin;
        bool list_ok = rl < 0.5 * std::min(L[0], std::min(L[1], L[2])) && skin > 0.0;
        if ((cm.compat || !complete || !list_ok) && precision == PREC_FP64) {
          mode = NB_CELLS;
          for (int q = 0; q < 3; ++q) S.n[q] = n[q];
          S.lc_side = side < 0 ? 0 : side;
        } else {
          mode = NB_LIST;
        }
      } else if (cm.kind == CM_LCBINARY) {
        // FP64: the reference's sub-cell stencil exactly (NB_CELLS on the lcbinary grid, which
        // grows when two atoms share a sub-cell); mixed: the complete Verlet list
        if ((int)lcb_n.size() != nsys) lcb_n.assign(nsys, {0, 0, 0});
        int* n = lcb_n[s].data();
        if (n[0] == 0)
          for (int q = 0; q < 3; ++q)
            n[q] = cm.mode_auto ? lcb_auto_n(L[q], cm.cutoff) : (q == 0 ? cm.nx : q == 1 ? cm.ny : cm.nz);
        if (n[0] <= 0 || n[1] <= 0 || n[2] <= 0) throw Error(1, "lcbinary: nx, ny and nz must be positive");
        double skin = opt_skin >= 0 ? opt_skin : (cm.skin >= 0 ? cm.skin : 0.1 * rc);
        rl = rc + skin;
        if (precision == PREC_FP64) {
          mode = NB_CELLS;
          for (int q = 0; q < 3; ++q) S.n[q] = n[q];
          S.lc_side = lcb_side(L, n, cm.cutoff);
        } else {
          mode = rl < 0.5 * std::min(L[0], std::min(L[1], L[2])) ? NB_LIST : NB_ALLPAIRS;
        }
      } else {  // verletlist
        if (std::fabs(cm.cutoff) < 1E-10) throw Error(3, "verletlist: No cutoff was defined");
        if (cm.skin >= 0 || opt_skin >= 0) {
          double skin = opt_skin >= 0 ? opt_skin : cm.skin;
          rl = std::max(cm.cutoff, rc) + skin;
          S.rebuild_policy = cm.rebuild;
        } else {
          rl = 1.08 * cm.cutoff;  // extcut, plugins/verletlist.cc:24-25
          S.rebuild_policy = REBUILD_BOTH;
        }
        if (!(rl > rc))
          throw Error(3, "verletlist: the list cutoff must exceed the potential cutoff");
        S.each = (int)std::max<int64_t>(1, cm.each);
        if (!(rl < 0.5 * std::min(L[0], std::min(L[1], L[2])))) mode = NB_ALLPAIRS;
      }
      if (mode == NB_ALLPAIRS && precision == PREC_MIXED)
        throw Error(1, "mixed precision needs every box edge longer than 2*(cutoff+skin)");
      S.mode = mode;
      if (mode == NB_LIST) {
        any_list = true;
        for (int q = 0; q < 3; ++q) {
          // cells at least (cutoff+skin)/stencil_r wide, with a 1e-4 margin that covers
          // binning by multiplication instead of division
          S.n[q] = std::max(1, (int)std::floor(L[q] * stencil_r / (rl * (1.0 + 1e-4))));
          if (S.n[q] > 1024) S.n[q] = 1024;
        }
        S.rlist2f = (float)(rl * rl * (1.0 + 1e-5));
        double sk = rl - rc;
        S.thresh2 = 0.25 * sk * sk * (1.0 - 1e-4);
        double V = L[0] * L[1] * L[2];
        double expect = 4.18879 * rl * rl * rl * (double)S.natoms / V;
        max_expect = std::max(max_expect, expect);
      } else if (mode == NB_ALLPAIRS) {
        S.n[0] = S.n[1] = S.n[2] = 1;
      }
      for (int q = 0; q < 3; ++q) {
        S.d[q] = L[q] / (double)S.n[q];
        S.df[q] = (float)S.d[q];
        S.dfc[q] = (float)((S.d[q] - (double)S.df[q]) / (double)S.df[q]);
      }
      S.ncells = S.n[0] * S.n[1] * S.n[2];
      for (int q = 0; q < 3; ++q) S.ninv[q] = (double)S.n[q] / L[q];
      S.cell_base = total_cells;
      total_cells += S.ncells;
      if (s == 0) {
        st.neighbor_mode = mode;
        st.list_radius = rl;
        for (int q = 0; q < 3; ++q) st.cell_grid[q] = S.n[q];
      }
    }
    for (int s = 1; s < nsys; ++s)
      if (sysd[s].mode != sysd[0].mode)
        throw Error(1, "every system of a batch must use the same neighbour mode (box too small for a Verlet list?)");
    // cell arrays and neighbour list
    free_cells();
    alloc_cells(total_cells);
    int maxnb = 0;
    if (any_list) {
      maxnb = (int)std::ceil(max_expect * 1.35) + 32;
      maxnb = (maxnb + 7) & ~7;
    }
    alloc_list(maxnb);
    upload_sysd();
    k_cell_centres<<<nblocks(total_cells, 256), 256, 0, stream>>>(D);  // reads the uploaded grids
    k_clear_state<<<nblocks(nsys, 128), 128, 0, stream>>>(D, nsys);
    launched(2);
    check_launch("clear");
    configured = true;
    forces_valid = false;
  }

  // Cell arrays of the current grids (sysd[*].cell_base / ncells) and the per-cell system map.
  void alloc_cells(int total) {
    D.cstart = alloc<int>(total, true);
    D.ccnt = alloc<int>(total, true);
    D.ccount = alloc<int>(total, true);
    D.ccursor = alloc<int>(total, true);
    std::vector<int> cs(total);
    for (int q = 0; q < nsys; ++q)
      for (int c = 0; c < sysd[q].ncells; ++c) cs[sysd[q].cell_base + c] = q;
    D.cell_sys = alloc<int>(total, true);
    CK(cudaMemcpyAsync(D.cell_sys, cs.data(), sizeof(int) * total, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    D.total_cells = total;
    D.ccentre = alloc<double>(3 * (size_t)total, true);
    std::vector<int> bs, bc;
    for (int q = 0; q < nsys; ++q)
      for (int c = 0; c < sysd[q].ncells; c += LIST_WARPS) {
        bs.push_back(q);
        bc.push_back(sysd[q].cell_base + c);
      }
    D.list_blocks = (int)bs.size();
    D.lblk_sys = alloc<int>(bs.size(), true);
    D.lblk_cell = alloc<int>(bc.size(), true);
    CK(cudaMemcpyAsync(D.lblk_sys, bs.data(), sizeof(int) * bs.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(D.lblk_cell, bc.data(), sizeof(int) * bc.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
  }

  void alloc_list(int maxnb) {
    D.maxnb = maxnb;
    st.list_capacity = maxnb;
    if (maxnb > 0) {
      long long nb = 0;
      for (int s = 0; s < nsys; ++s) {
        sysd[s].nl_base = nb;
        nb += (long long)sysd[s].natoms * maxnb;
      }
      D.nl = alloc<unsigned>((size_t)nb, true);
    } else {
      D.nl = nullptr;
    }
  }

  // --------------------------------------------------------------------------------------
  // Launch sequences
  // --------------------------------------------------------------------------------------

  void launch_decide(cudaStream_t s, int ucall_inc, int force_all, cudaGraphConditionalHandle h, int use_cond) {
    k_decide<<<nblocks(nsys, DECIDE_THREADS), DECIDE_THREADS, 0, s>>>(D, nsys, ucall_inc, force_all,
                                                                      (unsigned long long)h, use_cond);
    launched();
  }

  void launch_rebuild(cudaStream_t s) {
    Range r("gbmd:enqueue_rebuild");
    launch_rebuild_kernels(s);
    if (lcb_exact() && !capturing) lcb_grow_until_single(s);
  }

  void launch_rebuild_kernels(cudaStream_t s) {
    const unsigned nb = nblocks(N, 256);
    mark_begin(s, T_REBUILD);
    k_bin<<<nb, 256, 0, s>>>(D);
    k_scan<<<nsys, 1024, 0, s>>>(D);
    k_scatter<<<nb, 256, 0, s>>>(D);
    k_cellsort<<<nblocks(D.total_cells, SORT_WARPS), 32 * SORT_WARPS, 0, s>>>(D);
    k_permute<<<nb, 256, 0, s>>>(D);
    k_copyback<<<nb, 256, 0, s>>>(D);
    launched(6);
    if (any_list) {
      k_buildlist<<<D.list_blocks, 32 * LIST_WARPS, 0, s>>>(D);
      launched();
    }
    mark_end(s, T_REBUILD);
  }

  // decide_next / cond_next: the mixed path's tail kernel also decides the next step's rebuild
  // and sets that step's graph conditional (0: a k_decide launch does it instead).
  // raw: keep fixedvel atoms' accelerations (a bare UpdateForces outside an integrator step).
  void launch_force_passes(cudaStream_t s, int epi, int count_step, int decide_next = 0,
                           cudaGraphConditionalHandle cond_next = 0, int raw = 0) {
    const bool mixed = precision == PREC_MIXED;
    const int np = (int)pots.size();
    mark_begin(s, T_FORCE);
    int first_eam = -1;
    for (int p = 0; p < np; ++p)
      if (!pair_kind(pots[p].kind)) {
        first_eam = p;
        break;
      }
    for (int p = 0; p < np; ++p) {
      const PotParams& P = pots[p];
      StepParams sp;
      sp.dt = integ.dt;
      sp.half_dt = 0.5 * integ.dt;
      sp.half_dt2 = 0.5 * integ.dt * integ.dt;
      sp.epi = epi;
      sp.first = (p == 0);
      sp.last = (p == np - 1);
      sp.count_step = count_step;
      sp.kinetic = 1;
      sp.raw_acc = raw;
      const int mode = sysd[0].mode;
      const bool species = P.spc_sum >= 0;
      // Sutton-Chen exponent pairs of common metals get straight-line powers, and without a
      // species filter the many-body prefactor folded into the gathered embedding factor
      const bool sc96 = P.kind == POT_SC && P.int_n == 9 && P.int_m == 6;
      const bool sc126 = P.kind == POT_SC && P.int_n == 12 && P.int_m == 6;
      PotParams Pe = P;
      Pe.f[14] = (!species && (sc96 || sc126)) ? P.f[2] : 1.0f;  // scale of the density pass's copy
      // list rows through the shared-memory ring for ensembles and pair potentials, through
      // registers for a single EAM system (the faster of the two on the GB300 for each), unless
      // the option says otherwise
      const bool ring = list_feed == 2 || (list_feed == 0 && (nsys > 1 || pair_kind(P.kind)));
      if (!pair_kind(P.kind)) {
        int first = (p == first_eam);
        if (mixed && P.kind == POT_SC && P.int_m == 6)
          ring ? k_eam_density32<6, FEED_RING><<<ntiles, TILE, 0, s>>>(D, Pe)
               : k_eam_density32<6, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, Pe);
        else if (mixed)
          ring ? k_eam_density32<0, FEED_RING><<<ntiles, TILE, 0, s>>>(D, Pe)
               : k_eam_density32<0, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, Pe);
        else if (mode == NB_LIST)
          k_eam_density<NB_LIST><<<ntiles, TILE, 0, s>>>(D, P, first);
        else if (mode == NB_CELLS)
          k_eam_density<NB_CELLS><<<ntiles, TILE, 0, s>>>(D, P, first);
        else
          k_eam_density<NB_ALLPAIRS><<<ntiles, TILE, 0, s>>>(D, P, first);
        launched();
      }
      if (mixed) {
        if (pair_kind(P.kind) && lanes > 1) {
          const unsigned g = (unsigned)ntiles * lanes;
          if (lanes == 2)
            species ? k_force32_lanes<1, 2><<<g, TILE, 0, s>>>(D, P, sp) : k_force32_lanes<0, 2><<<g, TILE, 0, s>>>(D, P, sp);
          else if (lanes == 4)
            species ? k_force32_lanes<1, 4><<<g, TILE, 0, s>>>(D, P, sp) : k_force32_lanes<0, 4><<<g, TILE, 0, s>>>(D, P, sp);
          else if (lanes == 8)
            species ? k_force32_lanes<1, 8><<<g, TILE, 0, s>>>(D, P, sp) : k_force32_lanes<0, 8><<<g, TILE, 0, s>>>(D, P, sp);
          else if (lanes == 16)
            species ? k_force32_lanes<1, 16><<<g, TILE, 0, s>>>(D, P, sp) : k_force32_lanes<0, 16><<<g, TILE, 0, s>>>(D, P, sp);
          else
            species ? k_force32_lanes<1, 32><<<g, TILE, 0, s>>>(D, P, sp) : k_force32_lanes<0, 32><<<g, TILE, 0, s>>>(D, P, sp);
        } else if (pair_kind(P.kind)) {
          if (species)
            ring ? k_force32<PC_PAIR, 1, 0, 0, FEED_RING><<<ntiles, TILE, 0, s>>>(D, P, sp)
                 : k_force32<PC_PAIR, 1, 0, 0, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, P, sp);
          else
            ring ? k_force32<PC_PAIR, 0, 0, 0, FEED_RING><<<ntiles, TILE, 0, s>>>(D, P, sp)
                 : k_force32<PC_PAIR, 0, 0, 0, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, P, sp);
        } else {
          if (species)
            ring ? k_force32<PC_EAM, 1, 0, 0, FEED_RING><<<ntiles, TILE, 0, s>>>(D, Pe, sp)
                 : k_force32<PC_EAM, 1, 0, 0, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, Pe, sp);
          else if (sc96)
            ring ? k_force32<PC_EAM, 0, 9, 6, FEED_RING><<<ntiles, TILE, 0, s>>>(D, Pe, sp)
                 : k_force32<PC_EAM, 0, 9, 6, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, Pe, sp);
          else if (sc126)
            ring ? k_force32<PC_EAM, 0, 12, 6, FEED_RING><<<ntiles, TILE, 0, s>>>(D, Pe, sp)
                 : k_force32<PC_EAM, 0, 12, 6, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, Pe, sp);
          else
            ring ? k_force32<PC_EAM, 0, 0, 0, FEED_RING><<<ntiles, TILE, 0, s>>>(D, Pe, sp)
                 : k_force32<PC_EAM, 0, 0, 0, FEED_REGS><<<ntiles, TILE, 0, s>>>(D, Pe, sp);
        }
      } else if (mode == NB_LIST) {
        if (pair_kind(P.kind))
          k_force64<NB_LIST, PC_PAIR><<<ntiles, TILE, 0, s>>>(D, P, sp);
        else
          k_force64<NB_LIST, PC_EAM><<<ntiles, TILE, 0, s>>>(D, P, sp);
      } else if (mode == NB_CELLS) {
        if (pair_kind(P.kind))
          k_force64<NB_CELLS, PC_PAIR><<<ntiles, TILE, 0, s>>>(D, P, sp);
        else
          k_force64<NB_CELLS, PC_EAM><<<ntiles, TILE, 0, s>>>(D, P, sp);
      } else {
        if (pair_kind(P.kind))
          k_force64<NB_ALLPAIRS, PC_PAIR><<<ntiles, TILE, 0, s>>>(D, P, sp);
        else
          k_force64<NB_ALLPAIRS, PC_EAM><<<ntiles, TILE, 0, s>>>(D, P, sp);
      }
      launched();
    }
    mark_end(s, T_FORCE);
    if (mixed)
      k_tail<<<nblocks(nsys, TAIL_THREADS), TAIL_THREADS, 0, s>>>(D, count_step, decide_next,
                                                                  (unsigned long long)cond_next);
    else
      k_thermo<<<nsys, TILE, 0, s>>>(D, count_step);
    launched();
  }

  void ensure_ready() {
    for (const auto& P : pots)
      if (P.kind == POT_FASTLJ && precision == PREC_MIXED)
        throw Error(1, "fastlj has no mixed-precision form (an FP32 distance can fall into the neighbouring "
                       "table bin): use precision fp64");
    if (!configured) configure();
    CK(cudaSetDevice(device));
    if (!D.g32e && precision == PREC_MIXED)
      for (const auto& P : pots)
        if (!pair_kind(P.kind)) {
          D.g32e = alloc<float4>((size_t)N);  // the mixed EAM density pass writes it
          break;
        }
    if (integ.kind != INT_VV && !D.ist) {
      // history of the integrators other than velocityverlet, moved with the atoms at re-sorts
      D.ist = alloc<double>((size_t)IST_K * N);
      D.ist_alt = alloc<double>((size_t)IST_K * N);
      D.nh = alloc<double>((size_t)nsys * NH_LEN);
      CK(cudaMemsetAsync(D.ist, 0, sizeof(double) * IST_K * N, stream));
      CK(cudaMemsetAsync(D.nh, 0, sizeof(double) * nsys * NH_LEN, stream));
    }
  }

  // Reads the per-system error words and the list statistics (synchronises the stream).
  void check_errors() {
    CK(cudaStreamSynchronize(stream));
    collect_marks();
    std::vector<SysState> hs(nsys);
    CK(cudaMemcpyAsync(hs.data(), d_sst, sizeof(SysState) * nsys, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    int err = 0, maxc = 0;
    long long rb = 0;
    unsigned long long rech = 0;
    for (const auto& x : hs) {
      err |= x.error;
      maxc = std::max(maxc, x.max_count);
      rb += x.rebuilds;
      rech += x.rechecks;
    }
    st.max_neighbors = maxc;
    st.list_rebuilds = rb;
    st.fp_guard_rechecks = (int64_t)rech;
    if (err & ERR_OUTSIDE) throw Error(8, "RuntimeError: atom position is not finite or far outside the simulation box");
    if (err & ERR_LIST) throw Error(7, "neighbour list capacity exceeded (maxneighbors is too small!)");
    // VerletListCellManager throws once an atom reaches maxneighbors-1 list entries
    // (plugins/verletlist.cc:96-97)
    if (cm.kind == CM_VERLETLIST && maxnb_cap > 0 && maxc >= maxnb_cap - 1)
      throw Error(3, "PluginError: verletlist: maxneighbors is too small!");
  }
  long long maxnb_cap = 0;

  // First build: size the list from the measured maximum and rebuild if it did not fit.
  void first_build() {
    for (int attempt = 0; attempt < 4; ++attempt) {
      launch_decide(stream, attempt == 0 ? 1 + pending_ucalls : 0, 1, 0, 0);
      launch_rebuild(stream);
      check_launch("rebuild");
      CK(cudaStreamSynchronize(stream));
      std::vector<SysState> hs(nsys);
      CK(cudaMemcpyAsync(hs.data(), d_sst, sizeof(SysState) * nsys, cudaMemcpyDeviceToHost, stream));
      CK(cudaStreamSynchronize(stream));
      int maxc = 0, err = 0;
      for (const auto& x : hs) {
        maxc = std::max(maxc, x.max_count);
        err |= x.error;
      }
      if (err & ERR_OUTSIDE) throw Error(8, "RuntimeError: atom position is not finite or far outside the simulation box");
      pending_ucalls = 0;
      if (!any_list || maxc <= D.maxnb * 0.8) return;
      // grow: re-allocate the list with room to spare and rebuild from scratch
      int maxnb = (int)std::ceil(maxc * 1.4) + 16;
      maxnb = (maxnb + 7) & ~7;
      long long old_entries = 0;
      for (const auto& S : sysd) old_entries += (long long)S.natoms * D.maxnb;
      cell_bytes -= sizeof(unsigned) * (size_t)(old_entries ? old_entries : 1);
      dev_free(D.nl);
      cell_allocs.erase(std::find_if(cell_allocs.begin(), cell_allocs.end(),
                                     [&](const std::pair<void*, size_t>& a) { return a.first == (void*)D.nl; }));
      alloc_list(maxnb);
      upload_sysd();
      k_clear_state<<<nblocks(nsys, 128), 128, 0, stream>>>(D, nsys);
      launched();
    }
    throw Error(7, "could not size the neighbour list");
  }

  // One force evaluation at the current positions (CombinedPotential::UpdateForces).
  void update_forces() {
    ensure_ready();
    set_buffers(cbuf);
    if (!forces_valid_layout) {
      first_build();
      forces_valid_layout = true;
      launch_force_passes(stream, EPI_FORCES, 0);
    } else {
      launch_decide(stream, 1, 0, 0, 0);
      launch_rebuild(stream);
      launch_force_passes(stream, EPI_FORCES, 0);
    }
    check_launch("update_forces");
    st.force_evaluations++;
    check_errors();
    forces_valid = true;
    pend = false;
  }
  bool forces_valid_layout = false;

  // Stand-alone AdvancePosition from the committed positions into the other buffer.
  void launch_drift(cudaStream_t s) {
    set_buffers(cbuf);
    mark_begin(s, T_DRIFT);
    if (precision == PREC_MIXED)
      k_drift<1><<<ntiles, TILE, 0, s>>>(D, integ.dt, 0.5 * integ.dt * integ.dt);
    else
      k_drift<0><<<ntiles, TILE, 0, s>>>(D, integ.dt, 0.5 * integ.dt * integ.dt);
    mark_end(s, T_DRIFT);
    launched();
    pend = true;
  }

  // First half of a step: switch to the drifted buffer and decide whether to rebuild.
  void launch_step_head(cudaStream_t s, int ucall_inc, bool conditional, cudaGraphConditionalHandle h) {
    set_buffers(1 - cbuf);
    launch_decide(s, ucall_inc, 0, h, conditional ? 1 : 0);
    if (!conditional) launch_rebuild(s);
  }

  // Second half: fused force + kick + drift into the other buffer; commits the step.
  void launch_step_tail(cudaStream_t s, int decide_next = 0, cudaGraphConditionalHandle cond_next = 0) {
    launch_force_passes(s, EPI_KICK_DRIFT, 1, decide_next, cond_next);
    cbuf = 1 - cbuf;
  }

  void build_graph(int nsteps) {
    Range r("gbmd:capture_graph");
    std::lock_guard<std::recursive_mutex> lk(g_dev_mu);
    drop_graph();
    CK(cudaGraphCreate(&graph, 0));
    bool cond = graph_mode == 2;
    std::vector<cudaGraphConditionalHandle> handles(nsteps);
    if (cond) {
      for (int k = 0; k < nsteps; ++k) {
        if (cudaGraphConditionalHandleCreate(&handles[k], graph, 0, cudaGraphCondAssignDefault) != cudaSuccess) {
          cudaGetLastError();
          cond = false;
          break;
        }
      }
    }
    CK(cudaStreamBeginCaptureToGraph(stream, graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    int64_t saved = st.kernel_launches;
    const int cbuf0 = cbuf;
    capturing = true;
    // mixed path: the tail kernel of step k decides step k+1, so only the first step of the
    // graph launches k_decide
    const bool fused = precision == PREC_MIXED;
    int64_t base_launches = 0;
    try {
      for (int k = 0; k < nsteps; ++k) {
        set_buffers(1 - cbuf);
        int64_t before = st.kernel_launches;
        if (!(fused && k > 0)) launch_decide(stream, 2, 0, cond ? handles[k] : 0, cond ? 1 : 0);
        if (!cond) launch_rebuild(stream);
        base_launches += st.kernel_launches - before;
        if (cond) {
          cudaStreamCaptureStatus cs;
          cudaGraph_t g;
          const cudaGraphNode_t* deps = nullptr;
          size_t ndeps = 0;
          CK(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, &deps, nullptr, &ndeps));
          cudaGraphNodeParams cp = {};
          cp.type = cudaGraphNodeTypeConditional;
          cp.conditional.handle = handles[k];
          cp.conditional.type = cudaGraphCondTypeIf;
          cp.conditional.size = 1;
          cudaGraphNode_t cnode;
          CK(cudaGraphAddNode(&cnode, g, deps, nullptr, ndeps, &cp));
          cudaGraph_t body = cp.conditional.phGraph_out[0];
          CK(cudaStreamUpdateCaptureDependencies(stream, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
          CK(cudaStreamBeginCaptureToGraph(stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
          launch_rebuild(stream2);
          cudaGraph_t bout;
          CK(cudaStreamEndCapture(stream2, &bout));
        }
        const bool decide_next = fused && k + 1 < nsteps;
        before = st.kernel_launches;
        launch_step_tail(stream, decide_next ? 1 : 0, (decide_next && cond) ? handles[k + 1] : 0);
        base_launches += st.kernel_launches - before;
      }
    } catch (...) {
      capturing = false;
      cbuf = cbuf0;
      cudaGraph_t tmp;
      cudaStreamEndCapture(stream, &tmp);
      cudaGetLastError();
      st.kernel_launches = saved;
      drop_graph();
      throw;
    }
    capturing = false;
    cbuf = cbuf0;  // capture does not execute: the buffers flip when the graph runs
    cudaGraph_t out;
    CK(cudaStreamEndCapture(stream, &out));
    st.kernel_launches = saved;
    CK(cudaGraphInstantiate(&gexec, graph, 0));
    gsteps = nsteps;
    gparity = cbuf0;
    graph_cond = cond;
    graph_launches = base_launches;
  }
  bool graph_cond = false;
  int64_t graph_launches = 0;  // kernels one graph launch runs, rebuild chains not included

  // Integrator::Initialize of the integrators other than velocityverlet, at their first step
  // (SimulationBuilder::DoStep, liblpmd/simulation/simulationbuilder.cc:130-133).
  void init_integrator() {
    const double dt = integ.dt;
    const int k = integ.kind;
    const unsigned nb = nblocks(N, 256);
    set_buffers(cbuf);
    if (k == INT_EULER) return;  // no Initialize of its own
    if (k == INT_VERLET) {       // UseOldConfig: the backed-up positions; SetCellManager on the copy
      k_init_backup<INT_VERLET><<<nb, 256, 0, stream>>>(D, dt);
      launched();
      pending_ucalls += 1;
      return;
    }
    // leapfrog, beeman, nosehoover: UseOldConfig, then UpdateForces on the backed-up
    // configuration (two UpdateCell calls), whose accelerations seed the history
    if (k == INT_LEAPFROG)
      k_init_backup<INT_LEAPFROG><<<nb, 256, 0, stream>>>(D, dt);
    else
      k_init_backup<INT_BEEMAN><<<nb, 256, 0, stream>>>(D, dt);
    launched();
    launch_decide(stream, 2 + pending_ucalls, 1, 0, 0);
    pending_ucalls = 0;
    launch_rebuild(stream);
    launch_force_passes(stream, EPI_FORCES, 0, 0, 0, 1);
    if (k == INT_LEAPFROG)
      k_init_restore<INT_LEAPFROG><<<nb, 256, 0, stream>>>(D, dt);
    else
      k_init_restore<INT_BEEMAN><<<nb, 256, 0, stream>>>(D, dt);
    k_force_rebuild<<<1, 256, 0, stream>>>(D);
    launched(2);
    check_launch("integrator initialize");
    if (k == INT_NOSEHOOVER) init_nose_hoover();
  }

  // Nose-Hoover: friction 0 (nosehoover.cc:41), and each atom's rank among the atoms without
  // fixedpos in the reference's atom order, which sets how many friction increments it sees.
  void init_nose_hoover() {
    std::vector<int> tag(N);
    std::vector<unsigned char> fl(N, 0);
    CK(cudaMemcpyAsync(tag.data(), D.tag, sizeof(int) * N, cudaMemcpyDeviceToHost, stream));
    if (D.has_flags) CK(cudaMemcpyAsync(fl.data(), D.flags, N, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    std::vector<double> rank_by_tag(N, 0.0), nh((size_t)nsys * NH_LEN, 0.0);
    std::vector<unsigned char> fixed_by_tag(N, 0);
    for (long long i = 0, s = 0; i < N; ++i) {
      while (s + 1 < nsys && atom_base[s + 1] <= i) ++s;
      fixed_by_tag[atom_base[s] + tag[i]] = (fl[i] & FLAG_FIXEDPOS) ? 1 : 0;
    }
    for (int s = 0; s < nsys; ++s) {
      double r = 0.0;
      for (long long t = 0; t < natoms[s]; ++t) {
        if (!fixed_by_tag[atom_base[s] + t]) r += 1.0;
        rank_by_tag[atom_base[s] + t] = r;
      }
      nh[(size_t)s * NH_LEN + NH_NMOVE] = r;
    }
    double* d_rank = nullptr;
    CK(dev_malloc(&d_rank, sizeof(double) * std::max<long long>(N, 1)));
    CK(cudaMemcpyAsync(d_rank, rank_by_tag.data(), sizeof(double) * N, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(D.nh, nh.data(), sizeof(double) * nh.size(), cudaMemcpyHostToDevice, stream));
    k_set_rank<<<nblocks(N, 256), 256, 0, stream>>>(D, d_rank);
    launched();
    CK(cudaStreamSynchronize(stream));
    dev_free(d_rank);
  }

  // One step of an integrator other than velocityverlet (OneStepIntegrator::Advance /
  // TwoStepIntegrator::Advance), then the step's thermo record from the new velocities.
  void step_plain() {
    const double dt = integ.dt;
    const int k = integ.kind;
    const bool mixed = precision == PREC_MIXED;
    set_buffers(cbuf);
    if (k == INT_EULER || k == INT_LEAPFROG || k == INT_VERLET) {
      launch_decide(stream, 1 + pending_ucalls, 0, 0, 0);
      pending_ucalls = 0;
      launch_rebuild(stream);
      launch_force_passes(stream, EPI_FORCES, 0);
      if (k == INT_EULER)
        k_onestep<INT_EULER><<<ntiles, TILE, 0, stream>>>(D, dt);
      else if (k == INT_LEAPFROG)
        k_onestep<INT_LEAPFROG><<<ntiles, TILE, 0, stream>>>(D, dt);
      else
        k_onestep<INT_VERLET><<<ntiles, TILE, 0, stream>>>(D, dt);
      launched();
      cbuf = 1 - cbuf;
      set_buffers(cbuf);
    } else {
      // the step's first UpdateForces repeats the last evaluation at the same positions: only
      // its UpdateCell call is counted
      if (k == INT_NOSEHOOVER) {
        k_kinetic_clear<<<1, 256, 0, stream>>>(D);
        k_scale_kinetic<<<ntiles, TILE, 0, stream>>>(D, -1, 1);
        k_nh_friction<<<1, 256, 0, stream>>>(D, dt, integ.fmass, integ.t);
        k_twostep_position<INT_NOSEHOOVER><<<ntiles, TILE, 0, stream>>>(D, dt);
        launched(4);
      } else {
        k_twostep_position<INT_BEEMAN><<<ntiles, TILE, 0, stream>>>(D, dt);
        launched();
      }
      cbuf = 1 - cbuf;
      set_buffers(cbuf);
      launch_decide(stream, 2 + pending_ucalls, 0, 0, 0);
      pending_ucalls = 0;
      launch_rebuild(stream);
      launch_force_passes(stream, EPI_FORCES, 0);
      k_twostep_velocity<<<ntiles, TILE, 0, stream>>>(D, dt);
      launched();
    }
    if (mixed) {
      k_kinetic_slots_clear<<<1, 256, 0, stream>>>(D);
      k_step_kinetic<1><<<ntiles, TILE, 0, stream>>>(D);
      k_tail<<<nblocks(nsys, TAIL_THREADS), TAIL_THREADS, 0, stream>>>(D, 1, 0, 0ull);
      launched(3);
    } else {
      k_step_kinetic<0><<<ntiles, TILE, 0, stream>>>(D);
      k_thermo<<<nsys, TILE, 0, stream>>>(D, 1);
      launched(2);
    }
    check_launch("step");
  }

  void do_steps(int64_t nsteps) {
    ensure_ready();
    if (!have_integ) throw Error(4, "MissingComponent: integrator");
    if (nsteps <= 0) return;
    if (!forces_valid) update_forces();
    if (integ.kind != INT_VV) {
      if (!initialized) {
        init_integrator();
        initialized = true;
      }
      for (int64_t k = 0; k < nsteps; ++k) step_plain();
      st.steps += nsteps;
      st.force_evaluations += nsteps;
      check_errors();
      return;
    }
    if (!pend) launch_drift(stream);
    int first_extra = 0;
    if (!initialized) {
      // VelocityVerlet::Initialize -> UseOldConfig -> SetCellManager: one more UpdateCell call
      first_extra = 1;
      initialized = true;
    }
    int64_t done = 0;
    long long rb_before = st.list_rebuilds;
    if (first_extra) {
      launch_step_head(stream, 3, false, 0);
      launch_step_tail(stream);
      check_launch("step");
      done = 1;
    }
    const int gb = lcb_exact() ? 0 : graph_block;  // lcbinary grows its grid on the host
    if (graph_mode > 0 && gb > 0) {
      // a block of gb steps flips the buffers gb times: keep its parity even so one graph
      // serves every block
      const int gbe = gb & ~1;
      if (gbe > 0 && (cbuf != gparity || !gexec || gsteps != gbe) && nsteps - done >= gbe)
        build_graph(gbe);
      while (gbe > 0 && nsteps - done >= gbe && gparity == cbuf) {
        CK(cudaGraphLaunch(gexec, stream));
        st.kernel_launches += graph_launches;
        done += gbe;
      }
    }
    while (done < nsteps) {
      launch_step_head(stream, 2, false, 0);
      launch_step_tail(stream);
      check_launch("step");
      ++done;
    }
    st.steps += nsteps;
    st.force_evaluations += nsteps;
    check_errors();
    if (graph_cond) st.kernel_launches += (st.list_rebuilds - rb_before) * (6 + (any_list ? 1 : 0));
  }
};

// ------------------------------------------------------------------------------------------
// Engine API
// ------------------------------------------------------------------------------------------

Engine::Engine(int device, const std::vector<int64_t>& natoms, const std::vector<std::array<double, 3>>& cells)
    : natoms_(natoms), d_(new Impl) {
  try {
    d_->setup(device, natoms, cells);
  } catch (...) {
    delete d_;
    throw;
  }
}

Engine::~Engine() { delete d_; }

int wait_selftest(int device, long long polls) {
  if (polls < 1 || polls > WAIT_POLLS) throw Error(1, "polls must be in [1, 2^22]");
  CK(cudaSetDevice(device));
  int* d = nullptr;
  CK(dev_malloc(&d, sizeof(int)));
  int h = -1;
  k_wait_selftest<<<1, 32>>>(polls, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  dev_free(d);
  ck(e, "wait self-test");
  return h;
}

void Engine::scale_velocities(int sys, int mode, double target, double dt_over_tau) {
  Impl& I = *d_;
  if (sys >= I.nsys) throw Error(1, "system index out of range");
  if (mode != 0 && mode != 1) throw Error(1, "velocity scaling mode must be 0 (set temperature) or 1 (Berendsen)");
  if (!(target >= 0.0)) throw Error(1, "target temperature must be non-negative");
  if (!I.forces_valid) throw Error(4, "MissingComponent: no evaluated state yet (call update_forces or do_steps first)");
  CK(cudaSetDevice(I.device));
  I.set_buffers(I.cbuf);
  k_kinetic_clear<<<1, 256, 0, I.stream>>>(I.D);
  k_scale_kinetic<<<I.ntiles, TILE, 0, I.stream>>>(I.D, sys, mode);
  k_scale_velocities<<<nblocks(I.N, 256), 256, 0, I.stream>>>(I.D, sys, mode, target, dt_over_tau);
  I.launched(3);
  I.check_launch("scale_velocities");
  // the drift already queued for the next step used the old velocities: redo it
  I.pend = false;
  CK(cudaStreamSynchronize(I.stream));
}

void Engine::set_active(int sys, bool on) {
  Impl& I = *d_;
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  CK(cudaSetDevice(I.device));
  // a system coming back has no pending drift: re-evaluate the batch's forces (identical
  // values for the systems that kept running) and drift again before the next step
  if (on && !I.sysd[sys].active) I.forces_valid = false;
  I.sysd[sys].active = on ? 1 : 0;
  I.upload_sysd();
}

void Engine::set_atoms(int sys, const double* pos, const double* vel, const double* acc, const int32_t* Z,
                       const double* mass) {
  Range rg("gbmd:set_atoms");
  Impl& I = *d_;
  CK(cudaSetDevice(I.device));
  I.set_buffers(I.cbuf);
  I.pend = false;
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  const int n = (int)I.natoms[sys];
  if (n == 0) return;
  const size_t v3 = sizeof(double) * 3 * n;
  // staging in the permutation scratch (11 doubles per atom, idle outside a rebuild and
  // ordered with it on the stream): pos | vel | acc | mass (doubles) then Z (ints)
  {
    double* dp = I.D.sdbl;
    double* dv = dp + 3 * n;
    double* da = dv + 3 * n;
    double* dm = da + 3 * n;
    int* dz = (int*)(dm + n);
    if (pos) CK(cudaMemcpyAsync(dp, pos, v3, cudaMemcpyHostToDevice, I.stream));
    if (vel) CK(cudaMemcpyAsync(dv, vel, v3, cudaMemcpyHostToDevice, I.stream));
    else CK(cudaMemsetAsync(dv, 0, v3, I.stream));
    if (acc) CK(cudaMemcpyAsync(da, acc, v3, cudaMemcpyHostToDevice, I.stream));
    else CK(cudaMemsetAsync(da, 0, v3, I.stream));
    if (mass) CK(cudaMemcpyAsync(dm, mass, sizeof(double) * n, cudaMemcpyHostToDevice, I.stream));
    if (Z) CK(cudaMemcpyAsync(dz, Z, sizeof(int) * n, cudaMemcpyHostToDevice, I.stream));
    k_set_atoms<<<nblocks(n, 256), 256, 0, I.stream>>>(I.D, I.atom_base[sys], n, pos ? dp : nullptr, dv, da,
                                                        Z ? dz : nullptr, mass ? dm : nullptr);
    I.launched();
    I.check_launch("set_atoms");
    CK(cudaStreamSynchronize(I.stream));
  }
  I.forces_valid = false;
  I.forces_valid_layout = false;
}

void Engine::set_flags(int sys, const uint8_t* flags) {
  Impl& I = *d_;
  CK(cudaSetDevice(I.device));
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  const int n = (int)I.natoms[sys];
  int nfixed = 0;
  if (flags)
    for (int k = 0; k < n; ++k)
      if (flags[k] & (FLAG_FIXEDVEL | FLAG_FIXEDPOS)) ++nfixed;
  I.sysd[sys].nfree = n - nfixed;
  I.sysd[sys].kbn = 8.6173422E-05 * (double)(n - nfixed);
  if (n == 0) return;
  unsigned char* df = nullptr;
  CK(dev_malloc(&df, n));
  if (flags) CK(cudaMemcpyAsync(df, flags, n, cudaMemcpyHostToDevice, I.stream));
  k_set_flags<<<nblocks(n, 256), 256, 0, I.stream>>>(I.D, I.atom_base[sys], n, flags ? df : nullptr);
  I.launched();
  CK(cudaStreamSynchronize(I.stream));
  dev_free(df);
  if (nfixed) I.flags_any = true;
  I.D.has_flags = I.flags_any ? 1 : 0;
  I.upload_sysd();
  I.drop_graph();
}

void Engine::get_atoms(int sys, double* pos, double* vel, double* acc) {
  Range rg("gbmd:get_atoms");
  Impl& I = *d_;
  CK(cudaSetDevice(I.device));
  I.set_buffers(I.cbuf);
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  const int n = (int)I.natoms[sys];
  if (n == 0) return;
  const size_t v3 = sizeof(double) * 3 * n;
  double* stg = I.D.sdbl;  // staging in the permutation scratch (see set_atoms)
  k_get_atoms<<<nblocks(n, 256), 256, 0, I.stream>>>(I.D, I.atom_base[sys], n, stg, stg + 3 * n, stg + 6 * n);
  I.launched();
  if (pos) CK(cudaMemcpyAsync(pos, stg, v3, cudaMemcpyDeviceToHost, I.stream));
  if (vel) CK(cudaMemcpyAsync(vel, stg + 3 * n, v3, cudaMemcpyDeviceToHost, I.stream));
  if (acc) CK(cudaMemcpyAsync(acc, stg + 6 * n, v3, cudaMemcpyDeviceToHost, I.stream));
  ck(cudaStreamSynchronize(I.stream), "get_atoms");
}

void Engine::set_cell_manager(const CellManagerCfg& cfg) {
  d_->cm = cfg;
  d_->lcb_n.clear();
  d_->have_cm = true;
  d_->pending_ucalls = 1;  // Configuration::SetCellManager calls UpdateCell once
  d_->configured = false;
  d_->forces_valid = false;
  d_->forces_valid_layout = false;
}

void Engine::add_potential(const PotParams& p) {
  if (d_->pots.size() >= 8) throw Error(1, "at most 8 potentials");
  PotParams q = p;
  q.tab = nullptr;
  if (p.kind == POT_FASTLJ) {
    const long bins = (long)p.p[3];
    if (bins < 1 || bins > (1L << 24)) throw Error(1, "fastlj: bins must be in [1, 2^24]");
    std::vector<double> t = fastlj_table(p.p[0], p.p[1], p.p[2], bins);
    CK(cudaSetDevice(d_->device));
    double* d = d_->alloc<double>(t.size());
    CK(cudaMemcpy(d, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice));
    q.tab = d;
  }
  d_->pots.push_back(q);
  d_->configured = false;
  d_->forces_valid = false;
  d_->forces_valid_layout = false;
}

void Engine::set_integrator(const IntegratorCfg& cfg) {
  if (!(cfg.dt > 0.0) || !std::isfinite(cfg.dt)) throw Error(1, "integrator: dt must be positive");
  if (cfg.kind < INT_VV || cfg.kind > INT_NOSEHOOVER) throw Error(1, "unknown integrator");
  // A different integrator starts over with its own Initialize (its history is not the old
  // one's) from forces at the current positions (a one-step integrator leaves the previous
  // positions' accelerations).
  if (d_->have_integ && cfg.kind != d_->integ.kind) {
    d_->initialized = false;
    d_->forces_valid = false;
    d_->pend = false;
  }
  d_->integ = cfg;
  d_->have_integ = true;
  d_->drop_graph();
}

void Engine::set_precision(int precision) {
  if (precision != PREC_FP64 && precision != PREC_MIXED)
    throw Error(1, "unknown precision");
  if (precision != d_->precision) {
    d_->precision = precision;
    d_->configured = false;
    d_->forces_valid = false;
    d_->forces_valid_layout = false;
  }
}

void Engine::set_option(const std::string& key, const std::string& value) {
  Impl& I = *d_;
  char* end = nullptr;
  double v = std::strtod(value.c_str(), &end);
  if (end == value.c_str()) throw Error(1, "option " + key + ": not a number: " + value);
  if (key == "maxneighbors_cap") {
    I.maxnb_cap = (long long)v;
    return;
  }
  if (key == "time_kernels") {
    I.time_kernels = (int)v;
    return;
  }
  if (key == "stream_priority") {  // 1: highest, 0: lowest (default); replaces the stream
    I.set_priority(v != 0.0 ? 1 : 0);
    return;
  }
  if (key == "list_feed") {  // list rows of the mixed passes: 0 auto, 1 registers, 2 shared-memory ring
    const int f = (int)v;
    if (f < 0 || f > 2) throw Error(1, "list_feed must be 0 (auto), 1 (registers) or 2 (ring)");
    I.list_feed = f;
    I.drop_graph();
    return;
  }
  if (key == "lanes_per_atom") {  // mixed LJ force pass: 1 (one lane per atom), 2, 4, 8, 16 or 32 lanes per atom
    const int l = (int)v;
    if (l != 1 && l != 2 && l != 4 && l != 8 && l != 16 && l != 32)
      throw Error(1, "lanes_per_atom must be 1, 2, 4, 8, 16 or 32");
    I.lanes = l;
    I.drop_graph();
    return;
  }
  if (key == "skin") {
    I.opt_skin = v;
  } else if (key == "graph_block") {
    I.graph_block = (int)v;
  } else if (key == "graph_mode") {
    I.graph_mode = (int)v;
  } else if (key == "cell_scale" || key == "stencil") {
    if ((int)v != 1 && (int)v != 2) throw Error(1, "cell_scale must be 1 or 2");
    I.stencil_r = (int)v;
  } else {
    throw Error(1, "unknown option " + key);
  }
  I.configured = false;
  I.forces_valid = false;
  I.forces_valid_layout = false;
  I.drop_graph();
}

void Engine::update_forces() {
  Range r("gbmd:update_forces");
  d_->update_forces();
}
void Engine::do_steps(int64_t nsteps) {
  Range r("gbmd:do_steps");
  d_->do_steps(nsteps);
}
void Engine::synchronize() {
  CK(cudaSetDevice(d_->device));
  CK(cudaStreamSynchronize(d_->stream));
}

void Engine::thermo(int sys, double* out22) {
  Impl& I = *d_;
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  CK(cudaSetDevice(I.device));
  CK(cudaMemcpyAsync(out22, I.D.thermo_last + (size_t)sys * THERMO_LEN, sizeof(double) * THERMO_LEN,
                     cudaMemcpyDeviceToHost, I.stream));
  CK(cudaStreamSynchronize(I.stream));
}

int64_t Engine::thermo_log(int sys, double* out, int64_t cap) {
  Impl& I = *d_;
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  CK(cudaSetDevice(I.device));
  std::vector<double> all((size_t)I.log_cap * THERMO_LEN);
  CK(cudaMemcpyAsync(all.data(), I.D.thermo_log + (size_t)sys * I.log_cap * THERMO_LEN,
                     sizeof(double) * all.size(), cudaMemcpyDeviceToHost, I.stream));
  SysState hs;
  CK(cudaMemcpyAsync(&hs, I.d_sst + sys, sizeof(SysState), cudaMemcpyDeviceToHost, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  long long last = hs.step;
  long long first = std::max<long long>(1, last - I.log_cap + 1);
  if (!I.read_from.count(sys)) I.read_from[sys] = 1;
  first = std::max(first, I.read_from[sys]);
  int64_t c = 0;
  for (long long stp = first; stp <= last && c < cap; ++stp, ++c)
    std::memcpy(out + c * THERMO_LEN, all.data() + (stp % I.log_cap) * THERMO_LEN, sizeof(double) * THERMO_LEN);
  I.read_from[sys] = first + c;
  return c;
}

Stats Engine::stats() {
  Impl& I = *d_;
  if (I.configured) I.check_errors();
  Stats s = I.st;
  s.device_bytes = (int64_t)(I.bytes + I.cell_bytes);
  return s;
}

void* Engine::stream() const { return (void*)d_->stream; }

void Engine::neighbors(int sys, int full, double rcut, int64_t* counts, int64_t* idx, int64_t cap, int64_t* total) {
  Impl& I = *d_;
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  I.ensure_ready();
  if (!I.forces_valid) I.update_forces();
  I.set_buffers(I.cbuf);
  const SysDev& S = I.sysd[sys];
  const int n = S.natoms;
  if (S.mode == NB_LIST) {
    double rl = std::sqrt((double)S.rlist2f / (1.0 + 1e-5));
    if (rcut > rl * (1.0 - 1e-9))
      throw Error(1, "rcut exceeds the neighbour-list radius (cutoff + skin)");
  }
  int half = 0;
  if (!full) half = (I.cm.kind == CM_LINKEDCELL || I.cm.kind == CM_LCBINARY) ? 1 : 2;
  const double rc2 = rcut * rcut;
  const float lo = band_lo(rc2), hi = band_hi(rc2);
  const bool mixed = I.precision == PREC_MIXED;
  long long *dc = nullptr, *doff = nullptr, *didx = nullptr;
  CK(dev_malloc(&dc, sizeof(long long) * std::max(n, 1)));
  CK(dev_malloc(&doff, sizeof(long long) * std::max(n, 1)));
  auto launch = [&](long long* cnt, const long long* off, long long* ix) {
    const unsigned nb = nblocks(n, 128);
    if (n == 0) return;
    if (S.mode == NB_LIST) {
      if (mixed)
        k_export<NB_LIST, 1><<<nb, 128, 0, I.stream>>>(I.D, sys, rc2, lo, hi, half, cnt, off, ix);
      else
        k_export<NB_LIST, 0><<<nb, 128, 0, I.stream>>>(I.D, sys, rc2, lo, hi, half, cnt, off, ix);
    } else if (S.mode == NB_CELLS) {
      k_export<NB_CELLS, 0><<<nb, 128, 0, I.stream>>>(I.D, sys, rc2, lo, hi, half, cnt, off, ix);
    } else {
      k_export<NB_ALLPAIRS, 0><<<nb, 128, 0, I.stream>>>(I.D, sys, rc2, lo, hi, half, cnt, off, ix);
    }
    I.launched();
    I.check_launch("export");
  };
  try {
    launch(dc, nullptr, nullptr);
    std::vector<long long> hc(n), ho(n);
    CK(cudaMemcpyAsync(hc.data(), dc, sizeof(long long) * n, cudaMemcpyDeviceToHost, I.stream));
    CK(cudaStreamSynchronize(I.stream));
    long long t = 0;
    for (int k = 0; k < n; ++k) {
      ho[k] = t;
      t += hc[k];
    }
    if (counts)
      for (int k = 0; k < n; ++k) counts[k] = hc[k];
    if (total) *total = t;
    if (idx && t > 0) {
      if (cap < t) throw Error(9, "neighbour index buffer too small");
      CK(dev_malloc(&didx, sizeof(long long) * t));
      CK(cudaMemcpyAsync(doff, ho.data(), sizeof(long long) * n, cudaMemcpyHostToDevice, I.stream));
      launch(nullptr, doff, didx);
      CK(cudaMemcpyAsync(idx, didx, sizeof(long long) * t, cudaMemcpyDeviceToHost, I.stream));
      CK(cudaStreamSynchronize(I.stream));
    }
  } catch (...) {
    dev_free(dc);
    dev_free(doff);
    dev_free(didx);
    throw;
  }
  dev_free(dc);
  dev_free(doff);
  dev_free(didx);
}

void Engine::cell_sort(int sys, const int32_t n[3], int64_t* cell, int64_t* order) {
  Impl& I = *d_;
  if (sys < 0 || sys >= I.nsys) throw Error(1, "system index out of range");
  for (int q = 0; q < 3; ++q)
    if (n[q] <= 0) throw Error(1, "cell grid must be positive");
  I.ensure_ready();
  I.set_buffers(I.cbuf);
  I.pend = false;
  // Bin and sort on the requested grid with the rebuild kernels, then restore the config.
  std::vector<SysDev> saved = I.sysd;
  I.free_cells();
  int total = 0;
  for (int s = 0; s < I.nsys; ++s) {
    SysDev& S = I.sysd[s];
    S.mode = NB_CELLS;
    for (int q = 0; q < 3; ++q) S.n[q] = n[q];
    S.ncells = n[0] * n[1] * n[2];
    S.cell_base = total;
    total += S.ncells;
  }
  I.alloc_cells(total);
  I.D.nl = nullptr;
  bool any_list = I.any_list;
  I.any_list = false;
  I.upload_sysd();
  I.launch_decide(I.stream, 0, 1, 0, 0);
  I.launch_rebuild(I.stream);
  I.any_list = any_list;
  const int na = I.sysd[sys].natoms;
  long long *dc = nullptr, *dord = nullptr;
  CK(dev_malloc(&dc, sizeof(long long) * std::max(na, 1)));
  CK(dev_malloc(&dord, sizeof(long long) * std::max(na, 1)));
  if (na > 0) k_cells_out<<<nblocks(na, 128), 128, 0, I.stream>>>(I.D, sys, dc, dord);
  I.check_launch("cell_sort");
  std::vector<long long> hc(na), ho(na);
  CK(cudaMemcpyAsync(hc.data(), dc, sizeof(long long) * na, cudaMemcpyDeviceToHost, I.stream));
  CK(cudaMemcpyAsync(ho.data(), dord, sizeof(long long) * na, cudaMemcpyDeviceToHost, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  dev_free(dc);
  dev_free(dord);
  for (int k = 0; k < na; ++k) {
    if (cell) cell[k] = hc[k];
    if (order) order[k] = ho[k];
  }
  I.sysd = saved;
  I.configured = false;
  I.forces_valid = false;
  I.forces_valid_layout = false;
}

// ------------------------------------------------------------------------------------------
// Checkpoint / restore: the complete device state (both memory pools) and the host counters,
// so that a restored engine continues bit for bit.  Simulation::Dump/Restore
// (liblpmd/simulation/simulationbuilder.cc:195-293) write a 6-digit text file instead.
// ------------------------------------------------------------------------------------------

namespace {

struct CkptHeader {
  char magic[8];
  int64_t natoms_total;
  int32_t nsys, precision, total_cells, maxnb;
  int32_t cbuf, pend, initialized, forces_valid, forces_valid_layout, pending_ucalls, flags_any;
  int32_t n_allocs, n_cell_allocs, n_read_from;
  uint64_t config_hash;
  uint64_t body_bytes;
  Stats st;
};

constexpr char CKPT_MAGIC[8] = {'G', 'B', 'M', 'D', 'C', 'K', 'P', '1'};

uint64_t fnv(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t k = 0; k < n; ++k) h = (h ^ b[k]) * 1099511628211ull;
  return h;
}
template <class T>
uint64_t fnv_v(uint64_t h, T v) {
  return fnv(h, &v, sizeof(v));
}

}  // namespace

// Everything that determines the layout and the evolution besides the device state.
static uint64_t config_hash(const Engine::Impl& I) {
  uint64_t h = 1469598103934665603ull;
  for (auto n : I.natoms) h = fnv_v(h, (int64_t)n);
  for (const auto& c : I.cells)
    for (double v : c) h = fnv_v(h, v);
  h = fnv_v(h, I.precision);
  h = fnv_v(h, I.cm.kind);
  h = fnv_v(h, I.cm.cutoff);
  h = fnv_v(h, I.cm.nx);
  h = fnv_v(h, I.cm.ny);
  h = fnv_v(h, I.cm.nz);
  h = fnv_v(h, (int)I.cm.mode_auto);
  h = fnv_v(h, (int64_t)I.cm.maxneighbors);
  h = fnv_v(h, (int64_t)I.cm.each);
  h = fnv_v(h, I.cm.skin);
  h = fnv_v(h, I.opt_skin);
  h = fnv_v(h, I.stencil_r);
  h = fnv_v(h, I.integ.dt);
  h = fnv_v(h, I.integ.kind);
  h = fnv_v(h, I.integ.fmass);
  h = fnv_v(h, I.integ.t);
  for (auto P : I.pots) {  // PotParams is zero-filled before use; the table pointer is this engine's own
    P.tab = nullptr;
    h = fnv(h, &P, sizeof(P));
  }
  return h;
}

size_t Engine::checkpoint_size() {
  Impl& I = *d_;
  I.ensure_ready();
  size_t n = sizeof(CkptHeader) + sizeof(SysDev) * I.sysd.size() + 16 * I.read_from.size();
  for (auto& a : I.allocs) n += a.second;
  for (auto& a : I.cell_allocs) n += a.second;
  return n;
}

void Engine::checkpoint_save(void* buf, size_t bytes) {
  Impl& I = *d_;
  Range r("gbmd:checkpoint_save");
  const size_t need = checkpoint_size();
  if (!buf || bytes < need) throw Error(9, "checkpoint buffer too small: " + std::to_string(need) + " bytes needed");
  CK(cudaStreamSynchronize(I.stream));
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, CKPT_MAGIC, 8);
  h.natoms_total = I.N;
  h.nsys = I.nsys;
  h.precision = I.precision;
  h.total_cells = I.total_cells;
  h.maxnb = I.D.maxnb;
  h.cbuf = I.cbuf;
  h.pend = I.pend;
  h.initialized = I.initialized;
  h.forces_valid = I.forces_valid;
  h.forces_valid_layout = I.forces_valid_layout;
  h.pending_ucalls = I.pending_ucalls;
  h.flags_any = I.flags_any;
  h.n_allocs = (int32_t)I.allocs.size();
  h.n_cell_allocs = (int32_t)I.cell_allocs.size();
  h.n_read_from = (int32_t)I.read_from.size();
  h.config_hash = config_hash(I);
  h.body_bytes = need - sizeof(CkptHeader);
  h.st = I.st;
  char* o = (char*)buf;
  std::memcpy(o, &h, sizeof(h));
  o += sizeof(h);
  std::memcpy(o, I.sysd.data(), sizeof(SysDev) * I.sysd.size());
  o += sizeof(SysDev) * I.sysd.size();
  for (const auto& kv : I.read_from) {
    int64_t pair[2] = {kv.first, kv.second};
    std::memcpy(o, pair, 16);
    o += 16;
  }
  for (auto* pool : {&I.allocs, &I.cell_allocs})
    for (auto& a : *pool) {
      CK(cudaMemcpyAsync(o, a.first, a.second, cudaMemcpyDeviceToHost, I.stream));
      o += a.second;
    }
  CK(cudaStreamSynchronize(I.stream));
}

void Engine::checkpoint_load(const void* buf, size_t bytes) {
  Impl& I = *d_;
  Range r("gbmd:checkpoint_load");
  if (!buf || bytes < sizeof(CkptHeader)) throw Error(1, "checkpoint: truncated");
  CkptHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, CKPT_MAGIC, 8) != 0) throw Error(1, "checkpoint: not a gbmd checkpoint");
  if (bytes != sizeof(CkptHeader) + h.body_bytes) throw Error(1, "checkpoint: size mismatch");
  if (h.natoms_total != I.N || h.nsys != I.nsys) throw Error(1, "checkpoint: different systems");
  I.ensure_ready();
  if (h.total_cells != I.total_cells && I.lcb_exact() && h.config_hash == config_hash(I)) {
    // lcbinary grids only grow: adopt the saved ones (their counts are in the saved systems)
    std::vector<SysDev> saved(I.nsys);
    if (bytes < sizeof(CkptHeader) + sizeof(SysDev) * I.nsys) throw Error(1, "checkpoint: truncated");
    std::memcpy(saved.data(), (const char*)buf + sizeof(CkptHeader), sizeof(SysDev) * I.nsys);
    for (int q = 0; q < I.nsys; ++q)
      for (int a = 0; a < 3; ++a) I.lcb_n[q][a] = saved[q].n[a];
    I.lcb_apply_grids(I.stream);
  }
  if (h.config_hash != config_hash(I) || h.precision != I.precision || h.total_cells != I.total_cells)
    throw Error(1, "checkpoint: cell manager, potentials, integrator, precision or options differ");
  if (h.maxnb != I.D.maxnb) {  // the saved list had grown: give this engine the same capacity
    long long old_entries = 0;
    for (const auto& S : I.sysd) old_entries += (long long)S.natoms * I.D.maxnb;
    I.cell_bytes -= sizeof(unsigned) * (size_t)(old_entries ? old_entries : 1);
    dev_free(I.D.nl);
    I.cell_allocs.erase(std::find_if(I.cell_allocs.begin(), I.cell_allocs.end(),
                                     [&](const std::pair<void*, size_t>& a) { return a.first == (void*)I.D.nl; }));
    I.alloc_list(h.maxnb);
  }
  if (h.n_allocs != (int32_t)I.allocs.size() || h.n_cell_allocs != (int32_t)I.cell_allocs.size())
    throw Error(1, "checkpoint: device layout differs");
  const char* in = (const char*)buf + sizeof(h);
  std::vector<SysDev> sysd(I.nsys);
  std::memcpy(sysd.data(), in, sizeof(SysDev) * I.nsys);
  in += sizeof(SysDev) * I.nsys;
  std::map<int, long long> rf;
  for (int k = 0; k < h.n_read_from; ++k) {
    int64_t pair[2];
    std::memcpy(pair, in, 16);
    in += 16;
    rf[(int)pair[0]] = pair[1];
  }
  size_t body = 0;
  for (auto* pool : {&I.allocs, &I.cell_allocs})
    for (auto& a : *pool) body += a.second;
  if ((size_t)(in - (const char*)buf) + body != bytes) throw Error(1, "checkpoint: device layout differs");
  CK(cudaSetDevice(I.device));
  for (auto* pool : {&I.allocs, &I.cell_allocs})
    for (auto& a : *pool) {
      CK(cudaMemcpyAsync(a.first, in, a.second, cudaMemcpyHostToDevice, I.stream));
      in += a.second;
    }
  CK(cudaStreamSynchronize(I.stream));
  I.sysd = sysd;
  I.read_from = rf;
  I.cbuf = h.cbuf;
  I.pend = h.pend != 0;
  I.initialized = h.initialized != 0;
  I.forces_valid = h.forces_valid != 0;
  I.forces_valid_layout = h.forces_valid_layout != 0;
  I.pending_ucalls = h.pending_ucalls;
  I.flags_any = h.flags_any != 0;
  I.D.has_flags = I.flags_any ? 1 : 0;
  I.st = h.st;
  I.drop_graph();
  I.set_buffers(I.cbuf);
}

}  // namespace gbmd

// grid2d.cu - grid-wide persistent solve_split of small 2D grids (FP32,
// unfolded steps), and the multi-grid pass kernels of batches (end of the
// file; folded steps).
//
// One cooperative launch advances every grid of a batch (or the single grid
// of solve_split) through an outer step of solve_split (solve_split.m:49-80)
// with all SMs on every pass: the y pass of step i is a list of work items
// (grid, tile of y pencils) over all grids, dealt round-robin to the CTAs;
// a grid barrier; the x pass likewise (with the block-end epilogue at the
// last step of a block); a grid barrier; and at a block end the kinetic-
// energy sums (forward FFTs) of the grids whose mu is needed, a barrier, the
// block finalizer of every grid (solve_split.m:65-78, one CTA per grid), a
// barrier.  Each item runs the axis-pass body of the per-pass kernels
// (pass.cuh pass_body) on its tile, so the arithmetic is that of the
// per-pass path; the states (a few hundred KB per grid) stay in L2 between
// passes.  Against the cluster kernel (cluster2d.cuh, one cluster of at most
// 16 SMs per grid) a single grid gets every SM; against the per-pass path a
// pass costs a grid barrier instead of a kernel launch.
//
// The grid barrier is a monotone arrival counter in global memory (zeroed
// before each launch): each CTA's thread 0 releases its writes
// (__threadfence and a release reduction), and polls the counter with acquire loads; the
// poll is bounded (about a second), after which the CTA raises the failure
// flag and returns, and every other CTA stops at its next barrier.  The
// cooperative launch guarantees all CTAs are resident, so the barrier
// completes on any correct run.
#include <algorithm>
#include <type_traits>

#include "cluster2d.h"
#include "grid2d.h"
#include "pass.cuh"

namespace gpe {

// Both passes on the default plans (fewer instructions and exchanges than
// the alternative plans; the contiguous exchange of PlanAlt<256> also has
// 2-way bank conflicts).
template <int N>
using G2P = Plan<N>;
template <int N>
using G2Y = ContigLayout<G2P<N>, float>;
template <int N>
using G2X = StridedLayout<Plan<N>, float>;

#define X(v)                                                                                   \
  static_assert(G2Y<v>::THREADS == G2_THREADS && G2X<v>::THREADS == G2_THREADS,                \
                "grid2d kernel: every pass body of length " #v " runs on G2_THREADS threads");
GPE_C2_SIZES(X)
#undef X

template <class P, class L>
constexpr size_t g2_body_smem() {
  const size_t a = pass_smem_bytes<float, P, L, KIND_STEP>(), b = pass_smem_bytes<float, P, L, KIND_ENERGY>();
  return a > b ? a : b;
}
constexpr size_t g2_smem_max() {
  size_t m = 0;
#define X(v)                                                         \
  m = m > g2_body_smem<G2P<v>, G2Y<v>>() ? m : g2_body_smem<G2P<v>, G2Y<v>>(); \
  m = m > g2_body_smem<Plan<v>, G2X<v>>() ? m : g2_body_smem<Plan<v>, G2X<v>>();
  GPE_C2_SIZES(X)
#undef X
  return m;
}
constexpr size_t G2_SMEM = g2_smem_max();
// Resident CTAs per SM the kernel is compiled for (registers per thread =
// 65536 / (G2_THREADS * G2_MIN_BLOCKS), capped at 255).
#ifndef G2_MIN_BLOCKS
#define G2_MIN_BLOCKS 2
#endif

// Bounded grid barrier (see the file comment).  False: the wait ran out
// somewhere; the caller returns.
__device__ __forceinline__ bool g2_sync(const G2Args& a, unsigned& target) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    target += gridDim.x;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(a.bar) : "memory");
    int good = 1;
    for (long long it = 0;; ++it) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a.bar) : "memory");
      if ((int)(v - target) >= 0) break;
      if (*(volatile int*)a.fail) {
        good = 0;
        break;
      }
      if (it > (1LL << 22)) {
        good = 0;
        atomicExch(a.fail, 1);
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Grid of item `item`: the last g with off[g] <= item.
__device__ __forceinline__ int g2_find(const int* off, int ng, int item) {
  int lo = 0, hi = ng - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Pass arguments of grid G's y pass (axis 1) or x pass (axis 0).
__device__ __forceinline__ PassArgs<float> g2_args(const G2Grid& G, int axis) {
  PassArgs<float> p{};
  p.psi = static_cast<cx<float>*>(G.psi);
  p.V = static_cast<const float*>(G.V);
  p.php = static_cast<const cx<float>*>(G.php[axis]);
  p.tws = static_cast<const cx<float>*>(G.tws[axis]);
  p.k2p = static_cast<const float*>(G.k2p[axis]);
  p.partials = G.partials;
  p.sc = G.sc;
  p.cap = G.cap;
  p.npts = (long long)G.nx * G.ny;
  if (axis == 1) {
    p.n_batch = G.nx;
    p.stride = 1;
    p.inner = 1;
    p.outer = 0;
    p.kin_slot = S_KY;
  } else {
    p.n_batch = G.ny;
    p.stride = G.ny;
    p.inner = G.ny;
    p.outer = (long long)G.nx * G.ny;
    p.kin_slot = S_KX;
  }
  p.g = G.g;
  p.dre = G.dre;
  p.dim = G.dim;
  p.gr = (float)G.g;
  p.drer = (float)G.dre;
  p.dimr = (float)G.dim;
  return p;
}

// The pass bodies by axis length: one dispatcher per (axis, kind), each
// called from one place, so that every body is inlined once.
template <int AXIS, int KIND>
__device__ __forceinline__ void g2_body(int n, const PassArgs<float>& p, long long tile, unsigned char* smem,
                                        float s, float mu) {
  switch (n) {
#define X(v)                                                                        \
  case v:                                                                           \
    if constexpr (AXIS == 1)                                                        \
      pass_body<float, G2P<v>, G2Y<v>, KIND>(p, tile, smem, s, mu);        \
    else                                                                            \
      pass_body<float, Plan<v>, G2X<v>, KIND>(p, tile, smem, s, mu);                 \
    break;
    GPE_C2_SIZES(X)
#undef X
  }
}

// Sum of partials[0 .. n) over the CTA in FP64 (fixed order: thread t sums
// t, t + G2_THREADS, ..., then a fixed tree), broadcast to every thread.
__device__ __forceinline__ double g2_cta_sum(const double* p, int n, double* red) {
  double x = 0.0;
  for (int i = threadIdx.x; i < n; i += G2_THREADS) x += p[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < G2_THREADS / 32; ++w) s += red[w];
  __syncthreads();
  return s;
}

// The block finalizer of grid g (the arithmetic of aux_kernels.cu
// k_finalize_block): sums of the block-end epilogue (the tiles of the pass
// that ran it: x, or y after folded steps with an even n_rec) and, when mu
// is needed, the kinetic sums (y and x tiles); mu, the renormalisation
// factor, the history record of the outer step's last block.
__device__ void g2_finalize(const G2Args& a, int g, int jj, bool last, double* red) {
  const G2Grid& G = a.grids[g];
  DevScalars* sc = G.sc;
  if (__syncthreads_or(sc->stop != 0)) return;
  const bool need = G.feedback || last;
  const int cap = G.cap;
  const int ne = a.epi_y ? G.ytiles : G.xtiles;  // tiles of the pass that ran the epilogue
  const double n = g2_cta_sum(G.partials + S_N * cap, ne, red);
  const double vn = g2_cta_sum(G.partials + S_VN * cap, ne, red);
  const double n2 = g2_cta_sum(G.partials + S_N2 * cap, ne, red);
  double kin = 0.0;
  if (need) kin = g2_cta_sum(G.partials + S_KY * cap, G.ytiles, red) + g2_cta_sum(G.partials + S_KX * cap, G.xtiles, red);
  if (threadIdx.x != 0) return;
  const int outer = sc->outer;
  const int j = G.start + 1 + outer;                                  // solve_split.m:49
  const double time2 = (j - 1) * a.dt_outer + (jj - 1) * a.ddt * a.n_rec;  // solve_split.m:53
  const double w = G.weight;
  const double ncur = n * w;  // solve_split.m:67
  double muc, scale = 1.0, energy = 0.0;
  if (G.feedback) {  // solve_split.m:68-75
    double NNN = sc->NNN;
    if (G.tau > 0) NNN = sc->NN0 * exp(-time2 / G.tau);
    sc->NNN = NNN;
    scale = sqrt(NNN / ncur);
    const double s2 = scale * scale;
    muc = (s2 * (kin + vn) * w + s2 * s2 * G.g * n2 * w) / NNN;
    energy = s2 * (kin + vn) * w + 0.5 * s2 * s2 * G.g * n2 * w;
    sc->mu = muc;
  } else {  // solve_split.m:76-77
    muc = (kin + vn + G.g * n2) * w / ncur;
    energy = (kin + vn + 0.5 * G.g * n2) * w;
  }
  sc->energy = energy;
  sc->scale = scale;
  sc->ncur = ncur;
  sc->muc = muc;
  sc->sums[S_N] = n * w;
  sc->sums[S_VN] = vn * w;
  sc->sums[S_N2] = n2 * w;
  const bool bad = !isfinite(ncur) || !isfinite(muc) || !isfinite(scale);
  if (bad) {
    sc->nonfinite = 1;
    sc->status = NONFINITE;
    sc->stop = 1;
  }
  if (last && !bad) {
    double* h = G.hist + 3 * (size_t)outer;
    h[0] = muc;
    h[1] = ncur;
    h[2] = energy;
    sc->outer = outer + 1;
  }
}

__global__ void __launch_bounds__(G2_THREADS, G2_MIN_BLOCKS) k_grid2d(const G2Args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float s_sc[2];
  __shared__ double red[G2_THREADS / 32];
  __shared__ int s_item;
  unsigned target = 0;
  // Items are taken from a monotone counter (a.bar[1], zero at launch): the
  // phase with n items owns the values base .. base + n - 1; every CTA ends a
  // phase with one grab past its end, so the next phase's base is
  // base + n + gridDim.x on every CTA.  Items of uneven cost (grids of
  // different sizes) spread evenly over the CTAs.
  unsigned base = 0;
  auto grab = [&](unsigned n) -> int {
    if (threadIdx.x == 0) {
      const unsigned v = atomicAdd(a.bar + 1, 1u) - base;
      s_item = v < n ? (int)v : -1;
    }
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    return it;
  };
  const int ng = a.ngrids;
  const int ny_items = a.yoff[ng], nx_items = a.xoff[ng];
  // one item of a pass: the grid's pending scale and mu, the stop vote
  auto item_run = [&](auto axis_c, auto kind_c, const int* off, int pro, int epi, int item, bool skip_unneeded,
                      bool last) {
    constexpr int AXIS = decltype(axis_c)::value, KIND = decltype(kind_c)::value;
    const int g = g2_find(off, ng, item);
    const G2Grid& G = a.grids[g];
    if (threadIdx.x == 0) {
      s_sc[0] = (float)G.sc->scale;
      s_sc[1] = (float)G.sc->mu;
    }
    const bool skip = __syncthreads_or(G.sc->stop != 0) || (skip_unneeded && !(G.feedback || last));
    if (!skip) {
      PassArgs<float> p = g2_args(G, AXIS);
      p.kind = KIND;
      p.pro = pro;
      p.epi = epi;
      // the pass body reads V for a phase prologue only when side says so
      p.side = (pro == PRO_RT_HALF || pro == PRO_RT_FULL || epi == EPI_RT_END) ? 1 : 0;
      g2_body<AXIS, KIND>(AXIS == 1 ? G.ny : G.nx, p, item - off[g], smem, s_sc[0], s_sc[1]);
    }
    __syncthreads();  // shared memory and s_sc are reused by the next item
  };
  using Y = std::integral_constant<int, 1>;
  using Xa = std::integral_constant<int, 0>;
  using Step = std::integral_constant<int, KIND_STEP>;
  using Energy = std::integral_constant<int, KIND_ENERGY>;
  for (int o = 0; o < a.nouter; ++o) {
    for (int jj = 1; jj <= a.nb; ++jj) {
      const bool last = jj == a.nb;
      for (int i = 1; i <= a.n_rec; ++i) {
        const int pro = i == 1 ? PRO_RT_HALF : PRO_RT_FULL;  // solve_split.m:55-56 / 60-61
        for (int item = grab(ny_items); item >= 0; item = grab(ny_items))
          item_run(Y{}, Step{}, a.yoff, pro, EPI_NONE, item, false, last);
        base += ny_items + gridDim.x;
        if (!g2_sync(a, target)) return;
        const int epi = i == a.n_rec ? EPI_RT_END : EPI_NONE;  // solve_split.m:60-67
        for (int item = grab(nx_items); item >= 0; item = grab(nx_items))
          item_run(Xa{}, Step{}, a.xoff, PRO_NONE, epi, item, false, last);
        base += nx_items + gridDim.x;
        if (!g2_sync(a, target)) return;
      }
      // kinetic sums of the block-end state of the grids whose mu is needed
      for (int item = grab(ny_items + nx_items); item >= 0; item = grab(ny_items + nx_items)) {
        if (item < ny_items) item_run(Y{}, Energy{}, a.yoff, PRO_NONE, EPI_NONE, item, true, last);
        else item_run(Xa{}, Energy{}, a.xoff, PRO_NONE, EPI_NONE, item - ny_items, true, last);
      }
      base += ny_items + nx_items + gridDim.x;
      if (!g2_sync(a, target)) return;
      for (int g = blockIdx.x; g < ng; g += gridDim.x) g2_finalize(a, g, jj, last, red);
      if (!g2_sync(a, target)) return;
    }
  }
}

int grid2d_tile_pencils(int n, bool strided) {
  switch (n) {
#define X(v) \
  case v:    \
    return strided ? G2X<v>::FFTS : G2Y<v>::FFTS;
    GPE_C2_SIZES(X)
#undef X
  }
  return 0;
}

size_t grid2d_smem() { return G2_SMEM; }

int grid2d_max_ctas() {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  if (cudaFuncSetAttribute(k_grid2d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G2_SMEM) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_grid2d, G2_THREADS, G2_SMEM) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return per * sms;
}

cudaError_t launch_grid2d(const G2Args& a, int nctas, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)nctas);
  cfg.blockDim = dim3(G2_THREADS);
  cfg.dynamicSmemBytes = G2_SMEM;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_grid2d, a);
}

// ---- multi-grid pass kernels ------------------------------------------------------
// The work items of the grid-wide kernel, one launch per pass over the tiles
// of a group of grids of one shape (CTA = item): each (axis, kind, length)
// kernel has the register allocation and occupancy of the per-pass kernels,
// kernel boundaries replace the grid barriers, and the groups of a batch run
// on their own streams.  The launches of an outer step are one
// CUDA graph with programmatic dependent launch between them.

template <int AXIS, int KIND, int N>
__device__ __forceinline__ void g2m_item(const G2Args& a, int pro, int epi, int item, bool skip_unneeded, bool last,
                                         unsigned char* smem) {
  __shared__ float s_sc[2];
  const int* off = AXIS == 1 ? a.yoff : a.xoff;
  const int g = g2_find(off, a.ngrids, item);
  const G2Grid& G = a.grids[g];
  if (threadIdx.x == 0) {
    s_sc[0] = (float)G.sc->scale;
    s_sc[1] = (float)G.sc->mu;
  }
  if (__syncthreads_or(G.sc->stop != 0) || (skip_unneeded && !(G.feedback || last))) return;
  PassArgs<float> p = g2_args(G, AXIS);
  p.kind = KIND;
  p.pro = pro;
  p.epi = epi;
  // the pass body reads V for a phase prologue only when side says so
  p.side = (pro == PRO_RT_HALF || pro == PRO_RT_FULL || epi == EPI_RT_END) ? 1 : 0;
  p.fold = KIND == KIND_STEP_EXT ? 1 : 0;  // the extended kernel runs the folded passes
  if constexpr (AXIS == 1)
    pass_body<float, G2P<N>, G2Y<N>, KIND>(p, item - off[g], smem, s_sc[0], s_sc[1]);
  else
    pass_body<float, Plan<N>, G2X<N>, KIND>(p, item - off[g], smem, s_sc[0], s_sc[1]);
}

template <int AXIS, int N>
struct G2MBounds {
  using P = std::conditional_t<AXIS == 1, G2P<N>, Plan<N>>;
  using L = std::conditional_t<AXIS == 1, G2Y<N>, G2X<N>>;
  static constexpr int value = MinBlocks<float, P, L>::value;
};

// One pass (AXIS 1: y, 0: x) over the tiles of every grid of the group:
// KIND_STEP with the given prologue and epilogue, KIND_STEP_EXT (a folded
// pass: two steps' transforms with the full nonlinear step between them),
// or KIND_ENERGY (the kinetic sums of the grids whose mu is needed at this
// block end).
template <int AXIS, int KIND, int N>
__global__ void __launch_bounds__(G2_THREADS, G2MBounds<AXIS, N>::value)
    k_multi2d(const G2Args a, int pro, int epi, int last) {
  extern __shared__ __align__(16) unsigned char smem[];
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  g2m_item<AXIS, KIND, N>(a, pro, epi, (int)blockIdx.x, KIND == KIND_ENERGY, last != 0, smem);
}

// The block finalizer of every grid of the group: CTA g = grid g.
__global__ void __launch_bounds__(G2_THREADS) k_multi2d_final(const G2Args a, int jj, int last) {
  __shared__ double red[G2_THREADS / 32];
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  g2_finalize(a, (int)blockIdx.x, jj, last != 0, red);
}

static cudaError_t g2m_launch(const void* kern, void** args, int nblocks, size_t smem, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)nblocks);
  cfg.blockDim = dim3(G2_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, kern, args);
}

struct G2MKernels {
  const void* k[2][3];  // [axis][kind: 0 step, 1 energy, 2 folded step]
  size_t smem[2][3];
};

template <int N>
static G2MKernels g2m_kernels() {
  G2MKernels K;
  K.k[1][0] = (const void*)k_multi2d<1, KIND_STEP, N>;
  K.k[1][1] = (const void*)k_multi2d<1, KIND_ENERGY, N>;
  K.k[0][0] = (const void*)k_multi2d<0, KIND_STEP, N>;
  K.k[0][1] = (const void*)k_multi2d<0, KIND_ENERGY, N>;
  K.k[1][2] = (const void*)k_multi2d<1, KIND_STEP_EXT, N>;
  K.k[0][2] = (const void*)k_multi2d<0, KIND_STEP_EXT, N>;
  K.smem[1][2] = pass_smem_bytes<float, G2P<N>, G2Y<N>, KIND_STEP_EXT>();
  K.smem[0][2] = pass_smem_bytes<float, Plan<N>, G2X<N>, KIND_STEP_EXT>();
  K.smem[1][0] = pass_smem_bytes<float, G2P<N>, G2Y<N>, KIND_STEP>();
  K.smem[1][1] = pass_smem_bytes<float, G2P<N>, G2Y<N>, KIND_ENERGY>();
  K.smem[0][0] = pass_smem_bytes<float, Plan<N>, G2X<N>, KIND_STEP>();
  K.smem[0][1] = pass_smem_bytes<float, Plan<N>, G2X<N>, KIND_ENERGY>();
  return K;
}

static bool g2m_lookup(int n, G2MKernels* K) {
  switch (n) {
#define X(v)               \
  case v:                  \
    *K = g2m_kernels<v>(); \
    return true;
    GPE_C2_SIZES(X)
#undef X
  }
  return false;
}

cudaError_t launch_multi2d_block(const G2Args& a, int ny, int nx, int ny_items, int nx_items, int jj, bool last,
                                 bool energy, bool fold, cudaStream_t s) {
  G2MKernels KY, KX;
  if (!g2m_lookup(ny, &KY) || !g2m_lookup(nx, &KX)) return cudaErrorInvalidValue;
  const void* ky[3] = {KY.k[1][0], KY.k[1][1], KY.k[1][2]};
  const void* kx[3] = {KX.k[0][0], KX.k[0][1], KX.k[0][2]};
  const size_t sy[3] = {KY.smem[1][0], KY.smem[1][1], KY.smem[1][2]};
  const size_t sx[3] = {KX.smem[0][0], KX.smem[0][1], KX.smem[0][2]};
  for (int k = 0; k < 3; ++k) {
    cudaError_t e = cudaFuncSetAttribute(ky[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sy[k]);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kx[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx[k]);
    if (e != cudaSuccess) return e;
  }
  G2Args args = a;
  args.epi_y = fold && a.n_rec % 2 == 0 ? 1 : 0;  // the last step's order is x y
  int lst = last ? 1 : 0, j = jj, pnone = PRO_NONE, enone = EPI_NONE;
  cudaError_t e = cudaSuccess;
  if (fold) {
    // folded steps: y x for odd steps, x y for even ones; the shared axis of
    // consecutive steps is one folded pass (the extended kernel): 1 + n_rec
    // pass launches per block
    int pro = PRO_RT_HALF;  // solve_split.m:55-56
    void* ay[4] = {&args, &pro, &enone, &lst};
    e = g2m_launch(ky[0], ay, ny_items, sy[0], s);
    for (int i = 1; i <= a.n_rec && e == cudaSuccess; ++i) {
      const bool xa = i % 2 == 1;
      const int k = i < a.n_rec ? 2 : 0;
      int epi = i == a.n_rec ? EPI_RT_END : EPI_NONE;  // solve_split.m:60-67
      void* ar[4] = {&args, &pnone, &epi, &lst};
      e = xa ? g2m_launch(kx[k], ar, nx_items, sx[k], s) : g2m_launch(ky[k], ar, ny_items, sy[k], s);
    }
  }
  for (int i = 1; i <= a.n_rec && e == cudaSuccess && !fold; ++i) {
    int pro = i == 1 ? PRO_RT_HALF : PRO_RT_FULL;  // solve_split.m:55-56 / 60-61
    void* ay[4] = {&args, &pro, &enone, &lst};
    e = g2m_launch(ky[0], ay, ny_items, sy[0], s);
    int epi = i == a.n_rec ? EPI_RT_END : EPI_NONE;  // solve_split.m:60-67
    void* ax[4] = {&args, &pnone, &epi, &lst};
    if (e == cudaSuccess) e = g2m_launch(kx[0], ax, nx_items, sx[0], s);
  }
  if (e == cudaSuccess && energy) {
    void* ae[4] = {&args, &pnone, &enone, &lst};
    e = g2m_launch(ky[1], ae, ny_items, sy[1], s);
    if (e == cudaSuccess) e = g2m_launch(kx[1], ae, nx_items, sx[1], s);
  }
  if (e == cudaSuccess) {
    void* af[3] = {&args, &j, &lst};
    e = g2m_launch((const void*)k_multi2d_final, af, a.ngrids, 0, s);
  }
  return e;
}

}  // namespace gpe

// pass_launch.cuh - host launchers of the axis-pass kernel, explicitly
// instantiated per (precision, axis length) in the pass_*.cu files so that
// the FFT kernels compile in parallel translation units.
#pragma once
#include <string.h>

#include "pass_tma.cuh"

namespace gpe {

template <typename R, int N, int V>
PassGeom pass_geom(bool strided) {
  using P = typename PlanSel<N, V>::type;
  if (strided) {
    using L = StridedLayout<P, R>;
    return PassGeom{L::THREADS, L::FFTS, L::smem_bytes()};
  }
  using L = ContigLayout<P, R>;
  return PassGeom{L::THREADS, L::FFTS, L::smem_bytes()};
}

template <int N, int V>
PlanInfo plan_info() {
  using P = typename PlanSel<N, V>::type;
  PlanInfo pi{};
  pi.N = P::N;
  pi.T = P::T;
  pi.E = P::E;
  pi.nstages = P::NSTAGES;
  for (int s = 0; s < P::NSTAGES; ++s) pi.radix[s] = P::radix[s];
  return pi;
}

// Resident CTAs per SM of a kernel at a given dynamic shared-memory size,
// cached (the occupancy query costs a few microseconds of host time).
int resident_ctas(const void* kern, int threads, size_t smem);
// SMs of the current device (cached).
int device_sm_count();

template <typename R, class P, class L>
static cudaError_t launch_layout(const PassArgs<R>& a, cudaStream_t s) {
  auto kern = a.kind == KIND_ENERGY     ? pass_kernel<R, P, L, KIND_ENERGY>
              : a.kind == KIND_STEP_EXT ? pass_kernel<R, P, L, KIND_STEP_EXT>
                                        : pass_kernel<R, P, L, KIND_STEP>;
  const size_t smem = a.kind == KIND_ENERGY     ? pass_smem_bytes<R, P, L, KIND_ENERGY>()
                      : a.kind == KIND_STEP_EXT ? pass_smem_bytes<R, P, L, KIND_STEP_EXT>()
                                                : pass_smem_bytes<R, P, L, KIND_STEP>();
  // Above 32 KB of dynamic shared memory opt in explicitly: the static
  // reduction scratch counts toward the 48 KB default limit too.
  if (smem > 32 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const long long blocks = (a.n_batch + L::FFTS - 1) / L::FFTS;
  if (blocks > a.cap || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  PassArgs<R> b = a;
  b.pf_ahead = 0;
  if (a.prefetch) {
    const int wave = resident_ctas((const void*)kern, L::THREADS, smem) * device_sm_count();
    if (wave > 0 && blocks > wave) b.pf_ahead = wave;
  }
  if (!a.pdl) {
    kern<<<(unsigned)blocks, L::THREADS, smem, s>>>(b);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(L::THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, b);
}

template <typename R, int N, int V>
cudaError_t launch_pass(const PassArgs<R>& a, bool strided, cudaStream_t s) {
  using P = typename PlanSel<N, V>::type;
  if (strided) return launch_layout<R, P, StridedLayout<P, R>>(a, s);
  return launch_layout<R, P, ContigLayout<P, R>>(a, s);
}

// ---- TMA-staged persistent variant --------------------------------------

// Tensor map of a state (units = 2: complex) or side array (units = 1) of
// `unit`-byte reals laid out as tdim = (ny, nx, nz, components), with a box of
// `pencils` y positions by `len` positions along axis `ax` (1 = x, 2 = z).
// False when the driver offers no tensor maps or refuses the layout.
bool encode_tile_map(CUtensorMap* m, const void* base, int unit, int units, const long long* tdim, int pencils,
                     int ax, int len);

template <typename R, class P, class L>
static cudaError_t launch_tma_layout(const PassArgs<R>& a, cudaStream_t s, int sms) {
  using SMB = TmaSmem<L, R>;
  auto kern = a.kind == KIND_ENERGY ? pass_tma_kernel<R, P, L, KIND_ENERGY> : pass_tma_kernel<R, P, L, KIND_STEP>;
  const size_t smem = SMB::bytes(a.side != 0);
  if (smem > 32 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const long long ntiles = (a.n_batch + L::FFTS - 1) / L::FFTS;
  const int per_sm = resident_ctas((const void*)kern, L::THREADS, smem);
  long long grid = (long long)sms * (per_sm > 0 ? per_sm : 1);
  if (grid > ntiles) grid = ntiles;
  if (grid > a.cap) grid = a.cap;
  PassArgs<R> b = a;
  CUtensorMap tm_psi, tm_side;
  memset(&tm_psi, 0, sizeof(tm_psi));
  memset(&tm_side, 0, sizeof(tm_side));
  if constexpr (!L::CONTIG) {
    const int ax = a.stride == a.tdim[0] ? 1 : 2;
    const int len = P::N > 256 ? P::N / 2 : P::N;
    b.tma_tensor = a.tma_tensor && a.tdim[0] % L::FFTS == 0 &&
                   encode_tile_map(&tm_psi, a.psi, (int)sizeof(R), 2, a.tdim, L::FFTS, ax, len) &&
                   (a.side == 0 || encode_tile_map(&tm_side, a.side == 2 ? (const void*)a.aux : (const void*)a.V,
                                                   (int)sizeof(R), 1, a.tdim, L::FFTS, ax, len));
  } else {
    b.tma_tensor = 0;
  }
  kern<<<(unsigned)grid, L::THREADS, smem, s>>>(b, tm_psi, tm_side);
  return cudaGetLastError();
}

template <typename R, int N>
cudaError_t launch_pass_tma(const PassArgs<R>& a, bool strided, cudaStream_t s, int sms, int* grid_out) {
  using P = Plan<N>;
  cudaError_t e;
  if (strided) {
    using L = TStrided<P, R>;
    e = launch_tma_layout<R, P, L>(a, s, sms);
  } else {
    using L = TContig<P, R>;
    e = launch_tma_layout<R, P, L>(a, s, sms);
  }
  return e;
}

// CTAs a TMA pass launches (partial sums land in that many slots).
template <typename R, int N>
int pass_tma_grid(const PassArgs<R>& a, bool strided, int sms) {
  using P = Plan<N>;
  auto g = [&](auto L_) {
    using L = decltype(L_);
    using SMB = TmaSmem<L, R>;
    auto kern = a.kind == KIND_ENERGY ? pass_tma_kernel<R, P, L, KIND_ENERGY> : pass_tma_kernel<R, P, L, KIND_STEP>;
    const size_t smem = SMB::bytes(a.side != 0);
    if (smem > 32 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const long long ntiles = (a.n_batch + L::FFTS - 1) / L::FFTS;
    const int per_sm = resident_ctas((const void*)kern, L::THREADS, smem);
    long long grid = (long long)sms * (per_sm > 0 ? per_sm : 1);
    if (grid > ntiles) grid = ntiles;
    if (grid > a.cap) grid = a.cap;
    return (int)grid;
  };
  if (strided) return g(TStrided<P, R>{});
  return g(TContig<P, R>{});
}

// Pencils per tile of the TMA pass (strided tiles must not straddle rows).
template <typename R, int N>
int pass_tma_ffts(bool strided) {
  using P = Plan<N>;
  return strided ? TStrided<P, R>::FFTS : TContig<P, R>::FFTS;
}

// Dynamic shared memory of a TMA pass with side staging (the larger case).
template <typename R, int N>
size_t pass_tma_smem(bool strided) {
  using P = Plan<N>;
  return strided ? TmaSmem<TStrided<P, R>, R>::bytes(true) : TmaSmem<TContig<P, R>, R>::bytes(true);
}

#define GPE_INST_PASS(R, N)                                                                  \
  template PassGeom pass_geom<R, N>(bool);                                                   \
  template cudaError_t launch_pass<R, N>(const PassArgs<R>&, bool, cudaStream_t);            \
  template cudaError_t launch_pass_tma<R, N>(const PassArgs<R>&, bool, cudaStream_t, int, int*); \
  template int pass_tma_grid<R, N>(const PassArgs<R>&, bool, int);                          \
  template int pass_tma_ffts<R, N>(bool);                                                   \
  template size_t pass_tma_smem<R, N>(bool);

// Plan descriptions are precision independent: instantiated once (FP32 files).
#define GPE_INST_PLAN(N) template PlanInfo plan_info<N>();

// The alternative plan of N (FP32 direct passes only).
#define GPE_INST_PASS_ALT(N)                                                              \
  template PassGeom pass_geom<float, N, 1>(bool);                                         \
  template cudaError_t launch_pass<float, N, 1>(const PassArgs<float>&, bool, cudaStream_t); \
  template PlanInfo plan_info<N, 1>();

}  // namespace gpe

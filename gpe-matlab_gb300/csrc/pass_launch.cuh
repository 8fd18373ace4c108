// pass_launch.cuh - host launchers of the axis-pass kernel, explicitly
// instantiated per (precision, axis length) in the pass_*.cu files so that
// the FFT kernels compile in parallel translation units.
#pragma once
#include "pass.cuh"

namespace gpe {

template <typename R, int N>
PassGeom pass_geom(bool strided) {
  using P = Plan<N>;
  if (strided) {
    using L = StridedLayout<P, R>;
    return PassGeom{L::THREADS, L::FFTS, L::smem_bytes()};
  }
  using L = ContigLayout<P, R>;
  return PassGeom{L::THREADS, L::FFTS, L::smem_bytes()};
}

template <typename R, class P, class L>
static cudaError_t launch_layout(const PassArgs<R>& a, cudaStream_t s) {
  auto kern = pass_kernel<R, P, L>;
  const size_t smem = L::smem_bytes();
  // Above 32 KB of dynamic shared memory opt in explicitly: the static
  // reduction scratch counts toward the 48 KB default limit too.
  if (smem > 32 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const long long blocks = (a.n_batch + L::FFTS - 1) / L::FFTS;
  if (blocks > a.cap || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  kern<<<(unsigned)blocks, L::THREADS, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename R, int N>
cudaError_t launch_pass(const PassArgs<R>& a, bool strided, cudaStream_t s) {
  using P = Plan<N>;
  if (strided) return launch_layout<R, P, StridedLayout<P, R>>(a, s);
  return launch_layout<R, P, ContigLayout<P, R>>(a, s);
}

#define GPE_INST_PASS(R, N)                                                      \
  template PassGeom pass_geom<R, N>(bool);                                       \
  template cudaError_t launch_pass<R, N>(const PassArgs<R>&, bool, cudaStream_t);

}  // namespace gpe

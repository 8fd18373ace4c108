// pass_x2_launch.cuh - host launchers of the paired FP32 step pass, explicitly
// instantiated per axis length and plan in pass_x2_*.cu: on PlanAlt<N> for
// every length with an alternative plan (E = 8 or 12 points per pencil and
// thread), and on Plan<N> for 128, 256 and 512 (E = 16).  Each reads the
// tables of its plan.
#pragma once
#include "pass_launch.cuh"
#include "pass_x2.cuh"

namespace gpe {

template <class P, class L>
static cudaError_t launch_x2_layout(const PassArgs<float>& a, cudaStream_t s) {
  auto kern = a.fold ? pass_x2_kernel<P, L, true> : pass_x2_kernel<P, L, false>;
  const size_t smem = x2_smem_bytes<P, L>();
  if (smem > 32 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const long long blocks = (a.n_batch + L::PENCILS - 1) / L::PENCILS;
  if (blocks > a.cap || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  PassArgs<float> b = a;
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

template <int N, int V>
PassGeom pass_x2_geom(bool strided) {
  using P = typename PlanSel<N, V>::type;
  if (strided) return PassGeom{StridedX2<P>::THREADS, StridedX2<P>::PENCILS, x2_smem_bytes<P, StridedX2<P>>()};
  return PassGeom{ContigX2<P>::THREADS, ContigX2<P>::PENCILS, x2_smem_bytes<P, ContigX2<P>>()};
}

template <int N, int V>
cudaError_t launch_pass_x2(const PassArgs<float>& a, bool strided, cudaStream_t s) {
  using P = typename PlanSel<N, V>::type;
  if (strided) return launch_x2_layout<P, StridedX2<P>>(a, s);
  return launch_x2_layout<P, ContigX2<P>>(a, s);
}

#define GPE_INST_PASS_X2(N, V)                \
  template PassGeom pass_x2_geom<N, V>(bool); \
  template cudaError_t launch_pass_x2<N, V>(const PassArgs<float>&, bool, cudaStream_t);

}  // namespace gpe

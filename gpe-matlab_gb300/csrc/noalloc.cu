// noalloc.cu - gpe_norm_noalloc: integrate(|psi|^2) of a caller's device
// array without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a
// norm: a MATLAB MEX function working on gpuArray data whose memory belongs
// to MATLAB's own GPU allocator, a user callback running in the middle of a
// solve_split call, or an application that sizes and owns all device memory
// up front.  For them this entry point runs the same per-chunk reduction as
// the context-based norm, but its per-CTA partial sums live in a fixed
// file-scope device array instead of a context's scratch buffer.
//
// The array is NA_MAX_PARTIALS + 1 doubles (256 KB + 8 bytes): one partial
// sum per chunk of NA_CHUNK points plus a result slot, so one call handles at
// most NA_MAX_PARTIALS * NA_CHUNK = 134,217,728 points (512^3).  Every GPU
// that loads the library holds the array until the process exits.  All calls
// share it and it keeps the last call's values; nothing in it has to start at
// zero, because each call writes every partial and the result slot it later
// reads.  Calls that overlap on the GPU (different streams, or threads using
// the same device concurrently) race on the array and must be serialised by
// the caller.
//
// The value is integrate(|psi|^2), the particle number that solve_split
// calls ncur (solve_split.m:65-67 of GPE-MATLAB) and gpe_obs.norm reports:
// the square of MATLAB's grid.norm (norm.m:11).
//
// Before any CUDA call the input pointer is checked for the alignment of
// one complex element, and then asked of the driver: memory the GPU cannot
// address as device memory of the current device (plain or page-locked host
// memory, another device's memory) is refused with GPE_ERR_INVALID instead
// of being handed to a kernel.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/gpe.h"
#include "common.cuh"

namespace gpe {
namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CHUNK = 4096;  // points per CTA (16 per thread)
constexpr int NA_MAX_PARTIALS = 32768;
constexpr long long NA_MAX_POINTS = (long long)NA_MAX_PARTIALS * NA_CHUNK;
constexpr int NA_MAX_DEVICES = 64;

static __device__ __align__(256) double g_na_scratch[NA_MAX_PARTIALS + 1];

// Sum of |psi|^2 over chunk blockIdx.x: FP32/FP64 Kahan per thread, FP64
// across the CTA, one partial per CTA.
template <typename R>
__global__ void __launch_bounds__(NA_THREADS) k_na_partials(const cx<R>* __restrict__ psi, long long n,
                                                          double* partials) {
  const long long base = (long long)blockIdx.x * NA_CHUNK;
  R s = R(0), c = R(0);
#pragma unroll 4
  for (int k = 0; k < NA_CHUNK / NA_THREADS; ++k) {
    const long long i = base + threadIdx.x + (long long)k * NA_THREADS;
    if (i < n) {
      const cx<R> p = psi[i];
      const R y = (p.x * p.x + p.y * p.y) - c;
      const R t = s + y;
      c = (t - s) - y;
      s = t;
    }
  }
  double v = (double)s - (double)c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __shared__ double red[NA_THREADS / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < NA_THREADS / 32; ++w) tot += red[w];
    partials[blockIdx.x] = tot;
  }
}

// Deterministic FP64 Kahan sum of the partials, times the cell volume.
__global__ void __launch_bounds__(NA_THREADS) k_na_final(const double* partials, int nparts, double weight,
                                                       double* out) {
  double s = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < nparts; i += NA_THREADS) {
    const double y = partials[i] - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __shared__ double sh[NA_THREADS];
  sh[threadIdx.x] = s - c;
  __syncthreads();
  for (int o = NA_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0] * weight;
}

std::mutex g_na_mu;
double* g_na_ptr[NA_MAX_DEVICES] = {};

}  // namespace

// Thread-local message returned by gpe_last_error(NULL) (gpe_api.cu).
void set_thread_error(const std::string& msg);

static gpe_status na_fail(gpe_status st, const std::string& msg) {
  set_thread_error(msg);
  return st;
}

}  // namespace gpe

using namespace gpe;

// The device address of the scratch array on device `dev` (the current
// device), looked up once per device (the lookup needs that device current,
// and must not run inside a stream capture; the first call on each device
// does it).  The address stays valid for the life of the CUDA context: a
// cudaDeviceReset by the host application ends it, and this library (its
// contexts and this entry point alike) must not be used across one.
static gpe_status na_scratch(int dev, double** out) {
  if (dev < 0 || dev >= NA_MAX_DEVICES) return na_fail(GPE_ERR_INVALID, "device ordinal beyond 63");
  cudaError_t e;
  std::lock_guard<std::mutex> lock(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess || !p)
      return na_fail(GPE_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_na_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_na_ptr[dev];
  return GPE_OK;
}

extern "C" GPE_API gpe_status gpe_norm_noalloc(const void* d_psi, long long npoints, int precision, double weight,
                                               void* stream, double* norm_out) {
  if (!d_psi || !norm_out) return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: null pointer");
  if (precision != GPE_FP32 && precision != GPE_FP64)
    return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: precision must be GPE_FP32 or GPE_FP64");
  if (npoints <= 0) return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: npoints must be positive");
  if (npoints > NA_MAX_POINTS)
    return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: " + std::to_string(npoints) +
                                        " points exceed the fixed scratch of this entry point (at most " +
                                        std::to_string(NA_MAX_POINTS) + " points, i.e. 512^3)");
  // One complex element is 8 (FP32) or 16 (FP64) bytes; the kernel loads
  // whole elements, so a pointer off that boundary is refused here, before
  // any CUDA call.
  const uintptr_t align = precision == GPE_FP32 ? sizeof(cx<float>) : sizeof(cx<double>);
  if (reinterpret_cast<uintptr_t>(d_psi) % align != 0)
    return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: d_psi is not aligned to one complex element (" +
                                        std::to_string(align) + " bytes)");
  // The call waits on the host for its result (a copy to pageable memory
  // and a stream synchronisation), which a stream under capture cannot do:
  // refuse it with the first CUDA call, so the caller's capture survives.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap);
  if (e != cudaSuccess) return na_fail(GPE_ERR_CUDA, std::string("gpe_norm_noalloc: cudaStreamIsCapturing: ") +
                                                         cudaGetErrorString(e));
  if (cap != cudaStreamCaptureStatusNone)
    return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: the stream is capturing; this call waits on the host for its "
                                    "result");
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(GPE_ERR_CUDA, std::string("gpe_norm_noalloc: cudaGetDevice: ") +
                                                         cudaGetErrorString(e));
  // Only memory of the current device (or managed memory) goes to the kernel.
  cudaPointerAttributes pa{};
  e = cudaPointerGetAttributes(&pa, d_psi);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // the query's error is not sticky; clear it
    return na_fail(GPE_ERR_INVALID, std::string("gpe_norm_noalloc: d_psi is not a CUDA pointer (") +
                                        cudaGetErrorString(e) + ")");
  }
  if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged)
    return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: d_psi is host memory; pass device memory of the "
                                    "current device");
  if (pa.type == cudaMemoryTypeDevice && pa.device != dev)
    return na_fail(GPE_ERR_INVALID, "gpe_norm_noalloc: d_psi lives on device " + std::to_string(pa.device) +
                                        ", not on the current device " + std::to_string(dev));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* scratch = nullptr;
  gpe_status st = na_scratch(dev, &scratch);
  if (st != GPE_OK) return st;
  const int nparts = (int)((npoints + NA_CHUNK - 1) / NA_CHUNK);
  if (precision == GPE_FP32)
    k_na_partials<float><<<nparts, NA_THREADS, 0, s>>>(static_cast<const cx<float>*>(d_psi), npoints, scratch);
  else
    k_na_partials<double><<<nparts, NA_THREADS, 0, s>>>(static_cast<const cx<double>*>(d_psi), npoints, scratch);
  k_na_final<<<1, NA_THREADS, 0, s>>>(scratch, nparts, weight, scratch + NA_MAX_PARTIALS);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(norm_out, scratch + NA_MAX_PARTIALS, sizeof(double),
                                            cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return na_fail(GPE_ERR_CUDA, std::string("gpe_norm_noalloc: ") + cudaGetErrorString(e));
  return GPE_OK;
}

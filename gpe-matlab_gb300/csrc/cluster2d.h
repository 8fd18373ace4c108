// cluster2d.h - host-visible part of the persistent cluster kernel of small
// 2D grids (cluster2d.cuh): the launch arguments, the per-CTA shared-memory
// plan and the launchers.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "plans.cuh"

namespace gpe {

// Threads per CTA: 512 for FP32 (16 warps on the few pencils a CTA owns;
// GPE_C2_THREADS_F32 = 256 gives two CTAs per SM where shared memory
// allows), 256 for FP64, whose E = 16 double plans would spill at 128
// registers.
#ifndef GPE_C2_THREADS_F32
#define GPE_C2_THREADS_F32 512
#endif
template <typename R>
struct C2Threads {
  static constexpr int value = sizeof(R) == 8 ? 256 : GPE_C2_THREADS_F32;
  static constexpr int min_blocks = sizeof(R) == 8 ? 1 : 512 / GPE_C2_THREADS_F32;
};
__host__ __device__ constexpr int c2_threads(int esz) { return esz == 16 ? 256 : GPE_C2_THREADS_F32; }
constexpr int C2_RED_BYTES = 2048;  // [8] cluster-visible sums, [8] broadcast, [16][8] warp partials

// Axis lengths the cluster kernel handles, each on its alternative FFT plan
// where it has one (PlanAlt<N>: twice the threads per pencil and half the
// points per thread of Plan<N>, so that an FP32 CTA of 512 threads keeps 16
// warps busy on the few pencils a cluster CTA owns), else on Plan<N>.  Each
// needs the contiguous-axis padding p + p/16 and T <= 32.
// FP64 contexts keep Plan<N> (their per-pass kernels exist for Plan<N>
// only, and the context's tables must match them).
#define GPE_C2_SIZES(X) X(64) X(96) X(128) X(192) X(256) X(384)
// Plan variant (plans.cuh PlanSel) the cluster kernel of element size esz
// (bytes of one complex value) uses for length n: the context's tables.
__host__ __device__ inline int c2_plan_var(int n, int esz) { return (esz == 16 || n == 64 || n == 96) ? 0 : 1; }
template <typename R, int N>
using C2Plan = typename PlanSel<N, (sizeof(R) == 8 || N == 64 || N == 96) ? 0 : 1>::type;

__host__ __device__ inline int c2_T(int n, int esz) {
  switch (n) {
#define X(v) \
  case v:    \
    return esz == 16 ? C2Plan<double, v>::T : C2Plan<float, v>::T;
    GPE_C2_SIZES(X)
#undef X
  }
  return 0;
}
// Padded stride between pencils of the contiguous layout (ContigLayout::REG).
__host__ __device__ constexpr int c2_reg(int n) {
  const int r0 = n + ((n - 1) >> 4);
  return (r0 % 2 == 0) ? r0 + 1 : r0;
}

// Shared-memory plan of one CTA for an nx x ny grid on clusters of cs CTAs.
// vsm: the CTA also keeps its columns of V (cols x ny reals, constant over
// the launch) after the reduction scratch, so the y pass's nonlinear phase
// reads V from shared memory instead of L2 at every step.
struct C2Geom {
  int cols, cols_pad, rows, regy, home, xbuf;  // home/xbuf in complex elements
  size_t vofs;                                 // byte offset of the V columns (vsm)
  size_t vrofs;                                // byte offset of the V rows (vsm)
  int vrstride;                                // row stride of the V rows: nx + 2 (conflict-free)
  size_t bytes;
};
__host__ __device__ inline C2Geom c2_geom(int nx, int ny, int cs, int esz, int vsm = 0) {
  C2Geom g;
  g.cols = nx / cs;
  g.rows = ny / cs;
  const int fpi = c2_threads(esz) / c2_T(ny, esz);
  const int fpw = 32 / c2_T(ny, esz);  // pencils per warp: home holds whole warps' pencils
  g.cols_pad = (g.cols + fpw - 1) / fpw * fpw;
  g.regy = c2_reg(ny);
  g.home = g.cols_pad * g.regy;
  const int gx = c2_threads(esz) / c2_T(nx, esz);
  g.xbuf = gx * nx > fpi * g.regy ? gx * nx : fpi * g.regy;
  g.bytes = (size_t)(g.home + g.xbuf) * (size_t)esz + C2_RED_BYTES;
  g.vofs = g.bytes;
  if (vsm) g.bytes += (size_t)g.cols * ny * (size_t)(esz / 2);
  // V of the CTA's x-pass rows, [row][x] with stride nx + 2 (the x pass's
  // lanes read 16 rows x 2 columns: banks 2 row + column, all distinct)
  g.vrstride = nx + 2;
  g.vrofs = (g.bytes + 15) & ~(size_t)15;
  if (vsm) g.bytes = g.vrofs + (size_t)g.rows * g.vrstride * (size_t)(esz / 2);
  return g;
}

// One realisation (context) of the batch.
struct C2Grid {
  void* psi;                 // cx<R> state, ny x nx, y fastest
  const void* V;             // R potential
  const void* tws[2];        // stage twiddle rows of C2Plan<n>: [0] x axis, [1] y axis
  const void* php[2];        // kinetic factors exp(-k^2/2 dt)/n in slot order
  const void* k2p[2];        // k^2/2/n in slot order (energy sums)
  DevScalars* sc;
  double* hist;              // record (muc, ncur, energy) of outer step k at hist + 3*k
  int nx, ny;
  int feedback;              // gamma > 0 and mu_init == 0: mu and the norm feed back every block
  int start;                 // current_iter at the start of the run
  double weight, g, tau;     // cell volume, coupling, decay time (0: none)
  double dre, dim;           // complex time step dt = i ddt/(1 + i gamma)
};

struct C2Args {
  const C2Grid* grids;
  const int* order;  // grid indices in cluster order
  const int* offs;   // cluster c runs order[offs[c] .. offs[c+1])
  int n_rec, nb;     // steps per block, blocks per outer step
  int nouter;        // outer steps per launch
  int vsm;           // V columns in shared memory (C2Geom)
  int fold;          // folded steps (y x, x y, ...: 1 + n_rec passes per block)
  double ddt, dt_outer;
};

// Launch of k_cluster2d<R> on nclusters clusters of cs CTAs (cluster2d_f32.cu,
// cluster2d_f64.cu).
template <typename R>
cudaError_t launch_cluster2d(const C2Args& a, int nclusters, int cs, size_t smem, cudaStream_t s);
template <>
cudaError_t launch_cluster2d<float>(const C2Args& a, int nclusters, int cs, size_t smem, cudaStream_t s);
template <>
cudaError_t launch_cluster2d<double>(const C2Args& a, int nclusters, int cs, size_t smem, cudaStream_t s);
// Clusters of cs CTAs with `smem` bytes each that can be resident at once
// (0: this cluster shape does not fit the device).
template <typename R>
int cluster2d_max_clusters(int cs, size_t smem);
template <>
int cluster2d_max_clusters<float>(int cs, size_t smem);
template <>
int cluster2d_max_clusters<double>(int cs, size_t smem);

}  // namespace gpe

// cluster2d.cuh - persistent solve_split of many small 2D grids in one launch.
//
// The graph path runs a 2D split step as axis-pass launches per step and
// per grid: for grids of a few hundred KB (all of them L2-resident) that is
// launch- and latency-bound.  Here one launch advances every grid of
// a batch through a whole outer step of solve_split (solve_split.m:49-80):
//
//  * each grid is owned by one thread-block cluster of CS CTAs (CS = 8, or 16
//    where the device allows it), and a cluster works through its list of
//    grids one after the other;
//  * the grid's state is loaded once into the cluster's distributed shared
//    memory and stays there for all niter_inner steps: CTA r holds the y
//    pencils (MATLAB columns) of x in [r*cols, (r+1)*cols), cols = nx/CS, each
//    in the padded per-pencil layout of the contiguous-axis pass;
//  * y pass: each CTA transforms its own pencils in place (nonlinear prologue,
//    FFT_y, exp(-ky^2/2 dt)/ny, inverse FFT_y), exactly the arithmetic of the
//    y axis pass;
//  * x pass: CTA r takes the rows y in [r*rows, (r+1)*rows), rows = ny/CS,
//    GX at a time; the threads read the row's elements from the owning CTAs'
//    shared memory (ld.shared::cluster), transform them with a local exchange
//    buffer, apply the block-end epilogue and write them back
//    (st.shared::cluster), exactly the arithmetic of the x axis pass;
//  * folded steps (C2Args::fold): odd steps take y then x, even steps x then
//    y, and the shared axis of consecutive steps is one pass with the full
//    nonlinear step between its two transforms, so a block of n_rec steps is
//    1 + n_rec passes (the first y pass with the half-step prologue, the
//    last with the block-end epilogue);
//  * hardware cluster barriers separate the passes; at the end of a block
//    whose mu is needed (gamma > 0 feedback, or the last block of the outer
//    step) the kinetic-energy sums of both axes (Parseval, forward FFTs) and
//    the epilogue's n, Vn, n^2 sums are reduced over the cluster through
//    distributed shared memory and every CTA evaluates the block finalizer's
//    formulas (solve_split.m:65-78) on the same sums, so mu, the
//    renormalisation factor and the stop decision are identical in all of
//    them; CTA 0 writes the context's device scalars and history record.
//
// HBM/L2 traffic per grid and outer step: one load and one store of the
// state, the potential read once per step from L2.  No CTA ever waits on a
// flag written by another: the only waits are the cluster barriers, which
// every CTA of a cluster reaches the same number of times (all decisions are
// taken on values every CTA computes identically).
#pragma once
#include "cluster2d.h"
#include "pass.cuh"

namespace gpe {

#define X(v)                                                                                                 \
  static_assert(C2Plan<float, v>::PADSH == 4 && c2_reg(v) == ContigLayout<C2Plan<float, v>, float>::REG &&    \
                    C2Plan<float, v>::T <= 32 && 32 % C2Plan<float, v>::T == 0 &&                            \
                    C2Plan<double, v>::PADSH == 4 && c2_reg(v) == ContigLayout<C2Plan<double, v>, double>::REG && \
                    C2Plan<double, v>::T <= 32 && 32 % C2Plan<double, v>::T == 0,                            \
                "cluster kernel: contiguous layout of N = " #v);
GPE_C2_SIZES(X)
#undef X

// ---- cluster primitives (inline PTX, sm_90+) ---------------------------------
__device__ __forceinline__ uint32_t c2_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t c2_nrank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t c2_cluster_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
// All threads of all CTAs of the cluster; release/acquire at cluster scope,
// so shared-memory writes before it are visible to every CTA after it.
__device__ __forceinline__ void c2_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of the same shared-memory offset in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t c2_map(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ cx<float> c2_ld(uint32_t a, float) {
  float x, y;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(x), "=f"(y) : "r"(a) : "memory");
  return mk<float>(x, y);
}
__device__ __forceinline__ cx<double> c2_ld(uint32_t a, double) {
  double x, y;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "r"(a) : "memory");
  return mk<double>(x, y);
}
__device__ __forceinline__ void c2_st(uint32_t a, cx<float> v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void c2_st(uint32_t a, cx<double> v) {
  asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(a), "d"(v.x), "d"(v.y) : "memory");
}
__device__ __forceinline__ double c2_ld_f64(uint32_t a) {
  double x;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(x) : "r"(a) : "memory");
  return x;
}

// Exchange policy of the x pass: GX rows interleaved position-major in the
// local buffer ([position][row], conflict-free), CTA-wide barrier.
template <int GX>
struct C2XPol {
  int f;
  __device__ __forceinline__ int idx(int p) const { return p * GX + f; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  GPE_POL_CHECK_MEMBERS
};

// ---- the passes ----------------------------------------------------------------
// y pass over this CTA's pencils, in place in `home` (pencil pc at pc*regy).
// pa.fold = 1: a folded pass (the transform, the full nonlinear step, the
// transform again: the last pass of one step and the first of the next);
// pa.epi = EPI_RT_END: the block-end phases and the n, Vn, n^2 sums.
template <typename R, class P>
__device__ __forceinline__ void c2_y_step(cx<R>* home, const R* vloc, const C2Geom& g, const C2Grid& G, int col0,
                                          const PassArgs<R>& pa, R s, R mu, Kahan<R>* acc) {
  constexpr int T = P::T, E = P::E, N = P::N;
  constexpr int FPI = C2Threads<R>::value / T;
  using St = typename P::template St<R>;
  const int f = threadIdx.x / T, t = threadIdx.x % T;
  const cx<R>* tws = static_cast<const cx<R>*>(G.tws[1]);
  const cx<R>* php = static_cast<const cx<R>*>(G.php[1]);
  const R* V = static_cast<const R*>(G.V);
  for (int p0 = 0; p0 < g.cols; p0 += FPI) {
    const int pc = p0 + f;
    // A pencil lies within one warp (T <= 32), and home holds whole warps'
    // pencils: pencils past cols_pad leave their warp idle (warp-uniform),
    // the ones in [cols, cols_pad) run on scratch space.
    if (p0 + (int)(threadIdx.x / 32) * (32 / T) >= g.cols_pad) continue;
    const bool valid = pc < g.cols;
    typename ContigLayout<P, R>::Pol pol{pc * g.regy};
    GPE_POL_BOUNDS(pol, G.sc, g.home);
    cx<R> v[E];
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = valid ? home[GPE_SMI(pol, pol.idx(t + T * m))] : mk<R>(R(0), R(0));
    R sv[E];
    auto load_v = [&]() {
      if (vloc) {  // this CTA's V columns in shared memory
        const R* vs = vloc + pc * N + t;
#pragma unroll
        for (int m = 0; m < E; ++m) sv[m] = valid ? vs[T * m] : R(0);
      } else {
        const R* vs = V + (long long)(col0 + pc) * N + t;
#pragma unroll
        for (int m = 0; m < E; ++m) sv[m] = valid ? __ldg(vs + T * m) : R(0);
      }
    };
    if (pa.pro != PRO_NONE) {
      load_v();
      prologue<R, E>(v, sv, pa, valid, 0, 0, s, mu);
    }
    pol.sync();  // every lane has read its values before the exchanges reuse the pencil
#pragma unroll 1
    for (int rep = 0;; ++rep) {
      St::template forward<false>(v, home, pol, t, tws);
      apply_phase<T, E, false>(v, php, t);
      St::template inverse<false>(v, home, pol, t, tws);
      if (rep >= pa.fold) break;
      load_v();
      rt_full_phase<R, E>(v, sv, pa, mu);  // solve_split.m:60-61
    }
    if (pa.epi != EPI_NONE) {
      load_v();
      epilogue<R, E>(v, sv, pa, acc, valid, mu);
    }
#pragma unroll
    for (int m = 0; m < E; ++m) home[GPE_SMI(pol, pol.idx(t + T * m))] = v[m];
  }
}

// x pass over rows [rank*rows, (rank+1)*rows): elements read from and
// written back to the owning CTAs' pencils.  pa.fold and epi = EPI_RT_END as
// in the y pass.
template <typename R, class P>
__device__ __forceinline__ void c2_x_step(cx<R>* home, cx<R>* xbuf, const R* vrow, const C2Geom& g, const C2Grid& G,
                                          int rank, const PassArgs<R>& pa, R mu, Kahan<R>* acc) {
  constexpr int T = P::T, E = P::E, N = P::N;
  constexpr int GX = C2Threads<R>::value / T;
  using St = typename P::template St<R>;
  const int f = threadIdx.x % GX, t = threadIdx.x / GX;
  const cx<R>* tws = static_cast<const cx<R>*>(G.tws[0]);
  const cx<R>* php = static_cast<const cx<R>*>(G.php[0]);
  const R* V = static_cast<const R*>(G.V);
  const uint32_t hb = smem_u32(home);
  C2XPol<GX> pol{f};
  GPE_POL_BOUNDS(pol, G.sc, g.xbuf);
  const int c0 = t / g.cols, lc0 = t - c0 * g.cols;  // x = t lives in CTA c0, column lc0
  for (int r0 = 0; r0 < g.rows; r0 += GX) {
    // bounds-checked build: the thread's last x column lies inside the grid
    const bool valid = r0 + f < g.rows && bounds_ok(G.sc, BS_CLUSTER, t + (long long)T * (E - 1), G.nx);
    const int y = rank * g.rows + (valid ? r0 + f : 0);
    const uint32_t yoff = (uint32_t)padpos<4>(y) * (uint32_t)sizeof(cx<R>);
    cx<R> v[E];
    {
      int c = c0, lc = lc0;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        v[m] = valid ? c2_ld(c2_map(hb + (uint32_t)(lc * g.regy) * (uint32_t)sizeof(cx<R>) + yoff, c), R(0))
                     : mk<R>(R(0), R(0));
        lc += T;
        while (lc >= g.cols) {  // T may exceed cols: x = t + T*m lives in CTA x / cols
          lc -= g.cols;
          ++c;
        }
      }
    }
    R sv[E];
    auto load_v = [&]() {
      if (vrow) {  // this CTA's V rows in shared memory
        const int v0 = (r0 + f) * g.vrstride + t;
#pragma unroll
        for (int m = 0; m < E; ++m)
          sv[m] = valid && bounds_ok(G.sc, BS_SMEM, v0 + T * m, (long long)g.rows * g.vrstride) ? vrow[v0 + T * m]
                                                                                                : R(0);
      } else {
        const R* vs = V + (long long)t * G.ny + y;
#pragma unroll
        for (int m = 0; m < E; ++m) sv[m] = valid ? __ldg(vs + (long long)T * m * G.ny) : R(0);
      }
    };
#pragma unroll 1
    for (int rep = 0;; ++rep) {
      St::template forward<false>(v, xbuf, pol, t, tws);
      apply_phase<T, E, false>(v, php, t);
      St::template inverse<false>(v, xbuf, pol, t, tws);
      if (rep >= pa.fold) break;
      load_v();
      rt_full_phase<R, E>(v, sv, pa, mu);  // solve_split.m:60-61
    }
    if (pa.epi != EPI_NONE) {
      load_v();
      epilogue<R, E>(v, sv, pa, acc, valid, mu);
    }
    if (valid) {
      int c = c0, lc = lc0;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        c2_st(c2_map(hb + (uint32_t)(lc * g.regy) * (uint32_t)sizeof(cx<R>) + yoff, c), v[m]);
        lc += T;
        while (lc >= g.cols) {  // T may exceed cols: x = t + T*m lives in CTA x / cols
          lc -= g.cols;
          ++c;
        }
      }
    }
  }
}

// Kinetic-energy sum of the y axis over this CTA's pencils: forward FFT in
// the exchange buffer (the stored state is not touched), sum k^2/2/N |psi^|^2.
template <typename R, class P>
__device__ __forceinline__ void c2_y_energy(const cx<R>* home, cx<R>* xbuf, const C2Geom& g, const C2Grid& G,
                                            Kahan<R>& kin) {
  constexpr int T = P::T, E = P::E;
  constexpr int FPI = C2Threads<R>::value / T;
  using St = typename P::template St<R>;
  const int f = threadIdx.x / T, t = threadIdx.x % T;
  const cx<R>* tws = static_cast<const cx<R>*>(G.tws[1]);
  const R* k2p = static_cast<const R*>(G.k2p[1]);
  typename ContigLayout<P, R>::Pol pol{f * g.regy};
  GPE_POL_BOUNDS(pol, G.sc, g.xbuf);
  for (int p0 = 0; p0 < g.cols; p0 += FPI) {
    const int pc = p0 + f;
    if (p0 + (int)(threadIdx.x / 32) * (32 / T) >= g.cols_pad) continue;  // as in c2_y_step
    const bool valid = pc < g.cols;
    cx<R> v[E];
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int hi = pc * g.regy + padpos<4>(t + T * m);
      v[m] = valid && bounds_ok(G.sc, BS_SMEM, hi, g.home) ? home[hi] : mk<R>(R(0), R(0));
    }
    St::template forward<false>(v, xbuf, pol, t, tws);
    if (valid) {
#pragma unroll
      for (int m = 0; m < E; ++m) kin.add(__ldg(k2p + m * T + t) * norm2(v[m]));
    }
  }
}

// Kinetic-energy sum of the x axis over this CTA's rows (remote reads only).
template <typename R, class P>
__device__ __forceinline__ void c2_x_energy(const cx<R>* home, cx<R>* xbuf, const C2Geom& g, const C2Grid& G,
                                            int rank, Kahan<R>& kin) {
  constexpr int T = P::T, E = P::E;
  constexpr int GX = C2Threads<R>::value / T;
  using St = typename P::template St<R>;
  const int f = threadIdx.x % GX, t = threadIdx.x / GX;
  const cx<R>* tws = static_cast<const cx<R>*>(G.tws[0]);
  const R* k2p = static_cast<const R*>(G.k2p[0]);
  const uint32_t hb = smem_u32(home);
  C2XPol<GX> pol{f};
  GPE_POL_BOUNDS(pol, G.sc, g.xbuf);
  const int c0 = t / g.cols, lc0 = t - c0 * g.cols;
  for (int r0 = 0; r0 < g.rows; r0 += GX) {
    const bool valid = r0 + f < g.rows && bounds_ok(G.sc, BS_CLUSTER, t + (long long)T * (E - 1), G.nx);
    const int y = rank * g.rows + (valid ? r0 + f : 0);
    const uint32_t yoff = (uint32_t)padpos<4>(y) * (uint32_t)sizeof(cx<R>);
    cx<R> v[E];
    int c = c0, lc = lc0;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      v[m] = valid ? c2_ld(c2_map(hb + (uint32_t)(lc * g.regy) * (uint32_t)sizeof(cx<R>) + yoff, c), R(0))
                   : mk<R>(R(0), R(0));
      lc += T;
      while (lc >= g.cols) {
        lc -= g.cols;
        ++c;
      }
    }
    St::template forward<false>(v, xbuf, pol, t, tws);
    if (valid) {
#pragma unroll
      for (int m = 0; m < E; ++m) kin.add(__ldg(k2p + m * T + t) * norm2(v[m]));
    }
  }
}

// Runtime dispatch over the axis length.
template <typename R>
__device__ void c2_y_step_n(int n, cx<R>* home, const R* vloc, const C2Geom& g, const C2Grid& G, int col0,
                            const PassArgs<R>& pa, R s, R mu, Kahan<R>* acc) {
  switch (n) {
#define X(v)                                                             \
  case v:                                                                \
    c2_y_step<R, C2Plan<R, v>>(home, vloc, g, G, col0, pa, s, mu, acc);  \
    break;
    GPE_C2_SIZES(X)
#undef X
  }
}
template <typename R>
__device__ void c2_x_step_n(int n, cx<R>* home, cx<R>* xbuf, const R* vrow, const C2Geom& g, const C2Grid& G,
                            int rank, const PassArgs<R>& pa, R mu, Kahan<R>* acc) {
  switch (n) {
#define X(v)                                                                 \
  case v:                                                                    \
    c2_x_step<R, C2Plan<R, v>>(home, xbuf, vrow, g, G, rank, pa, mu, acc);   \
    break;
    GPE_C2_SIZES(X)
#undef X
  }
}
template <typename R>
__device__ void c2_energy_n(const cx<R>* home, cx<R>* xbuf, const C2Geom& g, const C2Grid& G, int rank,
                            Kahan<R>& ky, Kahan<R>& kx) {
  switch (G.ny) {
#define X(v)                                            \
  case v:                                               \
    c2_y_energy<R, C2Plan<R, v>>(home, xbuf, g, G, ky);      \
    break;
    GPE_C2_SIZES(X)
#undef X
  }
  __syncthreads();  // the y sums' exchanges are done before the x sums reuse the buffer
  switch (G.nx) {
#define X(v)                                                 \
  case v:                                                    \
    c2_x_energy<R, C2Plan<R, v>>(home, xbuf, g, G, rank, kx);     \
    break;
    GPE_C2_SIZES(X)
#undef X
  }
}

// CTA sum of NV per-thread compensated sums into red[0..NV) (FP64), as the
// pass kernels' FP32 pair reduction does.
template <typename R, int NV>
__device__ __forceinline__ void c2_cta_reduce(const Kahan<R>* acc, double* red, double* wpart) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double x;
    if constexpr (sizeof(R) == 4) {
      float h = acc[i].s, l = -acc[i].c;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, h, o);
        const float l2 = __shfl_down_sync(0xffffffffu, l, o);
        pair_add(h, l, h2, l2);
      }
      x = (double)h + (double)l;
    } else {
      x = acc[i].value();
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    }
    if (lane == 0) wpart[warp * 8 + i] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
    for (int w = 0; w < C2Threads<R>::value / 32; ++w) s += wpart[w * 8 + threadIdx.x];
    red[threadIdx.x] = s;
  }
}

template <typename R>
__global__ void __launch_bounds__(C2Threads<R>::value, C2Threads<R>::min_blocks) k_cluster2d(const C2Args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int rank = (int)c2_rank();
  const int cs = (int)c2_nrank();
  const int cid = (int)c2_cluster_id();
  // [0..7]: this CTA's block-end sums (read by the whole cluster), [8]:
  // broadcast of the finalizer's (scale, mu, stop) within the CTA, then the
  // warp partials of the CTA reduction.
  for (int k = a.offs[cid]; k < a.offs[cid + 1]; ++k) {
    const C2Grid& G = a.grids[a.order[k]];
    const C2Geom g = c2_geom(G.nx, G.ny, cs, (int)sizeof(cx<R>), a.vsm);
    R* vloc = a.vsm ? reinterpret_cast<R*>(smem + g.vofs) : nullptr;
    R* vrow = a.vsm ? reinterpret_cast<R*>(smem + g.vrofs) : nullptr;
    cx<R>* home = reinterpret_cast<cx<R>*>(smem);
    cx<R>* xbuf = home + g.home;
    double* red = reinterpret_cast<double*>(smem + (size_t)(g.home + g.xbuf) * sizeof(cx<R>));
    double* bc = red + 8;
    double* wpart = red + 16;
    DevScalars* sc = G.sc;
    // Every CTA reads the same values: nothing writes them before this
    // cluster's first finalizer of this grid, which comes after barriers.
    if (sc->stop) continue;
    R s = (R)sc->scale, mu = (R)sc->mu;
    double NNN = sc->NNN;
    const double NN0 = sc->NN0;
    const int outer0 = sc->outer;
    const int col0 = rank * g.cols;
    // state -> this CTA's pencils
    {
      const cx<R>* src = static_cast<const cx<R>*>(G.psi) + (long long)col0 * G.ny;
      const int total = g.cols * G.ny;
      for (int i = threadIdx.x; i < total; i += C2Threads<R>::value) {
        const int pc = i / G.ny, y = i - pc * G.ny;
        home[pc * g.regy + padpos<4>(y)] = src[i];
      }
      if (vloc) {  // this CTA's columns of V, dense [column][y]
        const R* vsrc = static_cast<const R*>(G.V) + (long long)col0 * G.ny;
        for (int i = threadIdx.x; i < total; i += C2Threads<R>::value) vloc[i] = vsrc[i];
        // and its x-pass rows y in [rank*rows, (rank+1)*rows), [row][x]
        const R* vg = static_cast<const R*>(G.V) + (long long)rank * g.rows;
        const int rtotal = g.rows * G.nx;
        for (int i = threadIdx.x; i < rtotal; i += C2Threads<R>::value) {
          const int x = i / g.rows, r = i - x * g.rows;
          vrow[r * g.vrstride + x] = vg[(long long)x * G.ny + r];
        }
      }
    }
    c2_sync();
    PassArgs<R> pa{};
    pa.gr = (R)G.g;
    pa.drer = (R)G.dre;
    pa.dimr = (R)G.dim;
    bool stopped = false;
    int done = 0;
    for (int o = 0; o < a.nouter && !stopped; ++o) {
      const int j = G.start + 1 + outer0 + o;  // solve_split.m:49
      const double time = (j - 1) * a.dt_outer;
      for (int jj = 1; jj <= a.nb && !stopped; ++jj) {
        const double time2 = time + (jj - 1) * a.ddt * a.n_rec;  // solve_split.m:53
        Kahan<R> acc[3];
        // Folded steps: step i takes the axes in the order y x (odd i) or
        // x y (even i), so the last pass of a step and the first of the
        // next are one folded pass with the full nonlinear step between its
        // transforms (solve_split.m:60-61): 1 + n_rec passes and cluster
        // barriers per block instead of 2 n_rec.  The kinetic factors of
        // the axes commute; only the rounding differs.
        // (a.fold = 0: y x every step, 2 n_rec passes)
        pa.pro = PRO_RT_HALF;  // solve_split.m:55-56
        pa.epi = EPI_NONE;
        pa.fold = 0;
        c2_y_step_n<R>(G.ny, home, vloc, g, G, col0, pa, s, mu, acc);
        c2_sync();
        pa.pro = PRO_NONE;
        for (int i = 1; i <= a.n_rec; ++i) {
          const bool xa = !a.fold || i % 2 == 1;
          if (!a.fold && i > 1) {
            pa.pro = PRO_RT_FULL;  // solve_split.m:60-61
            c2_y_step_n<R>(G.ny, home, vloc, g, G, col0, pa, s, mu, acc);
            c2_sync();
            pa.pro = PRO_NONE;
          }
          pa.fold = a.fold && i < a.n_rec ? 1 : 0;
          pa.epi = i == a.n_rec ? EPI_RT_END : EPI_NONE;  // solve_split.m:60-67
          if (xa) c2_x_step_n<R>(G.nx, home, xbuf, vrow, g, G, rank, pa, mu, acc);
          else c2_y_step_n<R>(G.ny, home, vloc, g, G, col0, pa, s, mu, acc);
          c2_sync();
        }
        const bool last = jj == a.nb;
        if (!(G.feedback || last)) {
          s = R(1);  // the block finalizer leaves no pending factor without feedback
          continue;
        }
        // kinetic sums of the block-end state, then the cluster reduction
        Kahan<R> kin[2];
        c2_energy_n<R>(home, xbuf, g, G, rank, kin[0], kin[1]);
        Kahan<R> all[5] = {acc[0], acc[1], acc[2], kin[0], kin[1]};
        c2_cta_reduce<R, 5>(all, red, wpart);
        c2_sync();
        if (threadIdx.x == 0) {
          double sums[5] = {0, 0, 0, 0, 0};
          for (int r = 0; r < cs; ++r) {
            const uint32_t rb = c2_map(smem_u32(red), (uint32_t)r);
            for (int q = 0; q < 5; ++q) sums[q] += c2_ld_f64(rb + 8u * q);
          }
          // the block finalizer (solve_split.m:65-78) on the cluster's sums
          const double w = G.weight, n = sums[0], vn = sums[1], n2 = sums[2], kinv = sums[3] + sums[4];
          const double ncur = n * w;  // solve_split.m:67
          double muc, scale = 1.0, energy;
          if (G.feedback) {  // solve_split.m:68-75
            if (G.tau > 0) NNN = NN0 * exp(-time2 / G.tau);
            scale = sqrt(NNN / ncur);
            const double s2 = scale * scale;
            muc = (s2 * (kinv + vn) * w + s2 * s2 * G.g * n2 * w) / NNN;
            energy = s2 * (kinv + vn) * w + 0.5 * s2 * s2 * G.g * n2 * w;
          } else {  // solve_split.m:76-77
            muc = (kinv + vn + G.g * n2) * w / ncur;
            energy = (kinv + vn + 0.5 * G.g * n2) * w;
          }
          const bool bad = !isfinite(ncur) || !isfinite(muc) || !isfinite(scale);
          if (rank == 0) {
            if (G.feedback) {
              sc->NNN = NNN;
              sc->mu = muc;
            }
            sc->energy = energy;
            sc->scale = scale;
            sc->ncur = ncur;
            sc->muc = muc;
            sc->sums[S_N] = n * w;
            sc->sums[S_VN] = vn * w;
            sc->sums[S_N2] = n2 * w;
            if (bad) {
              sc->nonfinite = 1;
              sc->status = NONFINITE;
              sc->stop = 1;
            }
            if (last && !bad) {
              double* h = G.hist + 3 * (size_t)(outer0 + o);
              h[0] = muc;
              h[1] = ncur;
              h[2] = energy;
            }
          }
          bc[0] = scale;
          bc[1] = G.feedback ? muc : (double)mu;
          bc[2] = bad ? 1.0 : 0.0;
          bc[3] = NNN;
        }
        __syncthreads();
        s = (R)bc[0];
        mu = (R)bc[1];
        stopped = bc[2] != 0.0;
        NNN = bc[3];
      }
      if (!stopped) ++done;
    }
    // pencils -> state (the remote accesses of the last pass are behind the
    // last cluster barrier)
    {
      cx<R>* dst = static_cast<cx<R>*>(G.psi) + (long long)col0 * G.ny;
      const int total = g.cols * G.ny;
      for (int i = threadIdx.x; i < total; i += C2Threads<R>::value) {
        const int pc = i / G.ny, y = i - pc * G.ny;
        dst[i] = home[pc * g.regy + padpos<4>(y)];
      }
    }
    if (rank == 0 && threadIdx.x == 0) sc->outer = outer0 + done;
    c2_sync();  // the next grid's load overwrites pencils the peers may still read
  }
  c2_sync();  // no CTA leaves while a peer may access its shared memory
}

}  // namespace gpe

namespace gpe {

// Launch configuration shared by the launcher and the occupancy query.
template <typename R>
cudaLaunchConfig_t c2_config(int nclusters, int cs, size_t smem, cudaStream_t s, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nclusters * cs));
  cfg.blockDim = dim3(C2Threads<R>::value);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

// Function attributes, set before the first occupancy query (and so before
// any launch or graph capture): the device's opt-in shared-memory maximum,
// whatever a launch asks for below it, and non-portable cluster sizes.
template <typename R>
cudaError_t c2_prepare() {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cluster2d<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cluster2d<R>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

template <typename R>
cudaError_t launch_cluster2d_impl(const C2Args& a, int nclusters, int cs, size_t smem, cudaStream_t s) {
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = c2_config<R>(nclusters, cs, smem, s, attr);
  return cudaLaunchKernelEx(&cfg, k_cluster2d<R>, a);
}

template <typename R>
int cluster2d_max_clusters_impl(int cs, size_t smem) {
  if (c2_prepare<R>() != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = c2_config<R>(1, cs, smem, nullptr, attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_cluster2d<R>, &cfg) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace gpe

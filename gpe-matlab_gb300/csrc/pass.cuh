// pass.cuh - one axis pass of the split step: load pencils, [prologue],
// FFT along the axis, kinetic factor, inverse FFT, [epilogue], store.
//
// The kinetic propagator exp(-kk*dt) of GPE-MATLAB (set_kinop.m:9,
// ssft_kin_step.m:17) factorises exactly over axes because
// kk = (kx^2 + ky^2 + kz^2)/2 (lib/@grid3d/init.m:76) and the 1D DFTs of an
// nD FFT commute, so one step is one pass per axis, each one HBM round trip.
// The potential/nonlinear phase factors of the step are fused as a prologue
// of the first (contiguous, y) pass and an epilogue of the last pass.
//
// Two memory layouts:
//  * Contig: the pencil is contiguous (MATLAB dim 1 = y).  The T threads of a
//    pencil are adjacent lanes, so each load instruction of a half warp reads
//    a 128-byte run.  Exchanges use a padded per-pencil shared-memory region.
//  * Strided: the pencil runs along x (stride ny) or z (stride nx*ny).  Lanes
//    are assigned to FFTS adjacent pencils (adjacent y), so every load of a
//    half warp again reads one 128-byte run; the shared-memory buffer is
//    interleaved [position][pencil], which makes every exchange conflict-free.
#pragma once
#include "plans.cuh"

namespace gpe {

template <typename R>
struct Kahan {
  R s = R(0), c = R(0);
  __device__ __forceinline__ void add(R x) {
    R y = x - c;
    R t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

template <int PADSH>
__host__ __device__ constexpr int padpos(int p) {
  if constexpr (PADSH < 0) return p;
  else return p + (p >> PADSH);
}

template <class P, typename R>
struct ContigLayout {
  static constexpr int T = P::T;
  static constexpr int FFTS = (T >= 256) ? 1 : 256 / T;
  static constexpr int THREADS = FFTS * T;
  static constexpr int REG0 = padpos<P::PADSH>(P::N - 1) + 1;
  static constexpr int REG = (REG0 % 2 == 0) ? REG0 + 1 : REG0;  // odd stride between pencils
  static constexpr size_t smem_bytes() { return sizeof(cx<R>) * (size_t)FFTS * REG; }
  struct Pol {
    int off;
    __device__ __forceinline__ int idx(int p) const { return off + padpos<P::PADSH>(p); }
    __device__ __forceinline__ void sync() const {
      if constexpr (T <= 32) __syncwarp();
      else __syncthreads();
    }
  };
  static __device__ __forceinline__ void map(int tid, int& f, int& t) {
    f = tid / T;
    t = tid % T;
  }
  static __device__ __forceinline__ Pol pol(int f) { return Pol{f * REG}; }
  static __device__ __forceinline__ long long base(const PassArgs<R>& a, long long b) {
    return b * (long long)P::N;
  }
  static __device__ __forceinline__ long long step(const PassArgs<R>&) { return 1; }
};

template <class P, typename R>
struct StridedLayout {
  static constexpr int T = P::T;
  static constexpr int G = 128 / (int)sizeof(cx<R>);  // pencils per 128-byte row
  static constexpr int F0 = (256 / T > G) ? 256 / T : G;
  static constexpr int FFTS = (F0 * T > 1024) ? 1024 / T : F0;
  static constexpr int THREADS = FFTS * T;
  static constexpr size_t smem_bytes() { return sizeof(cx<R>) * (size_t)FFTS * P::N; }
  struct Pol {
    int f;
    __device__ __forceinline__ int idx(int p) const { return p * FFTS + f; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
  };
  static __device__ __forceinline__ void map(int tid, int& f, int& t) {
    f = tid % FFTS;
    t = tid / FFTS;
  }
  static __device__ __forceinline__ Pol pol(int f) { return Pol{f}; }
  static __device__ __forceinline__ long long base(const PassArgs<R>& a, long long b) {
    return (b % a.inner) + (b / a.inner) * a.outer;
  }
  static __device__ __forceinline__ long long step(const PassArgs<R>& a) { return a.stride; }
};

// Sum `nred` per-thread values over the CTA in FP64 and store the CTA's
// partial of each to partials[slot*cap + blockIdx.x].
template <int THREADS>
__device__ __forceinline__ void cta_reduce_store(double* vals, const int* slots, int nred,
                                                 double* partials, int cap) {
  __shared__ double red[THREADS / 32 > 0 ? THREADS / 32 : 1][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i >= nred) break;
    double x = vals[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][i] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < nred; ++i) {
      double s = 0.0;
      for (int w = 0; w < (THREADS + 31) / 32; ++w) s += red[w][i];
      partials[(size_t)slots[i] * cap + blockIdx.x] = s;
    }
  }
}

template <typename R, class P, class L>
__global__ void __launch_bounds__(L::THREADS) pass_kernel(const PassArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<R>* sm = reinterpret_cast<cx<R>*>(smem_raw);
  if (a.sc->stop) return;  // grid-uniform: an earlier finalizer ended the run

  constexpr int T = P::T, E = P::E;
  using St = typename P::template St<R>;
  int f, t;
  L::map(threadIdx.x, f, t);
  const long long b = (long long)blockIdx.x * L::FFTS + f;
  const bool valid = b < a.n_batch;
  const long long base = valid ? L::base(a, b) : 0;
  const long long st = L::step(a);
  const auto pol = L::pol(f);

  cx<R> v[E];
#pragma unroll
  for (int m = 0; m < E; ++m)
    v[m] = valid ? a.psi[base + (long long)(t + T * m) * st] : mk<R>(R(0), R(0));

  Kahan<R> acc[4];
  int slots[4];
  int nred = 0;

  // ---- prologue ---------------------------------------------------------
  if (a.pro != PRO_NONE) {
    const R s = (R)a.sc->scale;
    const R mu = (R)a.sc->mu;
    const R g = (R)a.g, dre = (R)a.dre, dim = (R)a.dim;
    const bool needV = a.pro == PRO_RT_HALF || a.pro == PRO_RT_FULL || a.pro == PRO_ITP ||
                       (a.kind == KIND_ENERGY && a.energy_pot);
    R Vv[E];
#pragma unroll
    for (int m = 0; m < E; ++m)
      Vv[m] = (valid && needV) ? a.V[base + (long long)(t + T * m) * st] : R(0);
    if (a.kind == KIND_ENERGY && a.energy_pot) nred = 3;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      cx<R> p = v[m];
      if (a.pro == PRO_SCALE) {
        p = rmul(p, s);
        if (a.kind == KIND_ENERGY && a.energy_pot) {
          R n = norm2(p);
          acc[0].add(n);
          acc[1].add(Vv[m] * n);
          acc[2].add(n * n);
        }
      } else if (a.pro == PRO_RT_HALF) {
        p = rmul(p, s);
        R ex = (-(Vv[m] - mu) - g * norm2(p)) * R(0.5);
        p = cmul(cexp_real_times(ex, dre, dim), p);
      } else if (a.pro == PRO_RT_FULL) {
        R ex = -(Vv[m] - mu) - g * norm2(p);
        p = cmul(cexp_real_times(ex, dre, dim), p);
      } else if (a.pro == PRO_ITP) {
        p = rmul(p, s);
        R nl = rexp(-dre * R(0.5) * (norm2(p) * g + Vv[m]));
        if (valid) a.aux[base + (long long)(t + T * m) * st] = nl;
        p = rmul(p, nl);
      }
      v[m] = p;
    }
  }

  // ---- FFT along the axis -----------------------------------------------
  St::forward(v, sm, pol, t, a.tw);

  if (a.kind == KIND_ENERGY) {
    Kahan<R> kin;
#pragma unroll
    for (int m = 0; m < E; ++m) kin.add(__ldg(&a.k2h[St::spec_pos(t, m)]) * norm2(v[m]));
    double vals[4];
    if (nred == 3) {
      vals[0] = valid ? acc[0].value() : 0.0;
      vals[1] = valid ? acc[1].value() : 0.0;
      vals[2] = valid ? acc[2].value() : 0.0;
      slots[0] = S_N; slots[1] = S_VN; slots[2] = S_N2;
    }
    vals[nred] = valid ? kin.value() : 0.0;
    slots[nred] = a.kin_slot;
    cta_reduce_store<L::THREADS>(vals, slots, nred + 1, a.partials, a.cap);
    return;
  }

#pragma unroll
  for (int m = 0; m < E; ++m) v[m] = cmul(v[m], ldg(&a.phase[St::spec_pos(t, m)]));

  St::inverse(v, sm, pol, t, a.tw);

  // ---- epilogue ---------------------------------------------------------
  if (a.epi == EPI_RT_END) {
    const R mu = (R)a.sc->mu;
    const R g = (R)a.g, dre = (R)a.dre, dim = (R)a.dim;
    R Vv[E];
#pragma unroll
    for (int m = 0; m < E; ++m) Vv[m] = valid ? a.V[base + (long long)(t + T * m) * st] : R(0);
    nred = 3;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      cx<R> p = v[m];
      const R VV = Vv[m] - mu;
      p = cmul(cexp_real_times(-VV - g * norm2(p), dre, dim), p);            // solve_split.m:60-61
      p = cmul(cexp_real_times((VV + g * norm2(p)) * R(0.5), dre, dim), p);  // solve_split.m:63-64
      const R n = norm2(p);                                                  // solve_split.m:65
      acc[0].add(n);
      acc[1].add(Vv[m] * n);
      acc[2].add(n * n);
      v[m] = p;
    }
    slots[0] = S_N; slots[1] = S_VN; slots[2] = S_N2;
  } else if (a.epi == EPI_ITP) {
    nred = 1;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const R nl = valid ? a.aux[base + (long long)(t + T * m) * st] : R(0);
      v[m] = rmul(v[m], nl);  // groundstate_itp.m:42
      acc[0].add(norm2(v[m]));
    }
    slots[0] = S_N;
  }

  if (valid) {
#pragma unroll
    for (int m = 0; m < E; ++m) a.psi[base + (long long)(t + T * m) * st] = v[m];
  }
  if (nred > 0) {
    double vals[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) vals[i] = (i < nred && valid) ? acc[i].value() : 0.0;
    cta_reduce_store<L::THREADS>(vals, slots, nred, a.partials, a.cap);
  }
}

// Host-side launch description of a pass for one axis length.
struct PassGeom {
  int threads;
  int ffts;
  size_t smem;
};

template <typename R, int N>
PassGeom pass_geom(bool strided);

template <typename R, int N>
cudaError_t launch_pass(const PassArgs<R>& a, bool strided, cudaStream_t s);

}  // namespace gpe

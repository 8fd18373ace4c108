// pass_x2.cuh - the paired FP32 axis pass: two pencils per thread, every
// complex operation on packed FP32x2 lanes (fx2, common.cuh).
//
// Same split-step arithmetic and order as pass_kernel's KIND_STEP (pass.cuh):
// [prologue] -> FFT -> x exp(-k^2/2 dt)/N -> IFFT -> [epilogue], with the
// plan's radix schedule and its FFT tables (the tables of the scalar pass of
// the same plan; each entry is broadcast to both lanes).  Thread (f, t) holds
// the E points t + T*m of the pencils 2f and 2f+1 of its CTA's range as
// cx<fx2>{(re_A, re_B), (im_A, im_B)}: each packed instruction advances two
// pencils, so the FFT, the kinetic factor and the phase factors issue about
// half the instructions of the scalar pass, whose throughput is bounded by
// instruction issue rather than by HBM.  Shared-memory exchanges move one
// 16-byte element per position (both pencils).
//
// Layouts (both read the pair's two pencils with the loads of one pencil):
//  * ContigX2 (y): the pencils are contiguous; lanes t of one pair are
//    adjacent, exchange regions padded as p + (p >> PADSH) (chosen by
//    simulating the 16-byte exchange patterns, 8 lanes per shared-memory
//    phase: conflict-free for the E = 8 plans, 1.17x the ideal wavefronts
//    for E = 12).
//  * StridedX2 (x, z): the two pencils are adjacent elements of one row, so
//    one 16-byte load reads both; a CTA covers 2*FP adjacent pencils (at
//    least one 128-byte row); the exchange buffer is [position][pair].
#pragma once
#include "pass.cuh"

namespace gpe {

// Paired-lane padding shift of the contiguous exchange region.
template <class P>
constexpr int x2_padsh() {
  return P::E >= 16 ? 4 : 3;
}

template <class P>
struct ContigX2 {
  static constexpr int T = P::T;
  static_assert(T >= 8, "paired contiguous pass: a 16-byte shared-memory phase must stay within one pair");
  static constexpr int FP = (T >= GPE_DIRECT_CTA_THREADS) ? 1 : GPE_DIRECT_CTA_THREADS / T;
  static constexpr int THREADS = FP * T;
  static constexpr int PENCILS = 2 * FP;
  static constexpr int PADSH = x2_padsh<P>();
  static constexpr int REG = padpos<PADSH>(P::N - 1) + 1;
  __host__ __device__ static constexpr size_t smem_bytes() { return sizeof(cx<fx2>) * (size_t)FP * REG; }
  struct Pol {
    int off;
    __device__ __forceinline__ int idx(int p) const { return off + padpos<PADSH>(p); }
    __device__ __forceinline__ void sync() const {
      if constexpr (T <= 32) __syncwarp();
      else __syncthreads();
    }
    GPE_POL_CHECK_MEMBERS
  };
  static __device__ __forceinline__ void map(int tid, int& f, int& t) {
    f = tid / T;
    t = tid % T;
  }
  static __device__ __forceinline__ Pol pol(int f) { return Pol{f * REG}; }
  static __device__ __forceinline__ long long base(const PassArgs<float>&, long long b) { return b * (long long)P::N; }
  static __device__ __forceinline__ long long step(const PassArgs<float>&) { return 1; }
  // element offset of pencil B from pencil A
  static __device__ __forceinline__ long long pair_off(const PassArgs<float>&) { return P::N; }
  static __device__ __forceinline__ void load(const cx<float>* src, long long dm, long long pb, bool valid,
                                              cx<fx2>* v) {
#pragma unroll
    for (int m = 0; m < P::E; ++m) {
      const cx<float> a = valid ? ld_stream(src + m * dm) : mk<float>(0.f, 0.f);
      const cx<float> b = valid ? ld_stream(src + m * dm + pb) : mk<float>(0.f, 0.f);
      v[m] = mk<fx2>(fx2(a.x, b.x), fx2(a.y, b.y));
    }
  }
  static __device__ __forceinline__ void store(cx<float>* dst, long long dm, long long pb, const cx<fx2>* v) {
#pragma unroll
    for (int m = 0; m < P::E; ++m) {
      dst[m * dm] = mk<float>(v[m].x.v.x, v[m].y.v.x);
      dst[m * dm + pb] = mk<float>(v[m].x.v.y, v[m].y.v.y);
    }
  }
  // real side array (V, aux) of both pencils at element m
  static __device__ __forceinline__ fx2 load_side(const float* s, long long dm, long long pb, int m, bool valid) {
    if (!valid) return fx2(0.f);
    return fx2(ld_stream(s + m * dm), ld_stream(s + m * dm + pb));
  }
  static __device__ __forceinline__ void store_side(float* s, long long dm, long long pb, int m, fx2 x) {
    s[m * dm] = x.v.x;
    s[m * dm + pb] = x.v.y;
  }
  static __device__ __forceinline__ void prefetch(const PassArgs<float>& a, long long b0, long long cnt) {
    ContigLayout<P, float>::prefetch(a, b0, cnt);
  }
};

template <class P>
struct StridedX2 {
  static constexpr int T = P::T;
  // pairs per CTA: 16 bytes per pair, at least one 128-byte row, at least
  // GPE_DIRECT_CTA_THREADS threads, at most 1024
  static constexpr int F0 = (GPE_DIRECT_CTA_THREADS / T > 8) ? GPE_DIRECT_CTA_THREADS / T : 8;
  static constexpr int FP = (F0 * T > 1024) ? 1024 / T : F0;
  static constexpr int THREADS = FP * T;
  static constexpr int PENCILS = 2 * FP;
  __host__ __device__ static constexpr size_t smem_bytes() { return sizeof(cx<fx2>) * (size_t)FP * P::N; }
  struct Pol {
    int f;
    __device__ __forceinline__ int idx(int p) const { return p * FP + f; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    GPE_POL_CHECK_MEMBERS
  };
  static __device__ __forceinline__ void map(int tid, int& f, int& t) {
    f = tid % FP;
    t = tid / FP;
  }
  static __device__ __forceinline__ Pol pol(int f) { return Pol{f}; }
  static __device__ __forceinline__ long long base(const PassArgs<float>& a, long long b) {
    return (b % a.inner) + (b / a.inner) * a.outer;
  }
  static __device__ __forceinline__ long long step(const PassArgs<float>& a) { return a.stride; }
  static __device__ __forceinline__ long long pair_off(const PassArgs<float>&) { return 1; }
  // The pair's elements are adjacent and 16-byte aligned (even offsets,
  // checked on the host): one 16-byte load or store per position.
  static __device__ __forceinline__ void load(const cx<float>* src, long long dm, long long, bool valid, cx<fx2>* v) {
#pragma unroll
    for (int m = 0; m < P::E; ++m) {
      const float4 q = valid ? __ldcs(reinterpret_cast<const float4*>(src + m * dm)) : make_float4(0.f, 0.f, 0.f, 0.f);
      v[m] = mk<fx2>(fx2(q.x, q.z), fx2(q.y, q.w));
    }
  }
  static __device__ __forceinline__ void store(cx<float>* dst, long long dm, long long, const cx<fx2>* v) {
#pragma unroll
    for (int m = 0; m < P::E; ++m)
      *reinterpret_cast<float4*>(dst + m * dm) = make_float4(v[m].x.v.x, v[m].y.v.x, v[m].x.v.y, v[m].y.v.y);
  }
  static __device__ __forceinline__ fx2 load_side(const float* s, long long dm, long long, int m, bool valid) {
    if (!valid) return fx2(0.f);
    return fx2(__ldcs(reinterpret_cast<const float2*>(s + m * dm)));
  }
  static __device__ __forceinline__ void store_side(float* s, long long dm, long long, int m, fx2 x) {
    *reinterpret_cast<float2*>(s + m * dm) = x.v;
  }
  static __device__ __forceinline__ void prefetch(const PassArgs<float>& a, long long b0, long long cnt) {
    if (a.inner % PENCILS != 0) return;
    const long long o = base(a, b0);
    const int lines = (int)((cnt * (long long)sizeof(cx<float>) + 127) / 128);
    for (int i = threadIdx.x; i < P::N * lines; i += THREADS) {
      const int r = i / lines, l = i % lines;
      prefetch_l2_line(reinterpret_cast<const char*>(a.psi + o + (long long)r * a.stride) + l * 128);
    }
    if (a.side != 0) {
      const float* s = side_array(a);
      const int sl = (int)((cnt * (long long)sizeof(float) + 127) / 128);
      for (int i = threadIdx.x; i < P::N * sl; i += THREADS) {
        const int r = i / sl, l = i % sl;
        prefetch_l2_line(reinterpret_cast<const char*>(s + o + (long long)r * a.stride) + l * 128);
      }
    }
  }
};

// ---- packed elementwise math -------------------------------------------------

// exp(a * (dre + i dim)) of both lanes (cexp_real_times, common.cuh).
__device__ __forceinline__ cx<fx2> cexp_real_times_x2(fx2 a, float dre, float dim) {
  fx2 s, c;
  sincos_x2(a * fx2(dim), s, c);
  if (dre == 0.0f) return mk<fx2>(c, s);
  const fx2 m = exp_x2(a * fx2(dre));
  return mk<fx2>(m * c, m * s);
}

// The full nonlinear step of real time on both pencils (solve_split.m:60-61):
// the PRO_RT_FULL prologue, and the middle of a folded pass.
template <class L, int E>
__device__ __forceinline__ void rt_full_x2(cx<fx2>* v, const PassArgs<float>& a, bool valid, long long first,
                                           long long dm, long long pb, float mu) {
  const fx2 g(a.gr);
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const fx2 V = L::load_side(a.V + first, dm, pb, m, valid);
    const fx2 ex = fma2(-g, norm2(v[m]), fx2(mu) - V);
    v[m] = cmul(cexp_real_times_x2(ex, a.drer, a.dimr), v[m]);
  }
}

// Prologue of the first pass (pass.cuh prologue, on both pencils).
template <class L, int E>
__device__ __forceinline__ void prologue_x2(cx<fx2>* v, const PassArgs<float>& a, bool valid, long long first,
                                            long long dm, long long pb, float s, float mu) {
  const fx2 g(a.gr);
  const float dre = a.drer, dim = a.dimr;
  switch (a.pro) {
    case PRO_SCALE:
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = rmul(v[m], fx2(s));
      break;
    case PRO_RT_HALF:  // solve_split.m:55-56
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const fx2 V = L::load_side(a.V + first, dm, pb, m, valid);
        const cx<fx2> p = rmul(v[m], fx2(s));
        const fx2 ex = fma2(-g, norm2(p), fx2(mu) - V) * fx2(0.5f);
        v[m] = cmul(cexp_real_times_x2(ex, dre, dim), p);
      }
      break;
    case PRO_RT_FULL:  // solve_split.m:60-61
      rt_full_x2<L, E>(v, a, valid, first, dm, pb, mu);
      break;
    case PRO_ITP:  // groundstate_itp.m:36/76, :40
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const fx2 V = L::load_side(a.V + first, dm, pb, m, valid);
        const cx<fx2> p = rmul(v[m], fx2(s));
        const fx2 nl = exp_x2(fx2(-dre * 0.5f) * fma2(norm2(p), g, V));
        if (valid) L::store_side(a.aux + first, dm, pb, m, nl);
        v[m] = rmul(p, nl);
      }
      break;
    default:
      break;
  }
}

// Per-lane compensated sums, merged into one float pair at the end.
struct Kahan2 {
  fx2 s = fx2(0.f), c = fx2(0.f);
  __device__ __forceinline__ void add(fx2 x) {
    const fx2 y = x - c;
    const fx2 t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ Kahan<float> merged() const {
    float h = s.v.x, l = -c.v.x;
    pair_add(h, l, s.v.y, -c.v.y);
    Kahan<float> k;
    k.s = h;
    k.c = -l;
    return k;
  }
};

// Epilogue of the last pass (pass.cuh epilogue, on both pencils).
template <class L, int E>
__device__ __forceinline__ void epilogue_x2(cx<fx2>* v, const PassArgs<float>& a, Kahan2* acc, bool valid,
                                            long long first, long long dm, long long pb, float mu) {
  if (a.epi == EPI_RT_END) {
    const fx2 g(a.gr);
    const float dre = a.drer, dim = a.dimr;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const fx2 V = L::load_side(a.V + first, dm, pb, m, valid);
      cx<fx2> p = v[m];
      const fx2 VV = V - fx2(mu);
      p = cmul(cexp_real_times_x2(fma2(-g, norm2(p), -VV), dre, dim), p);            // solve_split.m:60-61
      p = cmul(cexp_real_times_x2(fma2(g, norm2(p), VV) * fx2(0.5f), dre, dim), p);  // solve_split.m:63-64
      const fx2 n = norm2(p);                                                       // solve_split.m:65
      if (valid) {
        acc[0].add(n);
        acc[1].add(V * n);
        acc[2].add(n * n);
      }
      v[m] = p;
    }
  } else if (a.epi == EPI_ITP) {
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const fx2 nl = L::load_side(a.aux + first, dm, pb, m, valid);
      v[m] = rmul(v[m], nl);  // groundstate_itp.m:42
      if (valid) acc[0].add(norm2(v[m]));
    }
  }
}

// Kinetic factors of the thread's slots, broadcast to both pencils (the
// scalar pass's table: [m/2][t] pairs of entries).
template <int T, int E, bool SMT>
__device__ __forceinline__ void apply_phase_x2(cx<fx2>* v, const cx<float>* __restrict__ php, int t) {
  const float4* r4 = reinterpret_cast<const float4*>(php) + t;
#pragma unroll
  for (int i = 0; i < E / 2; ++i) {
    const float4 q = ld_tab<SMT>(r4 + i * T);
    v[2 * i] = cmul(v[2 * i], mk<fx2>(fx2(q.x), fx2(q.y)));
    v[2 * i + 1] = cmul(v[2 * i + 1], mk<fx2>(fx2(q.z), fx2(q.w)));
  }
}

// Resident threads per SM the paired passes aim at: E <= 12 points per
// pencil (two pencils: 2E complex values per thread) at 768 (80 registers),
// E = 16 at 512 (128 registers).
#ifndef GPE_X2_THREADS_PER_SM
#define GPE_X2_THREADS_PER_SM 768
#endif
#ifndef GPE_X2_THREADS_PER_SM_E16
#define GPE_X2_THREADS_PER_SM_E16 512
#endif
template <class P, class L>
struct X2MinBlocks {
  static constexpr int TPS = P::E >= 16 ? GPE_X2_THREADS_PER_SM_E16 : GPE_X2_THREADS_PER_SM;
  static constexpr int value = L::THREADS <= TPS ? TPS / L::THREADS : 1;
};
template <class P>
struct X2SmemTables {
  static constexpr bool value = GPE_SMEM_TABLES && P::N <= 256;
};
template <class P, class L>
constexpr size_t x2_smem_bytes() {
  return L::smem_bytes() + (X2SmemTables<P>::value ? sizeof(cx<float>) * (size_t)(P::TW_LEN + P::N) : 0);
}

// The paired step pass (KIND_STEP; FOLD: the folded passes, a.fold = 1).
template <class P, class L, bool FOLD>
__global__ void __launch_bounds__(L::THREADS, X2MinBlocks<P, L>::value) pass_x2_kernel(const PassArgs<float> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<fx2>* sm = reinterpret_cast<cx<fx2>*>(smem_raw);
  // Programmatic dependent launch and the first-wave L2 hint as in pass_kernel.
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (a.pdl && a.pf_ahead > 0 && (long long)blockIdx.x < a.pf_ahead) {
    const long long b0 = (long long)blockIdx.x * L::PENCILS;
    if (b0 < a.n_batch) L::prefetch(a, b0, a.n_batch - b0 < L::PENCILS ? a.n_batch - b0 : (long long)L::PENCILS);
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __shared__ float scal[2];
  if (threadIdx.x == 0) {
    scal[0] = (float)a.sc->scale;
    scal[1] = (float)a.sc->mu;
  }
  if (__syncthreads_or(a.sc->stop != 0)) return;

  constexpr int T = P::T, E = P::E;
  using St = typename P::template St<fx2>;
  int f, t;
  L::map(threadIdx.x, f, t);
  const long long b = (long long)blockIdx.x * L::PENCILS + 2 * f;  // pencil A; B is its neighbour
  const bool valid0 = b < a.n_batch;  // n_batch is even: A and B are valid together
  const long long st = L::step(a);
  const long long first = (valid0 ? L::base(a, b) : 0) + (long long)t * st;
  const long long dm = (long long)T * st;
  const long long pb = L::pair_off(a);
  auto pol = L::pol(f);
  GPE_POL_BOUNDS(pol, a.sc, L::smem_bytes() / sizeof(cx<fx2>));
  // bounds-checked build: the pair's last element inside the pass's extent
  const bool valid = valid0 && bounds_ok(a.sc, BS_LOAD, first + (E - 1) * dm + pb, a.npts);

  cx<fx2> v[E];
  L::load(a.psi + first, dm, pb, valid, v);
  if (a.pf_ahead > 0) {
    const long long b0 = ((long long)blockIdx.x + a.pf_ahead) * L::PENCILS;
    if (b0 < a.n_batch) L::prefetch(a, b0, a.n_batch - b0 < L::PENCILS ? a.n_batch - b0 : (long long)L::PENCILS);
  }
  const cx<float>* tws = a.tws;
  const cx<float>* php = a.php;
  constexpr bool SMT = X2SmemTables<P>::value;
  if constexpr (SMT) {
    cx<float>* tab = reinterpret_cast<cx<float>*>(smem_raw + L::smem_bytes());  // 16-byte aligned
    const float4* g1 = reinterpret_cast<const float4*>(a.tws);
    float4* s1 = reinterpret_cast<float4*>(tab);
    for (int i = threadIdx.x; i < P::TW_LEN / 2; i += L::THREADS) s1[i] = __ldg(g1 + i);
    const float4* g2 = reinterpret_cast<const float4*>(a.php);
    float4* s2 = reinterpret_cast<float4*>(tab + P::TW_LEN);
    for (int i = threadIdx.x; i < P::N / 2; i += L::THREADS) s2[i] = __ldg(g2 + i);
    __syncthreads();
    tws = tab;
    php = tab + P::TW_LEN;
  }
  if (a.pro != PRO_NONE) prologue_x2<L, E>(v, a, valid, first, dm, pb, scal[0], scal[1]);
  if constexpr (FOLD) {
    // a folded pass: the transform, the full nonlinear step, the transform
    // again
#pragma unroll 1
    for (int rep = 0;; ++rep) {
      St::template forward<SMT>(v, sm, pol, t, tws);
      apply_phase_x2<T, E, SMT>(v, php, t);
      St::template inverse<SMT>(v, sm, pol, t, tws);
      if (rep == 1) break;
      rt_full_x2<L, E>(v, a, valid, first, dm, pb, scal[1]);
    }
  } else {
    St::template forward<SMT>(v, sm, pol, t, tws);
    apply_phase_x2<T, E, SMT>(v, php, t);
    St::template inverse<SMT>(v, sm, pol, t, tws);
  }
  Kahan2 acc[3];
  if (a.epi != EPI_NONE) epilogue_x2<L, E>(v, a, acc, valid, first, dm, pb, scal[1]);
  if (valid) L::store(a.psi + first, dm, pb, v);
  const int nred = a.epi == EPI_RT_END ? 3 : a.epi == EPI_ITP ? 1 : 0;
  if (nred > 0) {
    Kahan<float> k[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) k[i] = acc[i].merged();
    const int slots[4] = {S_N, S_VN, S_N2, 0};
    if (bounds_ok(a.sc, BS_PARTIAL, blockIdx.x, a.cap)) cta_reduce_store<L::THREADS>(k, slots, nred, a.partials, a.cap);
  }
}

// The paired pass applies to plain step passes whose pencil pairs are
// adjacent, 16-byte aligned elements: an even pencil count, and even row
// offsets and strides on the strided axes.
inline bool x2_applies(const PassArgs<float>& a, bool strided) {
  if (!(a.kind == KIND_STEP || (a.kind == KIND_STEP_EXT && a.fold)) || a.rot || a.skip_fwd || a.skip_inv ||
      a.mask_c)
    return false;
  if (a.n_batch % 2 != 0) return false;
  if (strided) return a.inner % 2 == 0 && a.outer % 2 == 0 && a.stride % 2 == 0;
  return true;
}

// V: the plan the paired pass runs on (plans.cuh PlanSel: 0 = Plan<N>,
// 1 = PlanAlt<N>).
template <int N, int V>
PassGeom pass_x2_geom(bool strided);
template <int N, int V>
cudaError_t launch_pass_x2(const PassArgs<float>& a, bool strided, cudaStream_t s);

}  // namespace gpe

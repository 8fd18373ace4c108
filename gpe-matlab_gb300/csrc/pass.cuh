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
#include "tma.cuh"

namespace gpe {

// Side array of a pass (V for the phase factors, aux for the ITP factor).
template <typename R>
__device__ __forceinline__ const R* side_array(const PassArgs<R>& a) {
  return a.side == 2 ? a.aux : a.V;
}

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

// Threads per CTA of the direct passes (pencils per CTA follow from it).
#ifndef GPE_DIRECT_CTA_THREADS
#define GPE_DIRECT_CTA_THREADS 256
#endif

template <class P, typename R>
struct ContigLayout {
  static constexpr bool CONTIG = true;
  static constexpr int T = P::T;
  static constexpr int FFTS = (T >= GPE_DIRECT_CTA_THREADS) ? 1 : GPE_DIRECT_CTA_THREADS / T;
  static constexpr int THREADS = FFTS * T;
  static constexpr int REG0 = padpos<P::PADSH>(P::N - 1) + 1;
  static constexpr int REG = (REG0 % 2 == 0) ? REG0 + 1 : REG0;  // odd stride between pencils
  __host__ __device__ static constexpr size_t smem_bytes() { return sizeof(cx<R>) * (size_t)FFTS * REG; }
  struct Pol {
    int off;
    __device__ __forceinline__ int idx(int p) const { return off + padpos<P::PADSH>(p); }
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
  static __device__ __forceinline__ long long base(const PassArgs<R>& a, long long b) {
    return b * (long long)P::N;
  }
  static __device__ __forceinline__ long long step(const PassArgs<R>&) { return 1; }
  // L2 prefetch of pencils b0 .. b0+cnt-1 (one contiguous run; with the side
  // array's run when the pass reads one).  N*sizeof(R) is a multiple of 16
  // for every planned N, so every chunk is 16-byte aligned and sized.
  static __device__ __forceinline__ void prefetch(const PassArgs<R>& a, long long b0, long long cnt) {
    constexpr size_t CH = 4096;
    const size_t bytes = (size_t)cnt * P::N * sizeof(cx<R>);
    const char* p = reinterpret_cast<const char*>(a.psi + b0 * P::N);
    for (size_t off = (size_t)threadIdx.x * CH; off < bytes; off += (size_t)THREADS * CH)
      prefetch_l2_bulk(p + off, (uint32_t)(bytes - off < CH ? bytes - off : CH));
    if (a.side != 0) {
      const size_t sb = (size_t)cnt * P::N * sizeof(R);
      const char* s = reinterpret_cast<const char*>(side_array(a) + b0 * P::N);
      for (size_t off = (size_t)threadIdx.x * CH; off < sb; off += (size_t)THREADS * CH)
        prefetch_l2_bulk(s + off, (uint32_t)(sb - off < CH ? sb - off : CH));
    }
  }
};

template <class P, typename R>
struct StridedLayout {
  static constexpr bool CONTIG = false;
  static constexpr int T = P::T;
  // Adjacent pencils per CTA: one 128-byte row.  (64-byte rows, which halve
  // the CTA of T > 16 plans, measured 5% faster on the 512^3 x pass and 28%
  // slower on the z pass, whose rows are 2 MB apart.)
  static constexpr int G = 128 / (int)sizeof(cx<R>);
  static constexpr int F0 = (GPE_DIRECT_CTA_THREADS / T > G) ? GPE_DIRECT_CTA_THREADS / T : G;
  static constexpr int FFTS = (F0 * T > 1024) ? 1024 / T : F0;
  static constexpr int THREADS = FFTS * T;
  __host__ __device__ static constexpr size_t smem_bytes() { return sizeof(cx<R>) * (size_t)FFTS * P::N; }
  struct Pol {
    int f;
    __device__ __forceinline__ int idx(int p) const { return p * FFTS + f; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    GPE_POL_CHECK_MEMBERS
  };
  static __device__ __forceinline__ void map(int tid, int& f, int& t) {
    f = tid % FFTS;
    t = tid / FFTS;
  }
  static __device__ __forceinline__ Pol pol(int f) { return Pol{f}; }
  // (32-bit and shift forms of this division made ptxas spill 130-150 bytes
  // in the strided step kernel, and it measured slower.)
  static __device__ __forceinline__ long long base(const PassArgs<R>& a, long long b) {
    return (b % a.inner) + (b / a.inner) * a.outer;
  }
  static __device__ __forceinline__ long long step(const PassArgs<R>& a) { return a.stride; }
  // L2 prefetch of pencils b0 .. b0+cnt-1: N rows of cnt adjacent elements,
  // one line-sized hint per 128 bytes of each row (and of the side array's
  // rows).  Skipped when a tile's pencils could straddle two row groups.
  static __device__ __forceinline__ void prefetch(const PassArgs<R>& a, long long b0, long long cnt) {
    if (a.inner % FFTS != 0) return;
    const long long o = base(a, b0);
    const int lines = (int)((cnt * (long long)sizeof(cx<R>) + 127) / 128);
    for (int i = threadIdx.x; i < P::N * lines; i += THREADS) {
      const int r = i / lines, l = i % lines;
      prefetch_l2_line(reinterpret_cast<const char*>(a.psi + o + (long long)r * a.stride) + l * 128);
    }
    if (a.side != 0) {
      const R* s = side_array(a);
      const int sl = (int)((cnt * (long long)sizeof(R) + 127) / 128);
      for (int i = threadIdx.x; i < P::N * sl; i += THREADS) {
        const int r = i / sl, l = i % sl;
        prefetch_l2_line(reinterpret_cast<const char*>(s + o + (long long)r * a.stride) + l * 128);
      }
    }
  }
};

// Error-free float addition (Knuth's TwoSum): a + b = s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// (h, l) += (h2, l2) for unevaluated float pairs h + l (double-float add).
__device__ __forceinline__ void pair_add(float& h, float& l, float h2, float l2) {
  float s, e;
  two_sum(h, h2, s, e);
  e += l + l2;
  h = s + e;
  l = e - (h - s);
}

// Sum `nred` per-thread values over the CTA in FP64 and store the CTA's
// partial of each to partials[slot*cap + idx] (idx: the tile, by default the
// CTA index).
template <int THREADS>
__device__ __forceinline__ void cta_reduce_store(double* vals, const int* slots, int nred,
                                                 double* partials, int cap, long long idx = -1);

// The same for per-thread compensated sums.  FP32: each thread's Kahan sum
// s - c is kept as the float pair (s, -c) and the warp combines pairs with
// double-float additions (FP32 pipe; the GPU's FP64 rate is a small fraction
// of its FP32 rate), converting to FP64 once per warp.
template <int THREADS, typename R>
__device__ __forceinline__ void cta_reduce_store(const Kahan<R>* acc, const int* slots, int nred,
                                                 double* partials, int cap, long long idx = -1) {
  if (idx < 0) idx = blockIdx.x;
  if constexpr (sizeof(R) == 8) {
    double vals[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) vals[i] = i < nred ? acc[i].value() : 0.0;
    cta_reduce_store<THREADS>(vals, slots, nred, partials, cap, idx);
  } else {
    __shared__ double red[THREADS / 32 > 0 ? THREADS / 32 : 1][4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i >= nred) break;
      float h = acc[i].s, l = -acc[i].c;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, h, o);
        const float l2 = __shfl_down_sync(0xffffffffu, l, o);
        pair_add(h, l, h2, l2);
      }
      if (lane == 0) red[warp][i] = (double)h + (double)l;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < nred; ++i) {
        double s = 0.0;
        for (int w = 0; w < (THREADS + 31) / 32; ++w) s += red[w][i];
        partials[(size_t)slots[i] * cap + idx] = s;
      }
    }
  }
}

template <int THREADS>
__device__ __forceinline__ void cta_reduce_store(double* vals, const int* slots, int nred,
                                                 double* partials, int cap, long long idx) {
  if (idx < 0) idx = blockIdx.x;
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
      partials[(size_t)slots[i] * cap + idx] = s;
    }
  }
}

// Multiply v[0..E) by the thread's kinetic factors.  The permuted table is
// stored slot-major so adjacent lanes read adjacent addresses: FP32 as
// [m/2][t] pairs of entries (16-byte vectors), FP64 as [m][t] entries.
// SMT: php points to shared memory.
template <int T, int E, bool SMT = false>
__device__ __forceinline__ void apply_phase(cx<float>* v, const cx<float>* __restrict__ php, int t) {
  const float4* r4 = reinterpret_cast<const float4*>(php) + t;
#pragma unroll
  for (int i = 0; i < E / 2; ++i) {
    const float4 q = ld_tab<SMT>(r4 + i * T);
    v[2 * i] = cmul(v[2 * i], mk<float>(q.x, q.y));
    v[2 * i + 1] = cmul(v[2 * i + 1], mk<float>(q.z, q.w));
  }
}
template <int T, int E, bool SMT = false>
__device__ __forceinline__ void apply_phase(cx<double>* v, const cx<double>* __restrict__ php, int t) {
#pragma unroll
  for (int m = 0; m < E; ++m) v[m] = cmul(v[m], ld_tab<SMT>(php + m * T + t));
}

// Occupancy hint: FP32 passes aim at GPE_FP32_THREADS_PER_SM resident
// threads per SM (the register budget per thread follows from it).
#ifndef GPE_FP32_THREADS_PER_SM
#define GPE_FP32_THREADS_PER_SM 768  // 80 registers: no spills; 1024 (64) spilled heavily
#endif
// FP32 step passes of length <= 256 keep their twiddle rows and kinetic
// factors in shared memory (after the exchange buffer): measured 4% faster
// at 256^3; at 512 the larger buffers cost occupancy and it was slower.
template <typename R, class P, int KIND>
struct SmemTables {
  static constexpr bool value = GPE_SMEM_TABLES && sizeof(R) == 4 && KIND != KIND_ENERGY && P::N <= 256;
};
template <typename R, class P, class L, int KIND>
constexpr size_t pass_smem_bytes() {
  return L::smem_bytes() + (SmemTables<R, P, KIND>::value ? sizeof(cx<R>) * (size_t)(P::TW_LEN + P::N) : 0);
}

// Plans with at most 8 points per thread hold half the data in registers and
// aim at 1024 threads per SM (64 registers).
template <typename R, class P, class L>
struct MinBlocks {
  static constexpr int TPS = P::E <= 8 ? 1024 : GPE_FP32_THREADS_PER_SM;
  static constexpr int value = (sizeof(R) == 4 && L::THREADS <= TPS) ? TPS / L::THREADS : 1;
};

// The full nonlinear step of real time, exp((-(V - mu) - g|psi|^2) dt) psi
// (solve_split.m:60-61), on one pencil's E values (sv: V).
template <typename R, int E>
__device__ __forceinline__ void rt_full_phase(cx<R>* v, const R* sv, const PassArgs<R>& a, R mu) {
  const R g = a.gr, dre = a.drer, dim = a.dimr;
  if constexpr (sizeof(R) == 4) {
    float ex[E];
#pragma unroll
    for (int m = 0; m < E; ++m) ex[m] = -(sv[m] - mu) - g * norm2(v[m]);
    apply_rt_phase<E>(v, ex, dre, dim);
  } else {
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const R ex = -(sv[m] - mu) - g * norm2(v[m]);
      v[m] = cmul(cexp_real_times(ex, dre, dim), v[m]);
    }
  }
}

// Prologue of the first pass on one pencil's E values (sv: V for the phase
// modes, unused otherwise).  The mode switch sits outside the unrolled loops
// so only the selected variant executes (branches inside an unrolled loop
// are if-converted, which ran every variant).
// s, mu: the pending scale and mu in R (read once per CTA).
template <typename R, int E>
__device__ __forceinline__ void prologue(cx<R>* v, const R* sv, const PassArgs<R>& a, bool valid,
                                         long long first, long long dm, R s, R mu) {
  const R g = a.gr, dre = a.drer, dim = a.dimr;
  switch (a.pro) {
    case PRO_SCALE:
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = rmul(v[m], s);
      break;
    case PRO_RT_HALF:  // solve_split.m:55-56
      if constexpr (sizeof(R) == 4) {
        float ex[E];
#pragma unroll
        for (int m = 0; m < E; ++m) {
          v[m] = rmul(v[m], s);
          ex[m] = (-(sv[m] - mu) - g * norm2(v[m])) * 0.5f;
        }
        apply_rt_phase<E>(v, ex, dre, dim);
      } else {
#pragma unroll
        for (int m = 0; m < E; ++m) {
          const cx<R> p = rmul(v[m], s);
          const R ex = (-(sv[m] - mu) - g * norm2(p)) * R(0.5);
          v[m] = cmul(cexp_real_times(ex, dre, dim), p);
        }
      }
      break;
    case PRO_RT_FULL:  // solve_split.m:60-61
      rt_full_phase<R, E>(v, sv, a, mu);
      break;
    case PRO_ITP:  // groundstate_itp.m:36/76, :40
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const cx<R> p = rmul(v[m], s);
        const R nl = rexp(-dre * R(0.5) * (norm2(p) * g + sv[m]));
        if (valid) a.aux[first + m * dm] = nl;
        v[m] = rmul(p, nl);
      }
      break;
    default:
      break;
  }
}

// Epilogue of the last pass; sums of valid pencils go to acc.
template <typename R, int E>
__device__ __forceinline__ void epilogue(cx<R>* v, const R* sv, const PassArgs<R>& a, Kahan<R>* acc,
                                         bool valid, R mu) {
  if (a.epi == EPI_RT_END) {
    const R g = a.gr, dre = a.drer, dim = a.dimr;
    if constexpr (sizeof(R) == 4) {
      // FP32: both phases through the packed sin/cos/exp of apply_rt_phase,
      // in halves of the thread's values (fewer live registers)
      constexpr int H = E % 4 == 0 ? E / 2 : E;
#pragma unroll
      for (int h = 0; h < E; h += H) {
        float ex[H];
#pragma unroll
        for (int m = 0; m < H; ++m) ex[m] = -(sv[h + m] - mu) - g * norm2(v[h + m]);  // solve_split.m:60-61
        apply_rt_phase<H>(v + h, ex, dre, dim);
#pragma unroll
        for (int m = 0; m < H; ++m) ex[m] = ((sv[h + m] - mu) + g * norm2(v[h + m])) * 0.5f;  // :63-64
        apply_rt_phase<H>(v + h, ex, dre, dim);
#pragma unroll
        for (int m = 0; m < H; ++m) {
          const R n = norm2(v[h + m]);  // solve_split.m:65
          if (valid) {
            acc[0].add(n);
            acc[1].add(sv[h + m] * n);
            acc[2].add(n * n);
          }
        }
      }
    } else {
#pragma unroll
      for (int m = 0; m < E; ++m) {
        cx<R> p = v[m];
        const R VV = sv[m] - mu;
        p = cmul(cexp_real_times(-VV - g * norm2(p), dre, dim), p);            // solve_split.m:60-61
        p = cmul(cexp_real_times((VV + g * norm2(p)) * R(0.5), dre, dim), p);  // solve_split.m:63-64
        const R n = norm2(p);                                                  // solve_split.m:65
        if (valid) {
          acc[0].add(n);
          acc[1].add(sv[m] * n);
          acc[2].add(n * n);
        }
        v[m] = p;
      }
    }
  } else if (a.epi == EPI_ITP) {
#pragma unroll
    for (int m = 0; m < E; ++m) {
      v[m] = rmul(v[m], sv[m]);  // groundstate_itp.m:42
      if (valid) acc[0].add(norm2(v[m]));
    }
  }
}

// One tile (FFTS pencils) of an axis pass: tile `tile` of the pass, with
// the pending scale s and mu of the run (read once per CTA by the caller).
// The pass kernel runs tile blockIdx.x; the grid-wide persistent kernel of
// small 2D grids (grid2d.cuh) runs many tiles per CTA.
template <typename R, class P, class L, int KIND>
__device__ __forceinline__ void pass_body(const PassArgs<R>& a, long long tile, unsigned char* smem_raw, R s_scale,
                                          R s_mu) {
  cx<R>* sm = reinterpret_cast<cx<R>*>(smem_raw);
  const R scal[2] = {s_scale, s_mu};
  constexpr int T = P::T, E = P::E;
  using St = typename P::template St<R>;
  int f, t;
  L::map(threadIdx.x, f, t);
  const long long b = tile * L::FFTS + f;
  const bool valid0 = b < a.n_batch;
  const long long st = L::step(a);
  // element m of this thread sits at offset m*dm from its first element
  const long long first = (valid0 ? L::base(a, b) : 0) + (long long)t * st;
  const long long dm = (long long)T * st;
  auto pol = L::pol(f);
  GPE_POL_BOUNDS(pol, a.sc, L::smem_bytes() / sizeof(cx<R>));
  // bounds-checked build: the thread's last element inside the pass's extent
  const bool valid = valid0 && bounds_ok(a.sc, BS_LOAD, first + (E - 1) * dm, a.npts);

  cx<R> v[E];
  {
    const cx<R>* __restrict__ src = a.psi + first;
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = valid ? ld_stream(src + m * dm) : mk<R>(R(0), R(0));
  }
  R sv[E];
  // With the own loads in flight, hint the tile of the CTA one wave of
  // resident CTAs later into L2, so that CTA's loads hit L2.
  if (a.pf_ahead > 0) {
    const long long b0 = (tile + a.pf_ahead) * L::FFTS;
    if (b0 < a.n_batch) L::prefetch(a, b0, a.n_batch - b0 < L::FFTS ? a.n_batch - b0 : (long long)L::FFTS);
  }
  // Step-pass tables in shared memory (SmemTables): copied while the pencil
  // loads are in flight, then read from shared memory.
  const cx<R>* tws = a.tws;
  const cx<R>* php = a.php;
  if constexpr (SmemTables<R, P, KIND>::value) {
    cx<R>* tab = reinterpret_cast<cx<R>*>(smem_raw + L::smem_bytes());  // 16-byte aligned
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

  if constexpr (KIND == KIND_ENERGY) {
    // <psi|L_axis psi> (+ the n, Vn, n^2 sums on request) of the state times
    // the pending scale (PRO_SCALE) or as stored (PRO_NONE).
    const R s = a.pro == PRO_SCALE ? scal[0] : R(1);
    Kahan<R> acc[3];
    const bool pot = a.energy_pot != 0;
    const R* __restrict__ vs = a.V + first;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      v[m] = rmul(v[m], s);
      if (pot) {
        const R n = norm2(v[m]);
        const R Vm = valid ? ld_stream(vs + m * dm) : R(0);
        acc[0].add(n);
        acc[1].add(Vm * n);
        acc[2].add(n * n);
      }
    }
    St::template forward<false>(v, sm, pol, t, a.tws);
    Kahan<R> kin;
    if (a.rotw) {
      // rotating frame (lap.m:8-9): weight k^2/2 -+ omega * coordinate * k
      const R w = valid ? a.rotw[(unsigned)b % (unsigned)a.rot_period] : R(0);
#pragma unroll
      for (int m = 0; m < E; ++m)
        kin.add((__ldg(a.k2p + m * T + t) + w * __ldg(a.kp + m * T + t)) * norm2(v[m]));
    } else {
#pragma unroll
      for (int m = 0; m < E; ++m) kin.add(__ldg(a.k2p + m * T + t) * norm2(v[m]));
    }
    Kahan<R> sums[4];
    int slots[4];
    int nred;
    if (pot) {
      if (valid) {
        sums[0] = acc[0];
        sums[1] = acc[1];
        sums[2] = acc[2];
        sums[3] = kin;
      }
      slots[0] = S_N; slots[1] = S_VN; slots[2] = S_N2; slots[3] = a.kin_slot;
      nred = 4;
    } else {
      if (valid) sums[0] = kin;
      slots[0] = a.kin_slot;
      nred = 1;
    }
    if (bounds_ok(a.sc, BS_PARTIAL, tile, a.cap)) cta_reduce_store<L::THREADS>(sums, slots, nred, a.partials, a.cap, tile);
  } else {
    // The side array (V for the phase factors, or the ITP factors) is read
    // right before the phase that uses it: a pass has a prologue or an
    // epilogue, never both, so it is never held across the FFTs.
    auto load_side = [&]() {
      const R* __restrict__ ss = (a.side == 2 ? a.aux : a.V) + first;
#pragma unroll
      for (int m = 0; m < E; ++m) sv[m] = valid ? ld_stream(ss + m * dm) : R(0);
    };
    if (a.pro != PRO_NONE) {
      if (a.side != 0) load_side();
      prologue<R, E>(v, sv, a, valid, first, dm, scal[0], scal[1]);
    }
    constexpr bool SMT = SmemTables<R, P, KIND>::value;
    if constexpr (KIND == KIND_STEP_EXT) {
      // a folded pass (a.fold = 1): the transform, the full nonlinear step,
      // the transform again (the state stays in registers between the steps)
#pragma unroll 1
      for (int rep = 0;; ++rep) {
        if (!a.skip_fwd) {
          St::template forward<SMT>(v, sm, pol, t, tws);
          apply_phase<T, E, SMT>(v, php, t);
          if (a.rot) {
            // rotating frame: the cross term of this pencil's transverse coordinate
            const unsigned ci = valid ? (unsigned)b % (unsigned)a.rot_period : 0u;
            apply_phase<T, E, false>(v, a.rot + (size_t)ci * P::N, t);
          }
          if (a.mask_c) {
            // energy cut-off, ekk .* (kk < ecut) (SGPEtask/solve_split.m:40-42)
            R kab = R(0);
            if (valid) {
              kab = __ldg(a.mask_a + b % a.mask_pa);
              if (a.mask_b) kab += __ldg(a.mask_b + b / a.mask_pa);
            }
#pragma unroll
            for (int m = 0; m < E; ++m)
              if (!(kab + __ldg(a.mask_c + m * T + t) < a.ecut)) v[m] = mk<R>(R(0), R(0));
          }
        }
        if (!a.skip_inv) St::template inverse<SMT>(v, sm, pol, t, tws);
        if (rep >= a.fold) break;
        load_side();
        rt_full_phase<R, E>(v, sv, a, scal[1]);
      }
    } else {
      St::template forward<SMT>(v, sm, pol, t, tws);
      apply_phase<T, E, SMT>(v, php, t);
      St::template inverse<SMT>(v, sm, pol, t, tws);
    }
    Kahan<R> acc[3];
    if (a.epi != EPI_NONE) {
      load_side();
      epilogue<R, E>(v, sv, a, acc, valid, scal[1]);
    }
    if (valid) {
      cx<R>* __restrict__ dst = a.psi + first;
#pragma unroll
      for (int m = 0; m < E; ++m) dst[m * dm] = v[m];
    }
    const int nred = a.epi == EPI_RT_END ? 3 : a.epi == EPI_ITP ? 1 : 0;
    if (nred > 0) {
      const int slots[4] = {S_N, S_VN, S_N2, 0};
      if (bounds_ok(a.sc, BS_PARTIAL, tile, a.cap)) cta_reduce_store<L::THREADS>(acc, slots, nred, a.partials, a.cap, tile);
    }
  }
}

// KIND is a template parameter so the step and energy variants are separate
// kernels, each with only its own live ranges and code.
template <typename R, class P, class L, int KIND>
__global__ void __launch_bounds__(L::THREADS, MinBlocks<R, P, L>::value) pass_kernel(const PassArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // Programmatic dependent launch: the next kernel in the stream may be
  // scheduled as soon as every CTA of this one has started.  A CTA of the
  // first wave, started early that way, hints its own tile into L2 while the
  // previous kernel drains (L2 is the point of coherence, so the hint cannot
  // hold stale data), then waits for that kernel's completion and memory
  // before it reads anything.  Without the launch attribute both are no-ops.
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (a.pdl && a.pf_ahead > 0 && (long long)blockIdx.x < a.pf_ahead) {
    const long long b0 = (long long)blockIdx.x * L::FFTS;
    if (b0 < a.n_batch) L::prefetch(a, b0, a.n_batch - b0 < L::FFTS ? a.n_batch - b0 : (long long)L::FFTS);
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // The pending scale and mu, converted to R once per CTA (the FP64 pipe of
  // this GPU is narrow: per-thread conversions showed up in the pass time).
  __shared__ R scal[2];
  if (threadIdx.x == 0) {
    scal[0] = (R)a.sc->scale;
    scal[1] = (R)a.sc->mu;
  }
  // An earlier finalizer (or a timed-out pass) ended the run; the block-wide
  // vote keeps the decision uniform within the CTA (and publishes scal).
  if (__syncthreads_or(a.sc->stop != 0)) return;
  pass_body<R, P, L, KIND>(a, (long long)blockIdx.x, smem_raw, scal[0], scal[1]);
}

// Host-side launch description of a pass for one axis length.
struct PassGeom {
  int threads;
  int ffts;
  size_t smem;
};

// V: plan variant (plans.cuh PlanSel): 0 = Plan<N>, 1 = PlanAlt<N>.
template <typename R, int N, int V = 0>
PassGeom pass_geom(bool strided);

template <int N, int V = 0>
PlanInfo plan_info();

template <typename R, int N>
cudaError_t launch_pass_tma(const PassArgs<R>& a, bool strided, cudaStream_t s, int sms, int* grid_out);
template <typename R, int N>
int pass_tma_grid(const PassArgs<R>& a, bool strided, int sms);
template <typename R, int N>
int pass_tma_ffts(bool strided);
template <typename R, int N>
size_t pass_tma_smem(bool strided);

template <typename R, int N, int V = 0>
cudaError_t launch_pass(const PassArgs<R>& a, bool strided, cudaStream_t s);

}  // namespace gpe

// pass_tma.cuh - persistent, TMA-staged variant of the axis pass.
//
// Each CTA walks a strided sequence of pencil tiles.  The tile (FFTS pencils
// of the state, plus the matching values of V or of the ITP factor array
// when the pass needs them) is fetched into shared memory by bulk
// asynchronous copies (cp.async.bulk, tracked by an mbarrier) one tile ahead,
// so the HBM transfer of tile k+1 overlaps the FFTs of tile k without
// holding registers.  The staging buffer of the current tile then serves as
// the FFT exchange buffer; results go back to HBM with coalesced stores.
//
// Tile geometry (no transposes in HBM):
//  * contiguous axis (y): FFTS whole pencils = one contiguous range, one
//    bulk copy; staged as [pencil][position];
//  * strided axes (x, z): FFTS adjacent pencils = N rows of FFTS contiguous
//    elements (128 bytes for FP32 and FP64), one bulk copy per row; staged as
//    [position][pencil], the strided pass's conflict-free exchange layout.
#pragma once
#include "pass.cuh"
#include "tma.cuh"

namespace gpe {

template <class P, typename R>
struct TContig {
  static constexpr bool CONTIG = true;
  static constexpr int T = P::T, N = P::N;
  static constexpr int FFTS = (T >= 128) ? 1 : 128 / T;
  static constexpr int THREADS = FFTS * T;
  static constexpr int REG0 = padpos<P::PADSH>(N - 1) + 1;
  static constexpr int REG = (REG0 % 2 == 0) ? REG0 + 1 : REG0;
  static constexpr int PSI_ELEMS = (FFTS * REG > FFTS * N) ? FFTS * REG : FFTS * N;
  static __device__ __forceinline__ void map(int tid, int& f, int& t) {
    f = tid / T;
    t = tid % T;
  }
  static __device__ __forceinline__ int stage_idx(int f, int p) { return f * N + p; }
  struct Pol {
    int off;
    __device__ __forceinline__ int idx(int p) const { return off + padpos<P::PADSH>(p); }
    __device__ __forceinline__ void sync() const {
      if constexpr (T <= 32) __syncwarp();
      else __syncthreads();
    }
    GPE_POL_CHECK_MEMBERS
  };
  static __device__ __forceinline__ Pol pol(int f) { return Pol{f * REG}; }
};

template <class P, typename R>
struct TStrided {
  static constexpr bool CONTIG = false;
  static constexpr int T = P::T, N = P::N;
  static constexpr int G = 128 / (int)sizeof(cx<R>);  // 128-byte rows
  static constexpr int FFTS = (G * T > 1024) ? 1024 / T : G;
  static constexpr int THREADS = FFTS * T;
  static constexpr int PSI_ELEMS = FFTS * N;
  static __device__ __forceinline__ void map(int tid, int& f, int& t) {
    f = tid % FFTS;
    t = tid / FFTS;
  }
  static __device__ __forceinline__ int stage_idx(int f, int p) { return p * FFTS + f; }
  struct Pol {
    int f;
    __device__ __forceinline__ int idx(int p) const { return p * FFTS + f; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    GPE_POL_CHECK_MEMBERS
  };
  static __device__ __forceinline__ Pol pol(int f) { return Pol{f}; }
};

// Shared-memory plan of a TMA pass: two psi buffers, two side buffers (if
// the pass reads V or the ITP factors), two mbarriers.
template <class L, typename R>
struct TmaSmem {
  static constexpr size_t PSI_BYTES = ((size_t)L::PSI_ELEMS * sizeof(cx<R>) + 127) / 128 * 128;
  static constexpr size_t SIDE_BYTES = ((size_t)L::FFTS * L::N * sizeof(R) + 127) / 128 * 128;
  static constexpr size_t bytes(bool side) { return 2 * PSI_BYTES + (side ? 2 * SIDE_BYTES : 0) + 16; }
};

#ifndef GPE_TMA_THREADS_PER_SM
#define GPE_TMA_THREADS_PER_SM 512
#endif
template <typename R, class L>
struct TmaMinBlocks {
  static constexpr int value = (sizeof(R) == 4 && L::THREADS <= 256) ? GPE_TMA_THREADS_PER_SM / L::THREADS : 1;
};

// Coordinates (y, x, z, component) of element offset e of the state tensor.
__device__ __forceinline__ void tensor_coords(const long long* d, long long e, int* c) {
  const long long plane = d[0] * d[1], vol = plane * d[2];
  c[0] = (int)(e % d[0]);
  c[1] = (int)((e / d[0]) % d[1]);
  c[2] = (int)((e / plane) % d[2]);
  c[3] = (int)(e / vol);
}

template <typename R, class P, class L, int KIND>
__global__ void __launch_bounds__(L::THREADS, TmaMinBlocks<R, L>::value)
    pass_tma_kernel(const PassArgs<R> a, const __grid_constant__ CUtensorMap tm_psi,
                    const __grid_constant__ CUtensorMap tm_side) {
  extern __shared__ __align__(128) unsigned char smem[];
  // Another CTA may set stop on a timeout while this one starts: the
  // block-wide vote keeps the early exit uniform within the CTA.
  if (__syncthreads_or(a.sc->stop != 0)) return;

  constexpr int T = P::T, E = P::E, N = P::N, FFTS = L::FFTS;
  using St = typename P::template St<R>;
  using SM = TmaSmem<L, R>;
  const bool side = a.side != 0;
  const R* __restrict__ side_src = a.side == 2 ? a.aux : a.V;
  cx<R>* psib[2] = {reinterpret_cast<cx<R>*>(smem), reinterpret_cast<cx<R>*>(smem + SM::PSI_BYTES)};
  R* sideb[2] = {reinterpret_cast<R*>(smem + 2 * SM::PSI_BYTES),
                 reinterpret_cast<R*>(smem + 2 * SM::PSI_BYTES + SM::SIDE_BYTES)};
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * SM::PSI_BYTES + (side ? 2 * SM::SIDE_BYTES : 0));

  const long long ntiles = (a.n_batch + FFTS - 1) / FFTS;
  int f, t;
  L::map(threadIdx.x, f, t);

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // pend[s]: a copy into slot s is in flight (set by every thread alike).
  // With the test knob a.tma_stall the barrier is armed for bytes that are
  // never issued, so nothing is ever in flight and the wait runs out.
  bool pend[2] = {false, false};
  const int polls = a.tma_stall > 0 ? a.tma_stall : (1 << 22);
  auto issue = [&](long long tile, int slot) {
    const long long b0 = tile * FFTS;
    if (a.tma_stall > 0) {
      if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar[slot], 16u);
      return;
    }
    pend[slot] = true;
    if constexpr (L::CONTIG) {
      if (threadIdx.x == 0) {
        const long long np = (a.n_batch - b0 < FFTS) ? a.n_batch - b0 : FFTS;
        const uint32_t pb = (uint32_t)(np * N * sizeof(cx<R>));
        const uint32_t sb = side ? (uint32_t)(np * N * sizeof(R)) : 0u;
        mbar_arrive_expect_tx(&bar[slot], pb + sb);
        tma_load_1d(psib[slot], a.psi + b0 * N, pb, &bar[slot]);
        if (side) tma_load_1d(sideb[slot], side_src + b0 * N, sb, &bar[slot]);
      }
    } else if (a.tma_tensor) {
      // one box per tile (two for N = 512: a box spans at most 256
      // elements per dimension), landing as [position][pencil]
      if (threadIdx.x == 0) {
        const long long base = (b0 % a.inner) + (b0 / a.inner) * a.outer;
        int cc[4];
        tensor_coords(a.tdim, base, cc);
        const int ax = a.stride == a.tdim[0] ? 1 : 2;  // x pencils step by ny, z pencils by nx*ny
        constexpr int NB = N > 256 ? 2 : 1, BOX = N / NB;
        mbar_arrive_expect_tx(&bar[slot], (uint32_t)(N * FFTS * (sizeof(cx<R>) + (side ? sizeof(R) : 0))));
#pragma unroll
        for (int h = 0; h < NB; ++h) {
          int q[4] = {cc[0], cc[1], cc[2], cc[3]};
          q[ax] += h * BOX;
          // the maps count real units: a complex element is two of them
          tma_load_4d(psib[slot] + h * BOX * FFTS, &tm_psi, 2 * q[0], q[1], q[2], q[3], &bar[slot]);
          if (side) tma_load_4d(sideb[slot] + h * BOX * FFTS, &tm_side, q[0], q[1], q[2], q[3], &bar[slot]);
        }
      }
    } else {
      const long long base = (b0 % a.inner) + (b0 / a.inner) * a.outer;
      if (threadIdx.x == 0)
        mbar_arrive_expect_tx(&bar[slot], (uint32_t)(N * FFTS * (sizeof(cx<R>) + (side ? sizeof(R) : 0))));
      for (int p = threadIdx.x; p < N; p += L::THREADS) {
        tma_load_1d(psib[slot] + p * FFTS, a.psi + base + p * a.stride, FFTS * sizeof(cx<R>), &bar[slot]);
        if (side)
          tma_load_1d(sideb[slot] + p * FFTS, side_src + base + p * a.stride, FFTS * sizeof(R), &bar[slot]);
      }
    }
  };

  Kahan<R> acc[4];
  long long tile = blockIdx.x;
  if (tile < ntiles) issue(tile, 0);
  for (int k = 0; tile < ntiles; tile += gridDim.x, ++k) {
    const int slot = k & 1;
    const long long next = tile + gridDim.x;
    if (next < ntiles) issue(next, slot ^ 1);
    const bool ok = mbar_wait(&bar[slot], (uint32_t)((k >> 1) & 1), polls);
    if (!__syncthreads_and(ok)) {
      // A copy did not land in time: flag it, give every copy still in
      // flight (this slot's and the next tile's) a bounded chance to finish
      // so the CTA does not exit under them, and stop.
      if (threadIdx.x == 0) {
        atomicExch(&a.sc->timeout, 1);
        atomicExch(&a.sc->stop, 1);
      }
      if (pend[slot]) mbar_wait(&bar[slot], (uint32_t)((k >> 1) & 1));
      if (pend[slot ^ 1]) mbar_wait(&bar[slot ^ 1], (uint32_t)(((k + 1) >> 1) & 1));
      return;
    }
    pend[slot] = false;

    const long long b = tile * FFTS + f;
    const bool valid = b < a.n_batch;
    long long first = 0, dm = 0;
    if constexpr (L::CONTIG) {
      first = (valid ? b * N : 0) + t;
      dm = T;
    } else {
      first = (valid ? (b % a.inner) + (b / a.inner) * a.outer : 0) + (long long)t * a.stride;
      dm = (long long)T * a.stride;
    }
    cx<R> v[E];
    R sv[E];
    {
      const cx<R>* stg = psib[slot];
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = stg[L::stage_idx(f, t + T * m)];
    }
    // Side values come from their own staging buffer, which the exchanges do
    // not touch, so they are read right before the phase that needs them.
    auto load_side = [&]() {
      const R* ss = sideb[slot];
#pragma unroll
      for (int m = 0; m < E; ++m) sv[m] = ss[L::stage_idx(f, t + T * m)];
    };
    __syncthreads();  // staging reads done before the exchanges reuse the buffer

    auto pol = L::pol(f);
    GPE_POL_BOUNDS(pol, a.sc, L::PSI_ELEMS);
    cx<R>* xb = psib[slot];
    if constexpr (KIND == KIND_ENERGY) {
      const R s = a.pro == PRO_SCALE ? (R)a.sc->scale : R(1);
      if (a.energy_pot) load_side();
#pragma unroll
      for (int m = 0; m < E; ++m) {
        v[m] = rmul(v[m], s);
        if (a.energy_pot && valid) {
          const R n = norm2(v[m]);
          acc[0].add(n);
          acc[1].add(sv[m] * n);
          acc[2].add(n * n);
        }
      }
      St::template forward<false>(v, xb, pol, t, a.tws);
      if (valid) {
#pragma unroll
        for (int m = 0; m < E; ++m) acc[3].add(__ldg(a.k2p + m * T + t) * norm2(v[m]));
      }
    } else {
      if (a.pro != PRO_NONE) {
        if (side) load_side();
        prologue<R, E>(v, sv, a, valid, first, dm, (R)a.sc->scale, (R)a.sc->mu);
      }
      St::template forward<false>(v, xb, pol, t, a.tws);
      apply_phase<T, E>(v, a.php, t);
      St::template inverse<false>(v, xb, pol, t, a.tws);
      if (a.epi != EPI_NONE) {
        load_side();
        epilogue<R, E>(v, sv, a, acc, valid, (R)a.sc->mu);
      }
      if (valid && bounds_ok(a.sc, BS_STORE, first + (E - 1) * dm, a.npts)) {
        cx<R>* __restrict__ dst = a.psi + first;
#pragma unroll
        for (int m = 0; m < E; ++m) dst[m * dm] = v[m];
      }
    }
    fence_proxy_async_smem();
    __syncthreads();  // the buffer is free for the copy issued next iteration
  }

  if constexpr (KIND == KIND_ENERGY) {
    double vals[4];
    int slots[4];
    int n = 0;
    if (a.energy_pot) {
      vals[0] = acc[0].value();
      vals[1] = acc[1].value();
      vals[2] = acc[2].value();
      slots[0] = S_N; slots[1] = S_VN; slots[2] = S_N2;
      n = 3;
    }
    vals[n] = acc[3].value();
    slots[n] = a.kin_slot;
    cta_reduce_store<L::THREADS>(vals, slots, n + 1, a.partials, a.cap);
  } else {
    const int nr = a.epi == EPI_RT_END ? 3 : a.epi == EPI_ITP ? 1 : 0;
    if (nr > 0) {
      double vals[4] = {acc[0].value(), acc[1].value(), acc[2].value(), 0.0};
      const int slots[4] = {S_N, S_VN, S_N2, 0};
      cta_reduce_store<L::THREADS>(vals, slots, nr, a.partials, a.cap);
    }
  }
}

}  // namespace gpe

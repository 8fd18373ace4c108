// plans.cuh - FFT plans per axis length.
//
// A plan fixes the threads per pencil T, the points per thread E = N/T, the
// radix of every Stockham stage (each radix divides E) and the padding of the
// shared-memory exchange buffer of the contiguous-axis pass (PADSH: position p
// lives at p + (p >> PADSH); -1 = no padding).  The padding was chosen by
// counting shared-memory wavefronts of each exchange pattern.
#pragma once
#include "fft.cuh"

namespace gpe {

template <int N_, int T_, int PADSH_, int... RADS>
struct PlanT {
  static constexpr int N = N_;
  static constexpr int T = T_;
  static constexpr int E = N_ / T_;
  static constexpr int PADSH = PADSH_;
  static constexpr int NSTAGES = sizeof...(RADS);
  static constexpr int radix[sizeof...(RADS)] = {RADS...};
  template <typename R>
  using St = Stages<R, N_, T_, 1, 0, RADS...>;
  static constexpr int prod() { return (RADS * ...); }
  // Complex entries of the stage twiddle rows (the layout the host builds:
  // stage s >= 1 takes even(Ns * R_s) entries), at least 2.
  static constexpr int tw_len() {
    const int r[] = {RADS...};
    int off = 0, Ns = r[0];
    for (int s = 1; s < (int)sizeof...(RADS); ++s) {
      off += (Ns * r[s] + 1) & ~1;
      Ns *= r[s];
    }
    return off < 2 ? 2 : off;
  }
  static constexpr int TW_LEN = tw_len();
  static_assert(prod() == N_, "radices must multiply to N");
  static_assert((((N_ / T_) % RADS == 0) && ...), "every radix must divide E");
};

template <int N>
struct Plan;  // only the lengths below are supported

template <> struct Plan<8>    : PlanT<8, 1, -1, 8> {};
template <> struct Plan<12>   : PlanT<12, 1, -1, 4, 3> {};
template <> struct Plan<16>   : PlanT<16, 1, -1, 16> {};
template <> struct Plan<24>   : PlanT<24, 2, 4, 4, 6> {};
template <> struct Plan<32>   : PlanT<32, 2, 4, 16, 2> {};
template <> struct Plan<48>   : PlanT<48, 4, 4, 4, 4, 3> {};
template <> struct Plan<64>   : PlanT<64, 4, 4, 16, 4> {};
template <> struct Plan<96>   : PlanT<96, 4, 4, 8, 4, 3> {};
template <> struct Plan<128>  : PlanT<128, 8, 4, 16, 8> {};
template <> struct Plan<192>  : PlanT<192, 8, 4, 8, 8, 3> {};
template <> struct Plan<256>  : PlanT<256, 16, 4, 16, 16> {};
template <> struct Plan<384>  : PlanT<384, 16, 4, 8, 8, 6> {};
template <> struct Plan<512>  : PlanT<512, 32, 4, 16, 16, 2> {};
template <> struct Plan<768>  : PlanT<768, 32, 4, 8, 8, 6, 2> {};
template <> struct Plan<1024> : PlanT<1024, 64, 4, 16, 16, 4> {};

// Alternative plans: twice the threads per pencil, half the points per thread
// (fewer registers, more resident warps; one more shared-memory exchange).
// The autotuner times both plans of an axis pass and keeps the faster one
// (FP32 passes; FP64 passes use Plan<N>).
template <int N>
struct PlanAlt;
template <> struct PlanAlt<128> : PlanT<128, 16, 4, 8, 4, 4> {};
template <> struct PlanAlt<192> : PlanT<192, 16, 4, 4, 4, 4, 3> {};
template <> struct PlanAlt<256> : PlanT<256, 32, 4, 8, 8, 4> {};
template <> struct PlanAlt<384> : PlanT<384, 32, 4, 4, 4, 4, 6> {};
template <> struct PlanAlt<512> : PlanT<512, 64, 4, 8, 8, 8> {};

// Plan variant V of length N: 0 = Plan<N>, 1 = PlanAlt<N>.
template <int N, int V>
struct PlanSel {
  using type = Plan<N>;
};
template <int N>
struct PlanSel<N, 1> {
  using type = PlanAlt<N>;
};

// The axis lengths with an alternative plan.
#define GPE_FOR_EACH_ALT(X) X(128) X(192) X(256) X(384) X(512)

// Host-side description of a plan: the tables the pass kernels read are
// built from it (stage twiddle rows, per-thread permuted kinetic factors).
struct PlanInfo {
  int N, T, E, nstages;
  int radix[8];
};

// Twiddle rows of stage s (s >= 1, Ns = R_0*...*R_{s-1}) start at
// sum over earlier stages s' >= 1 of even(Ns' * R_s'); row k holds
// exp(-2 pi i r k/(Ns R_s)) for r = 0..R_s-1.
inline int stage_rows_offset(const PlanInfo& p, int s) {
  int off = 0, Ns = p.radix[0];
  for (int q = 1; q < s; ++q) {
    off += (Ns * p.radix[q] + 1) & ~1;
    Ns *= p.radix[q];
  }
  return off;
}

// Natural-order spectrum position that register slot m of thread t holds
// after the forward transform (the last stage's scatter position).
inline int plan_spec_pos(const PlanInfo& p, int t, int m) {
  const int Rl = p.radix[p.nstages - 1];
  const int Ns = p.N / Rl;
  const int NB = p.E / Rl;
  const int b = m % NB, r = m / NB;
  const int j = t + p.T * b;
  return (j / Ns) * Ns * Rl + (j % Ns) + r * Ns;
}

// The axis lengths with a plan (host-side check before any launch).
#define GPE_FOR_EACH_N(X) \
  X(8) X(12) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024)

}  // namespace gpe

// fft.cuh - register/shared-memory Stockham FFT engine for one pencil.
//
// T threads cooperate on one pencil of N = T*E points; thread t holds the E
// points at positions t + T*m (m = 0..E-1), the "own" layout, which is also
// the layout pencils are loaded and stored in.
//
// Forward transform: Stockham autosort stages with radices R_0..R_{S-1}
// (Ns = R_0*...*R_{s-1}).  Stage s reads a[j + r*N/R] (own layout, j = t + T*b),
// multiplies by w^(r*(j mod Ns)), w = exp(-2 pi i/(Ns R)), applies a radix-R DFT
// and writes position (j/Ns)*Ns*R + (j mod Ns) + r*Ns.  Between stages the
// scattered outputs go through shared memory back to the own layout.  After
// the last stage each thread holds natural-order spectrum values at the
// positions it wrote, so the kinetic factor is applied in registers.
//
// Inverse transform: the adjoint network (stages in reverse, conjugate DFT,
// conjugate twiddles after the butterfly).  Its first stage reads exactly the
// positions the last forward stage left in registers, so forward + inverse
// cost 2*(S-1) shared-memory exchanges and no extra one in between.  The 1/N
// of MATLAB's ifft is folded into the kinetic factor table.
#pragma once
#include "common.cuh"

namespace gpe {

// ---- radix-R DFT butterflies, in place on u[0..R-1] --------------------
// DIR = -1: forward (exp(-2 pi i/R)), DIR = +1: inverse without 1/R.
template <typename R, int DIR>
__device__ __forceinline__ cx<R> mul_mi(cx<R> a) {  // a * (DIR * i)
  return DIR < 0 ? mk<R>(a.y, -a.x) : mk<R>(-a.y, a.x);
}

template <typename R, int DIR>
__device__ __forceinline__ void dft2(cx<R>& a, cx<R>& b) {
  cx<R> t = a;
  a = t + b;
  b = t - b;
}

template <typename R, int DIR>
__device__ __forceinline__ void dft4(cx<R>& a0, cx<R>& a1, cx<R>& a2, cx<R>& a3) {
  cx<R> t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = mul_mi<R, DIR>(a1 - a3);
  a0 = t0 + t2;
  a2 = t0 - t2;
  a1 = t1 + t3;
  a3 = t1 - t3;
}

// Irrational butterfly constants.  FP64 uses the correctly rounded values.
// FP32 cannot hold these unit complex numbers with |z| = 1 exactly: the
// nearest floats of (cos pi/8, sin pi/8), (1, 1)/sqrt(2) and (-1/2, sqrt(3)/2)
// all lie inside the unit circle (|z|^2 - 1 = -3e-8 .. -6e-8), which shrank
// the norm of every FP32 pass by a fixed ~1e-7.  Each FP32 constant is
// instead a neighbour within one ulp (angle error < 2e-8 rad) picked so that
// the modulus errors of the constant multiplications inside one butterfly
// (and one forward + inverse pair) cancel to first order.
template <typename R>
struct BK;
template <>
struct BK<double> {
  static constexpr double c16 = 0.92387953251128675613, s16 = 0.38268343236508977173;
  static constexpr double c2 = 0.70710678118654752440, c2b = 0.70710678118654752440;
  static constexpr double h3 = 0.86602540378443864676, h3b = 0.86602540378443864676;
};
template <>
struct BK<float> {
  // |(c16, s16)|^2 - 1 = +5.3e-8 offsets the four 1/sqrt(2) products of a
  // radix-16 butterfly (2 c2^2 - 1 = -3.4e-8 each).
  static constexpr float c16 = 0.9238795638084412f, s16 = 0.3826834261417389f;
  static constexpr float c2 = 0.7071067690849304f;   // 2 c^2 - 1 = -3.4e-8
  static constexpr float c2b = 0.7071068286895752f;  // 2 c^2 - 1 = +1.3e-7, one use in four
  static constexpr float h3 = 0.8660253882408142f;   // 1/4 + h^2 - 1 = -2.7e-8
  static constexpr float h3b = 0.866025447845459f;   // 1/4 + h^2 - 1 = +7.6e-8, one use in four
};
template <>
struct BK<fx2> : BK<float> {};  // paired lanes: the FP32 constants, broadcast

// a * (SC*C + i*SS*S) for constants C, S and signs SC, SS in {+1, -1}.
template <typename R, int SC, int SS>
__device__ __forceinline__ cx<R> rotk(cx<R> a, R C, R S) {
  const R cc = SC > 0 ? C : -C, ss = SS > 0 ? S : -S;
  return mk<R>(a.x * cc - a.y * ss, a.x * ss + a.y * cc);
}

template <typename R, int DIR>
__device__ __forceinline__ void dft3(cx<R>& a0, cx<R>& a1, cx<R>& a2) {
  cx<R> t = a1 + a2;
  cx<R> d = a1 - a2;
  cx<R> m = mk<R>(a0.x - R(0.5) * t.x, a0.y - R(0.5) * t.y);
  const R hx = d.x * BK<R>::h3, hy = d.y * BK<R>::h3;  // sin(2 pi/3) * d
  // forward: X1 = m - i h d, X2 = m + i h d
  cx<R> s = DIR < 0 ? mk<R>(hy, -hx) : mk<R>(-hy, hx);
  a0 = a0 + t;
  a1 = m + s;
  a2 = m - s;
}

// a * exp(DIR*2 pi i q/8), q in 0..3; ALT selects the second 1/sqrt(2).
template <typename R, int DIR, bool ALT = false>
__device__ __forceinline__ cx<R> w8(cx<R> a, int q) {
  const R c = ALT ? BK<R>::c2b : BK<R>::c2;
  if (q == 0) return a;
  if (q == 2) return mul_mi<R, DIR>(a);
  if (q == 1) {  // (c, DIR*c)
    return DIR < 0 ? mk<R>((a.x + a.y) * c, (a.y - a.x) * c) : mk<R>((a.x - a.y) * c, (a.x + a.y) * c);
  }
  // q == 3: (-c, DIR*c)
  return DIR < 0 ? mk<R>((a.y - a.x) * c, -((a.x + a.y) * c)) : mk<R>(-((a.x + a.y) * c), (a.x - a.y) * c);
}

template <typename R, int DIR>
__device__ __forceinline__ void dft8(cx<R>* u) {
  cx<R> e0 = u[0], e1 = u[2], e2 = u[4], e3 = u[6];
  cx<R> o0 = u[1], o1 = u[3], o2 = u[5], o3 = u[7];
  dft4<R, DIR>(e0, e1, e2, e3);
  dft4<R, DIR>(o0, o1, o2, o3);
  o1 = w8<R, DIR>(o1, 1);
  o2 = w8<R, DIR>(o2, 2);
  o3 = w8<R, DIR, (DIR > 0)>(o3, 3);  // forward + inverse: three c2, one c2b
  u[0] = e0 + o0; u[4] = e0 - o0;
  u[1] = e1 + o1; u[5] = e1 - o1;
  u[2] = e2 + o2; u[6] = e2 - o2;
  u[3] = e3 + o3; u[7] = e3 - o3;
}

template <typename R, int DIR>
__device__ __forceinline__ cx<R> w16(cx<R> a, int q) {  // a * exp(DIR*2 pi i q/16), q = n2*k1 < 10
  constexpr int D = DIR < 0 ? -1 : 1;
  switch (q) {
    case 0: return a;
    case 1: return rotk<R, 1, D>(a, BK<R>::c16, BK<R>::s16);    // ( cos pi/8,  D sin pi/8)
    case 2: return w8<R, DIR>(a, 1);                            // ( c2,  D c2)
    case 3: return rotk<R, 1, D>(a, BK<R>::s16, BK<R>::c16);    // ( sin pi/8,  D cos pi/8)
    case 4: return mul_mi<R, DIR>(a);
    case 6: return w8<R, DIR>(a, 3);                            // (-c2,  D c2)
    case 9: return rotk<R, -1, -D>(a, BK<R>::c16, BK<R>::s16);  // (-cos pi/8, -D sin pi/8)
    default: return a;  // q = 5, 7, 8 never occur (q = n2*k1, n2,k1 < 4)
  }
}

template <typename R, int DIR>
__device__ __forceinline__ void dft16(cx<R>* u) {
  // 16 = 4 x 4: inner DFT4 over n1 (stride 4), twiddle W16^(n2 k1), outer DFT4 over n2.
  cx<R> b[16];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    cx<R> a0 = u[n2], a1 = u[n2 + 4], a2 = u[n2 + 8], a3 = u[n2 + 12];
    dft4<R, DIR>(a0, a1, a2, a3);
    b[n2 * 4 + 0] = a0;
    b[n2 * 4 + 1] = w16<R, DIR>(a1, n2 * 1);
    b[n2 * 4 + 2] = w16<R, DIR>(a2, n2 * 2);
    b[n2 * 4 + 3] = w16<R, DIR>(a3, n2 * 3);
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cx<R> a0 = b[0 * 4 + k1], a1 = b[1 * 4 + k1], a2 = b[2 * 4 + k1], a3 = b[3 * 4 + k1];
    dft4<R, DIR>(a0, a1, a2, a3);
    u[k1] = a0;
    u[k1 + 4] = a1;
    u[k1 + 8] = a2;
    u[k1 + 12] = a3;
  }
}

template <typename R, int DIR>
__device__ __forceinline__ void dft6(cx<R>* u) {
  // 6 = 2 x 3: DFT3 of even and odd samples, twiddle W6^k, radix-2 combine.
  cx<R> e0 = u[0], e1 = u[2], e2 = u[4];
  cx<R> o0 = u[1], o1 = u[3], o2 = u[5];
  dft3<R, DIR>(e0, e1, e2);
  dft3<R, DIR>(o0, o1, o2);
  // W6^1 = (1/2, DIR*h), W6^2 = (-1/2, DIR*h), h = sin(2 pi/3); with the two
  // DFT3s: three uses of h3, one of h3b.
  const R h1x = o1.x * BK<R>::h3b, h1y = o1.y * BK<R>::h3b;
  const R h2x = o2.x * BK<R>::h3, h2y = o2.y * BK<R>::h3;
  o1 = DIR < 0 ? mk<R>(R(0.5) * o1.x + h1y, R(0.5) * o1.y - h1x) : mk<R>(R(0.5) * o1.x - h1y, R(0.5) * o1.y + h1x);
  o2 = DIR < 0 ? mk<R>(-R(0.5) * o2.x + h2y, -R(0.5) * o2.y - h2x)
               : mk<R>(-R(0.5) * o2.x - h2y, -R(0.5) * o2.y + h2x);
  u[0] = e0 + o0; u[3] = e0 - o0;
  u[1] = e1 + o1; u[4] = e1 - o1;
  u[2] = e2 + o2; u[5] = e2 - o2;
}

template <typename R, int RAD, int DIR>
__device__ __forceinline__ void dft(cx<R>* u) {
  if constexpr (RAD == 2) dft2<R, DIR>(u[0], u[1]);
  else if constexpr (RAD == 3) dft3<R, DIR>(u[0], u[1], u[2]);
  else if constexpr (RAD == 4) dft4<R, DIR>(u[0], u[1], u[2], u[3]);
  else if constexpr (RAD == 6) dft6<R, DIR>(u);
  else if constexpr (RAD == 8) dft8<R, DIR>(u);
  else if constexpr (RAD == 16) dft16<R, DIR>(u);
  else static_assert(RAD == 2, "unsupported radix");
}

// ---- Stockham stages ----------------------------------------------------
// Smem policy SM provides: idx(p) -> shared-memory element index of position
// p of this thread's pencil, and sync().
template <int Ns, int RAD>
__device__ __forceinline__ int scatter_pos(int j, int r) {
  return (j / Ns) * Ns * RAD + (j % Ns) + r * Ns;
}

// u[r] *= w_r (DIR < 0) or u[r] *= conj(w_r) (DIR > 0), r = 1..RAD-1, where
// w_r = exp(-2 pi i r k/(Ns RAD)) comes from the stage's twiddle rows.  The
// rows are stored k-fastest so that adjacent lanes (adjacent k) read adjacent
// addresses: FP32 stages of even radix as [r/2][k] pairs of entries (one
// 16-byte vector load gives w_{2i}, w_{2i+1}), otherwise as [r][k] entries.
// SMT: the rows are in shared memory (plain loads), else in global memory.
template <int Ns, int RAD, int DIR, bool SMT>
__device__ __forceinline__ void apply_row(cx<float>* u, const cx<float>* __restrict__ rows, int k) {
  if constexpr (RAD % 2 == 0) {
    const float4* r4 = reinterpret_cast<const float4*>(rows) + k;
#pragma unroll
    for (int i = 0; i < RAD / 2; ++i) {
      const float4 q = ld_tab<SMT>(r4 + i * Ns);
      if (i > 0) u[2 * i] = DIR < 0 ? cmul(u[2 * i], mk<float>(q.x, q.y)) : cmulc(u[2 * i], mk<float>(q.x, q.y));
      u[2 * i + 1] = DIR < 0 ? cmul(u[2 * i + 1], mk<float>(q.z, q.w)) : cmulc(u[2 * i + 1], mk<float>(q.z, q.w));
    }
  } else {
#pragma unroll
    for (int r = 1; r < RAD; ++r) {
      const cx<float> w = ld_tab<SMT>(rows + r * Ns + k);
      u[r] = DIR < 0 ? cmul(u[r], w) : cmulc(u[r], w);
    }
  }
}
// Paired lanes: the FP32 rows, each entry broadcast to both pencils.
template <int Ns, int RAD, int DIR, bool SMT>
__device__ __forceinline__ void apply_row(cx<fx2>* u, const cx<float>* __restrict__ rows, int k) {
  if constexpr (RAD % 2 == 0) {
    const float4* r4 = reinterpret_cast<const float4*>(rows) + k;
#pragma unroll
    for (int i = 0; i < RAD / 2; ++i) {
      const float4 q = ld_tab<SMT>(r4 + i * Ns);
      const cx<fx2> w0 = mk<fx2>(fx2(q.x), fx2(q.y)), w1 = mk<fx2>(fx2(q.z), fx2(q.w));
      if (i > 0) u[2 * i] = DIR < 0 ? cmul(u[2 * i], w0) : cmulc(u[2 * i], w0);
      u[2 * i + 1] = DIR < 0 ? cmul(u[2 * i + 1], w1) : cmulc(u[2 * i + 1], w1);
    }
  } else {
#pragma unroll
    for (int r = 1; r < RAD; ++r) {
      const cx<float> q = ld_tab<SMT>(rows + r * Ns + k);
      const cx<fx2> w = mk<fx2>(fx2(q.x), fx2(q.y));
      u[r] = DIR < 0 ? cmul(u[r], w) : cmulc(u[r], w);
    }
  }
}
template <int Ns, int RAD, int DIR, bool SMT>
__device__ __forceinline__ void apply_row(cx<double>* u, const cx<double>* __restrict__ rows, int k) {
#pragma unroll
  for (int r = 1; r < RAD; ++r) {
    const cx<double> w = ld_tab<SMT>(rows + r * Ns + k);
    u[r] = DIR < 0 ? cmul(u[r], w) : cmulc(u[r], w);
  }
}

template <typename R, int N, int T, int Ns, int RAD, bool SMT>
__device__ __forceinline__ void fwd_stage(cx<R>* v, int t, const cx<Tab<R>>* __restrict__ rows) {
  constexpr int E = N / T;
  constexpr int NB = E / RAD;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    cx<R> u[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) u[r] = v[b + r * NB];
    if constexpr (Ns > 1) apply_row<Ns, RAD, -1, SMT>(u, rows, (t + T * b) % Ns);
    dft<R, RAD, -1>(u);
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[b + r * NB] = u[r];
  }
}

template <typename R, int N, int T, int Ns, int RAD, bool SMT>
__device__ __forceinline__ void inv_stage(cx<R>* v, int t, const cx<Tab<R>>* __restrict__ rows) {
  constexpr int E = N / T;
  constexpr int NB = E / RAD;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    cx<R> u[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) u[r] = v[b + r * NB];
    dft<R, RAD, +1>(u);
    if constexpr (Ns > 1) apply_row<Ns, RAD, +1, SMT>(u, rows, (t + T * b) % Ns);
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[b + r * NB] = u[r];
  }
}

// Scattered outputs of stage (Ns, RAD) -> own layout.
template <typename R, int N, int T, int Ns, int RAD, class SM>
__device__ __forceinline__ void xchg_scatter_to_own(cx<R>* v, cx<R>* sm, const SM& pol, int t) {
  constexpr int E = N / T;
  constexpr int NB = E / RAD;
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int r = 0; r < RAD; ++r) sm[GPE_SMI(pol, pol.idx(scatter_pos<Ns, RAD>(t + T * b, r)))] = v[b + r * NB];
  pol.sync();
#pragma unroll
  for (int m = 0; m < E; ++m) v[m] = sm[GPE_SMI(pol, pol.idx(t + T * m))];
  pol.sync();
}

// Own layout -> the scattered positions stage (Ns, RAD) wrote.
template <typename R, int N, int T, int Ns, int RAD, class SM>
__device__ __forceinline__ void xchg_own_to_scatter(cx<R>* v, cx<R>* sm, const SM& pol, int t) {
  constexpr int E = N / T;
  constexpr int NB = E / RAD;
#pragma unroll
  for (int m = 0; m < E; ++m) sm[GPE_SMI(pol, pol.idx(t + T * m))] = v[m];
  pol.sync();
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[b + r * NB] = sm[GPE_SMI(pol, pol.idx(scatter_pos<Ns, RAD>(t + T * b, r)))];
  pol.sync();
}

// OFF: offset of this stage's twiddle rows (used when Ns > 1).
template <typename R, int N, int T, int Ns, int OFF, int RAD, int... REST>
struct Stages {
  static constexpr int NEXT_OFF = (Ns > 1) ? OFF + ((Ns * RAD + 1) & ~1) : OFF;
  // SMT: tws points to shared memory.
  template <bool SMT, class SM>
  static __device__ __forceinline__ void forward(cx<R>* v, cx<R>* sm, const SM& pol, int t,
                                                 const cx<Tab<R>>* __restrict__ tws) {
    fwd_stage<R, N, T, Ns, RAD, SMT>(v, t, tws + OFF);
    if constexpr (sizeof...(REST) > 0) {
      xchg_scatter_to_own<R, N, T, Ns, RAD>(v, sm, pol, t);
      Stages<R, N, T, Ns * RAD, NEXT_OFF, REST...>::template forward<SMT>(v, sm, pol, t, tws);
    }
  }
  template <bool SMT, class SM>
  static __device__ __forceinline__ void inverse(cx<R>* v, cx<R>* sm, const SM& pol, int t,
                                                 const cx<Tab<R>>* __restrict__ tws) {
    if constexpr (sizeof...(REST) > 0) {
      Stages<R, N, T, Ns * RAD, NEXT_OFF, REST...>::template inverse<SMT>(v, sm, pol, t, tws);
      xchg_own_to_scatter<R, N, T, Ns, RAD>(v, sm, pol, t);
    }
    inv_stage<R, N, T, Ns, RAD, SMT>(v, t, tws + OFF);
  }
};

}  // namespace gpe

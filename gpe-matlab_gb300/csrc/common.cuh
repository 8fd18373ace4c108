// common.cuh - shared types of libgpe's device code.
//
// State arrays hold interleaved complex values in MATLAB column-major order
// (iy + ny*(ix + nx*iz), lib/@grid3d/init.m:75-79 of GPE-MATLAB).  The FFT
// axis passes read and write that layout directly; nothing is transposed in
// HBM.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gpe {

template <typename R>
struct __align__(2 * sizeof(R)) cx {
  R x, y;
};

template <typename R>
__host__ __device__ __forceinline__ cx<R> mk(R a, R b) {
  cx<R> r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename R>
__device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__device__ __forceinline__ cx<R> cmul(cx<R> a, cx<R> b) {
  return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename R>
__device__ __forceinline__ cx<R> cmulc(cx<R> a, cx<R> b) {
  return mk<R>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename R>
__device__ __forceinline__ cx<R> rmul(cx<R> a, R s) { return mk<R>(a.x * s, a.y * s); }
template <typename R>
__device__ __forceinline__ R norm2(cx<R> a) { return a.x * a.x + a.y * a.y; }

// Two FP32 lanes processed by one packed instruction (sm_100+ FADD2, FMUL2,
// FFMA2: two FP32 results per issue slot).  The paired pass kernels hold two
// pencils per thread in structure-of-arrays form, cx<fx2>{re of both, im of
// both}, so every complex operation of the FFT is lane-uniform: one packed
// instruction does the work of two scalar ones.  Broadcast and negated
// operands cost nothing extra (they are operand modifiers of the packed ops).
struct fx2 {
  float2 v;
  fx2() = default;
  __host__ __device__ __forceinline__ fx2(float a) : v{a, a} {}
  __host__ __device__ __forceinline__ fx2(float a, float b) : v{a, b} {}
  __host__ __device__ __forceinline__ explicit fx2(float2 a) : v(a) {}
};
__device__ __forceinline__ fx2 operator+(fx2 a, fx2 b) { return fx2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ fx2 operator-(fx2 a) { return fx2(-a.v.x, -a.v.y); }
__device__ __forceinline__ fx2 operator-(fx2 a, fx2 b) { return fx2(__fadd2_rn(a.v, make_float2(-b.v.x, -b.v.y))); }
__device__ __forceinline__ fx2 operator*(fx2 a, fx2 b) { return fx2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ fx2 fma2(fx2 a, fx2 b, fx2 c) { return fx2(__ffma2_rn(a.v, b.v, c.v)); }

// Element type of the FFT tables a pass of lane type R reads (the paired
// kernels read the FP32 tables and broadcast each entry to both lanes).
template <typename R>
struct TabOf {
  using type = R;
};
template <>
struct TabOf<fx2> {
  using type = float;
};
template <typename R>
using Tab = typename TabOf<R>::type;

// Read-only (non-coherent cache) loads of table entries.
__device__ __forceinline__ cx<float> ldg(const cx<float>* p) {
  float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return mk<float>(v.x, v.y);
}
__device__ __forceinline__ cx<double> ldg(const cx<double>* p) {
  double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return mk<double>(v.x, v.y);
}

// Loads of FFT table entries (twiddle rows, kinetic factors): SMT = the
// tables were copied to shared memory (plain loads), else global memory
// through the read-only data cache.  GPE_SMEM_TABLES=0 disables the copy.
#ifndef GPE_SMEM_TABLES
#define GPE_SMEM_TABLES 1
#endif
template <bool SMT, typename T>
__device__ __forceinline__ T ld_tab(const T* p) {
  if constexpr (SMT) return *p;
  else return __ldg(p);
}
template <bool SMT>
__device__ __forceinline__ cx<float> ld_tab(const cx<float>* p) {
  const float2 v = ld_tab<SMT>(reinterpret_cast<const float2*>(p));
  return mk<float>(v.x, v.y);
}
template <bool SMT>
__device__ __forceinline__ cx<double> ld_tab(const cx<double>* p) {
  const double2 v = ld_tab<SMT>(reinterpret_cast<const double2*>(p));
  return mk<double>(v.x, v.y);
}

// Counter-based random numbers for the stochastic GPE: Philox4x32 with 10
// rounds (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC'11): round = two 32x32->64 multiplies by M0, M1 and xors with
// the key, which is bumped by the Weyl constants W0, W1 between rounds.
struct Philox4 {
  unsigned x, y, z, w;
};
__host__ __device__ inline void mulhilo32(unsigned a, unsigned b, unsigned& hi, unsigned& lo) {
  const unsigned long long p = (unsigned long long)a * b;
  hi = (unsigned)(p >> 32);
  lo = (unsigned)p;
}
__host__ __device__ inline Philox4 philox4x32_10(Philox4 c, unsigned k0, unsigned k1) {
  const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    unsigned hi0, lo0, hi1, lo1;
    mulhilo32(M0, c.x, hi0, lo0);
    mulhilo32(M1, c.z, hi1, lo1);
    c = Philox4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}
// Two standard normal variates for (seed, step, point index) by Box-Muller
// on 24-bit uniforms u1 in (0, 1], u2 in [0, 1) from the first two words.
template <typename R>
__device__ __forceinline__ cx<R> gauss2(unsigned long long seed, unsigned long long step, unsigned long long idx) {
  const Philox4 r = philox4x32_10(Philox4{(unsigned)idx, (unsigned)(idx >> 32), (unsigned)step, (unsigned)(step >> 32)},
                                  (unsigned)seed, (unsigned)(seed >> 32));
  const R u1 = (R)((r.x >> 8) + 1u) * (R)5.9604644775390625e-08;  // 2^-24
  const R u2 = (R)(r.y >> 8) * (R)5.9604644775390625e-08;
  R s, c;
  if constexpr (sizeof(R) == 4) {
    sincospif(2.0f * u2, &s, &c);
    const float rad = sqrtf(-2.0f * logf(u1));
    return mk<float>(rad * c, rad * s);
  } else {
    sincospi(2.0 * u2, &s, &c);
    const double rad = sqrt(-2.0 * log(u1));
    return mk<double>(rad * c, rad * s);
  }
}

// Loads of streamed data (state, potential) that a pass reads once: marked
// evict-first so they do not push the FFT tables out of L1.
#ifndef GPE_STREAM_LOADS
#define GPE_STREAM_LOADS 1
#endif
__device__ __forceinline__ cx<float> ld_stream(const cx<float>* p) {
#if GPE_STREAM_LOADS
  float2 v = __ldcs(reinterpret_cast<const float2*>(p));
  return mk<float>(v.x, v.y);
#else
  return *p;
#endif
}
__device__ __forceinline__ cx<double> ld_stream(const cx<double>* p) {
#if GPE_STREAM_LOADS
  double2 v = __ldcs(reinterpret_cast<const double2*>(p));
  return mk<double>(v.x, v.y);
#else
  return *p;
#endif
}
template <typename R>
__device__ __forceinline__ R ld_stream(const R* p) {
#if GPE_STREAM_LOADS
  return __ldcs(p);
#else
  return *p;
#endif
}

// sin and cos of x in FP32.  For |x| <= 65536 (any physically meaningful
// phase per step): Cody-Waite reduction x = q*pi/2 + r with pi/2 split into
// two floats (q*hi is exact inside the FMA), then the Taylor series of sin
// to r^9 and of cos to r^10 on |r| <= pi/4 (truncation < 2e-9), and the
// quadrant rotation.  Larger arguments take sincosf.
__device__ __forceinline__ void sincos_bounded(float x, float* sp, float* cp) {
  if (!(fabsf(x) <= 65536.0f)) {
    sincosf(x, sp, cp);
    return;
  }
  const float q = rintf(x * 0.636619772f);  // 2/pi
  float r = fmaf(q, -1.57079637e+00f, x);   // pi/2 rounded to float
  r = fmaf(q, 4.37113900e-08f, r);          // minus (pi/2 - float(pi/2))
  const float r2 = r * r;
  float s = fmaf(r2, 2.75573192e-06f, -1.98412698e-04f);  // 1/9!, -1/7!
  s = fmaf(r2, s, 8.33333333e-03f);                       // 1/5!
  s = fmaf(r2, s, -1.66666667e-01f);                      // -1/3!
  s = fmaf(r2 * r, s, r);
  float c = fmaf(r2, -2.75573192e-07f, 2.48015873e-05f);  // -1/10!, 1/8!
  c = fmaf(r2, c, -1.38888889e-03f);                      // -1/6!
  c = fmaf(r2, c, 4.16666667e-02f);                       // 1/4!
  c = fmaf(r2, c, -0.5f);
  c = fmaf(r2, c, 1.0f);
  const int qi = (int)q;
  float ss = (qi & 1) ? c : s;
  float cc = (qi & 1) ? s : c;
  if (qi & 2) ss = -ss;
  if ((qi + 1) & 2) cc = -cc;
  *sp = ss;
  *cp = cc;
}

// exp(a * (dre + i dim)) for real a: the nonlinear / potential phase factor
// of the split step, with complex time step dt = i*ddt/(1 + i*gamma).
__device__ __forceinline__ cx<float> cexp_real_times(float a, float dre, float dim) {
  float s, c;
  sincos_bounded(a * dim, &s, &c);
  float m = (dre == 0.0f) ? 1.0f : expf(a * dre);
  return mk<float>(m * c, m * s);
}
__device__ __forceinline__ cx<double> cexp_real_times(double a, double dre, double dim) {
  double s, c;
  sincos(a * dim, &s, &c);
  double m = (dre == 0.0) ? 1.0 : exp(a * dre);
  return mk<double>(m * c, m * s);
}
// sin and cos of two lanes: the reduction and polynomials of sincos_bounded
// on packed lanes.  q = rint(x * 2/pi) by adding and removing 1.5 * 2^23
// (exact round-to-nearest for |x * 2/pi| < 2^22); the low bits of the
// shifted value are q's quadrant.  In range: |x| <= 65536 in both lanes.
__device__ __forceinline__ void quadrant(int qi, float s, float c, float& ss, float& cc) {
  ss = (qi & 1) ? c : s;
  cc = (qi & 1) ? s : c;
  if (qi & 2) ss = -ss;
  if ((qi + 1) & 2) cc = -cc;
}
__device__ __forceinline__ void sincos_x2_inrange(fx2 x, fx2& sp, fx2& cp) {
  const fx2 shifted = fma2(x, fx2(0.636619772f), fx2(12582912.0f));  // 2/pi; 1.5 * 2^23
  const fx2 q = shifted - fx2(12582912.0f);
  fx2 r = fma2(q, fx2(-1.57079637e+00f), x);  // pi/2 rounded to float
  r = fma2(q, fx2(4.37113900e-08f), r);       // minus (pi/2 - float(pi/2))
  const fx2 r2 = r * r;
  fx2 s = fma2(r2, fx2(2.75573192e-06f), fx2(-1.98412698e-04f));
  s = fma2(r2, s, fx2(8.33333333e-03f));
  s = fma2(r2, s, fx2(-1.66666667e-01f));
  s = fma2(r2 * r, s, r);
  fx2 c = fma2(r2, fx2(-2.75573192e-07f), fx2(2.48015873e-05f));
  c = fma2(r2, c, fx2(-1.38888889e-03f));
  c = fma2(r2, c, fx2(4.16666667e-02f));
  c = fma2(r2, c, fx2(-0.5f));
  c = fma2(r2, c, fx2(1.0f));
  float s0, c0, s1, c1;
  quadrant(__float_as_int(shifted.v.x), s.v.x, c.v.x, s0, c0);
  quadrant(__float_as_int(shifted.v.y), s.v.y, c.v.y, s1, c1);
  sp = fx2(s0, s1);
  cp = fx2(c0, c1);
}
// Lanes with |x| > 65536 take the scalar function.
__device__ __forceinline__ void sincos_x2(fx2 x, fx2& sp, fx2& cp) {
  if (!(fabsf(x.v.x) <= 65536.0f && fabsf(x.v.y) <= 65536.0f)) {
    float s0, c0, s1, c1;
    sincos_bounded(x.v.x, &s0, &c0);
    sincos_bounded(x.v.y, &s1, &c1);
    sp = fx2(s0, s1);
    cp = fx2(c0, c1);
    return;
  }
  sincos_x2_inrange(x, sp, cp);
}

// exp of two lanes with |x| <= 1/4 (the damping factors of a split step):
// Taylor series to x^7, truncation < 4e-10 relative.
__device__ __forceinline__ fx2 exp_x2_small(fx2 x) {
  fx2 p = fma2(x, fx2(1.98412698e-04f), fx2(1.38888889e-03f));  // 1/7!, 1/6!
  p = fma2(x, p, fx2(8.33333333e-03f));                         // 1/5!
  p = fma2(x, p, fx2(4.16666667e-02f));                         // 1/4!
  p = fma2(x, p, fx2(1.66666667e-01f));                         // 1/3!
  p = fma2(x, p, fx2(0.5f));
  p = fma2(x, p, fx2(1.0f));
  return fma2(x, p, fx2(1.0f));
}
// Any argument: lanes beyond 1/4 take expf.
__device__ __forceinline__ fx2 exp_x2(fx2 x) {
  if (fabsf(x.v.x) <= 0.25f && fabsf(x.v.y) <= 0.25f) return exp_x2_small(x);
  return fx2(expf(x.v.x), expf(x.v.y));
}

// The FP32 phase factors exp(ex[m] (dre + i dim)) applied to v[m], m < E
// (the real-time prologues of the step passes).  One range check per thread
// (max |ex| against 65536/|dim| and 1/4/|dre|, true for every split step of a
// physical run) selects the branch-free path that evaluates two factors at a
// time on packed lanes; otherwise cexp_real_times, one at a time.
template <int E>
__device__ __forceinline__ void apply_rt_phase(cx<float>* v, const float* ex, float dre, float dim) {
  static_assert(E % 2 == 0, "pairs of points");
  float mx = 0.0f;
#pragma unroll
  for (int m = 0; m < E; ++m) mx = fmaxf(mx, fabsf(ex[m]));
  if (mx * fabsf(dim) <= 65536.0f && mx * fabsf(dre) <= 0.25f) {
#pragma unroll
    for (int m = 0; m < E; m += 2) {
      const fx2 a(ex[m], ex[m + 1]);
      fx2 s, c;
      sincos_x2_inrange(a * fx2(dim), s, c);
      if (dre != 0.0f) {
        const fx2 mm = exp_x2_small(a * fx2(dre));
        c = mm * c;
        s = mm * s;
      }
      v[m] = cmul(mk<float>(c.v.x, s.v.x), v[m]);
      v[m + 1] = cmul(mk<float>(c.v.y, s.v.y), v[m + 1]);
    }
  } else {
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = cmul(cexp_real_times(ex[m], dre, dim), v[m]);
  }
}

__device__ __forceinline__ float rexp(float a) { return expf(a); }
__device__ __forceinline__ double rexp(double a) { return exp(a); }

// Device-resident scalars of one solver context.  Everything that the
// reference keeps in MATLAB scalars between array operations (mu, the renorm
// factor, ncur, the ITP residual) lives here so that whole blocks of steps
// run without a host round trip.
struct DevScalars {
  double scale;       // pending multiplicative factor of the stored state
  double mu;          // chemical potential subtracted from V (VV = V - mu)
  double ncur;        // integrate(|psi|^2) at the last block end / iteration
  double muc;         // mu reported at the last block end
  double NNN;         // target norm (NN0 or NN0*exp(-t/tau))
  double NN0;
  double delta;       // last ITP residual
  double best_delta;  // smallest residual seen in the current ITP phase
  double mu_itp;      // last MU(i)
  double mu2, ee;     // last MU2(i), EE(i) before division by Ntotal
  double maxabs;      // max |psi| at the last ITP check
  double dtmin;       // groundstate_itp.m:35,63-65
  double sums[8];     // last finalized sums (see Slot), weighted by the cell volume
  double energy;      // get_energy of the state at the last block end (solve_split)
  double scale2;      // two-component ITP: pending factor of component 2 (scale: component 1)
  int stop;           // nonzero: pass kernels and finalizers do nothing
  int iter;           // ITP iterations completed
  int stall;          // ITP checks in a row without a 10% residual drop
  int status;         // StopReason
  int nonfinite;      // a reduction produced NaN/Inf
  int timeout;        // a bounded device-side wait gave up
  int fin_count;      // CTAs of a multi-CTA finalizer that are done (0 between launches)
  int outer;         // outer steps the cluster kernel has completed in this run (history slot)
  int bounds_site;   // bounds-checked build: the first site that met an index out of range (0: none)
  long long bounds_index;  // ... and that index
};

enum StopReason { RUNNING = 0, CONVERGED = 1, SWITCH_FP64 = 2, HALVE_DT = 3, NONFINITE = 4 };

// Bounds-checked build (-DGPE_CHECK=1, a separate library): every global
// index of the axis-pass kernels is checked against its array's length and
// every shared-memory index against its buffer; the first violation is
// recorded in the context's device scalars (bounds_site, bounds_index), the
// access is skipped (a load reads 0, a store is dropped), and the run
// returns GPE_ERR_BOUNDS.  Nothing out of range is ever accessed.  Sites:
enum BoundsSite {
  BS_NONE = 0,
  BS_LOAD = 1,       // state load of a pass
  BS_STORE = 2,      // state store of a pass
  BS_SIDE = 3,       // V / ITP-factor load
  BS_AUX_STORE = 4,  // ITP-factor store
  BS_SMEM = 5,       // shared-memory exchange index
  BS_PARTIAL = 6,    // per-tile partial sum slot
  BS_CLUSTER = 7,    // cluster kernel: distributed shared memory rank or offset
};
#ifndef GPE_CHECK
#define GPE_CHECK 0
#endif
// The shared-memory exchange policies (fft.cuh) carry their buffer's
// length in checked builds: GPE_SMI(pol, i) is i, or 0 after recording i.
#if GPE_CHECK
#define GPE_SMI(pol, i) (pol).checked(i)
#define GPE_POL_CHECK_MEMBERS                                                                     \
  DevScalars* chk_sc = nullptr;                                                                   \
  int chk_lim = 0;                                                                                \
  __device__ __forceinline__ int checked(int i) const { return bounds_ok(chk_sc, BS_SMEM, i, chk_lim) ? i : 0; }
#define GPE_POL_BOUNDS(pol, scp, n) ((pol).chk_sc = (scp), (pol).chk_lim = (int)(n))
#else
#define GPE_SMI(pol, i) (i)
#define GPE_POL_CHECK_MEMBERS
#define GPE_POL_BOUNDS(pol, scp, n) ((void)0)
#endif
// True when 0 <= i < n; otherwise records (site, i) once in *sc.
__device__ __forceinline__ bool bounds_ok(DevScalars* sc, int site, long long i, long long n) {
#if GPE_CHECK
  if (i >= 0 && i < n) return true;
  if (atomicCAS(&sc->bounds_site, 0, site) == 0) sc->bounds_index = i;
  return false;
#else
  (void)sc, (void)site, (void)i, (void)n;
  return true;
#endif
}

// Reduction slots of the per-CTA partial-sum buffer.
enum Slot {
  S_N = 0,     // sum |psi|^2
  S_VN = 1,    // sum V |psi|^2
  S_N2 = 2,    // sum |psi|^4
  S_KX = 3,    // sum over x pencils of (1/nx) sum_k kx^2/2 |psi_hat|^2
  S_KY = 4,
  S_KZ = 5,
  S_MAXD = 6,  // max | |psi| - |psi_prev| |
  S_MAXA = 7,  // max |psi|
  NSLOTS = 8,
  S_FIN = 8,   // scratch of the multi-CTA finalizer (chunk sums); buffer has NSLOTS + 1 slots
};

// Prologue applied right after a pencil is loaded (first axis pass).
enum Prologue {
  PRO_NONE = 0,
  PRO_SCALE = 1,    // psi *= scale
  PRO_RT_HALF = 2,  // psi = exp((-VV - g|s psi|^2) dt/2) s psi   (solve_split.m:55-56)
  PRO_RT_FULL = 3,  // psi = exp((-VV - g|psi|^2) dt) psi         (solve_split.m:60-61)
  PRO_ITP = 4       // nl = exp(-dt/2 (g|s psi|^2 + V)); aux = nl; psi = nl s psi
                    // (groundstate_itp.m:36/76 then :40)
};
// Epilogue applied before a pencil is stored (last axis pass).
enum Epilogue {
  EPI_NONE = 0,
  EPI_RT_END = 1,  // full NL, inverse half NL, sums n, Vn, n^2 (solve_split.m:60-67)
  EPI_ITP = 2      // psi *= aux, sum n (groundstate_itp.m:42-44)
};

// KIND_STEP_EXT: a step pass with the rotating-frame cross terms, the energy
// cut-off mask or only one of its halves; a separate kernel, so that the
// plain step kernel keeps its register allocation.
enum PassKind { KIND_STEP = 0, KIND_ENERGY = 1, KIND_STEP_EXT = 2 };

template <typename R>
struct PassArgs {
  cx<R>* psi;              // state, updated in place
  const R* V;              // total potential V(t)
  R* aux;                  // ITP: nonlinear factor written by pass 1, read by the last
  const cx<R>* php;        // kinetic factor exp(-k^2/2 dt)/N of this axis, in the
                           // spectrum-slot order of the threads (pass.cuh apply_phase)
  const cx<R>* tws;        // stage twiddle rows of the plan (plans.cuh)
  const R* k2p;            // k^2/2/N in the same permuted order (energy pass)
  double* partials;        // [NSLOTS][cap] per-CTA partial sums
  DevScalars* sc;
  long long n_batch;       // number of pencils
  long long stride;        // element stride along the axis
  long long inner, outer;  // pencil b starts at (b % inner) + (b / inner) * outer
  int cap;                 // partials capacity per slot
  int kind;                // PassKind
  int pro, epi;            // Prologue / Epilogue
  int side;                // TMA pass: 0 none, 1 stage V, 2 stage aux with the tile
  int kin_slot;            // energy pass: slot of the kinetic sum
  int energy_pot;          // energy pass: also accumulate n, Vn, n^2
  double g;                // coupling
  double dre, dim;         // time step (real, imag) of the phase factors
  R gr, drer, dimr;        // g, dre, dim rounded to R by the host (no FP64 work per thread)
  int prefetch = 0;        // direct pass: 1 = prefetch the tile one wave ahead into L2
  int pf_ahead = 0;        // set by the launcher: resident CTAs of the launch (one wave)
  int pdl = 0;             // launch with programmatic stream serialisation (host side)
  // Rotating frame (x and y passes; null/0 otherwise).  Pencil b has the
  // transverse grid index b % rot_period (y for x pencils, x for y pencils).
  const cx<R>* rot = nullptr;  // step: [transverse index][slot] cross-term factors
  const R* rotw = nullptr;     // energy: per transverse index weight (-+omega * coordinate)
  const R* kp = nullptr;       // energy: k/N in the spectrum-slot order
  int rot_period = 0;
  // Non-separable kinetic factor (the stochastic GPE's energy cut-off): a
  // step pass may run only its forward half (skip_inv: position m*T+t of the
  // pencil then holds spectrum slot m*T+t) or only its inverse half
  // (skip_fwd, reading that order back), and the middle pass zeroes the
  // modes with kk >= ecut, kk = mask_a[b % mask_pa] + mask_b[b / mask_pa]
  // (the pencil's transverse axes, by stored position; mask_b optional) +
  // mask_c[slot] (the pass's own axis).  Tables hold k^2/2 in slot order.
  int skip_fwd = 0, skip_inv = 0;
  const R* mask_a = nullptr;
  const R* mask_b = nullptr;
  const R* mask_c = nullptr;
  long long mask_pa = 1;
  R ecut = R(0);
  // TMA pass, test of the timeout path only (0 = off): arm the barriers for
  // copies that are never issued and give up after this many polls.
  int tma_stall = 0;
  // Elements of the arrays the pass reads and writes (bounds-checked build).
  long long npts = 0;
  // TMA pass, strided axes: the state (and side array) as 4D tensors
  // (y, x, z, component) of extents tdim, copied one box per tile through
  // the kernel's tensor-map parameters (tma_tensor = 1); otherwise one bulk
  // copy per 128-byte row.
  int tma_tensor = 0;
  long long tdim[4] = {1, 1, 1, 1};
  // Step pass (scalar kernels): 1 = transform, the full nonlinear step
  // (PRO_RT_FULL's phase, V read from L2), transform again: the passes of
  // this axis that end one split step and begin the next, when consecutive
  // steps take the axes in opposite orders.
  int fold = 0;
};

}  // namespace gpe

// spinor_kernels.cu - the elementwise, reduction and finalizer kernels of the
// coherently coupled two-component split step (lib/@GPEtaskSpinor of
// GPE-MATLAB).  The state holds component 1 at [0, P) and component 2 at
// [P, 2P); the kinetic factors are the ordinary axis passes run over both.
#include "aux_kernels.cuh"

namespace gpe {

constexpr int SP_THREADS = 256;

// cosh and sinh of a + ib.
template <typename R>
__device__ __forceinline__ void ccosh_csinh(R a, R b, cx<R>& ch, cx<R>& sh) {
  R sb, cb, sa, ca;
  if constexpr (sizeof(R) == 4) {
    sincosf(b, &sb, &cb);
    sa = sinhf(a);
    ca = coshf(a);
  } else {
    sincos(b, &sb, &cb);
    sa = sinh(a);
    ca = cosh(a);
  }
  ch = mk<R>(ca * cb, sa * sb);
  sh = mk<R>(sa * cb, ca * sb);
}

// One nonlinear + coupling factor of solve_split.m:77-91 at every point:
//   t_j  = V_j - mu + sum_k g(j,k) |psi_k|^2
//   psi1 <- exp(-t_1 dt) (cosom psi1 - sinomp psi2)
//   psi2 <- exp(-t_2 dt) (cosom psi2 - sinomm psi1)
// with the step-constant cosom/sinomm/sinomp of :61-64, or with nlincpl != 0
// cosh/sinh of dt*(coupling + nlincpl (|psi1|^2 + |psi2|^2)) (:84-89).
// `first`: the state still carries the pending renormalisation factor.
template <typename R>
__global__ void __launch_bounds__(SP_THREADS) k_spinor_nl(cx<R>* __restrict__ psi, const R* __restrict__ V,
                                                          long long P, const DevScalars* sc, int first,
                                                          const SpinorNL<R> q) {
  __shared__ R scal[2];
  if (threadIdx.x == 0) {
    scal[0] = first ? (R)sc->scale : R(1);
    scal[1] = (R)sc->mu;
  }
  if (__syncthreads_or(sc->stop != 0)) return;
  const R s = scal[0], mu = scal[1];
  for (long long i = (long long)blockIdx.x * SP_THREADS + threadIdx.x; i < P; i += (long long)gridDim.x * SP_THREADS) {
    const cx<R> p1 = rmul(psi[i], s), p2 = rmul(psi[i + P], s);
    const R n1 = norm2(p1), n2 = norm2(p2);
    const R t1 = V[i] - mu + q.g11 * n1 + q.g12 * n2;
    const R t2 = V[i + P] - mu + q.g21 * n1 + q.g22 * n2;
    cx<R> co = q.cosom, sm = q.sinomm, sp = q.sinomp;
    if (q.nl) {
      const R tr = q.cre + q.nlincpl * (n1 + n2), ti = q.cim;
      ccosh_csinh<R>(q.dre * tr - q.dim * ti, q.dre * ti + q.dim * tr, co, sm);
      sp = sm;
    }
    const cx<R> a1 = cmul(co, p1) - cmul(sp, p2);
    const cx<R> a2 = cmul(co, p2) - cmul(sm, p1);
    psi[i] = cmul(cexp_real_times(-t1, q.dre, q.dim), a1);
    psi[i + P] = cmul(cexp_real_times(-t2, q.dre, q.dim), a2);
  }
}

// Imaginary-time step of GPEtaskSpinor.groundstate_itp (groundstate_itp.m:
// 63-81), real dt.  First, from the state before the kinetic half step, the
// factors f_j = exp(-(V_j + sum_k g(j,k) |s_k psi_k|^2) dt) (s_k: pending
// factors; `split`: the two-component ITP keeps one per component, scale and
// scale2, GPEtask2comp/groundstate_itp.m:58-59, otherwise both are scale).
template <typename R>
__global__ void __launch_bounds__(SP_THREADS) k_spinor_itp_factors(const cx<R>* __restrict__ psi,
                                                                  const R* __restrict__ V, long long P,
                                                                  const DevScalars* sc, SpinorNL<R> q,
                                                                  R* __restrict__ f, int split) {
  __shared__ R s0[2];
  if (threadIdx.x == 0) {
    s0[0] = (R)sc->scale;
    s0[1] = (R)(split ? sc->scale2 : sc->scale);
  }
  if (__syncthreads_or(sc->stop != 0)) return;
  const R sa = s0[0], sb = s0[1], dt = q.dre;
  for (long long i = (long long)blockIdx.x * SP_THREADS + threadIdx.x; i < P; i += (long long)gridDim.x * SP_THREADS) {
    const R n1 = norm2(psi[i]) * sa * sa, n2 = norm2(psi[i + P]) * sb * sb;
    f[i] = rexp(-(V[i] + q.g11 * n1 + q.g12 * n2) * dt);
    f[i + P] = rexp(-(V[i + P] + q.g21 * n1 + q.g22 * n2) * dt);
  }
}

// Then, after the kinetic half step, psi1 <- f1 (cosom s psi1 - sinomp s psi2),
// psi2 <- f2 (cosom s psi2 - sinomm s psi1) (:72-73); the caller resets the
// pending factor.
template <typename R>
__global__ void __launch_bounds__(SP_THREADS) k_spinor_itp_couple(cx<R>* __restrict__ psi, const R* __restrict__ f,
                                                                 long long P, const DevScalars* sc, SpinorNL<R> q,
                                                                 int split) {
  __shared__ R s0[2];
  if (threadIdx.x == 0) {
    s0[0] = (R)sc->scale;
    s0[1] = (R)(split ? sc->scale2 : sc->scale);
  }
  if (__syncthreads_or(sc->stop != 0)) return;
  const R sa = s0[0], sb = s0[1];
  for (long long i = (long long)blockIdx.x * SP_THREADS + threadIdx.x; i < P; i += (long long)gridDim.x * SP_THREADS) {
    const cx<R> p1 = rmul(psi[i], sa), p2 = rmul(psi[i + P], sb);
    psi[i] = rmul(cmul(q.cosom, p1) - cmul(q.sinomp, p2), f[i]);
    psi[i + P] = rmul(cmul(q.cosom, p2) - cmul(q.sinomm, p1), f[i + P]);
  }
}

// The pending factors of the two-component ITP applied to the stored state
// (component 1 times scale, component 2 times scale2); the caller resets them.
template <typename R>
__global__ void __launch_bounds__(SP_THREADS) k_mix_apply_scales(cx<R>* __restrict__ psi, long long P,
                                                                const DevScalars* sc) {
  __shared__ R s0[2];
  if (threadIdx.x == 0) {
    s0[0] = (R)sc->scale;
    s0[1] = (R)sc->scale2;
  }
  __syncthreads();
  const R sa = s0[0], sb = s0[1];
  for (long long i = (long long)blockIdx.x * SP_THREADS + threadIdx.x; i < P; i += (long long)gridDim.x * SP_THREADS) {
    psi[i] = rmul(psi[i], sa);
    psi[i + P] = rmul(psi[i + P], sb);
  }
}

// Compensated per-thread sum in the context precision.
template <typename R>
struct KSum {
  R s = R(0), c = R(0);
  __device__ __forceinline__ void add(R x) {
    const R y = x - c;
    const R t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// The sums of GPEtaskSpinor.applyham / inner (GPEtaskSpinor.m:53-89) other
// than the kinetic ones, one partial per CTA and sum at out[k*gridDim.x + b]:
// n1, n2, V1 n1, V2 n2, n1^2, n2^2, n1 n2, Re and Im of conj(psi1) psi2.
template <typename R>
__global__ void __launch_bounds__(SP_THREADS) k_spinor_sums(const cx<R>* __restrict__ psi, const R* __restrict__ V,
                                                            long long P, const DevScalars* sc, double* out) {
  if (sc->stop) return;
  KSum<R> acc[SP_NSUMS];
  for (long long i = (long long)blockIdx.x * SP_THREADS + threadIdx.x; i < P; i += (long long)gridDim.x * SP_THREADS) {
    const cx<R> p1 = psi[i], p2 = psi[i + P];
    const R n1 = norm2(p1), n2 = norm2(p2);
    acc[0].add(n1);
    acc[1].add(n2);
    acc[2].add(V[i] * n1);
    acc[3].add(V[i + P] * n2);
    acc[4].add(n1 * n1);
    acc[5].add(n2 * n2);
    acc[6].add(n1 * n2);
    acc[7].add(p1.x * p2.x + p1.y * p2.y);
    acc[8].add(p1.x * p2.y - p1.y * p2.x);
  }
  __shared__ double sh[SP_NSUMS][SP_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < SP_NSUMS; ++k) {
    double v = acc[k].value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < SP_NSUMS) {
    double v = 0.0;
    for (int w = 0; w < SP_THREADS / 32; ++w) v += sh[threadIdx.x][w];
    out[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = v;
  }
}

constexpr int FIN_T = 256;

// Sum of n partials in a fixed order over the CTA (deterministic): strided
// per-thread sums, then a shared-memory tree.  Every thread gets the result.
__device__ double cta_sum_fixed(const double* p, int n, double* sh) {
  double v = 0.0;
  for (int i = (int)threadIdx.x; i < n; i += FIN_T) v += p[i];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = FIN_T / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Start of a run (mode 0, solve_split.m:29-37,52-57), block end (mode 1,
// :100-113) or observables (mode 2): NN0, renormalisation, mu.
__global__ void k_finalize_spinor(const SpinorFinalArgs a, DevScalars* sc) {
  if (a.mode != 2 && sc->stop) return;
  __shared__ double sh[FIN_T];
  double s[SP_NSUMS];
  for (int k = 0; k < SP_NSUMS; ++k) s[k] = cta_sum_fixed(a.sums + (size_t)k * a.nsum, a.nsum, sh);
  double kin = 0.0;
  for (int ax = 0; ax < 3; ++ax)
    if (a.nblk_kin[ax] > 0) kin += cta_sum_fixed(a.partials + (size_t)(S_KX + ax) * a.cap, a.nblk_kin[ax], sh);
  if (threadIdx.x != 0) return;
  const double w = a.weight;
  const double ncur = (s[0] + s[1]) * w;
  const double ev = (s[2] + s[3]) * w;
  const double eint = (a.g[0] * s[4] + (a.g[1] + a.g[2]) * s[6] + a.g[3] * s[5]) * w;
  // <psi1|c psi2> + <psi2|conj(c) psi1> = 2 Re(c * sum conj(psi1) psi2)
  const double ecpl = 2.0 * (a.cre * s[7] - a.cim * s[8]) * w;
  const double quad = kin * w + ev + ecpl;
  if (a.mode == 3) {
    // ITP (groundstate_itp.m:90-99): MU2 = <psi|H psi>/Ntotal and EE =
    // get_energy/Ntotal of the state times the pending factor
    const double s = sc->scale, s2 = s * s;
    if (a.hist) *a.hist = (s2 * quad + s2 * s2 * eint) / a.Ntotal;
    if (a.obs) *a.obs = (s2 * quad + 0.5 * s2 * s2 * eint) / a.Ntotal;
    return;
  }
  if (a.mode == 2) {
    a.obs[0] = ncur;
    a.obs[1] = kin * w;
    a.obs[2] = ev;
    a.obs[3] = eint;
    a.obs[4] = ecpl;
    return;
  }
  if (a.mode == 0) {
    const double NN0 = a.Ntotal > 0 ? a.Ntotal : ncur;
    sc->NN0 = NN0;
    sc->NNN = NN0;
    sc->mu = (quad + eint) / NN0;
    sc->scale = 1.0;
    if (!isfinite(sc->mu)) {
      sc->nonfinite = 1;
      sc->status = NONFINITE;
      sc->stop = 1;
    }
    return;
  }
  double scale = 1.0, NNN = sc->NNN;
  if (a.renorm) {
    if (a.tau > 0) NNN = sc->NN0 * exp(-a.time2 / a.tau);
    sc->NNN = NNN;
    scale = sqrt(NNN / ncur);
  }
  const double s2 = scale * scale;
  const double mu = (s2 * quad + s2 * s2 * eint) / NNN;
  const double energy = s2 * quad + 0.5 * s2 * s2 * eint;  // get_energy halves g (GPEtaskSpinor.m:98-110)
  sc->energy = energy;
  sc->scale = scale;
  sc->mu = mu;
  sc->muc = mu;
  sc->ncur = ncur;
  if (!isfinite(ncur) || !isfinite(mu) || !isfinite(scale)) {
    sc->nonfinite = 1;
    sc->status = NONFINITE;
    sc->stop = 1;
  }
  if (a.hist) {
    a.hist[0] = mu;
    a.hist[1] = ncur;
    a.hist[2] = energy;
  }
}

// GPEtask2comp/groundstate_itp.m:82-90: n_j = integrate(|psi_j|^2) from the
// per-CTA partials of each component, m_j = sqrt(N_j/n_j) kept pending as
// scale / scale2, MU1(i) = log(m1)/dt, MU2(i) = log(m2)/dt.
__global__ void k_finalize_mix(const MixFinalArgs a, DevScalars* sc) {
  if (sc->stop) return;
  __shared__ double sh[FIN_T];
  const double n1 = cta_sum_fixed(a.part1, a.nblk1, sh) * a.weight;
  const double n2 = cta_sum_fixed(a.part2, a.nblk2, sh) * a.weight;
  if (threadIdx.x != 0) return;
  const double m1 = sqrt(a.N1 / n1), m2 = sqrt(a.N2 / n2);
  sc->scale = m1;
  sc->scale2 = m2;
  sc->ncur = n1 + n2;
  sc->iter = a.iter;
  sc->mu_itp = log(m1) / a.dt;
  a.MU1[a.iter - 1] = log(m1) / a.dt;
  a.MU2[a.iter - 1] = log(m2) / a.dt;
  if (!isfinite(n1) || !isfinite(n2) || !isfinite(m1) || !isfinite(m2) || !(n1 > 0.0) || !(n2 > 0.0)) {
    sc->nonfinite = 1;
    sc->status = NONFINITE;
    sc->stop = 1;
  }
}

template <typename R>
void launch_spinor_nl(cx<R>* psi, const R* V, long long P, const DevScalars* sc, int first, const SpinorNL<R>& q,
                      cudaStream_t s) {
  k_spinor_nl<R><<<elem_grid(P, SP_THREADS), SP_THREADS, 0, s>>>(psi, V, P, sc, first, q);
}

template <typename R>
int launch_spinor_sums(const cx<R>* psi, const R* V, long long P, const DevScalars* sc, double* out,
                       cudaStream_t s) {
  const int grid = elem_grid(P, SP_THREADS);
  k_spinor_sums<R><<<grid, SP_THREADS, 0, s>>>(psi, V, P, sc, out);
  return grid;
}

template <typename R>
void launch_spinor_itp_factors(const cx<R>* psi, const R* V, long long P, const DevScalars* sc, const SpinorNL<R>& q,
                               R* f, int split, cudaStream_t s) {
  k_spinor_itp_factors<R><<<elem_grid(P, SP_THREADS), SP_THREADS, 0, s>>>(psi, V, P, sc, q, f, split);
}
template <typename R>
void launch_spinor_itp_couple(cx<R>* psi, const R* f, long long P, const DevScalars* sc, const SpinorNL<R>& q,
                              int split, cudaStream_t s) {
  k_spinor_itp_couple<R><<<elem_grid(P, SP_THREADS), SP_THREADS, 0, s>>>(psi, f, P, sc, q, split);
}
template <typename R>
void launch_mix_apply_scales(cx<R>* psi, long long P, const DevScalars* sc, cudaStream_t s) {
  k_mix_apply_scales<R><<<elem_grid(P, SP_THREADS), SP_THREADS, 0, s>>>(psi, P, sc);
}
void launch_finalize_mix(const MixFinalArgs& a, DevScalars* sc, cudaStream_t s) {
  k_finalize_mix<<<1, FIN_T, 0, s>>>(a, sc);
}

void launch_finalize_spinor(const SpinorFinalArgs& a, DevScalars* sc, cudaStream_t s) {
  k_finalize_spinor<<<1, FIN_T, 0, s>>>(a, sc);
}

#define INST_SPINOR(R)                                                                                     \
  template void launch_spinor_nl<R>(cx<R>*, const R*, long long, const DevScalars*, int, const SpinorNL<R>&, \
                                    cudaStream_t);                                                         \
  template int launch_spinor_sums<R>(const cx<R>*, const R*, long long, const DevScalars*, double*, cudaStream_t); \
  template void launch_spinor_itp_factors<R>(const cx<R>*, const R*, long long, const DevScalars*,                \
                                             const SpinorNL<R>&, R*, int, cudaStream_t);                          \
  template void launch_spinor_itp_couple<R>(cx<R>*, const R*, long long, const DevScalars*, const SpinorNL<R>&,   \
                                            int, cudaStream_t);                                                   \
  template void launch_mix_apply_scales<R>(cx<R>*, long long, const DevScalars*, cudaStream_t);
INST_SPINOR(float)
INST_SPINOR(double)

}  // namespace gpe

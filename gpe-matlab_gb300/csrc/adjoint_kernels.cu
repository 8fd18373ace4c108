// adjoint_kernels.cu - elementwise kernels of the discrete adjoint of the
// split step (gradient of an overlap loss with respect to V).
//
// At gamma = 0 every nonlinear factor of solve_split.m:55-64 is a pure phase,
// so |psi| is unchanged by it and the merged block (half step, n_rec x
// [kinetic, full step], inverse half step) is exactly (N K N)^n_rec with
// N(psi) = exp(-i (V - mu + g|psi|^2) dt/2) psi.  mu only adds a global phase,
// which an overlap loss |<target|psi(T)>|^2 does not see, so it is dropped.
//
// Adjoint of one factor N (input x, output y = exp(-i theta) x,
// theta = (V + g|x|^2) h): with lam = dL/dy* (Wirtinger),
//   u = exp(i theta) lam,  s = 2 Im(conj(u) x),
//   dL/dx* = u + g h s x,   dL/dV += s h.
// The kinetic factor K has a symbol that depends on k^2 only, so its adjoint
// is conj o K o conj; the kernels can write their result conjugated so the
// next kinetic pass runs unchanged.
#include "aux_kernels.cuh"

namespace gpe {

constexpr int ADJ_THREADS = 256;

template <typename R>
__global__ void k_nl_phase(cx<R>* __restrict__ psi, const R* __restrict__ V, long long n, R g, R h) {
  for (long long i = (long long)blockIdx.x * ADJ_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * ADJ_THREADS) {
    const cx<R> p = psi[i];
    const R th = (V[i] + g * norm2(p)) * h;
    R s, c;
    if constexpr (sizeof(R) == 4) sincos_bounded(th, &s, &c);
    else sincos(th, &s, &c);
    psi[i] = mk<R>(p.x * c + p.y * s, p.y * c - p.x * s);  // exp(-i th) p
  }
}

// Adjoint of the nonlinear halves that touch the step-boundary state x = x_m.
// first:  the opening half of step m, y = N(x) (input x);
// second: the closing half of step m-1, x = N(phi).  Its input phi has
//         |phi| = |x|, so theta = (V + g|x|^2) h and phi = exp(i theta) x:
//         s = 2 Im(conj(lam) x), dL/dphi* = exp(i theta) (lam + g h s x).
// Applying first then second is the backward order (step m before m-1).
template <typename R>
__global__ void k_adj_nl(cx<R>* __restrict__ lam, const cx<R>* __restrict__ x, const R* __restrict__ V,
                         double* __restrict__ dLdV, long long n, R g, R h, int first, int second, int conj_in,
                         int conj_out) {
  const R gh = g * h;
  for (long long i = (long long)blockIdx.x * ADJ_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * ADJ_THREADS) {
    const cx<R> xi = x[i];
    cx<R> l = lam[i];
    if (conj_in) l.y = -l.y;
    const R th = (V[i] + g * norm2(xi)) * h;
    R sn, cs;
    if constexpr (sizeof(R) == 4) sincos_bounded(th, &sn, &cs);
    else sincos(th, &sn, &cs);
    R acc = R(0);
    if (first) {
      const cx<R> u = mk<R>(l.x * cs - l.y * sn, l.x * sn + l.y * cs);  // exp(i th) lam
      const R s = R(2) * (u.x * xi.y - u.y * xi.x);                    // 2 Im(conj(u) x)
      l = mk<R>(u.x + gh * s * xi.x, u.y + gh * s * xi.y);
      acc += s;
    }
    if (second) {
      const R s = R(2) * (l.x * xi.y - l.y * xi.x);                    // 2 Im(conj(lam) x)
      const cx<R> w = mk<R>(l.x + gh * s * xi.x, l.y + gh * s * xi.y);
      l = mk<R>(w.x * cs - w.y * sn, w.x * sn + w.y * cs);
      acc += s;
    }
    if (conj_out) l.y = -l.y;
    lam[i] = l;
    dLdV[i] += (double)acc * (double)h;
  }
}

// partials[2*b], partials[2*b+1] = sum over this CTA's points of conj(a) b
template <typename R>
__global__ void k_inner(const cx<R>* __restrict__ a, const cx<R>* __restrict__ b, long long n,
                        double* __restrict__ partials) {
  double re = 0.0, im = 0.0;
  for (long long i = (long long)blockIdx.x * ADJ_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * ADJ_THREADS) {
    const cx<R> p = a[i], q = b[i];
    re += (double)p.x * q.x + (double)p.y * q.y;
    im += (double)p.x * q.y - (double)p.y * q.x;
  }
  __shared__ double sh[2][ADJ_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = re;
    sh[1][threadIdx.x >> 5] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0, s = 0.0;
    for (int w = 0; w < ADJ_THREADS / 32; ++w) {
      r += sh[0][w];
      s += sh[1][w];
    }
    partials[2 * blockIdx.x] = r;
    partials[2 * blockIdx.x + 1] = s;
  }
}

// out = (cr + i ci) * in
template <typename R>
__global__ void k_cscale(cx<R>* __restrict__ out, const cx<R>* __restrict__ in, long long n, double cr, double ci) {
  const R a = (R)cr, b = (R)ci;
  for (long long i = (long long)blockIdx.x * ADJ_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * ADJ_THREADS) {
    const cx<R> p = in[i];
    out[i] = mk<R>(a * p.x - b * p.y, a * p.y + b * p.x);
  }
}

template <typename R>
void launch_nl_phase(cx<R>* psi, const R* V, long long n, double g, double h, cudaStream_t s) {
  k_nl_phase<R><<<elem_grid(n, ADJ_THREADS), ADJ_THREADS, 0, s>>>(psi, V, n, (R)g, (R)h);
}
template <typename R>
void launch_adj_nl(cx<R>* lam, const cx<R>* x, const R* V, double* dLdV, long long n, double g, double h,
                   int first, int second, int conj_in, int conj_out, cudaStream_t s) {
  k_adj_nl<R><<<elem_grid(n, ADJ_THREADS), ADJ_THREADS, 0, s>>>(lam, x, V, dLdV, n, (R)g, (R)h, first, second,
                                                               conj_in, conj_out);
}
template <typename R>
int launch_inner(const cx<R>* a, const cx<R>* b, long long n, double* partials, cudaStream_t s) {
  const int grid = elem_grid(n, ADJ_THREADS);
  k_inner<R><<<grid, ADJ_THREADS, 0, s>>>(a, b, n, partials);
  return grid;
}
template <typename R>
void launch_cscale(cx<R>* out, const cx<R>* in, long long n, double cr, double ci, cudaStream_t s) {
  k_cscale<R><<<elem_grid(n, ADJ_THREADS), ADJ_THREADS, 0, s>>>(out, in, n, cr, ci);
}

// ---- stochastic GPE (lib/@SGPEtask/solve_split.m:57-66) ----------------------
// psi <- exp((mu - V - g|s psi|^2) dt') s psi with dt' = (dre + i dim) * frac
// (frac = 1/2 at a block start, 1 after a kinetic step), s = the pending scale
// at a block start, then psi <- psi + sigma (n1 + i n2) with n1, n2 the
// normal variates of gauss2(seed, step, point index).
template <typename R>
__global__ void k_sgpe_nl_noise(cx<R>* __restrict__ psi, const R* __restrict__ V, long long n, DevScalars* sc,
                                R g, R dre, R dim, int half, R sigma, unsigned long long seed,
                                unsigned long long step) {
  if (sc->stop) return;
  const R s = half ? (R)sc->scale : R(1);
  const R mu = (R)sc->mu;
  const R f = half ? R(0.5) : R(1);
  for (long long i = (long long)blockIdx.x * ADJ_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * ADJ_THREADS) {
    cx<R> p = psi[i];
    p = mk<R>(p.x * s, p.y * s);
    const R a = (mu - V[i] - g * norm2(p)) * f;
    p = cmul(cexp_real_times(a, dre, dim), p);
    if (sigma != R(0)) {
      const cx<R> z = gauss2<R>(seed, step, (unsigned long long)i);
      p = mk<R>(p.x + sigma * z.x, p.y + sigma * z.y);
    }
    psi[i] = p;
  }
}

template <typename R>
void launch_sgpe_nl_noise(cx<R>* psi, const R* V, long long n, DevScalars* sc, double g, double dre, double dim,
                          int half, double sigma, unsigned long long seed, unsigned long long step, cudaStream_t s) {
  k_sgpe_nl_noise<R><<<elem_grid(n, ADJ_THREADS), ADJ_THREADS, 0, s>>>(psi, V, n, sc, (R)g, (R)dre, (R)dim, half,
                                                                      (R)sigma, seed, step);
}

// The block end of solve_split.m:60-65 as one elementwise pass: the last
// step's full factor exp((mu - V - g|p|^2) dt), the inverse half step
// exp((V - mu + g|p|^2) dt/2), and per CTA the sums n, V n, n^2 into the
// partial slots S_N, S_VN, S_N2 (what the pass epilogue EPI_RT_END does).
template <typename R>
__global__ void __launch_bounds__(ADJ_THREADS) k_rt_block_end(cx<R>* __restrict__ psi, const R* __restrict__ V,
                                                             long long n, const DevScalars* sc, R g, R dre, R dim,
                                                             double* partials, int cap) {
  if (sc->stop) return;
  const R mu = (R)sc->mu;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (long long i = (long long)blockIdx.x * ADJ_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * ADJ_THREADS) {
    cx<R> p = psi[i];
    const R VV = V[i] - mu;
    p = cmul(cexp_real_times(-VV - g * norm2(p), dre, dim), p);
    p = cmul(cexp_real_times((VV + g * norm2(p)) * R(0.5), dre, dim), p);
    psi[i] = p;
    const double nn = (double)norm2(p);
    a0 += nn;
    a1 += (double)V[i] * nn;
    a2 += nn * nn;
  }
  __shared__ double sh[3][ADJ_THREADS];
  sh[0][threadIdx.x] = a0;
  sh[1][threadIdx.x] = a1;
  sh[2][threadIdx.x] = a2;
  __syncthreads();
  for (int o = ADJ_THREADS / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[(size_t)S_N * cap + blockIdx.x] = sh[0][0];
    partials[(size_t)S_VN * cap + blockIdx.x] = sh[1][0];
    partials[(size_t)S_N2 * cap + blockIdx.x] = sh[2][0];
  }
}

template <typename R>
int launch_rt_block_end(cx<R>* psi, const R* V, long long n, const DevScalars* sc, double g, double dre, double dim,
                        double* partials, int cap, cudaStream_t s) {
  const int nb = elem_grid(n, ADJ_THREADS);
  k_rt_block_end<R><<<nb, ADJ_THREADS, 0, s>>>(psi, V, n, sc, (R)g, (R)dre, (R)dim, partials, cap);
  return nb;
}

__global__ void k_selftest_noise(float* out, long long n, unsigned long long seed, unsigned long long step) {
  for (long long i = (long long)blockIdx.x * ADJ_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * ADJ_THREADS) {
    const cx<float> z = gauss2<float>(seed, step, (unsigned long long)i);
    out[2 * i] = z.x;
    out[2 * i + 1] = z.y;
  }
}
cudaError_t launch_selftest_noise(float* out, long long n, unsigned long long seed, unsigned long long step,
                                  cudaStream_t s) {
  k_selftest_noise<<<elem_grid(n, ADJ_THREADS), ADJ_THREADS, 0, s>>>(out, n, seed, step);
  return cudaGetLastError();
}

#define INST_ADJ(R)                                                                                     \
  template void launch_nl_phase<R>(cx<R>*, const R*, long long, double, double, cudaStream_t);         \
  template void launch_adj_nl<R>(cx<R>*, const cx<R>*, const R*, double*, long long, double, double,   \
                                 int, int, int, int, cudaStream_t);                                    \
  template int launch_inner<R>(const cx<R>*, const cx<R>*, long long, double*, cudaStream_t);          \
  template void launch_cscale<R>(cx<R>*, const cx<R>*, long long, double, double, cudaStream_t);        \
  template void launch_sgpe_nl_noise<R>(cx<R>*, const R*, long long, DevScalars*, double, double, double, int, \
                                        double, unsigned long long, unsigned long long, cudaStream_t);     \
  template int launch_rt_block_end<R>(cx<R>*, const R*, long long, const DevScalars*, double, double, double,  \
                                      double*, int, cudaStream_t);
INST_ADJ(float)
INST_ADJ(double)

}  // namespace gpe

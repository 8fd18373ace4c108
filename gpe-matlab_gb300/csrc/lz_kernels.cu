// lz_kernels.cu - the angular-momentum operator of an array (position
// dependent) omega: the Crank-Nicolson Lz update of ssft_kin_step.m:3-11 and
// the -omega*Lz energy term of applyh0 (GPEtask.m:92-94) in GPE-MATLAB.
//
// lz(phi) = -i (x d/dy - y d/dx) phi (lib/@grid2d/lz.m:4-8) with the 4th-order
// first derivatives of grid1d.m:52-57, (-f(i+2) + 8 f(i+1) - 8 f(i-1) +
// f(i-2)) / (12 h), zero outside the grid (convn 'same'); both derivatives
// take the x spacing (derivx.m / derivy.m pass obj.dx).  In 3D they act
// within every z slice.  Layout: point (ix, iy, iz) at iy + ny*(ix + nx*iz).
#include "aux_kernels.cuh"

namespace gpe {

constexpr int LZ_T = 256;

template <typename R>
__device__ __forceinline__ cx<R> ld0(const cx<R>* s, long long i, bool in) {
  return in ? s[i] : mk<R>(R(0), R(0));
}

// x d/dy - y d/dx of s at linear index i = (ix, iy) of its slice.
template <typename R>
__device__ __forceinline__ cx<R> lz_w(const cx<R>* __restrict__ s, long long i, int ix, int iy, const LzGeom& g) {
  const long long sy = 1, sx = g.ny;
  const R c8 = R(8), inv = R(1) / (R(12) * (R)g.h);
  auto d = [&](long long st, int k, int n) {
    const cx<R> p2 = ld0(s, i + 2 * st, k + 2 < n), p1 = ld0(s, i + st, k + 1 < n);
    const cx<R> m1 = ld0(s, i - st, k - 1 >= 0), m2 = ld0(s, i - 2 * st, k - 2 >= 0);
    return mk<R>((-p2.x + c8 * p1.x - c8 * m1.x + m2.x) * inv, (-p2.y + c8 * p1.y - c8 * m1.y + m2.y) * inv);
  };
  const cx<R> dy = d(sy, iy, g.ny), dx = d(sx, ix, g.nx);
  const R X = (R)(g.x0 + ix * g.hxg), Y = (R)(g.y0 + iy * g.hyg);
  return mk<R>(X * dy.x - Y * dx.x, X * dy.y - Y * dx.y);
}

// out = phi + c * omega * lz(src), c complex (lz = -i w); omega from the
// array om, or the scalar oms where om is null.
template <typename R>
__global__ void __launch_bounds__(LZ_T) k_lz_cn(cx<R>* out, const cx<R>* phi, const cx<R>* __restrict__ src,
                                               const R* __restrict__ om, R oms, long long n, LzGeom g, R cre,
                                               R cim) {
  const long long nxy = (long long)g.nx * g.ny;
  for (long long i = (long long)blockIdx.x * LZ_T + threadIdx.x; i < n; i += (long long)gridDim.x * LZ_T) {
    const long long r = i % nxy;
    const int ix = (int)(r / g.ny), iy = (int)(r % g.ny);
    const cx<R> w = lz_w<R>(src, i, ix, iy, g);
    const cx<R> lz = mk<R>(w.y, -w.x);  // -i w
    const R o = om ? om[i] : oms;
    const cx<R> t = mk<R>(o * (cre * lz.x - cim * lz.y), o * (cre * lz.y + cim * lz.x));
    const cx<R> p = phi[i];
    out[i] = mk<R>(p.x + t.x, p.y + t.y);
  }
}

// Per CTA: sum of real(conj(psi) * (-omega lz(psi))) = -omega Im(conj(psi) w),
// times scale^2 when the state carries a pending factor; omega per point (om)
// or the scalar oms when om is null.
template <typename R>
__global__ void __launch_bounds__(LZ_T) k_lz_energy(const cx<R>* __restrict__ psi, const R* __restrict__ om,
                                                   double oms, long long n, LzGeom g, const DevScalars* sc,
                                                   int use_scale, double* out) {
  if (sc->stop) return;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * LZ_T + threadIdx.x; i < n; i += (long long)gridDim.x * LZ_T) {
    const long long r = i % ((long long)g.nx * g.ny);
    const int ix = (int)(r / g.ny), iy = (int)(r % g.ny);
    const cx<R> w = lz_w<R>(psi, i, ix, iy, g);
    const cx<R> p = psi[i];
    const double o = om ? (double)om[i] : oms;
    acc += -o * ((double)p.x * w.y - (double)p.y * w.x);
  }
  __shared__ double sh[LZ_T];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = LZ_T / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double s = use_scale ? sc->scale : 1.0;
    out[blockIdx.x] = sh[0] * s * s;
  }
}

template <typename R>
void launch_lz_cn(cx<R>* out, const cx<R>* phi, const cx<R>* src, const R* om, double oms, long long n,
                  const LzGeom& g, double cre, double cim, cudaStream_t st) {
  k_lz_cn<R><<<elem_grid(n, LZ_T), LZ_T, 0, st>>>(out, phi, src, om, (R)oms, n, g, (R)cre, (R)cim);
}

template <typename R>
int launch_lz_energy(const cx<R>* psi, const R* om, double oms, long long n, const LzGeom& g, const DevScalars* sc,
                     int use_scale, double* out, cudaStream_t st) {
  const int nb = elem_grid(n, LZ_T);
  k_lz_energy<R><<<nb, LZ_T, 0, st>>>(psi, om, oms, n, g, sc, use_scale, out);
  return nb;
}

#define INST_LZ(R)                                                                                     \
  template void launch_lz_cn<R>(cx<R>*, const cx<R>*, const cx<R>*, const R*, double, long long,         \
                                const LzGeom&, double, double, cudaStream_t);                          \
  template int launch_lz_energy<R>(const cx<R>*, const R*, double, long long, const LzGeom&, const DevScalars*, int, \
                                   double*, cudaStream_t);
INST_LZ(float)
INST_LZ(double)

}  // namespace gpe

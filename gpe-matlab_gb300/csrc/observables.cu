// observables.cu - observables evaluated on the device at callbacks:
// vortex-core detection on a 2D slice of the state (lib/util/detect_core.m of
// GPE-MATLAB) and the Thomas-Fermi initial guess (lib/@GPEtask/
// groundstate_tf.m).  Both are off the split-step hot path; they read the
// state where it lies instead of copying it to the host.
//
// Slice layout: nx columns (x) by ny rows (y), point (ix, iy) at
// base + iy + ny*ix, which is MATLAB's column-major order of the ny x nx
// slice, so the order of find() is the linear index order here.
#include "aux_kernels.cuh"

namespace gpe {

constexpr int OB_T = 256;           // threads per CTA
constexpr int CORE_CHUNK = 4 * OB_T;  // slice points per compaction chunk

template <typename R>
__device__ __forceinline__ double dens(const cx<R>* s, int ny, int ix, int iy) {
  const cx<R> p = s[iy + (long long)ny * ix];
  return (double)p.x * (double)p.x + (double)p.y * (double)p.y;
}

// One dimension of MATLAB's del2: the central second difference of n at
// interior k, linear extrapolation at k = 0 and k = n-1 (n > 3).
template <typename F>
__device__ __forceinline__ double d2_extrap(F f, int k, int n) {
  auto c = [&](int j) { return f(j + 1) - 2.0 * f(j) + f(j - 1); };
  if (k == 0) return 2.0 * c(1) - c(2);
  if (k == n - 1) return 2.0 * c(n - 2) - c(n - 3);
  return c(k);
}

// |del2(|psi|^2, hx, hy)| at (ix, iy) (detect_core.m:18), times 4.
template <typename R>
__device__ __forceinline__ double ddphi(const cx<R>* s, int nx, int ny, int ix, int iy, double hx2, double hy2) {
  const double dxx = d2_extrap([&](int j) { return dens<R>(s, ny, j, iy); }, ix, nx) / hx2;
  const double dyy = d2_extrap([&](int j) { return dens<R>(s, ny, ix, j); }, iy, ny) / hy2;
  return fabs(dxx + dyy);
}

template <typename R>
__global__ void __launch_bounds__(OB_T) k_core_ddmax(const cx<R>* s, int nx, int ny, double hx2, double hy2,
                                                    double* blockmax) {
  double m = 0.0;
  const long long n = (long long)nx * ny;
  for (long long L = (long long)blockIdx.x * OB_T + threadIdx.x; L < n; L += (long long)gridDim.x * OB_T)
    m = fmax(m, ddphi<R>(s, nx, ny, (int)(L / ny), (int)(L % ny), hx2, hy2));
  __shared__ double sh[OB_T];
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int o = OB_T / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) blockmax[blockIdx.x] = sh[0];
}

// thr = 0.01 * max(ddphi) (detect_core.m:25).
__global__ void k_core_thr(const double* blockmax, int nb, double* thr) {
  __shared__ double sh[OB_T];
  double m = 0.0;
  for (int i = threadIdx.x; i < nb; i += OB_T) m = fmax(m, blockmax[i]);
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int o = OB_T / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *thr = 0.01 * sh[0];
}

// res1 of detect_core.m:19-25 at every slice point: the phase winding around
// the plaquette with corners (i,j), (i-1,j), (i-1,j-1), (i,j-1) in MATLAB's
// (row = y, column = x) indices, circular, where ddphi > thr; and per chunk
// of CORE_CHUNK consecutive points the counts of positive and negative ones.
template <typename R>
__global__ void __launch_bounds__(OB_T) k_core_charge(const cx<R>* s, int nx, int ny, double hx2, double hy2,
                                                     const double* thr, signed char* q, int* cnt) {
  const long long n = (long long)nx * ny;
  const double t = *thr;
  __shared__ int cp, cm;
  if (threadIdx.x == 0) cp = cm = 0;
  __syncthreads();
  int mp = 0, mm = 0;
  for (int r = 0; r < CORE_CHUNK / OB_T; ++r) {
    const long long L = (long long)blockIdx.x * CORE_CHUNK + r * OB_T + threadIdx.x;
    if (L >= n) break;
    const int ix = (int)(L / ny), iy = (int)(L % ny);
    const int ixm = ix == 0 ? nx - 1 : ix - 1, iym = iy == 0 ? ny - 1 : iy - 1;
    auto ang = [&](int a, int b) {
      const cx<R> p = s[b + (long long)ny * a];
      return atan2((double)p.y, (double)p.x);  // angle(phi)
    };
    const double a0 = ang(ix, iy), a1 = ang(ix, iym), a2 = ang(ixm, iym), a3 = ang(ixm, iy);
    const double d[4] = {a0 - a3, a1 - a0, a2 - a1, a3 - a2};  // angs - circshift(angs,[0 0 1])
    int c = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) c += (d[k] > M_PI) - (d[k] < -M_PI);
    if (c != 0 && !(ddphi<R>(s, nx, ny, ix, iy, hx2, hy2) > t)) c = 0;
    q[L] = (signed char)c;
    mp += c > 0;
    mm += c < 0;
  }
  if (mp) atomicAdd(&cp, mp);
  if (mm) atomicAdd(&cm, mm);
  __syncthreads();
  if (threadIdx.x == 0) {
    cnt[2 * blockIdx.x] = cp;
    cnt[2 * blockIdx.x + 1] = cm;
  }
}

// Exclusive prefix sums of the chunk counts (one CTA, chunk order), totals
// at off[2*nchunk], off[2*nchunk+1].
__global__ void k_core_scan(const int* cnt, int nchunk, int* off) {
  if (threadIdx.x != 0) return;
  int sp = 0, sm = 0;
  for (int c = 0; c < nchunk; ++c) {
    off[2 * c] = sp;
    off[2 * c + 1] = sm;
    sp += cnt[2 * c];
    sm += cnt[2 * c + 1];
  }
  off[2 * nchunk] = sp;
  off[2 * nchunk + 1] = sm;
}

// refine_core (detect_core.m:51-66, after C.L. Phillips et al., Phys. Rev. E
// 91, 023311 (2015)) at 0-based (row r, column c), already clamped to >= 1:
// the generalized eigenproblem A v = lambda B v of the bilinear model of the
// plaquette, solved in closed form; the first root (in ascending order) with
// lambda and v1/v2 in (0, 1) gives [x - hy*lambda, y - hx*v1/v2].  No such
// (real) root: [0, 0].
template <typename R>
__device__ void refine_core(const cx<R>* s, int ny, int r, int c, double xc, double yc, double hx, double hy,
                            double* out) {
  auto P = [&](int rr, int cc) { return s[rr + (long long)ny * cc]; };
  const cx<R> prc = P(r, c), pr1c = P(r - 1, c), prc1 = P(r, c - 1), pr1c1 = P(r - 1, c - 1);
  const double A11 = -((double)pr1c.x - prc.x), A12 = -(double)prc.x;
  const double A21 = -((double)pr1c.y - prc.y), A22 = -(double)prc.y;
  const double B11 = (double)prc.x - pr1c.x - prc1.x + pr1c1.x, B12 = (double)prc1.x - prc.x;
  const double B21 = (double)prc.y - pr1c.y - prc1.y + pr1c1.y, B22 = (double)prc1.y - prc.y;
  const double qa = B11 * B22 - B12 * B21;
  const double qb = -(A11 * B22 + A22 * B11 - A12 * B21 - A21 * B12);
  const double qc = A11 * A22 - A12 * A21;
  double lam[2];
  int nl = 0;
  if (qa == 0.0) {
    if (qb != 0.0) lam[nl++] = -qc / qb;
  } else {
    const double disc = qb * qb - 4.0 * qa * qc;
    if (disc >= 0.0) {
      const double qq = -0.5 * (qb + copysign(sqrt(disc), qb));
      double l1 = qq / qa, l2 = qq != 0.0 ? qc / qq : l1;
      if (l2 < l1) {
        const double tmp = l1;
        l1 = l2;
        l2 = tmp;
      }
      lam[nl++] = l1;
      lam[nl++] = l2;
    }
  }
  out[0] = 0.0;
  out[1] = 0.0;
  for (int i = 0; i < nl; ++i) {
    const double l = lam[i];
    double num = -(A12 - l * B12), den = A11 - l * B11;
    if (num == 0.0 && den == 0.0) {
      num = -(A22 - l * B22);
      den = A21 - l * B21;
    }
    if (den == 0.0) continue;
    const double v = num / den;
    if (l > 0.0 && l < 1.0 && v > 0.0 && v < 1.0) {
      out[0] = xc - hy * l;
      out[1] = yc - hx * v;
      return;
    }
  }
}

// Writes the cores in chunk order (detect_core.m:29-47): [x - dx/2, y - dy/2]
// for positive and [x - dx/2, y - dx/2] for negative ones (the reference
// subtracts dx from y there), or the refined positions.
template <typename R>
__global__ void __launch_bounds__(OB_T) k_core_write(const cx<R>* s, int nx, int ny, const signed char* q,
                                                    const int* off, CoreGeom geo, double* pos, int cap_pos,
                                                    double* neg, int cap_neg) {
  const long long n = (long long)nx * ny;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ int wp[OB_T / 32], wm[OB_T / 32];
  int basep = off[2 * blockIdx.x], basem = off[2 * blockIdx.x + 1];
  for (int r = 0; r < CORE_CHUNK / OB_T; ++r) {
    const long long L = (long long)blockIdx.x * CORE_CHUNK + r * OB_T + threadIdx.x;
    const int c = L < n ? q[L] : 0;
    const unsigned bp = __ballot_sync(0xffffffffu, c > 0), bm = __ballot_sync(0xffffffffu, c < 0);
    if (lane == 0) {
      wp[warp] = __popc(bp);
      wm[warp] = __popc(bm);
    }
    __syncthreads();
    int op = basep, om = basem;
    for (int w = 0; w < warp; ++w) {
      op += wp[w];
      om += wm[w];
    }
    const unsigned lt = (1u << lane) - 1u;
    if (c != 0) {
      const int ix = (int)(L / ny), iy = (int)(L % ny);
      const double xc = geo.x0 + ix * geo.hxg, yc = geo.y0 + iy * geo.hyg;
      double xy[2];
      if (geo.refine) {
        const int rr = iy < 1 ? 1 : iy, cc = ix < 1 ? 1 : ix;
        refine_core<R>(s, ny, rr, cc, geo.x0 + cc * geo.hxg, geo.y0 + rr * geo.hyg, geo.hx, geo.hy, xy);
      } else {
        xy[0] = xc - geo.hx / 2;
        xy[1] = yc - (c > 0 ? geo.hy : geo.hx) / 2;
      }
      if (c > 0) {
        const int k = op + __popc(bp & lt);
        if (k < cap_pos) {
          pos[2 * k] = xy[0];
          pos[2 * k + 1] = xy[1];
        }
      } else {
        const int k = om + __popc(bm & lt);
        if (k < cap_neg) {
          neg[2 * k] = xy[0];
          neg[2 * k + 1] = xy[1];
        }
      }
    }
    for (int w = 0; w < OB_T / 32; ++w) {
      basep += wp[w];
      basem += wm[w];
    }
    __syncthreads();
  }
}

template <typename R>
cudaError_t launch_detect_core(const cx<R>* slice, int nx, int ny, const CoreGeom& geo, CoreScratch& w,
                               double* pos, int cap_pos, double* neg, int cap_neg, cudaStream_t st) {
  const long long n = (long long)nx * ny;
  const double hx2 = geo.hx * geo.hx, hy2 = geo.hy * geo.hy;
  const int nb = elem_grid(n, OB_T);
  k_core_ddmax<R><<<nb, OB_T, 0, st>>>(slice, nx, ny, hx2, hy2, w.blockmax);
  k_core_thr<<<1, OB_T, 0, st>>>(w.blockmax, nb, w.thr);
  const int nchunk = (int)((n + CORE_CHUNK - 1) / CORE_CHUNK);
  k_core_charge<R><<<nchunk, OB_T, 0, st>>>(slice, nx, ny, hx2, hy2, w.thr, w.q, w.cnt);
  k_core_scan<<<1, 32, 0, st>>>(w.cnt, nchunk, w.off);
  k_core_write<R><<<nchunk, OB_T, 0, st>>>(slice, nx, ny, w.q, w.off, geo, pos, cap_pos, neg, cap_neg);
  return cudaGetLastError();
}

int core_chunks(long long n) { return (int)((n + CORE_CHUNK - 1) / CORE_CHUNK); }

// ---- Thomas-Fermi guess (groundstate_tf.m) --------------------------------
__global__ void __launch_bounds__(OB_T) k_minmax(const double* V, long long n, double* out) {
  double lo = INFINITY, hi = -INFINITY;
  for (long long i = (long long)blockIdx.x * OB_T + threadIdx.x; i < n; i += (long long)gridDim.x * OB_T) {
    lo = fmin(lo, V[i]);
    hi = fmax(hi, V[i]);
  }
  __shared__ double a[OB_T], b[OB_T];
  a[threadIdx.x] = lo;
  b[threadIdx.x] = hi;
  __syncthreads();
  for (int o = OB_T / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      a[threadIdx.x] = fmin(a[threadIdx.x], a[threadIdx.x + o]);
      b[threadIdx.x] = fmax(b[threadIdx.x], b[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = a[0];
    out[2 * blockIdx.x + 1] = b[0];
  }
}

// sum((mu - V) .* (V < mu)) per CTA (groundstate_tf.m:26-27).
__global__ void __launch_bounds__(OB_T) k_tf_sum(const double* V, long long n, double mu, double* out) {
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * OB_T + threadIdx.x; i < n; i += (long long)gridDim.x * OB_T) {
    const double v = V[i];
    if (v < mu) acc += mu - v;
  }
  __shared__ double sh[OB_T];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = OB_T / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// phi = sqrt(vvv / g) (groundstate_tf.m:37), imaginary part 0.
template <typename R>
__global__ void __launch_bounds__(OB_T) k_tf_state(cx<R>* psi, const double* V, long long n, double mu, double g) {
  for (long long i = (long long)blockIdx.x * OB_T + threadIdx.x; i < n; i += (long long)gridDim.x * OB_T) {
    const double v = V[i];
    psi[i] = mk<R>((R)sqrt((v < mu ? mu - v : 0.0) / g), R(0));
  }
}

int launch_minmax(const double* V, long long n, double* out, cudaStream_t st) {
  const int nb = elem_grid(n, OB_T);
  k_minmax<<<nb, OB_T, 0, st>>>(V, n, out);
  return nb;
}
int launch_tf_sum(const double* V, long long n, double mu, double* out, cudaStream_t st) {
  const int nb = elem_grid(n, OB_T);
  k_tf_sum<<<nb, OB_T, 0, st>>>(V, n, mu, out);
  return nb;
}
template <typename R>
void launch_tf_state(cx<R>* psi, const double* V, long long n, double mu, double g, cudaStream_t st) {
  k_tf_state<R><<<elem_grid(n, OB_T), OB_T, 0, st>>>(psi, V, n, mu, g);
}

#define INST_OBS(R)                                                                                      \
  template cudaError_t launch_detect_core<R>(const cx<R>*, int, int, const CoreGeom&, CoreScratch&, double*, \
                                             int, double*, int, cudaStream_t);                           \
  template void launch_tf_state<R>(cx<R>*, const double*, long long, double, double, cudaStream_t);
INST_OBS(float)
INST_OBS(double)

}  // namespace gpe

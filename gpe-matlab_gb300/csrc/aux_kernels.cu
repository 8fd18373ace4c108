// aux_kernels.cu - finalizers (the scalar logic of solve_split and
// groundstate_itp, run on the device so blocks of steps need no host round
// trip), grid reductions and elementwise conversions.
#include <math.h>

#include <mutex>
#include <vector>

#include <cudaTypedefs.h>

#include "aux_kernels.cuh"

namespace gpe {

static int g_sm_count = 0;

int device_sm_count() {
  if (g_sm_count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 152;
  }
  return g_sm_count;
}

int elem_grid(long long n, int threads) {
  device_sm_count();
  long long want = (n + threads - 1) / threads;
  long long cap = (long long)g_sm_count * 8;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

constexpr int FIN_THREADS = 256;

// Deterministic block-wide Kahan sums of K arrays p[k][0..n[k]) by
// FIN_THREADS threads in one sweep (the K chains interleave, so the loads of
// all arrays are in flight together); fixed-order warp and CTA combination.
// Every thread returns the K sums.
template <int K>
__device__ void block_sums(const double* const* p, const int* n, double* out) {
  __shared__ double sh[K][FIN_THREADS / 32];
  double s[K], c[K];
  int nmax = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    s[k] = c[k] = 0.0;
    nmax = n[k] > nmax ? n[k] : nmax;
  }
  for (int i = threadIdx.x; i < nmax; i += FIN_THREADS) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (i < n[k]) {
        const double y = __ldcg(p[k] + i) - c[k];  // written by other CTAs: read from L2
        const double t = s[k] + y;
        c[k] = (t - s[k]) - y;
        s[k] = t;
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = s[k] - c[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k][warp] = x;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double r = 0.0;
    for (int w = 0; w < FIN_THREADS / 32; ++w) r += sh[k][w];
    out[k] = r;
  }
  __syncthreads();
}

__device__ double block_sum(const double* p, int n) {
  double r;
  block_sums<1>(&p, &n, &r);
  return r;
}

__device__ double block_max(const double* p, int n) {
  __shared__ double sh[FIN_THREADS];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += FIN_THREADS) m = fmax(m, p[i]);
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int o = FIN_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ void flag_nonfinite(DevScalars* sc) {
  sc->nonfinite = 1;
  sc->status = NONFINITE;
  sc->stop = 1;
}

// solve_split.m:65-78 for one block.
// Up to FIN_GRID CTAs (one per FIN_CHUNK partials of the longest slot): CTA b
// sums chunk b of every slot's partials; the last CTA to finish sums the
// chunk results (fixed chunking and order: deterministic) and runs the
// scalar logic.  Spreading the FP64 Kahan sums over SMs keeps the finalizer
// short on a GPU whose FP64 rate per SM is low; small grids use one CTA.
constexpr int FIN_GRID = 32;
constexpr int FIN_CHUNK = 256;

__global__ void k_finalize_block(const BlockFinalArgs a, DevScalars* sc) {
  // programmatic dependent launch (see the pass kernel): let the next pass be
  // scheduled now, read nothing before the previous kernel has completed
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (sc->stop) return;  // set only by earlier kernels: the same for every CTA
  const int cap = a.cap;
  const double* p[6] = {a.partials + S_N * cap,        a.partials + S_VN * cap,       a.partials + S_N2 * cap,
                        a.partials + (S_KX + 0) * cap, a.partials + (S_KX + 1) * cap, a.partials + (S_KX + 2) * cap};
  const int cnt[6] = {a.nblk_epi, a.nblk_epi, a.nblk_epi, a.nblk_kin[0], a.nblk_kin[1], a.nblk_kin[2]};
  const double* pc[6];
  int nc[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int chunk = (cnt[k] + (int)gridDim.x - 1) / (int)gridDim.x;
    const int lo = min(cnt[k], (int)blockIdx.x * chunk), hi = min(cnt[k], lo + chunk);
    pc[k] = p[k] + lo;
    nc[k] = hi - lo;
  }
  double sums[6];
  block_sums<6>(pc, nc, sums);
  // [6][FIN_GRID] chunk sums, in the buffer's scratch slot (the slots read
  // above stay read-only)
  double* scratch = const_cast<double*>(a.partials) + (size_t)S_FIN * cap;
  __shared__ int last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 6; ++k) scratch[k * FIN_GRID + blockIdx.x] = sums[k];
    __threadfence();
    last = atomicAdd(&sc->fin_count, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const double* q[6];
  int nq[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    q[k] = scratch + k * FIN_GRID;
    nq[k] = (int)gridDim.x;
  }
  block_sums<6>(q, nq, sums);
  if (threadIdx.x == 0) sc->fin_count = 0;
  const double n = sums[0], vn = sums[1], n2 = sums[2];
  const double kin = sums[3] + sums[4] + sums[5];  // axes without a pass contribute 0
  if (threadIdx.x != 0) return;
  const double w = a.weight;
  const double ncur = n * w;  // solve_split.m:67
  double muc, scale = 1.0, energy = 0.0;
  if (a.feedback) {  // solve_split.m:68-75
    double NNN = sc->NNN;
    if (a.tau > 0) NNN = sc->NN0 * exp(-a.time2 / a.tau);
    sc->NNN = NNN;
    scale = sqrt(NNN / ncur);
    const double s2 = scale * scale;
    muc = (s2 * (kin + vn) * w + s2 * s2 * a.g * n2 * w) / NNN;
    energy = s2 * (kin + vn) * w + 0.5 * s2 * s2 * a.g * n2 * w;  // of the renormalised state
    sc->mu = muc;
  } else if (a.fixed_mu) {  // SGPEtask solve_split.m:52,78
    muc = sc->mu;
  } else {  // solve_split.m:76-77
    muc = (kin + vn + a.g * n2) * w / ncur;
    energy = (kin + vn + 0.5 * a.g * n2) * w;
  }
  sc->energy = energy;
  sc->scale = scale;
  sc->ncur = ncur;
  sc->muc = muc;
  sc->sums[S_N] = n * w;
  sc->sums[S_VN] = vn * w;
  sc->sums[S_N2] = n2 * w;
  if (!isfinite(ncur) || !isfinite(muc) || !isfinite(scale)) flag_nonfinite(sc);
  if (a.hist_mu) {
    *a.hist_mu = muc;
    *a.hist_n = ncur;
    if (a.hist_ok) *a.hist_ok = 1;
    if (a.hist_e) *a.hist_e = a.fixed_mu ? NAN : energy;
  }
}

// groundstate_itp.m:44-52 for one iteration.
__global__ void k_finalize_itp(const ItpFinalArgs a, DevScalars* sc) {
  if (sc->stop) return;
  const double n = block_sum(a.partials + S_N * a.cap, a.nblk) * a.weight;
  if (threadIdx.x != 0) return;
  double m, MU;
  if (a.Ntotal > 0) {
    m = sqrt(a.Ntotal / n);
    MU = log(m) / a.dt;
  } else {
    m = exp(a.mu_init * a.dt);
    MU = n * m * m;
  }
  sc->scale = m;
  sc->ncur = n;
  sc->iter = a.iter;
  sc->mu_itp = MU;
  a.MU[a.iter - 1] = MU;
  if (!isfinite(n) || !isfinite(m) || n <= 0.0) flag_nonfinite(sc);
}

// groundstate_itp.m:54-74 at a check iteration.
__global__ void k_finalize_check(const CheckFinalArgs a, DevScalars* sc) {
  if (sc->stop) return;
  const int cap = a.cap;
  const double maxd = block_max(a.partials + S_MAXD * cap, a.nblk_check);
  const double maxa = block_max(a.partials + S_MAXA * cap, a.nblk_check);
  double vn = 0.0, n2 = 0.0, kin = 0.0;
  if (a.nblk_pot > 0) {
    vn = block_sum(a.partials + S_VN * cap, a.nblk_pot);
    n2 = block_sum(a.partials + S_N2 * cap, a.nblk_pot);
  }
  for (int ax = 0; ax < 3; ++ax)
    if (a.nblk_kin[ax] > 0) kin += block_sum(a.partials + (S_KX + ax) * cap, a.nblk_kin[ax]);
  if (threadIdx.x != 0) return;
  const int i = a.iter - 1;
  const double w = a.weight;
  double mu2 = 0.0;
  if (a.nblk_pot > 0) {
    mu2 = (kin + vn + a.g * n2) * w;  // real(inner(phi, applyham(phi)))
    a.MU2[i] = mu2;
    a.EE[i] = (kin + vn + 0.5 * a.g * n2) * w;  // get_energy, GPEtask.m:97-107
    sc->mu2 = mu2;
    sc->ee = a.EE[i];
  }
  const double delta = maxd / (a.dt * 10.0);  // groundstate_itp.m:61
  sc->delta = delta;
  sc->maxabs = maxa;
  if (!isfinite(delta)) {
    flag_nonfinite(sc);
    return;
  }
  if (delta < a.eps) {  // groundstate_itp.m:63-72
    if (a.want_mu2) sc->dtmin = a.dt * sqrt(a.eps / fabs(a.MU[i] - a.MU2[i] / a.nnn));
    sc->stop = 1;
    sc->status = (!a.adjust || a.dt < sc->dtmin) ? CONVERGED : HALVE_DT;
    return;
  }
  if (a.fp32_phase) {
    // FP32 rounding puts a floor under delta (a few ulps of max|psi| per
    // 10*dt); leave the FP32 phase once below switch_delta or on a stall.
    if (delta < a.switch_delta) {
      sc->stop = 1;
      sc->status = SWITCH_FP64;
      return;
    }
    if (delta < 0.9 * sc->best_delta) {
      sc->best_delta = delta;
      sc->stall = 0;
    } else if (++sc->stall >= 3) {
      sc->stop = 1;
      sc->status = SWITCH_FP64;
    }
  }
}

// Observables / initial mu of solve_split (solve_split.m:41-46).
__global__ void k_finalize_obs(const ObsFinalArgs a, DevScalars* sc) {
  const int cap = a.cap;
  const double n = block_sum(a.partials + S_N * cap, a.nblk_pot);
  const double vn = block_sum(a.partials + S_VN * cap, a.nblk_pot);
  const double n2 = block_sum(a.partials + S_N2 * cap, a.nblk_pot);
  double k[3] = {0.0, 0.0, 0.0};
  for (int ax = 0; ax < 3; ++ax)
    if (a.nblk_kin[ax] > 0) k[ax] = block_sum(a.partials + (S_KX + ax) * cap, a.nblk_kin[ax]);
  if (threadIdx.x != 0) return;
  const double w = a.weight;
  sc->sums[S_N] = n * w;
  sc->sums[S_VN] = vn * w;
  sc->sums[S_N2] = n2 * w;
  sc->sums[S_KX] = k[0] * w;
  sc->sums[S_KY] = k[1] * w;
  sc->sums[S_KZ] = k[2] * w;
  if (a.div != 0.0) {
    const double muc = (k[0] + k[1] + k[2] + vn + a.g * n2) * w / a.div;
    sc->muc = muc;
    if (a.set_mu) sc->mu = a.mu_init > 0 ? a.mu_init : muc;
  }
}

__global__ void k_finalize_norm0(const double* partials, int cap, int nblk, double weight, double Ntotal,
                                 DevScalars* sc) {
  const double n = block_sum(partials + S_N * cap, nblk) * weight;
  if (threadIdx.x != 0) return;
  sc->ncur = n;
  sc->sums[S_N] = n;
  if (Ntotal > 0) {
    // process_init_state: sqrt(Ntotal)*normalize(phi0) (GPEtask.m:159-160,
    // normalize.m:13-15, norm.m:11).  The stored state already carries the
    // pending factor sc->scale, which norm() included.
    sc->scale = sc->scale * (sqrt(Ntotal) * (1.0 / sqrt(n)));
    if (!isfinite(sc->scale) || n <= 0.0) flag_nonfinite(sc);
  }
}

__global__ void k_reset_scalars(DevScalars* sc) {
  sc->stop = 0;
  sc->status = RUNNING;
  sc->nonfinite = 0;
  sc->timeout = 0;
  sc->bounds_site = 0;
  sc->bounds_index = 0;
  sc->stall = 0;
  sc->best_delta = INFINITY;
}

__global__ void k_set_scale_one(DevScalars* sc) {
  sc->scale = 1.0;
  sc->scale2 = 1.0;
}

void launch_finalize_block(const BlockFinalArgs& a, DevScalars* sc, cudaStream_t s) {
  int longest = a.nblk_epi;
  for (int ax = 0; ax < 3; ++ax) longest = a.nblk_kin[ax] > longest ? a.nblk_kin[ax] : longest;
  int grid = (longest + FIN_CHUNK - 1) / FIN_CHUNK;
  grid = grid < 1 ? 1 : grid > FIN_GRID ? FIN_GRID : grid;
  if (!a.pdl) {
    k_finalize_block<<<grid, FIN_THREADS, 0, s>>>(a, sc);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(FIN_THREADS);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_finalize_block, a, sc);
}
void launch_finalize_itp(const ItpFinalArgs& a, DevScalars* sc, cudaStream_t s) {
  k_finalize_itp<<<1, FIN_THREADS, 0, s>>>(a, sc);
}
void launch_finalize_check(const CheckFinalArgs& a, DevScalars* sc, cudaStream_t s) {
  k_finalize_check<<<1, FIN_THREADS, 0, s>>>(a, sc);
}
void launch_finalize_obs(const ObsFinalArgs& a, DevScalars* sc, cudaStream_t s) {
  k_finalize_obs<<<1, FIN_THREADS, 0, s>>>(a, sc);
}
void launch_finalize_norm0(const double* partials, int cap, int nblk, double weight, double Ntotal,
                           DevScalars* sc, cudaStream_t s) {
  k_finalize_norm0<<<1, FIN_THREADS, 0, s>>>(partials, cap, nblk, weight, Ntotal, sc);
}
void launch_reset_scalars(DevScalars* sc, cudaStream_t s) { k_reset_scalars<<<1, 1, 0, s>>>(sc); }
void launch_set_scale_one(DevScalars* sc, cudaStream_t s) { k_set_scale_one<<<1, 1, 0, s>>>(sc); }

// ---- grid reductions and elementwise kernels ------------------------------
constexpr int EL_THREADS = 256;

template <typename R>
__device__ __forceinline__ void block_store2(double a, double b, double* pa, double* pb, bool is_max) {
  __shared__ double sh[2][EL_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double xa = __shfl_down_sync(0xffffffffu, a, o);
    double xb = __shfl_down_sync(0xffffffffu, b, o);
    a = is_max ? fmax(a, xa) : a + xa;
    b = is_max ? fmax(b, xb) : b + xb;
  }
  if (lane == 0) {
    sh[0][warp] = a;
    sh[1][warp] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ra = sh[0][0], rb = sh[1][0];
    for (int w = 1; w < EL_THREADS / 32; ++w) {
      ra = is_max ? fmax(ra, sh[0][w]) : ra + sh[0][w];
      rb = is_max ? fmax(rb, sh[1][w]) : rb + sh[1][w];
    }
    if (pa) pa[blockIdx.x] = ra;
    if (pb) pb[blockIdx.x] = rb;
  }
}

template <typename R>
__global__ void k_norm(const cx<R>* __restrict__ psi, long long n, const DevScalars* sc, double* partials,
                       int cap) {
  const R s = (R)sc->scale;
  double tot = 0.0;
  for (long long i0 = (long long)blockIdx.x * EL_THREADS * 16; i0 < n; i0 += (long long)gridDim.x * EL_THREADS * 16) {
    R acc = R(0), c = R(0);
    for (int k = 0; k < 16; ++k) {
      long long i = i0 + threadIdx.x + (long long)k * EL_THREADS;
      if (i < n) {
        cx<R> p = psi[i];
        R y = (p.x * p.x + p.y * p.y) * s * s - c;
        R t = acc + y;
        c = (t - acc) - y;
        acc = t;
      }
    }
    tot += (double)acc - (double)c;
  }
  block_store2<R>(tot, 0.0, partials + S_N * cap, nullptr, false);
}

template <typename R>
__global__ void k_itp_check(const cx<R>* __restrict__ psi, R* __restrict__ absprev, long long n,
                            const DevScalars* sc, double* partials, int cap) {
  if (sc->stop) return;
  const R s = (R)sc->scale;
  double md = 0.0, ma = 0.0;
  for (long long i = (long long)blockIdx.x * EL_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * EL_THREADS) {
    cx<R> p = psi[i];
    R a = sqrt(p.x * p.x + p.y * p.y) * s;
    R d = fabs(a - absprev[i]);  // groundstate_itp.m:61
    absprev[i] = a;              // groundstate_itp.m:62
    md = fmax(md, (double)d);
    ma = fmax(ma, (double)a);
  }
  block_store2<R>(md, ma, partials + S_MAXD * cap, partials + S_MAXA * cap, true);
}

template <typename R>
__global__ void k_abs_init(const cx<R>* __restrict__ psi, R* __restrict__ absprev, long long n,
                           const DevScalars* sc) {
  const R s = (R)sc->scale;
  for (long long i = (long long)blockIdx.x * EL_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * EL_THREADS) {
    cx<R> p = psi[i];
    absprev[i] = sqrt(p.x * p.x + p.y * p.y) * s;
  }
}

template <typename R>
__global__ void k_apply_scale(cx<R>* __restrict__ psi, long long n, const DevScalars* sc) {
  const double sd = sc->scale;
  if (sd == 1.0) return;
  const R s = (R)sd;
  for (long long i = (long long)blockIdx.x * EL_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * EL_THREADS) {
    cx<R> p = psi[i];
    psi[i] = mk<R>(p.x * s, p.y * s);
  }
}

template <typename RI, typename RO>
__global__ void k_convert_cx(const cx<RI>* __restrict__ in, cx<RO>* __restrict__ out, long long n,
                             const DevScalars* sc) {
  const double s = sc ? sc->scale : 1.0;
  for (long long i = (long long)blockIdx.x * EL_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * EL_THREADS) {
    cx<RI> p = in[i];
    if (s == 1.0) {
      out[i] = mk<RO>((RO)p.x, (RO)p.y);
    } else {
      out[i] = mk<RO>((RO)((double)p.x * s), (RO)((double)p.y * s));
    }
  }
}

template <typename RI, typename RO>
__global__ void k_convert_re(const RI* __restrict__ in, RO* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * EL_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * EL_THREADS)
    out[i] = (RO)in[i];
}

template <typename R>
int launch_norm(const cx<R>* psi, long long n, DevScalars* sc, double* partials, int cap, cudaStream_t s) {
  int grid = (int)((n + EL_THREADS * 16 - 1) / (EL_THREADS * 16));
  int lim = elem_grid(n, EL_THREADS);
  if (grid > lim) grid = lim;
  if (grid > cap) grid = cap;
  k_norm<R><<<grid, EL_THREADS, 0, s>>>(psi, n, sc, partials, cap);
  return grid;
}
template <typename R>
int launch_itp_check(const cx<R>* psi, R* absprev, long long n, DevScalars* sc, double* partials, int cap,
                     cudaStream_t s) {
  int grid = elem_grid(n, EL_THREADS);
  if (grid > cap) grid = cap;
  k_itp_check<R><<<grid, EL_THREADS, 0, s>>>(psi, absprev, n, sc, partials, cap);
  return grid;
}
template <typename R>
void launch_abs_init(const cx<R>* psi, R* absprev, long long n, DevScalars* sc, cudaStream_t s) {
  k_abs_init<R><<<elem_grid(n, EL_THREADS), EL_THREADS, 0, s>>>(psi, absprev, n, sc);
}
template <typename R>
void launch_apply_scale(cx<R>* psi, long long n, DevScalars* sc, cudaStream_t s) {
  k_apply_scale<R><<<elem_grid(n, EL_THREADS), EL_THREADS, 0, s>>>(psi, n, sc);
}
template <typename RI, typename RO>
void launch_convert_cx(const cx<RI>* in, cx<RO>* out, long long n, const DevScalars* sc, cudaStream_t s) {
  k_convert_cx<RI, RO><<<elem_grid(n, EL_THREADS), EL_THREADS, 0, s>>>(in, out, n, sc);
}
template <typename RI, typename RO>
void launch_convert_re(const RI* in, RO* out, long long n, cudaStream_t s) {
  k_convert_re<RI, RO><<<elem_grid(n, EL_THREADS), EL_THREADS, 0, s>>>(in, out, n);
}

#define INST_R(R)                                                                                         \
  template int launch_norm<R>(const cx<R>*, long long, DevScalars*, double*, int, cudaStream_t);         \
  template int launch_itp_check<R>(const cx<R>*, R*, long long, DevScalars*, double*, int, cudaStream_t); \
  template void launch_abs_init<R>(const cx<R>*, R*, long long, DevScalars*, cudaStream_t);              \
  template void launch_apply_scale<R>(cx<R>*, long long, DevScalars*, cudaStream_t);
INST_R(float)
INST_R(double)
#define INST_CONV(RI, RO)                                                                                 \
  template void launch_convert_cx<RI, RO>(const cx<RI>*, cx<RO>*, long long, const DevScalars*,          \
                                          cudaStream_t);                                                  \
  template void launch_convert_re<RI, RO>(const RI*, RO*, long long, cudaStream_t);
INST_CONV(float, float)
INST_CONV(float, double)
INST_CONV(double, float)
INST_CONV(double, double)

}  // namespace gpe

namespace gpe {
// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on the driver library).
bool encode_tile_map(CUtensorMap* m, const void* base, int unit, int units, const long long* tdim, int pencils,
                     int ax, int len) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool looked = false;
  static std::mutex mu;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!looked) {
      looked = true;
      void* p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
              cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
        fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
      else
        (void)cudaGetLastError();
    }
  }
  if (!fn) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)(units * tdim[0]), (cuuint64_t)tdim[1], (cuuint64_t)tdim[2],
                              (cuuint64_t)tdim[3]};
  const cuuint64_t row = (cuuint64_t)(units * unit) * (cuuint64_t)tdim[0];
  const cuuint64_t strides[3] = {row, row * (cuuint64_t)tdim[1], row * (cuuint64_t)tdim[1] * (cuuint64_t)tdim[2]};
  const cuuint32_t box[4] = {(cuuint32_t)(units * pencils), (cuuint32_t)(ax == 1 ? len : 1),
                             (cuuint32_t)(ax == 2 ? len : 1), 1u};
  const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
  const CUtensorMapDataType dt = unit == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  return fn(m, dt, 4, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

// Occupancy cache for the TMA passes (host side).
int resident_ctas(const void* kern, int threads, size_t smem) {
  struct Key {
    const void* k;
    size_t smem;
    int dev;
    int val;
  };
  static std::mutex mu;
  static std::vector<Key> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  for (auto& e : cache)
    if (e.k == kern && e.smem == smem && e.dev == dev) return e.val;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem) != cudaSuccess) n = 1;
  cache.push_back({kern, smem, dev, n});
  return n;
}
}  // namespace gpe

namespace gpe {
// Self-test of the FP32 device trigonometry used by the phase factors.
__global__ void k_selftest_trig(const float* x, float* s, float* c, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    sincos_bounded(x[i], &s[i], &c[i]);
}
cudaError_t launch_selftest_trig(const float* x, float* s, float* c, long long n, cudaStream_t st) {
  k_selftest_trig<<<elem_grid(n, 256), 256, 0, st>>>(x, s, c, n);
  return cudaGetLastError();
}
}  // namespace gpe

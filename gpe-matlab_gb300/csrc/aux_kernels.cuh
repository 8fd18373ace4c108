// aux_kernels.cuh - declarations of the elementwise, reduction and
// finalizer kernels (aux_kernels.cu) used by the host drivers.
#pragma once
#include "common.cuh"

namespace gpe {

// Grid of the elementwise kernels: a multiple of the SM count.
int elem_grid(long long n, int threads);

// Per-block finalizer of solve_split (solve_split.m:65-78).
struct BlockFinalArgs {
  const double* partials;
  int cap;
  int nblk_epi;          // CTAs of the block-end pass (slots n, Vn, n2)
  int nblk_kin[3];       // CTAs of the kinetic-energy passes (x, y, z), 0 = skipped
  double weight, g;
  int feedback;          // gamma > 0 && mu_init == 0
  double tau, time2;
  double* hist_mu;       // nullptr or &history[j]
  double* hist_n;
  int* hist_ok;
  int fixed_mu = 0;      // report sc->mu (the stochastic GPE's mu_init) instead of <psi|H psi>/N
  double* hist_e = nullptr;  // get_energy of the block-end state (GPEtask.m:97-107), or nullptr
  int pdl = 0;               // launch with programmatic stream serialisation
};

struct ItpFinalArgs {
  const double* partials;
  int cap, nblk;
  double weight, dt, Ntotal, mu_init;
  int iter;              // 1-based iteration index
  double* MU;
};

struct CheckFinalArgs {
  const double* partials;
  int cap;
  int nblk_check;        // CTAs of itp_check (slots maxd, maxa)
  int nblk_pot;          // CTAs of the energy y pass with potential sums (0 = none)
  int nblk_kin[3];
  double weight, g, dt, eps, nnn;
  int iter;
  int want_mu2;
  int adjust;
  int fp32_phase;        // 1: end the phase on delta < switch_delta or a stall
  double switch_delta;
  const double* MU;
  double* MU2;
  double* EE;
};

struct ObsFinalArgs {
  const double* partials;
  int cap, nblk_pot;
  int nblk_kin[3];
  double weight, g;
  double div;            // muc = mu_integral / div (0: not stored)
  int set_mu;            // also set sc->mu (solve_split.m:42-46)
  double mu_init;
};

// Two-component (spinor) split step, spinor_kernels.cu.
template <typename R>
struct SpinorNL {
  R g11, g12, g21, g22;         // interaction matrix
  R dre, dim;                   // complex time step dt
  cx<R> cosom, sinomm, sinomp;  // step-constant coupling factors (nl == 0)
  int nl;                       // nlincpl != 0: per-point factors of cre + i cim + nlincpl*n
  R nlincpl, cre, cim;
};
constexpr int SP_NSUMS = 9;     // n1 n2 V1n1 V2n2 n1^2 n2^2 n1n2 Re/Im conj(psi1)psi2
struct SpinorFinalArgs {
  const double* sums;           // [SP_NSUMS][nsum] partials of launch_spinor_sums
  int nsum;
  const double* partials;       // kinetic partials (slots S_KX..S_KZ)
  int cap;
  int nblk_kin[3];
  double weight;
  double g[4];
  double cre, cim;
  int mode;                     // 0: run start, 1: block end, 2: observables, 3: ITP (MU2 -> hist, EE -> obs)
  double Ntotal;                // mode 0
  int renorm;                   // mode 1: gamma > 0
  double tau, time2;
  double* hist;                 // mode 1: (mu, ncur, energy) or nullptr
  double* obs;                  // mode 2: norm, ekin, epot, eint, ecpl
};
template <typename R>
void launch_spinor_nl(cx<R>* psi, const R* V, long long P, const DevScalars* sc, int first, const SpinorNL<R>& q,
                      cudaStream_t s);
template <typename R>
int launch_spinor_sums(const cx<R>* psi, const R* V, long long P, const DevScalars* sc, double* out,
                       cudaStream_t s);
void launch_finalize_spinor(const SpinorFinalArgs& a, DevScalars* sc, cudaStream_t s);
// Spinor ITP: the factors exp(-(V_j + sum_k g(j,k) |psi_k|^2) dt) into f (2P)
// and, after the kinetic half step, the coupling rotation times them.
// `split`: component 2 carries its own pending factor scale2 (two-component ITP).
template <typename R>
void launch_spinor_itp_factors(const cx<R>* psi, const R* V, long long P, const DevScalars* sc, const SpinorNL<R>& q,
                               R* f, int split, cudaStream_t s);
template <typename R>
void launch_spinor_itp_couple(cx<R>* psi, const R* f, long long P, const DevScalars* sc, const SpinorNL<R>& q,
                              int split, cudaStream_t s);
// Incoherent two-component ITP (GPEtask2comp): per-component norms and factors.
struct MixFinalArgs {
  const double* part1;          // per-CTA sums of |psi_1|^2
  const double* part2;          // per-CTA sums of |psi_2|^2
  int nblk1, nblk2;
  double weight, dt, N1, N2;
  int iter;                     // 1-based iteration index
  double* MU1;
  double* MU2;
};
template <typename R>
void launch_mix_apply_scales(cx<R>* psi, long long P, const DevScalars* sc, cudaStream_t s);
void launch_finalize_mix(const MixFinalArgs& a, DevScalars* sc, cudaStream_t s);

// Array-omega angular momentum, lz_kernels.cu.
struct LzGeom {
  int nx, ny;       // slice size (z slices are independent)
  double h;         // derivative spacing (grid1d deriv1 with obj.dx for both axes)
  double x0, y0;    // coordinates of ix = 0, iy = 0
  double hxg, hyg;  // grid spacings of the coordinates
};
// out = phi + (cre + i cim) * omega * lz(src), omega = om[i] or the scalar
// oms when om is null; out may be phi, never src.
template <typename R>
void launch_lz_cn(cx<R>* out, const cx<R>* phi, const cx<R>* src, const R* om, double oms, long long n,
                  const LzGeom& g, double cre, double cim, cudaStream_t st);
// The block end of solve_split as an elementwise pass (the last step's full
// nonlinear factor, the inverse half step, sums n, Vn, n^2 per CTA into the
// partial slots): the pass epilogue EPI_RT_END for runs whose last kinetic
// pass cannot carry it.  Returns CTAs.
template <typename R>
int launch_rt_block_end(cx<R>* psi, const R* V, long long n, const DevScalars* sc, double g, double dre, double dim,
                        double* partials, int cap, cudaStream_t s);
// Per-CTA sums of real(conj(psi) (-omega lz psi)) (times scale^2 if use_scale),
// omega per point (om) or the scalar oms (om null); returns CTAs.
template <typename R>
int launch_lz_energy(const cx<R>* psi, const R* om, double oms, long long n, const LzGeom& g, const DevScalars* sc,
                     int use_scale, double* out, cudaStream_t st);

// On-device observables, observables.cu.
struct CoreGeom {
  double x0, y0;    // coordinates of column 0 and row 0 of the slice
  double hxg, hyg;  // grid spacings (coordinate of column ix = x0 + ix*hxg)
  double hx, hy;    // detect_core.m:13-14 spacings (del2 and the position offsets)
  int refine;
};
struct CoreScratch {
  double* blockmax;   // elem_grid(n) doubles
  double* thr;        // 1 double
  signed char* q;     // n charges
  int* cnt;           // 2 * chunks
  int* off;           // 2 * chunks + 2 (totals last)
};
int core_chunks(long long n);
template <typename R>
cudaError_t launch_detect_core(const cx<R>* slice, int nx, int ny, const CoreGeom& geo, CoreScratch& w,
                               double* pos, int cap_pos, double* neg, int cap_neg, cudaStream_t st);
int launch_minmax(const double* V, long long n, double* out, cudaStream_t st);
int launch_tf_sum(const double* V, long long n, double mu, double* out, cudaStream_t st);
template <typename R>
void launch_tf_state(cx<R>* psi, const double* V, long long n, double mu, double g, cudaStream_t st);

void launch_finalize_block(const BlockFinalArgs& a, DevScalars* sc, cudaStream_t s);
void launch_finalize_itp(const ItpFinalArgs& a, DevScalars* sc, cudaStream_t s);
void launch_finalize_check(const CheckFinalArgs& a, DevScalars* sc, cudaStream_t s);
void launch_finalize_obs(const ObsFinalArgs& a, DevScalars* sc, cudaStream_t s);
// scale = Ntotal > 0 ? sqrt(Ntotal / (sum_n*w)) : 1 (GPEtask.m:159-160); returns CTAs read.
void launch_finalize_norm0(const double* partials, int cap, int nblk, double weight, double Ntotal,
                           DevScalars* sc, cudaStream_t s);
void launch_reset_scalars(DevScalars* sc, cudaStream_t s);
void launch_set_scale_one(DevScalars* sc, cudaStream_t s);
cudaError_t launch_selftest_trig(const float* x, float* s, float* c, long long n, cudaStream_t st);

// Discrete adjoint pieces (adjoint_kernels.cu).
template <typename R>
void launch_nl_phase(cx<R>* psi, const R* V, long long n, double g, double h, cudaStream_t s);
template <typename R>
void launch_adj_nl(cx<R>* lam, const cx<R>* x, const R* V, double* dLdV, long long n, double g, double h,
                   int first, int second, int conj_in, int conj_out, cudaStream_t s);
template <typename R>
int launch_inner(const cx<R>* a, const cx<R>* b, long long n, double* partials, cudaStream_t s);
template <typename R>
void launch_cscale(cx<R>* out, const cx<R>* in, long long n, double cr, double ci, cudaStream_t s);

// Stochastic GPE nonlinear factor + noise (adjoint_kernels.cu).
template <typename R>
void launch_sgpe_nl_noise(cx<R>* psi, const R* V, long long n, DevScalars* sc, double g, double dre, double dim,
                          int half, double sigma, unsigned long long seed, unsigned long long step, cudaStream_t s);
cudaError_t launch_selftest_noise(float* out, long long n, unsigned long long seed, unsigned long long step,
                                  cudaStream_t s);

template <typename R>
int launch_norm(const cx<R>* psi, long long n, DevScalars* sc, double* partials, int cap, cudaStream_t s);
template <typename R>
int launch_itp_check(const cx<R>* psi, R* absprev, long long n, DevScalars* sc, double* partials, int cap,
                     cudaStream_t s);
template <typename R>
void launch_abs_init(const cx<R>* psi, R* absprev, long long n, DevScalars* sc, cudaStream_t s);
// psi *= sc->scale (in place); the caller resets the scale afterwards.
template <typename R>
void launch_apply_scale(cx<R>* psi, long long n, DevScalars* sc, cudaStream_t s);
// out = in (element type conversion), optionally times sc->scale.
template <typename RI, typename RO>
void launch_convert_cx(const cx<RI>* in, cx<RO>* out, long long n, const DevScalars* sc, cudaStream_t s);
template <typename RI, typename RO>
void launch_convert_re(const RI* in, RO* out, long long n, cudaStream_t s);

}  // namespace gpe

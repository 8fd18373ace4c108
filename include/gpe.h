/*
 * gpe.h - C ABI of libgpe, a GB300-native (sm_103a) split-step Fourier solver
 * for the Gross-Pitaevskii equation.  It is a drop-in for the hot path of
 * GPE-MATLAB's GPEtask.groundstate_itp / GPEtask.solve_split on grid2d/grid3d.
 *
 * Plain C types only: host buffers are caller-owned and copied in or out
 * before the call returns; device buffers, kernels, tables and the CUDA
 * stream are owned by the context.  Every call returns a gpe_status; the
 * message of the last failure is available from gpe_last_error().  No call
 * exits or aborts the process.
 *
 * Array layout is MATLAB's: ny x nx (x nz) column-major meshgrid arrays, so
 * element (iy, ix, iz) sits at linear index iy + ny*(ix + nx*iz)
 * (lib/@grid2d/init.m:30-34, lib/@grid3d/init.m:75-79 of GPE-MATLAB).
 * Complex arrays are interleaved (re, im) pairs, as MATLAB R2018a+ and
 * gpuArray store them.
 *
 * Threading: one context is used by one host thread at a time; separate
 * contexts may be used concurrently from different threads.
 */
#ifndef GPE_H
#define GPE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPE_ABI_VERSION 1

#if defined(__GNUC__)
#define GPE_API __attribute__((visibility("default")))
#else
#define GPE_API
#endif

typedef struct gpe_ctx gpe_ctx;

typedef enum {
    GPE_OK = 0,
    GPE_ERR_INVALID = 1,     /* bad argument: null pointer, size, parameter   */
    GPE_ERR_UNSUPPORTED = 2, /* e.g. an axis length without an FFT plan       */
    GPE_ERR_CUDA = 3,        /* CUDA runtime error (see gpe_last_error)       */
    GPE_ERR_ALLOC = 4,       /* device or pinned allocation failed            */
    GPE_ERR_STATE = 5,       /* call out of order (no potential, no state)    */
    GPE_ERR_TIMEOUT = 6,     /* a bounded device-side wait expired            */
    GPE_ERR_NONFINITE = 7,   /* NaN/Inf met in a reduction (norm, mu, delta)  */
    GPE_ERR_NO_DEVICE = 8,   /* no CUDA device, or not an sm_103 device       */
    GPE_ERR_CALLBACK = 9,    /* a host callback returned nonzero              */
    GPE_ERR_BOUNDS = 10      /* bounds-checked build only: a kernel index was
                              * out of range (the access was skipped)        */
} gpe_status;

enum { GPE_FP32 = 1, GPE_FP64 = 2 };

/* Grid: replaces grid2d(xmax,nx,ymax,ny) / grid3d(...) construction,
 * lib/@grid2d/init.m:1-38 and lib/@grid3d/init.m:1-47.  Per axis the caller
 * passes dx = x(2)-x(1) and span = x(end)-x(1) exactly as the MATLAB grid
 * computes them; the wave numbers are [0:n/2, -(n/2-1):-1]*2*pi/(span+dx)
 * (init.m:27-28) and the integration weight is prod(dx) (init.m:36). */
typedef struct {
    int ndims;        /* 2 (grid2d) or 3 (grid3d)                               */
    int n[3];         /* nx, ny, nz (nz ignored in 2D); even, 2^a*3^b, 8..1024  */
    double dx[3];     /* grid spacing per axis (x, y, z)                        */
    double span[3];   /* x(end)-x(1) per axis                                   */
    int precision;    /* GPE_FP32 or GPE_FP64: arithmetic type of the step      */
    int device;       /* CUDA device ordinal                                    */
} gpe_grid_desc;

/* Public properties of GPEtask that the hot path reads,
 * lib/@GPEtask/GPEtask.m:4-34 (defaults in brackets). */
typedef struct {
    double g;               /* coupling coefficient                      [0]    */
    double gamma;           /* phenomenological damping                  [0]    */
    double decay_rate;      /* 1/e decay time of N, 0 = none             [0]    */
    double Ntotal;          /* particle number, <= 0: keep the state norm [0]   */
    double mu_init;         /* fixed chemical potential, 0 = from state  [0]    */
    int n_recalc;           /* steps per potential / mu refresh          [10]   */
    int itp_max_iter;       /* ITP iteration cap                         [5000] */
    int itp_min_iter;       /* ITP iterations before the first check     [50]   */
    int itp_adjust_stepsize;/* halve dt on convergence until dt < dtmin  [0]    */
    double omega;           /* rotation frequency of a rotating frame    [0]:
                               set_kinop.m:5-7, ssft_kin_step.m:12-15, lap.m:8-10
                               (scalar omega; the adjoint needs omega = 0)       */
} gpe_params;

/* Imaginary-time propagation, lib/@GPEtask/groundstate_itp.m:1-112. */
typedef struct {
    double dt;              /* imaginary time step                               */
    double eps;             /* convergence threshold on the residual delta       */
    int want_mu2;           /* compute MU2 = <psi|H psi> at checks (nargout>=3)  */
    int want_energy;        /* compute EE = energy at checks (nargout>=4)        */
    int fp64_polish;        /* FP32 contexts: once FP32 rounding stalls delta,
                               finish the iteration in FP64 (default 1)         */
    double switch_delta;    /* FP32 phase ends once delta < switch_delta
                               (0 = 2e-4), or when delta stalls                  */
} gpe_itp_params;

typedef struct {
    int iters;              /* number of iterations run (length of MU)           */
    int converged;          /* 1 if delta < eps was reached                      */
    int fp32_iters;         /* iterations run in FP32 before the FP64 polish     */
    double final_dt;        /* dt at exit (differs if itp_adjust_stepsize)       */
    double last_delta;      /* last residual delta                               */
    double ms_main;         /* device time of the iterations in the context's
                               precision (CUDA events on the context stream)     */
    double ms_fp64;         /* device time of the FP64 polish, conversions
                               included (0 without one)                          */
} gpe_itp_result;

/* Host callbacks of solve_split.  Both run on the calling thread. */
/* Fill V_out (nx*ny*nz doubles, MATLAB order) with getVtotal(time),
 * GPEtask.m:62-71; called once per block of n_recalc steps
 * (solve_split.m:53-54).  Return 0 on success. */
typedef int (*gpe_vtd_fn)(void *user, double time, double *V_out);
/* ext_callback (GPEtask.m:115-142): called after each outer step j with the
 * block time, mu and norm; the state may be read with gpe_get_state().
 * Return 0 to continue; nonzero stops the run after this outer step. */
typedef int (*gpe_step_fn)(void *user, int step, double time, double mu, double n);

/* Real-time split step, lib/@GPEtask/solve_split.m:1-84. */
typedef struct {
    double ddt;             /* real time step                                    */
    int niter_inner;        /* steps per outer step                              */
    int niter_outer;        /* run outer steps current_iter+1 .. niter_outer      */
    gpe_vtd_fn vtd;         /* NULL: the potential set by gpe_set_potential      */
    void *vtd_user;
    gpe_step_fn on_step;    /* NULL: no per-outer-step host synchronisation       */
    void *step_user;
} gpe_split_params;

/* Gradient of an overlap loss through the split step (no counterpart in the
 * reference; differentiates the gamma = 0 step of solve_split.m:55-64). */
typedef struct {
    double ddt;             /* real time step                                    */
    int nsteps;             /* steps of the forward window                       */
    int checkpoint_every;   /* states kept every K steps; <= 0: K ~ sqrt(nsteps) */
    double mem_budget;      /* device bytes for stored states; <= 0: 60e9        */
    int precision;          /* 0: the context's; GPE_FP64 on an FP32 context runs
                             * the sweep in FP64 from the FP32 state             */
} gpe_adjoint_params;

/* Stochastic GPE, lib/@SGPEtask (SGPEtask.m:1-48, solve_split.m:1-81). */
typedef struct {
    double T;                  /* temperature                                   [0] */
    double ecut;               /* energy cut-off: with T > 0 and ecut > 0 the kinetic
                                  factor is exp(-kk*dt) .* (kk < ecut)
                                  (solve_split.m:40-42); 0: no cut-off              */
    unsigned long long seed;   /* noise stream: Philox4x32-10 keyed by seed with the
                                  counter (grid point, global step index)           */
} gpe_sgpe_params;

/* Dynamics bookkeeping properties, GPEtask.m:18-24. */
typedef struct {
    int current_iter;
    double current_time;
    double current_mu;
    double current_n;
} gpe_current;

/* <psi|H psi> pieces, GPEtask.m:73-107.  With omega the rotating-frame term
 * is part of ekin: scalar omega real(inner(psi, lap(psi, omega)))
 * (lap.m:8-10), an omega array <psi|-omega lz psi> added to the kinetic sum
 * (GPEtask.m:92-94).  Spinor contexts (GPEtaskSpinor.m:53-110): sums over
 * both components, eint = sum_jk g(j,k) integrate(|psi_j|^2 |psi_k|^2), ecpl =
 * the coupling term 2 Re(coupling * inner(psi_1, psi_2)) (0 for one
 * component), and a scalar omega adds -omega <psi_j|lz psi_j> with grid1d's
 * stencil to ekin (GPEtaskSpinor.m:72-74). */
typedef struct {
    double norm;            /* integrate(|psi|^2)                                */
    double ekin;            /* real(inner(psi, lap(psi)))                        */
    double epot;            /* integrate(V |psi|^2)                              */
    double eint;            /* g * integrate(|psi|^4)                            */
    double mu_integral;     /* real(inner(psi, applyham(psi)))
                               = ekin + epot + eint + ecpl                       */
    double energy;          /* get_energy(psi) = ekin + epot + eint/2 + ecpl     */
    double ecpl;            /* coherent coupling energy (spinor)                 */
} gpe_obs;

/* Coherently coupled two-component condensate, lib/@GPEtaskSpinor
 * (GPEtaskSpinor.m:4-8; solve_split.m:61-91).  The other properties
 * (gamma, decay_rate, Ntotal, n_recalc, scalar omega) come from
 * gpe_set_params, whose g is not used by a spinor context. */
typedef struct {
    double g[4];            /* interaction matrix g(j,k) at g[2*(j-1)+(k-1)]     */
    double coupling_re;     /* coupling (Rabi frequency), complex      [0]       */
    double coupling_im;
    double nlincpl;         /* density-dependent coupling               [0]       */
} gpe_spinor_params;

/* Per-kernel-class timings collected while profiling is enabled. */
typedef struct {
    char name[48];
    long long launches;
    double total_ms;
    double bytes_per_launch;   /* algorithmic HBM bytes of one launch          */
} gpe_kernel_stat;

/* ---- context ---------------------------------------------------------- */
/* grid2d/grid3d init + GPEtask constructor (GPEtask.m:41-60). */
GPE_API gpe_status gpe_create(const gpe_grid_desc *desc, gpe_ctx **out);
/* A two-component (GPEtaskSpinor) context on the same grid.  Its state,
 * potential and Vtd buffers hold both components, component 1 then 2
 * (2*nx*ny*nz points: MATLAB's {phi1, phi2} / {V1, V2} concatenated);
 * gpe_solve_split runs GPEtaskSpinor.solve_split and gpe_observables its
 * applyham/get_energy, gpe_groundstate_itp its groundstate_itp and
 * gpe_groundstate_itp_2comp GPEtask2comp's.  Scalar omega follows
 * GPEtaskSpinor: solve_split keeps the plain kinetic factor (its
 * solve_split.m has no omega) and mu / the observables add -omega <psi|lz psi>
 * with grid1d's stencil (GPEtaskSpinor.m:72-74).  The adjoint, SGPE,
 * batching, the autotuner, gpe_set_omega_field and gpe_groundstate_tf return
 * GPE_ERR_UNSUPPORTED on it. */
GPE_API gpe_status gpe_create_spinor(const gpe_grid_desc *desc, gpe_ctx **out);
/* Array omega (GPEtask.omega as an array, ssft_kin_step.m:3-11,
 * set_kinop.m:3-4, GPEtask.m:92-94): omega per grid point (nx*ny*nz doubles,
 * MATLAB order) and the Crank-Nicolson iteration count n_crank [3].  The
 * kinetic step becomes exp(-kk dt/2), n_crank iterations of
 * lphi = phi + dt/2 omega lz(lphi), phi += dt omega lz(lphi), exp(-kk dt/2);
 * energies and mu add <psi|-omega lz psi> (reported inside ekin).  lz uses
 * grid1d's 4th-order derivatives with zero outside the grid.  NULL returns
 * to scalar omega (gpe_params.omega, which must be 0 while an array is set). */
GPE_API gpe_status gpe_set_omega_field(gpe_ctx *ctx, const double *omega, int n_crank);
GPE_API gpe_status gpe_set_spinor_params(gpe_ctx *ctx, const gpe_spinor_params *p);
GPE_API gpe_status gpe_get_spinor_params(const gpe_ctx *ctx, gpe_spinor_params *p);
/* Incoherent two-component mixture (GPEtask2comp), imaginary time:
 * lib/@GPEtask2comp/groundstate_itp.m:1-157 on a spinor context from its
 * current state, with the spinor's g (coupling and nlincpl must be 0).
 * Each component j relaxes with its own kinetic factor
 * exp(-kk dt/2/M_j) (:29-30) and is renormalised to its own N_j (:82-90);
 * MU1(i) = log(sqrt(N1/n1))/dt, MU2(i) likewise for component 2 (not the
 * <psi|H psi> of gpe_groundstate_itp).  EE(i) = get_energy/Ntotal
 * (GPEtask2comp.m:107-118, Ntotal from gpe_set_params) when want_energy, else
 * MU2(i) (:98-102); the convergence test of :113-135 runs on EE.  MU1, MU2,
 * EE (each may be NULL) receive up to cap entries; the iteration cap is
 * gpe_params.itp_max_iter (the reference's is 500000, :136).  Scalar omega
 * (2D grids; :31-36, 61-80): the half step is exp(-(kx^2/2 - kx y omega)
 * dt/2/M_j) then exp(-(ky^2/2 + ky x omega) dt/2/M_j) before the nonlinear
 * factor and the same in reverse order after it; EE then uses
 * lap(phi, omega).  prm->want_mu2, fp64_polish and switch_delta are not used. */
GPE_API gpe_status gpe_groundstate_itp_2comp(gpe_ctx *ctx, const gpe_itp_params *prm,
                               double N1, double N2, double M1, double M2,
                               double *MU1, double *MU2, double *EE, int cap,
                               gpe_itp_result *res);
GPE_API void gpe_destroy(gpe_ctx *ctx);
/* Message of the last failed call on ctx (ctx may be NULL: last failure of
 * gpe_create on this thread). Never NULL. */
GPE_API const char *gpe_last_error(const gpe_ctx *ctx);
GPE_API int gpe_abi_version(void);
/* 1 if a usable sm_103 CUDA device is present, else 0. */
GPE_API int gpe_device_available(void);

/* ---- properties (GPEtask.m:4-34) -------------------------------------- */
GPE_API void gpe_default_params(gpe_params *p);
GPE_API gpe_status gpe_set_params(gpe_ctx *ctx, const gpe_params *p);
GPE_API gpe_status gpe_get_params(const gpe_ctx *ctx, gpe_params *p);
GPE_API gpe_status gpe_get_current(const gpe_ctx *ctx, gpe_current *cur);
GPE_API gpe_status gpe_set_current(gpe_ctx *ctx, const gpe_current *cur);
/* history.mu / history.n (GPEtask.m:123-126): up to cap entries, *len = count */
GPE_API gpe_status gpe_get_history(const gpe_ctx *ctx, double *mu, double *n, int cap, int *len);
/* get_energy(psi) (GPEtask.m:97-107, GPEtaskSpinor.m:98-110) of the state
 * at the end of every outer step, from the block-end sums on the device (an
 * addition: the reference's history keeps mu and n only); NaN for SGPE runs,
 * whose blocks evaluate no energy. */
GPE_API gpe_status gpe_get_history_energy(const gpe_ctx *ctx, double *E, int cap, int *len);
GPE_API gpe_status gpe_clear_history(gpe_ctx *ctx);

/* ---- data ------------------------------------------------------------- */
/* Vtrap / getVtotal (GPEtask.m:44-46, 62-71): nx*ny*nz real values. */
GPE_API gpe_status gpe_set_potential(gpe_ctx *ctx, const double *V);
GPE_API gpe_status gpe_set_potential_f32(gpe_ctx *ctx, const float *V);
/* init_state / current_state: nx*ny*nz interleaved complex values. */
GPE_API gpe_status gpe_set_state(gpe_ctx *ctx, const double *psi);
GPE_API gpe_status gpe_set_state_f32(gpe_ctx *ctx, const float *psi);
GPE_API gpe_status gpe_get_state(gpe_ctx *ctx, double *psi);
GPE_API gpe_status gpe_get_state_f32(gpe_ctx *ctx, float *psi);
/* Device-resident variants (gpuArray inputs): d_psi is a device pointer on
 * the context's device holding interleaved complex values of `precision`. */
GPE_API gpe_status gpe_set_state_device(gpe_ctx *ctx, const void *d_psi, int precision);
GPE_API gpe_status gpe_get_state_device(gpe_ctx *ctx, void *d_psi, int precision);

/* Page-lock (pin) a caller-owned host buffer so state copies run at full
 * link bandwidth and asynchronously; unregister before freeing it. */
GPE_API gpe_status gpe_host_register(void *ptr, size_t bytes);
GPE_API gpe_status gpe_host_unregister(void *ptr);

/* ---- hot path --------------------------------------------------------- */
/* groundstate_itp.m:1-112 from the current state (process_init_state for an
 * array phi0 is applied: psi <- sqrt(Ntotal)*normalize(psi) when Ntotal > 0).
 * MU, MU2, EE (each may be NULL) receive up to cap entries, already divided
 * by Ntotal as the reference returns them.  On return the state holds the
 * ground state (init_state = phi, groundstate_itp.m:111).
 * Spinor context: lib/@GPEtaskSpinor/groundstate_itp.m:1-145 (MU from the
 * total norm, MU2 = <psi|H psi>/Ntotal, EE = get_energy/Ntotal).  Scalar
 * omega (2D grids, :30-33, 61-80): each kinetic half step is
 * exp(-(kx^2/2 - kx y omega) dt/2) then exp(-(ky^2/2 + ky x omega) dt/2), and
 * MU2/EE add -omega <psi|lz psi> with grid1d's 4th-order lz
 * (GPEtaskSpinor.m:72-74). */
GPE_API gpe_status gpe_groundstate_itp(gpe_ctx *ctx, const gpe_itp_params *prm,
                               double *MU, double *MU2, double *EE, int cap,
                               gpe_itp_result *res);
/* solve_split.m:1-84 from the current state; resumes at current_iter.
 * Spinor context: lib/@GPEtaskSpinor/solve_split.m:1-119 (kinetic half step
 * at each block start, per step the nonlinear and coupling factor then the
 * kinetic step, the inverse half step at the block end; blocks of n_recalc
 * steps, floor(niter_inner/n_recalc) of them; renormalised to Ntotal (with
 * decay) when gamma > 0; mu = <psi|H psi>/N at each block end with V at
 * current_time, as GPEtaskSpinor.applyham evaluates it).  vtd fills 2*P
 * doubles (V1 then V2). */
GPE_API gpe_status gpe_solve_split(gpe_ctx *ctx, const gpe_split_params *prm);
/* solve_split on `count` independent contexts (any grid sizes, same device,
 * same n_recalc and current_iter) advanced together: one block of n_recalc
 * steps of every context is captured into a CUDA graph whose per-context
 * chains run concurrently, and replayed.  Each context keeps its own state,
 * V, parameters, history and current_*.  Not available in a batch: vtd and
 * on_step callbacks (must be NULL) and decay_rate > 0.  Errors are reported
 * on ctxs[0]. */
GPE_API gpe_status gpe_solve_split_batch(gpe_ctx **ctxs, int count, const gpe_split_params *prm);
/* Discrete adjoint of `nsteps` split steps (the gamma = 0 operator sequence
 * of solve_split.m:55-64: per step exp(-i(V+g|psi|^2)ddt/2), kinetic
 * exp(-i k^2 ddt/2), the nonlinear half again; mu is a global phase and is
 * left out) from the current state psi0 at the current V:
 *   loss = 1 - |<target|psi(T)>|^2 / (<target|target> <psi0|psi0>)
 * with <a|b> = integrate(conj(a) b).  psi_target: nx*ny*nz interleaved
 * complex doubles; dLdV: nx*ny*nz doubles, dloss/dV at each grid point;
 * loss may be NULL.  Forward states are kept every checkpoint_every steps
 * and each segment is recomputed once in the backward sweep; the stored
 * states must fit mem_budget (else GPE_ERR_ALLOC).  The context state,
 * current_* and history are left unchanged.  gamma must be 0. */
GPE_API gpe_status gpe_adjoint_grad(gpe_ctx *ctx, const gpe_adjoint_params *prm, const double *psi_target,
                                    double *dLdV, double *loss);
/* SGPEtask.solve_split (lib/@SGPEtask/solve_split.m:1-81) from the current
 * state: mu = mu_init throughout, no renormalisation, and before every
 * kinetic step psi += sqrt(T*gamma*ddt/weight) * (n1 + i*n2) with n1, n2
 * standard normal variates (solve_split.m:49,55).  With T > 0 and ecut > 0
 * the modes with kk >= ecut are zeroed in every kinetic step (five axis
 * passes in 3D, three in 2D, instead of three and two; kk is summed in the
 * context's precision, so a mode within rounding of ecut may fall either
 * way).  history.mu holds mu_init, history.n the norm.  Vtd and on_step work as in gpe_solve_split; omega must
 * be 0 (the reference's rotating SGPE uses the Lz Crank-Nicolson branch). */
GPE_API gpe_status gpe_solve_sgpe(gpe_ctx *ctx, const gpe_split_params *prm, const gpe_sgpe_params *sg);
/* applyham / get_energy pieces for the current state at the current V. */
GPE_API gpe_status gpe_observables(gpe_ctx *ctx, gpe_obs *obs);

/* ---- observables on the device ------------------------------------------ */
/* lib/util/detect_core.m:1-67 on the 2D slice z_index (0 in 2D) of the
 * current state (component 0 or 1 of a spinor context): cores where the
 * phase winds around a plaquette and |del2(|psi|^2)| exceeds 1% of its
 * maximum.  pos/neg receive up to cap_pos/cap_neg (x, y) pairs in MATLAB's
 * find() order: [x - dx/2, y - dy/2] for positive and [x - dx/2, y - dx/2]
 * for negative cores as the reference writes them, or with refine != 0 the
 * sub-cell positions of refine_core (the first qualifying real root in
 * ascending order; no real root in (0,1): [0, 0]).  n_pos/n_neg receive the
 * counts, which may exceed the caps. */
GPE_API gpe_status gpe_detect_core(gpe_ctx *ctx, int component, int z_index, int refine,
                                   double *pos, int cap_pos, int *n_pos,
                                   double *neg, int cap_neg, int *n_neg);
/* lib/@GPEtask/groundstate_tf.m:1-37 against the potential last set: bisect
 * mu until (mur-mul)/mu <= eps (bounds = {mul, mur}, or NULL for min/max of
 * V), set the state to sqrt(vvv/g) with vvv of the last evaluated mu, and
 * return mu.  g must be positive. */
GPE_API gpe_status gpe_groundstate_tf(gpe_ctx *ctx, double eps, double N, const double *bounds, double *mu);

/* ---- profiling and timing (CUDA events on the context stream) ---------- */
GPE_API gpe_status gpe_synchronize(gpe_ctx *ctx);
GPE_API gpe_status gpe_timer_start(gpe_ctx *ctx);
GPE_API gpe_status gpe_timer_stop(gpe_ctx *ctx, double *ms);
GPE_API gpe_status gpe_profile_enable(gpe_ctx *ctx, int on);
GPE_API gpe_status gpe_profile_read(gpe_ctx *ctx, gpe_kernel_stat *out, int cap, int *n);
/* Axis-pass implementation: 0 (default) = direct-load passes that also
 * prefetch the next wave's tiles into L2, 1 = TMA-staged persistent passes
 * where the tile geometry allows, 2 = direct-load passes without prefetch.
 * All compute the same result; the knob exists for measurement. */
GPE_API gpe_status gpe_set_pass_variant(gpe_ctx *ctx, int variant);
/* integrate(|psi|^2) = sum |psi_i|^2 * weight of a caller-owned device array
 * d_psi (npoints interleaved complex values of `precision`, on the current
 * device), written to the host double *norm_out, on `stream` (a
 * cudaStream_t; NULL = default stream).  This is the particle number the
 * reference's solve_split calls ncur (solve_split.m:65-67) and gpe_obs.norm
 * reports, i.e. the SQUARE of MATLAB's grid.norm (norm.m:11).  No
 * counterpart in the reference: an addition for callers that cannot allocate
 * device memory at that point (MEX code on gpuArray memory owned by MATLAB's
 * allocator, code inside a solve_split callback, applications that own all
 * device memory).  It allocates nothing: its partial sums live in a fixed
 * 256 KB device array inside the library, so it accepts at most 134,217,728
 * points (512^3) and rejects larger inputs with GPE_ERR_INVALID.  Before any
 * device work, d_psi must be aligned to one complex element (8 bytes FP32,
 * 16 bytes FP64) and must be device memory of the current device (or managed
 * memory); host memory and another device's memory are refused with
 * GPE_ERR_INVALID.  The first call on each device looks up that array's
 * address and should come before any stream capture; the address lives as
 * long as the device's CUDA context, so no call may follow a cudaDeviceReset.
 * Each call waits on the host for its result; a call on a stream that is
 * being captured is refused with GPE_ERR_INVALID.  All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * Errors: gpe_last_error(NULL). */
GPE_API gpe_status gpe_norm_noalloc(const void *d_psi, long long npoints, int precision, double weight,
                                    void *stream, double *norm_out);
/* FFT plan autotuner (FP32 contexts).  Axis lengths 128, 192, 256, 384 and
 * 512 have two FFT plans (threads per pencil T and radix schedule) and a
 * paired step pass (two pencils per thread on packed FP32x2 arithmetic) on
 * the alternative plan, and 128, 256, 512 also on the default plan; the
 * tuner times these on each axis pass of this grid and keeps the fastest (a
 * non-default one must win by 5%), caching choices per device and grid
 * shape.
 * mode 0: default plans, no tuning; 1: tune now; 2 (default): tune on the
 * first groundstate_itp / solve_split / observables / adjoint call when the
 * grid has >= 2^20 points, and for every context of solve_split_batch;
 * 3: use the alternative plan wherever one exists (testing, measurement);
 * 4: the paired passes on the alternative plan wherever one exists;
 * 5: the paired passes on the default plan wherever they exist;
 * 16 + m (m = 0..7): the alternative plan on the axes of bit mask m (bit 0 =
 * x, 1 = y, 2 = z), the default elsewhere (reproducing a tuned choice);
 * 32 + m / 48 + m: the paired passes on the alternative / default plan on
 * the axes of bit mask m.
 * chosen (may be NULL) receives the plan variant of axes x, y, z (0 default,
 * 1 alternative, 2 paired on the alternative, 3 paired on the default, -1
 * for a length with one plan, FP64 contexts, 2D z). */
GPE_API gpe_status gpe_autotune(gpe_ctx *ctx, int mode, int *chosen);
/* Diagnostic: the stochastic GPE's noise variates for points 0..n-1 of step
 * `step` (FP32, interleaved n1, n2 per point), on device 0. */
GPE_API gpe_status gpe_selftest_noise(unsigned long long seed, unsigned long long step, long long n, float *out);
/* Diagnostic: the FP32 device sin/cos used by the phase factors, on n host
 * values (device 0).  Lets tests bound its error against FP64 references. */
GPE_API gpe_status gpe_selftest_trig(const float *x, float *s, float *c, long long n);
/* Launch counters of this library's kernels since the context was created. */
GPE_API long long gpe_kernel_launches(const gpe_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* GPE_H */

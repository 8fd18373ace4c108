// gpe_mex.cpp - MEX gateway from MATLAB's GPEtask class to libgpe (C ABI,
// include/gpe.h).  Build (MATLAB R2018a+, interleaved complex API):
//
//   mex -R2018a -I../../include gpe_mex.cpp -L.. -lgpe
//
// UNVERIFIED: this machine has no MATLAB (no mex.h, no libmx), so this file
// has not been compiled.  It uses only documented MEX C API calls, and every
// libgpe call it makes is exercised by the Python tests through the same ABI.
//
// Usage (see @GPEtaskGB300):
//   h = gpe_mex('create', ndims, n, dx, span, precision)   % precision 'single'|'double'
//   gpe_mex('destroy', h)
//   gpe_mex('set_params', h, g, gamma, decay_rate, Ntotal, mu_init, n_recalc,
//           itp_max_iter, itp_min_iter, itp_adjust_stepsize)
//   gpe_mex('set_current', h, iter, time, mu, n)
//   [iter, time, mu, n] = gpe_mex('current', h)
//   [mu, n] = gpe_mex('history', h)
//   gpe_mex('set_potential', h, V)                    % real double, grid size
//   gpe_mex('set_state', h, psi)                      % complex double or single
//   psi = gpe_mex('get_state', h, 'double'|'single')
//   [MU, MU2, EE, iters, converged] = gpe_mex('itp', h, dt, eps, want_mu2, want_energy)
//   gpe_mex('split', h, ddt, niter_inner, niter_outer, task)
//       task: the calling GPEtaskGB300 object; if it has a time-dependent
//       potential the gateway calls task.getVtotal(time) once per block, and
//       after every outer step it calls task.gb300_step(step, time, mu, n).
//   obs = gpe_mex('observables', h)                   % [norm ekin epot eint mu_int energy ecpl]
//   gpe_mex('sgpe', h, ddt, nin, nout, task, timedep, T, ecut, seed)   % SGPEtask.solve_split
//   h = gpe_mex('create_spinor', ndims, n, dx, span, precision)      % GPEtaskSpinor context
//   gpe_mex('set_spinor_params', h, g, coupling, nlincpl)
//   [MU1, MU2, EE] = gpe_mex('itp_2comp', h, dt, eps, want_energy, [N1 N2], [M1 M2])   % GPEtask2comp ITP
//       spinor contexts take [phi1(:); phi2(:)] and [V1(:); V2(:)] in set_state /
//       set_potential / getVtotal, and get_state returns them stacked the same way
//   gpe_mex('set_state_gpu', h, psi_gpuArray)                            % device to device
//   psi = gpe_mex('get_state_gpu', h, 'double'|'single', size)           % a new gpuArray
//   [resp, resm] = gpe_mex('detect_core', h, z_index, refine, component)   % detect_core.m on the device
//   mu = gpe_mex('groundstate_tf', h, eps, N[, mul, mur])                 % groundstate_tf.m on the device
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "gpe.h"
#include "gpu/mxGPUArray.h"
#include "mex.h"

namespace {

gpe_ctx* handle(const mxArray* a) {
  if (!mxIsUint64(a) || mxGetNumberOfElements(a) != 1) mexErrMsgIdAndTxt("gpe:handle", "invalid gpe handle");
  return reinterpret_cast<gpe_ctx*>(*static_cast<uint64_t*>(mxGetData(a)));
}

void check(gpe_ctx* c, gpe_status st) {
  if (st != GPE_OK) {
    std::string id = "gpe:status" + std::to_string((int)st);
    mexErrMsgIdAndTxt(id.c_str(), "%s", gpe_last_error(c));
  }
}

double scalar(const mxArray* a) { return mxGetScalar(a); }

std::string str(const mxArray* a) {
  char buf[64];
  if (mxGetString(a, buf, sizeof(buf)) != 0) mexErrMsgIdAndTxt("gpe:arg", "expected a string");
  return buf;
}

struct SplitCtx {
  const mxArray* task;
  size_t npts;
};

// getVtotal(time) of the MATLAB task, once per block (solve_split.m:53-54).
int vtd_cb(void* user, double time, double* V_out) {
  SplitCtx* s = static_cast<SplitCtx*>(user);
  mxArray* in[2] = {const_cast<mxArray*>(s->task), mxCreateDoubleScalar(time)};
  mxArray* out[1] = {nullptr};
  if (mexCallMATLAB(1, out, 2, in, "gb300_vtotal") != 0) return 1;
  int rc = 0;
  if (!mxIsDouble(out[0]) || mxIsComplex(out[0]) || mxGetNumberOfElements(out[0]) != s->npts) rc = 1;
  else memcpy(V_out, mxGetDoubles(out[0]), s->npts * sizeof(double));
  mxDestroyArray(in[1]);
  mxDestroyArray(out[0]);
  return rc;
}

// ext_callback bookkeeping in MATLAB (GPEtask.m:115-142).  task.gb300_step
// returns nonzero to end the run after this outer step (SGPEtask: the user
// callback returned 'TERM', @SGPEtask/solve_split.m:77-80).
int step_cb(void* user, int step, double time, double mu, double n) {
  SplitCtx* s = static_cast<SplitCtx*>(user);
  mxArray* in[5] = {const_cast<mxArray*>(s->task), mxCreateDoubleScalar(step), mxCreateDoubleScalar(time),
                    mxCreateDoubleScalar(mu), mxCreateDoubleScalar(n)};
  mxArray* out[1] = {nullptr};
  int rc = mexCallMATLAB(1, out, 5, in, "gb300_step");
  for (int i = 1; i < 5; ++i) mxDestroyArray(in[i]);
  if (rc == 0 && out[0]) {
    if (mxGetNumberOfElements(out[0]) == 1 && mxGetScalar(out[0]) != 0.0) rc = 1;
    mxDestroyArray(out[0]);
  }
  return rc;
}

}  // namespace

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs < 1) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex(command, ...)");
  const std::string cmd = str(prhs[0]);

  if (cmd == "create" || cmd == "create_spinor") {
    // create_spinor: a two-component (GPEtaskSpinor) context; its state, V and
    // Vtd arrays are [phi1(:); phi2(:)] / [V1(:); V2(:)]
    if (nrhs != 6) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('create', ndims, n, dx, span, precision)");
    gpe_grid_desc d;
    memset(&d, 0, sizeof(d));
    d.ndims = (int)scalar(prhs[1]);
    const double* n = mxGetDoubles(prhs[2]);
    const double* dx = mxGetDoubles(prhs[3]);
    const double* span = mxGetDoubles(prhs[4]);
    for (int a = 0; a < d.ndims && a < 3; ++a) {
      d.n[a] = (int)n[a];
      d.dx[a] = dx[a];
      d.span[a] = span[a];
    }
    d.precision = str(prhs[5]) == "single" ? GPE_FP32 : GPE_FP64;
    d.device = 0;
    gpe_ctx* c = nullptr;
    check(nullptr, cmd == "create" ? gpe_create(&d, &c) : gpe_create_spinor(&d, &c));
    plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
    *static_cast<uint64_t*>(mxGetData(plhs[0])) = reinterpret_cast<uint64_t>(c);
    return;
  }

  if (nrhs < 2) mexErrMsgIdAndTxt("gpe:usage", "missing handle");
  gpe_ctx* c = handle(prhs[1]);

  if (cmd == "destroy") {
    gpe_destroy(c);
  } else if (cmd == "set_params") {
    if (nrhs != 11 && nrhs != 12) mexErrMsgIdAndTxt("gpe:usage", "set_params needs 9 or 10 values");
    gpe_params p;
    gpe_default_params(&p);
    p.g = scalar(prhs[2]);
    p.gamma = scalar(prhs[3]);
    p.decay_rate = scalar(prhs[4]);
    p.Ntotal = scalar(prhs[5]);
    p.mu_init = scalar(prhs[6]);
    p.n_recalc = (int)scalar(prhs[7]);
    p.itp_max_iter = (int)scalar(prhs[8]);
    p.itp_min_iter = (int)scalar(prhs[9]);
    p.itp_adjust_stepsize = (int)scalar(prhs[10]);
    if (nrhs == 12) p.omega = scalar(prhs[11]);  // scalar rotating frame
    check(c, gpe_set_params(c, &p));
  } else if (cmd == "set_current") {
    gpe_current cur;
    cur.current_iter = (int)scalar(prhs[2]);
    cur.current_time = scalar(prhs[3]);
    cur.current_mu = scalar(prhs[4]);
    cur.current_n = scalar(prhs[5]);
    check(c, gpe_set_current(c, &cur));
  } else if (cmd == "current") {
    gpe_current cur;
    check(c, gpe_get_current(c, &cur));
    plhs[0] = mxCreateDoubleScalar(cur.current_iter);
    if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(cur.current_time);
    if (nlhs > 2) plhs[2] = mxCreateDoubleScalar(cur.current_mu);
    if (nlhs > 3) plhs[3] = mxCreateDoubleScalar(cur.current_n);
  } else if (cmd == "history") {
    int len = 0;
    check(c, gpe_get_history(c, nullptr, nullptr, 0, &len));
    plhs[0] = mxCreateDoubleMatrix(1, len, mxREAL);
    mxArray* nn = mxCreateDoubleMatrix(1, len, mxREAL);
    check(c, gpe_get_history(c, mxGetDoubles(plhs[0]), mxGetDoubles(nn), len, &len));
    if (nlhs > 1) plhs[1] = nn;
    else mxDestroyArray(nn);
  } else if (cmd == "set_omega_field") {
    // gpe_mex('set_omega_field', h, omega, n_crank): array omega (omega = [] returns to scalar)
    if (nrhs != 4) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('set_omega_field', h, omega, n_crank)");
    const bool none = mxGetNumberOfElements(prhs[2]) == 0;
    if (!none && (!mxIsDouble(prhs[2]) || mxIsComplex(prhs[2]))) mexErrMsgIdAndTxt("gpe:arg", "omega must be real double");
    check(c, gpe_set_omega_field(c, none ? nullptr : mxGetDoubles(prhs[2]), (int)scalar(prhs[3])));
  } else if (cmd == "set_spinor_params") {
    // gpe_mex('set_spinor_params', h, g (2x2), coupling (complex scalar), nlincpl)
    if (nrhs != 5) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('set_spinor_params', h, g, coupling, nlincpl)");
    if (!mxIsDouble(prhs[2]) || mxGetNumberOfElements(prhs[2]) != 4) mexErrMsgIdAndTxt("gpe:arg", "g must be 2x2 double");
    const double* g = mxGetDoubles(prhs[2]);  // column-major: g(1,1) g(2,1) g(1,2) g(2,2)
    gpe_spinor_params sp;
    memset(&sp, 0, sizeof(sp));
    sp.g[0] = g[0];
    sp.g[1] = g[2];
    sp.g[2] = g[1];
    sp.g[3] = g[3];
    if (mxIsComplex(prhs[3])) {
      const mxComplexDouble* cp = mxGetComplexDoubles(prhs[3]);
      sp.coupling_re = cp[0].real;
      sp.coupling_im = cp[0].imag;
    } else {
      sp.coupling_re = scalar(prhs[3]);
    }
    sp.nlincpl = scalar(prhs[4]);
    check(c, gpe_set_spinor_params(c, &sp));
  } else if (cmd == "set_potential") {
    if (!mxIsDouble(prhs[2]) || mxIsComplex(prhs[2])) mexErrMsgIdAndTxt("gpe:arg", "V must be real double");
    check(c, gpe_set_potential(c, mxGetDoubles(prhs[2])));
  } else if (cmd == "set_state") {
    const mxArray* psi = prhs[2];
    if (!mxIsComplex(psi)) mexErrMsgIdAndTxt("gpe:arg", "psi must be complex (use complex(psi))");
    if (mxIsSingle(psi)) check(c, gpe_set_state_f32(c, reinterpret_cast<const float*>(mxGetComplexSingles(psi))));
    else check(c, gpe_set_state(c, reinterpret_cast<const double*>(mxGetComplexDoubles(psi))));
  } else if (cmd == "set_state_gpu") {
    // gpe_mex('set_state_gpu', h, psi): psi a complex gpuArray (single or
    // double, interleaved on the device); copied device to device
    mxInitGPU();
    const mxGPUArray* g = mxGPUCreateFromMxArray(prhs[2]);
    if (mxGPUGetComplexity(g) != mxCOMPLEX) {
      mxGPUDestroyGPUArray(g);
      mexErrMsgIdAndTxt("gpe:arg", "psi must be complex (use complex(psi))");
    }
    const int prec = mxGPUGetClassID(g) == mxSINGLE_CLASS ? GPE_FP32 : GPE_FP64;
    const gpe_status st = gpe_set_state_device(c, mxGPUGetDataReadOnly(g), prec);
    mxGPUDestroyGPUArray(g);
    check(c, st);
  } else if (cmd == "get_state_gpu") {
    // psi = gpe_mex('get_state_gpu', h, cls, dims): the state as a new complex gpuArray
    if (nrhs < 4) mexErrMsgIdAndTxt("gpe:usage", "get_state_gpu needs the class and the size");
    mxInitGPU();
    const std::string cls = str(prhs[2]);
    const double* sz = mxGetDoubles(prhs[3]);
    const mwSize nd = mxGetNumberOfElements(prhs[3]) > 2 ? 3 : 2;
    mwSize dims[3] = {(mwSize)sz[0], (mwSize)sz[1], nd > 2 ? (mwSize)sz[2] : 1};
    mxGPUArray* g = mxGPUCreateGPUArray(nd, dims, cls == "single" ? mxSINGLE_CLASS : mxDOUBLE_CLASS, mxCOMPLEX,
                                        MX_GPU_DO_NOT_INITIALIZE);
    const gpe_status st = gpe_get_state_device(c, mxGPUGetData(g), cls == "single" ? GPE_FP32 : GPE_FP64);
    if (st != GPE_OK) {
      mxGPUDestroyGPUArray(g);
      check(c, st);
    }
    plhs[0] = mxGPUCreateMxArrayOnGPU(g);
    mxGPUDestroyGPUArray(g);
  } else if (cmd == "get_state") {
    // dims come from the caller's grid: psi = gpe_mex('get_state', h, cls, size(grid.mesh.x))
    const std::string cls = nrhs > 2 ? str(prhs[2]) : "double";
    if (nrhs < 4) mexErrMsgIdAndTxt("gpe:usage", "get_state needs the grid size");
    const double* sz = mxGetDoubles(prhs[3]);
    mwSize dims[3] = {(mwSize)sz[0], (mwSize)sz[1], mxGetNumberOfElements(prhs[3]) > 2 ? (mwSize)sz[2] : 1};
    const mwSize nd = mxGetNumberOfElements(prhs[3]) > 2 ? 3 : 2;
    if (cls == "single") {
      plhs[0] = mxCreateNumericArray(nd, dims, mxSINGLE_CLASS, mxCOMPLEX);
      check(c, gpe_get_state_f32(c, reinterpret_cast<float*>(mxGetComplexSingles(plhs[0]))));
    } else {
      plhs[0] = mxCreateNumericArray(nd, dims, mxDOUBLE_CLASS, mxCOMPLEX);
      check(c, gpe_get_state(c, reinterpret_cast<double*>(mxGetComplexDoubles(plhs[0]))));
    }
  } else if (cmd == "itp") {
    gpe_itp_params p;
    memset(&p, 0, sizeof(p));
    p.dt = scalar(prhs[2]);
    p.eps = scalar(prhs[3]);
    p.want_mu2 = (int)scalar(prhs[4]);
    p.want_energy = (int)scalar(prhs[5]);
    p.fp64_polish = 1;
    gpe_params prm;
    check(c, gpe_get_params(c, &prm));
    const int cap = prm.itp_max_iter;
    mxArray* MU = mxCreateDoubleMatrix(cap, 1, mxREAL);
    mxArray* MU2 = mxCreateDoubleMatrix(cap, 1, mxREAL);
    mxArray* EE = mxCreateDoubleMatrix(cap, 1, mxREAL);
    gpe_itp_result res;
    check(c, gpe_groundstate_itp(c, &p, mxGetDoubles(MU), mxGetDoubles(MU2), mxGetDoubles(EE), cap, &res));
    mxSetM(MU, res.iters);
    mxSetM(MU2, res.iters);
    mxSetM(EE, res.iters);
    plhs[0] = MU;
    if (nlhs > 1) plhs[1] = MU2;
    else mxDestroyArray(MU2);
    if (nlhs > 2) plhs[2] = EE;
    else mxDestroyArray(EE);
    if (nlhs > 3) plhs[3] = mxCreateDoubleScalar(res.iters);
    if (nlhs > 4) plhs[4] = mxCreateDoubleScalar(res.converged);
    if (!res.converged) mexWarnMsgIdAndTxt("gpe:itp", "Convergence not reached");
  } else if (cmd == "itp_2comp") {
    // [MU1, MU2, EE] = gpe_mex('itp_2comp', h, dt, eps, want_energy, [N1 N2], [M1 M2])
    if (nrhs != 7) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('itp_2comp', h, dt, eps, want_energy, [N1 N2], [M1 M2])");
    gpe_itp_params p;
    memset(&p, 0, sizeof(p));
    p.dt = scalar(prhs[2]);
    p.eps = scalar(prhs[3]);
    p.want_energy = (int)scalar(prhs[4]);
    if (mxGetNumberOfElements(prhs[5]) != 2 || mxGetNumberOfElements(prhs[6]) != 2 || !mxIsDouble(prhs[5]) ||
        !mxIsDouble(prhs[6]))
      mexErrMsgIdAndTxt("gpe:usage", "itp_2comp: [N1 N2] and [M1 M2] are two doubles each");
    const double* Nj = mxGetDoubles(prhs[5]);
    const double* Mj = mxGetDoubles(prhs[6]);
    gpe_params prm;
    check(c, gpe_get_params(c, &prm));
    const int cap = prm.itp_max_iter;
    mxArray* MU1 = mxCreateDoubleMatrix(cap, 1, mxREAL);
    mxArray* MU2 = mxCreateDoubleMatrix(cap, 1, mxREAL);
    mxArray* EE = mxCreateDoubleMatrix(cap, 1, mxREAL);
    gpe_itp_result res;
    check(c, gpe_groundstate_itp_2comp(c, &p, Nj[0], Nj[1], Mj[0], Mj[1], mxGetDoubles(MU1), mxGetDoubles(MU2),
                                       mxGetDoubles(EE), cap, &res));
    mxSetM(MU1, res.iters);
    mxSetM(MU2, res.iters);
    mxSetM(EE, res.iters);
    plhs[0] = MU1;
    if (nlhs > 1) plhs[1] = MU2;
    else mxDestroyArray(MU2);
    if (nlhs > 2) plhs[2] = EE;
    else mxDestroyArray(EE);
    if (!res.converged) mexWarnMsgIdAndTxt("gpe:itp", "Convergence not reached");
  } else if (cmd == "split") {
    if (nrhs != 7) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('split', h, ddt, nin, nout, task, timedep)");
    SplitCtx s{prhs[5], (size_t)mxGetScalar(mxGetProperty(prhs[5], 0, "gb300_npts"))};
    gpe_split_params p;
    memset(&p, 0, sizeof(p));
    p.ddt = scalar(prhs[2]);
    p.niter_inner = (int)scalar(prhs[3]);
    p.niter_outer = (int)scalar(prhs[4]);
    if (scalar(prhs[6]) != 0) {
      p.vtd = vtd_cb;
      p.vtd_user = &s;
    }
    p.on_step = step_cb;
    p.step_user = &s;
    check(c, gpe_solve_split(c, &p));
  } else if (cmd == "sgpe") {
    // gpe_mex('sgpe', h, ddt, nin, nout, task, timedep, T, ecut, seed): SGPEtask.solve_split
    if (nrhs != 10) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('sgpe', h, ddt, nin, nout, task, timedep, T, ecut, seed)");
    SplitCtx s{prhs[5], (size_t)mxGetScalar(mxGetProperty(prhs[5], 0, "gb300_npts"))};
    gpe_split_params p;
    memset(&p, 0, sizeof(p));
    p.ddt = scalar(prhs[2]);
    p.niter_inner = (int)scalar(prhs[3]);
    p.niter_outer = (int)scalar(prhs[4]);
    if (scalar(prhs[6]) != 0) {
      p.vtd = vtd_cb;
      p.vtd_user = &s;
    }
    p.on_step = step_cb;
    p.step_user = &s;
    gpe_sgpe_params sg;
    memset(&sg, 0, sizeof(sg));
    sg.T = scalar(prhs[7]);
    sg.ecut = scalar(prhs[8]);
    sg.seed = (unsigned long long)scalar(prhs[9]);
    check(c, gpe_solve_sgpe(c, &p, &sg));
  } else if (cmd == "observables") {
    gpe_obs o;
    check(c, gpe_observables(c, &o));
    plhs[0] = mxCreateDoubleMatrix(1, 7, mxREAL);
    double* r = mxGetDoubles(plhs[0]);
    r[0] = o.norm;
    r[1] = o.ekin;
    r[2] = o.epot;
    r[3] = o.eint;
    r[4] = o.mu_integral;
    r[5] = o.energy;
    r[6] = o.ecpl;
  } else if (cmd == "detect_core") {
    // [resp, resm] = gpe_mex('detect_core', h, z_index, refine, component): detect_core.m
    // of the current device state (slice z_index, 1-based as in MATLAB; 1 in 2D)
    if (nrhs != 5) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('detect_core', h, z_index, refine, component)");
    const int z = (int)scalar(prhs[2]) - 1, refine = (int)scalar(prhs[3]), comp = (int)scalar(prhs[4]) - 1;
    int np = 0, nm = 0;
    check(c, gpe_detect_core(c, comp, z, refine, nullptr, 0, &np, nullptr, 0, &nm));
    std::vector<double> p(2 * (size_t)std::max(np, 1)), m(2 * (size_t)std::max(nm, 1));
    check(c, gpe_detect_core(c, comp, z, refine, p.data(), np, &np, m.data(), nm, &nm));
    // k x 2 column-major results from (x, y) pairs
    plhs[0] = mxCreateDoubleMatrix(np, 2, mxREAL);
    for (int k = 0; k < np; ++k) {
      mxGetDoubles(plhs[0])[k] = p[2 * k];
      mxGetDoubles(plhs[0])[np + k] = p[2 * k + 1];
    }
    if (nlhs > 1) {
      plhs[1] = mxCreateDoubleMatrix(nm, 2, mxREAL);
      for (int k = 0; k < nm; ++k) {
        mxGetDoubles(plhs[1])[k] = m[2 * k];
        mxGetDoubles(plhs[1])[nm + k] = m[2 * k + 1];
      }
    }
  } else if (cmd == "groundstate_tf") {
    // mu = gpe_mex('groundstate_tf', h, eps, N[, mul, mur]): the state becomes the TF profile
    if (nrhs != 4 && nrhs != 6) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('groundstate_tf', h, eps, N[, mul, mur])");
    double b[2] = {0.0, 0.0}, mu = 0.0;
    if (nrhs == 6) {
      b[0] = scalar(prhs[4]);
      b[1] = scalar(prhs[5]);
    }
    check(c, gpe_groundstate_tf(c, scalar(prhs[2]), scalar(prhs[3]), nrhs == 6 ? b : nullptr, &mu));
    plhs[0] = mxCreateDoubleScalar(mu);
  } else if (cmd == "adjoint") {
    // [loss, dLdV] = gpe_mex('adjoint', h, target, ddt, nsteps, K, budget, precision)
    // precision: 0 = the context's, 2 = FP64 sweep.  dLdV has the grid's shape.
    if (nrhs != 8) mexErrMsgIdAndTxt("gpe:usage", "gpe_mex('adjoint', h, target, ddt, nsteps, K, budget, prec)");
    const mxArray* tg = prhs[2];
    if (!mxIsDouble(tg) || !mxIsComplex(tg)) mexErrMsgIdAndTxt("gpe:arg", "target must be complex double");
    gpe_adjoint_params p;
    memset(&p, 0, sizeof(p));
    p.ddt = scalar(prhs[3]);
    p.nsteps = (int)scalar(prhs[4]);
    p.checkpoint_every = (int)scalar(prhs[5]);
    p.mem_budget = scalar(prhs[6]);
    p.precision = (int)scalar(prhs[7]);
    mxArray* g = mxCreateNumericArray(mxGetNumberOfDimensions(tg), mxGetDimensions(tg), mxDOUBLE_CLASS, mxREAL);
    double loss = 0.0;
    check(c, gpe_adjoint_grad(c, &p, reinterpret_cast<const double*>(mxGetComplexDoubles(tg)), mxGetDoubles(g),
                              &loss));
    plhs[0] = mxCreateDoubleScalar(loss);
    if (nlhs > 1) plhs[1] = g;
    else mxDestroyArray(g);
  } else if (cmd == "autotune") {
    // chosen = gpe_mex('autotune', h, mode): FFT plan per axis (x, y, z)
    int ch[3];
    check(c, gpe_autotune(c, (int)scalar(prhs[2]), ch));
    plhs[0] = mxCreateDoubleMatrix(1, 3, mxREAL);
    for (int k = 0; k < 3; ++k) mxGetDoubles(plhs[0])[k] = ch[k];
  } else {
    mexErrMsgIdAndTxt("gpe:usage", "unknown command '%s'", cmd.c_str());
  }
}

// spinor_driver.cuh - host driver of the coherently coupled two-component
// split step (GPEtaskSpinor.solve_split, lib/@GPEtaskSpinor/solve_split.m of
// GPE-MATLAB) and its observables (GPEtaskSpinor.m:53-110).  Included by
// gpe_api.cu after the single-component drivers, whose pass, table and
// scalar helpers it uses.
//
// Per block of n_recalc steps (solve_split.m:66-113):
//   K/2 passes | (NL+coupling, K passes) x n_rec, the last K taking the
//   half-step factors (ekk .* ekkm = exp(-kk dt/2)) | kinetic sums, spinor
//   sums, finalizer (ncur, renormalisation factor kept pending, mu)
// The pending factor is applied by the next block's first NL kernel (the K/2
// passes before it are linear) or by materialize() when the state is read.
#pragma once

// The step constants of solve_split.m:61-64: cosom = cosh(dt |c|),
// sinomm/sinomp = sinh(dt |c|) exp(-/+ i angle(c)), in FP64, rounded once.
template <typename R>
SpinorNL<R> spinor_nl_consts(const gpe_ctx* c, double dre, double dim) {
  const gpe_spinor_params& p = c->spin;
  SpinorNL<R> q;
  q.g11 = (R)p.g[0];
  q.g12 = (R)p.g[1];
  q.g21 = (R)p.g[2];
  q.g22 = (R)p.g[3];
  q.dre = (R)dre;
  q.dim = (R)dim;
  const std::complex<double> dt(dre, dim), cpl(p.coupling_re, p.coupling_im);
  const double ac = std::abs(cpl), cang = std::arg(cpl);
  const std::complex<double> co = std::cosh(dt * ac), sh = std::sinh(dt * ac);
  const std::complex<double> sm = sh * std::exp(std::complex<double>(0.0, -cang));
  const std::complex<double> sp = sh * std::exp(std::complex<double>(0.0, cang));
  q.cosom = mk<R>((R)co.real(), (R)co.imag());
  q.sinomm = mk<R>((R)sm.real(), (R)sm.imag());
  q.sinomp = mk<R>((R)sp.real(), (R)sp.imag());
  q.nl = p.nlincpl != 0.0;
  q.nlincpl = (R)p.nlincpl;
  q.cre = (R)p.coupling_re;
  q.cim = (R)p.coupling_im;
  return q;
}

// GPEtaskSpinor's rotating frame outside the ITP's kinetic factors: its
// solve_split steps with the plain kinetic factor (solve_split.m:42-44 have no
// omega) and its applyham adds -omega lz with grid1d's stencil
// (GPEtaskSpinor.m:72-74).  While one is alive the kinetic tables and the
// energy passes of a context with scalar omega follow those rules.
struct SpinorOmegaScope {
  gpe_ctx* c;
  bool adi_off, lz_scalar;
  explicit SpinorOmegaScope(gpe_ctx* ctx) : c(ctx), adi_off(ctx->adi_off), lz_scalar(ctx->lz_scalar) {
    if (c->prm.omega != 0.0) {
      c->adi_off = true;
      c->lz_scalar = true;
    }
  }
  ~SpinorOmegaScope() {
    c->adi_off = adi_off;
    c->lz_scalar = lz_scalar;
  }
};

// Kinetic sums over both components, the spinor sums against Vsum and the
// finalizer in `mode` (0 run start, 1 block end, 2 observables).
template <typename R>
gpe_status spinor_finalize(gpe_ctx* c, Field& f, const R* Vsum, int mode, double time2, double* hist,
                           bool renorm, double* obs) {
  int nk[3] = {0, 0, 0};
  CHECK(energy_passes<R>(c, f, false, nk, nullptr));
  int ns;
  {
    Launch L(c, PC_NORM, (double)c->PS * (2 * sizeof(R) + sizeof(R)));
    ns = launch_spinor_sums<R>((const cx<R>*)f.psi, Vsum, c->P, c->sc, c->spin_part, c->stream);
    CU(cudaGetLastError());
  }
  SpinorFinalArgs a{};
  a.sums = c->spin_part;
  a.nsum = ns;
  a.partials = c->partials;
  a.cap = c->cap;
  for (int k = 0; k < 3; ++k) a.nblk_kin[k] = nk[k];
  a.weight = c->weight;
  for (int k = 0; k < 4; ++k) a.g[k] = c->spin.g[k];
  a.cre = c->spin.coupling_re;
  a.cim = c->spin.coupling_im;
  a.mode = mode;
  a.Ntotal = c->prm.Ntotal;
  a.renorm = renorm;
  a.tau = c->prm.decay_rate;
  a.time2 = time2;
  a.hist = hist;
  a.obs = obs;
  Launch L(c, PC_FINALIZE, 0);
  launch_finalize_spinor(a, c->sc, c->stream);
  CU(cudaGetLastError());
  return GPE_OK;
}

// getVtotal(time) of a time-dependent potential into the copy that the mu
// sums read (GPEtaskSpinor.applyham evaluates V at current_time,
// GPEtaskSpinor.m:53-58, while the step uses the block's time).
template <typename R>
gpe_status spinor_vmu(gpe_ctx* c, const gpe_split_params* prm, double time) {
  const size_t n = (size_t)c->PS;
  if (!c->Vmu) CU(cudaMalloc(&c->Vmu, n * sizeof(double)));
  if (sizeof(R) == 8) c->VmuR = nullptr;
  else if (!c->VmuR) CU(cudaMalloc(&c->VmuR, n * sizeof(R)));
  std::vector<double> h(n);
  if (prm->vtd(prm->vtd_user, time, h.data()) != 0)
    return fail(c, GPE_ERR_CALLBACK, "solve_split: potential callback failed");
  CU(cudaMemcpyAsync(c->Vmu, h.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (sizeof(R) == 4) {
    Launch L(c, PC_ELEMENTWISE, (double)n * 12);
    launch_convert_re<double, float>(c->Vmu, (float*)c->VmuR, (long long)n, c->stream);
    CU(cudaGetLastError());
  }
  CU(cudaStreamSynchronize(c->stream));  // h is pageable and goes out of scope
  return GPE_OK;
}

template <typename R>
const R* spinor_vmu_ptr(gpe_ctx* c) {
  return sizeof(R) == 8 ? (const R*)c->Vmu : (const R*)c->VmuR;
}

// GPEtaskSpinor.solve_split (solve_split.m:1-119) from the current state.
template <typename R>
gpe_status spinor_split_impl(gpe_ctx* c, const gpe_split_params* prm) {
  Field& f = c->main;
  const double ddt = prm->ddt, gam = c->prm.gamma;
  const int n_rec = c->prm.n_recalc;
  if (n_rec < 1) return fail(c, GPE_ERR_INVALID, "n_recalc must be >= 1");
  // jj = 1:niter_inner/n_rec (solve_split.m:66): floor(niter_inner/n_rec) blocks
  if (prm->niter_inner < n_rec)
    return fail(c, GPE_ERR_INVALID, "solve_split (spinor): niter_inner < n_recalc runs no block (solve_split.m:66)");
  const int nb = prm->niter_inner / n_rec;
  const int start = c->cur.current_iter, nout = prm->niter_outer;
  const std::complex<double> dtc = ddt * std::complex<double>(0.0, 1.0) / std::complex<double>(1.0, gam);  // :41
  const double dre = dtc.real(), dim = dtc.imag();
  SpinorOmegaScope scope(c);  // omega: plain kinetic factors, mu with -omega lz
  CHECK(set_kinop<R>(c, f, dre, dim));
  CHECK(materialize<R>(c));
  launch_reset_scalars(c->sc, c->stream);
  const bool vtd = prm->vtd != nullptr;
  if (vtd) CHECK(spinor_vmu<R>(c, prm, c->cur.current_time));
  // NN0 (:29-37) and mu = sum_j real(inner(phi_j, hphi_j))/NN0 (:52-57)
  CHECK(spinor_finalize<R>(c, f, vtd ? spinor_vmu_ptr<R>(c) : (const R*)f.V, 0, 0.0, nullptr, false, nullptr));
  const SpinorNL<R> q = spinor_nl_consts<R>(c, dre, dim);
  const std::vector<AxisPass> full = axis_passes(c);
  std::vector<AxisPass> half = full;
  for (auto& ap : half) ap.half = 1;
  const int nsteps_out = std::max(0, nout - start);
  const size_t hlen = 3 * (size_t)std::max(1, nsteps_out);  // (mu, ncur, energy) per outer step
  if (c->d_hist_len < hlen) {
    cudaFree(c->d_hist);
    c->d_hist = nullptr;
    CU(cudaMalloc(&c->d_hist, hlen * sizeof(double)));
    c->d_hist_len = hlen;
  }
  CU(cudaMemsetAsync(c->d_hist, 0, hlen * sizeof(double), c->stream));
  const double dt_outer = ddt * prm->niter_inner;
  int vk = 0, last_j = start;
  double time2 = c->cur.current_time;
  bool stopped = false;
  for (int j = start + 1; j <= nout && !stopped; ++j) {
    const double time = (j - 1) * dt_outer;
    for (int jj = 1; jj <= nb; ++jj) {
      time2 = time + (jj - 1) * ddt * n_rec;
      if (vtd) CHECK(vtd_upload<R>(c, prm, time2, vk));  // VV = getVtotal(time2) (:69)
      for (const auto& ap : half) CHECK(run_pass<R>(c, f, ap, KIND_STEP, PRO_NONE, EPI_NONE, 0, dre, dim, nullptr));
      for (int i = 1; i <= n_rec; ++i) {
        {
          Launch L(c, PC_NL_PHASE, (double)c->PS * (4 * sizeof(R) + sizeof(R)));
          launch_spinor_nl<R>((cx<R>*)f.psi, (const R*)f.V, c->P, c->sc, i == 1, q, c->stream);
          CU(cudaGetLastError());
        }
        for (const auto& ap : (i == n_rec ? half : full))
          CHECK(run_pass<R>(c, f, ap, KIND_STEP, PRO_NONE, EPI_NONE, 0, dre, dim, nullptr));
      }
      double* hist = (jj == nb) ? c->d_hist + 3 * (size_t)(j - start - 1) : nullptr;
      CHECK(spinor_finalize<R>(c, f, vtd ? spinor_vmu_ptr<R>(c) : (const R*)f.V, 1, time2, hist, gam > 0,
                               nullptr));
    }
    last_j = j;
    // ext_callback (:115): current_time = time2 from here on
    if (prm->on_step || vtd) {
      DevScalars h;
      CHECK(read_scalars(c, &h));
      if (h.nonfinite) break;
      c->cur.current_iter = j;
      c->cur.current_time = time2;
      c->cur.current_mu = h.muc;
      c->cur.current_n = h.ncur;
      if ((int)c->hist_mu.size() < j) {
        c->hist_mu.resize(j, 0.0);
        c->hist_n.resize(j, 0.0);
        c->hist_e.resize(j, 0.0);
      }
      c->hist_mu[j - 1] = h.muc;
      c->hist_n[j - 1] = h.ncur;
      c->hist_e[j - 1] = h.energy;
      if (prm->on_step && prm->on_step(prm->step_user, j, time2, h.muc, h.ncur) != 0) stopped = true;
      if (vtd && !stopped && j < nout) CHECK(spinor_vmu<R>(c, prm, time2));
    }
  }
  DevScalars h;
  CHECK(read_scalars(c, &h));
  if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "solve_split: non-finite norm or chemical potential");
  if (last_j > start) {
    std::vector<double> dh(3 * (size_t)(last_j - start));
    CU(cudaMemcpy(dh.data(), c->d_hist, dh.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if ((int)c->hist_mu.size() < last_j) {
      c->hist_mu.resize(last_j, 0.0);
      c->hist_n.resize(last_j, 0.0);
      c->hist_e.resize(last_j, 0.0);
    }
    for (int j = start + 1; j <= last_j; ++j) {
      c->hist_mu[j - 1] = dh[3 * (size_t)(j - start - 1)];
      c->hist_n[j - 1] = dh[3 * (size_t)(j - start - 1) + 1];
      c->hist_e[j - 1] = dh[3 * (size_t)(j - start - 1) + 2];
    }
    c->cur.current_iter = last_j;
    c->cur.current_time = time2;
    c->cur.current_mu = h.muc;
    c->cur.current_n = h.ncur;
  }
  return GPE_OK;
}

// applyham / get_energy pieces of both components at the current V.
template <typename R>
gpe_status spinor_observables(gpe_ctx* c, gpe_obs* o) {
  SpinorOmegaScope scope(c);  // -omega lz inside ekin
  CHECK(materialize<R>(c));
  launch_reset_scalars(c->sc, c->stream);
  double* obs = c->spin_part + (size_t)SP_NSUMS * 8 * c->sms;
  CHECK(spinor_finalize<R>(c, c->main, (const R*)c->main.V, 2, 0.0, nullptr, false, obs));
  double v[5];
  CU(cudaMemcpyAsync(v, obs, sizeof(v), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  o->norm = v[0];
  o->ekin = v[1];
  o->epot = v[2];
  o->eint = v[3];
  o->ecpl = v[4];
  o->mu_integral = v[1] + v[2] + v[3] + v[4];
  o->energy = v[1] + v[2] + 0.5 * v[3] + v[4];  // get_energy halves g (GPEtaskSpinor.m:98-110)
  return GPE_OK;
}

// GPEtaskSpinor.groundstate_itp (lib/@GPEtaskSpinor/groundstate_itp.m:1-145;
// omega != 0 on 2D grids) from the current state.  Per iteration: the nonlinear factors of
// the state before the kinetic half step, the half step, the coupling rotation
// times the factors, the half step, normalisation to Ntotal (MU = log(m)/dt),
// and with want_mu2 / want_energy MU2 and EE of every iteration (otherwise
// MU2 = MU and EE = MU2, as with fewer outputs there).  Every 10 iterations
// after iswitch + 10 the host tests delta = (|EE(i)-EE(i-9)|/9 +
// |EE(i)-EE(i-1)|)/dt < eps: then it stops if dt < eps or dt < 5e-6, or
// divides dt by 1.5.  The arrays returned drop the last iteration (:132-141).
template <typename R>
gpe_status spinor_itp_impl(gpe_ctx* c, const gpe_itp_params* prm, double* MU, double* MU2, double* EE, int cap,
                           gpe_itp_result* res) {
  Field& f = c->main;
  const long long P = c->P;
  const int maxit = std::max(1, c->prm.itp_max_iter);
  const bool want_mu2 = prm->want_mu2 != 0, want_e = prm->want_energy != 0;
  double dt = prm->dt;
  const double eps = prm->eps;
  if (!(c->prm.Ntotal > 0)) return fail(c, GPE_ERR_INVALID, "groundstate_itp (spinor): Ntotal must be positive");
  // f_j buffer (2P) and the per-iteration MU, MU2, EE arrays on the device
  if (!f.aux) CU(cudaMalloc(&f.aux, (size_t)c->PS * sizeof(R)));
  const size_t hlen = 3 * (size_t)maxit;
  if (c->d_hist_len < hlen) {
    cudaFree(c->d_hist);
    c->d_hist = nullptr;
    CU(cudaMalloc(&c->d_hist, hlen * sizeof(double)));
    c->d_hist_len = hlen;
  }
  double* dMU = c->d_hist;
  double* dMU2 = c->d_hist + maxit;
  double* dEE = c->d_hist + 2 * (size_t)maxit;
  CHECK(materialize<R>(c));
  launch_reset_scalars(c->sc, c->stream);
  // Rotating frame (2D, :30-33, 61-80): the kinetic half step is the x factor
  // then the y factor, on both sides of the nonlinear factor; energies use
  // lap without omega plus -omega lz with grid1d's stencil (GPEtaskSpinor.m:72-74).
  const bool rot = c->prm.omega != 0.0;
  SpinorOmegaScope scope(c);
  auto set_tables = [&](double h) -> gpe_status {
    if (rot) return rot_half_tables<R>(c, f, 0.5 * h, f.rth[0]);
    return set_kinop<R>(c, f, h, 0.0);
  };
  CHECK(set_tables(dt));
  SpinorNL<R> q = spinor_nl_consts<R>(c, dt, 0.0);  // cosh / sinh(dt |c|) with the coupling phase (:45-48)
  std::vector<AxisPass> half = rot ? rot_xy_passes(c, false) : axis_passes(c);
  if (!rot)
    for (auto& ap : half) ap.half = 1;
  auto kinetic = [&]() -> gpe_status {
    Field fr = rot ? rot_view(f, f.rth[0]) : f;
    for (const auto& ap : half) CHECK(run_pass<R>(c, fr, ap, KIND_STEP, PRO_NONE, EPI_NONE, 0, dt, 0.0, nullptr));
    return GPE_OK;
  };
  auto ee_of = [&](int i, std::vector<double>& host, int lo) { return host[i - lo]; };
  int i = 1, iswitch = 20;
  bool converged = false;
  double last_delta = NAN;
  std::vector<double> win;
  for (;; ++i) {
    {
      Launch L(c, PC_NL_PHASE, (double)c->PS * (2 * sizeof(R) + 2 * sizeof(R)));
      launch_spinor_itp_factors<R>((const cx<R>*)f.psi, (const R*)f.V, P, c->sc, q, (R*)f.aux, 0, c->stream);
    }
    CHECK(kinetic());
    {
      Launch L(c, PC_NL_PHASE, (double)c->PS * (4 * sizeof(R) + sizeof(R)));
      launch_spinor_itp_couple<R>((cx<R>*)f.psi, (const R*)f.aux, P, c->sc, q, 0, c->stream);
      launch_set_scale_one(c->sc, c->stream);
    }
    CHECK(kinetic());
    int nb;
    {
      Launch L(c, PC_NORM, (double)c->PS * 2 * sizeof(R));
      nb = launch_norm<R>((const cx<R>*)f.psi, c->PS, c->sc, c->partials, c->cap, c->stream);
    }
    ItpFinalArgs a{c->partials, c->cap, nb, c->weight, dt, c->prm.Ntotal, 0.0, i, dMU};
    {
      Launch L(c, PC_FINALIZE, 0);
      launch_finalize_itp(a, c->sc, c->stream);  // scale = m = sqrt(Ntotal/ntot), MU(i) = log(m)/dt
    }
    if (want_mu2 || want_e)
      CHECK(spinor_finalize<R>(c, f, (const R*)f.V, 3, 0.0, want_mu2 ? dMU2 + (i - 1) : nullptr, false,
                               want_e ? dEE + (i - 1) : nullptr));
    CU(cudaGetLastError());
    if ((i - iswitch) > 10 && i % 10 == 0) {
      // EE(i-9 .. i): EE = MU2 without want_energy, MU2 = MU without want_mu2
      const double* src = want_e ? dEE : (want_mu2 ? dMU2 : dMU);
      win.resize(10);
      CU(cudaMemcpyAsync(win.data(), src + (i - 10), 10 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      DevScalars h;
      CHECK(read_scalars(c, &h));  // synchronises
      if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "groundstate_itp (spinor): non-finite norm");
      const double e_i = ee_of(i, win, i - 9), e_i1 = ee_of(i - 1, win, i - 9), e_i9 = ee_of(i - 9, win, i - 9);
      const double delta = (std::abs(e_i - e_i9) / 9 + std::abs(e_i - e_i1)) / dt;
      last_delta = delta;
      if (delta < eps) {
        if (dt < eps || dt < 5e-6) {
          converged = true;
          break;
        }
        dt = dt / 1.5;
        CHECK(set_tables(dt));
        q = spinor_nl_consts<R>(c, dt, 0.0);
        iswitch = i;
      }
    }
    if (i >= maxit) break;  // the reference warns (:123-126)
  }
  DevScalars h;
  CHECK(read_scalars(c, &h));
  if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "groundstate_itp (spinor): non-finite norm");
  CHECK(materialize<R>(c));  // the state times its normalisation factor
  const int n_out = i - 1;   // MU(1:i-1) (:132-141)
  const int k = std::min(n_out, cap);
  std::vector<double> hm(std::max(k, 1));
  if (k > 0) {
    CU(cudaMemcpy(hm.data(), dMU, k * sizeof(double), cudaMemcpyDeviceToHost));
    if (MU) std::copy(hm.begin(), hm.begin() + k, MU);
    std::vector<double> h2(k), he(k);
    if (want_mu2) CU(cudaMemcpy(h2.data(), dMU2, k * sizeof(double), cudaMemcpyDeviceToHost));
    else h2 = std::vector<double>(hm.begin(), hm.begin() + k);
    if (want_e) CU(cudaMemcpy(he.data(), dEE, k * sizeof(double), cudaMemcpyDeviceToHost));
    else he = h2;
    if (MU2) std::copy(h2.begin(), h2.end(), MU2);
    if (EE) std::copy(he.begin(), he.end(), EE);
  }
  if (res) {
    res->iters = n_out;
    res->converged = converged;
    res->fp32_iters = 0;
    res->final_dt = dt;
    res->last_delta = last_delta;  // the last convergence test's delta (NaN: none ran)
    res->ms_main = 0.0;  // not timed on this path
    res->ms_fp64 = 0.0;
  }
  if (!converged) c->err = "groundstate_itp: Convergence not reached";
  return GPE_OK;
}

// GPEtask2comp.groundstate_itp (lib/@GPEtask2comp/groundstate_itp.m:1-157;
// omega != 0 on 2D grids) from the current state of a spinor context, coupling = 0.  Per
// iteration: the factors exp(-(V_j + sum_k g(j,k)|psi_k|^2) dt) from the state
// before the step (:58-59), the kinetic half step with each component's own
// exp(-kk dt/2/M_j) (:67-68; one launch over both components when M1 == M2),
// the factors, the kinetic half step again (:78-79), the two norms and the
// finalizer (m_j = sqrt(N_j/n_j) kept pending per component, MU1(i), MU2(i),
// :82-90).  With want_energy the factors are applied at once and EE(i) =
// get_energy/Ntotal (:98-99); the convergence test of :113-135 runs on EE
// (MU2 without want_energy, :101).
template <typename R>
gpe_status mix_itp_impl(gpe_ctx* c, const gpe_itp_params* prm, double N1, double N2, double M1, double M2,
                        double* MU1, double* MU2, double* EE, int cap, gpe_itp_result* res) {
  Field& f = c->main;
  const long long P = c->P;
  const int maxit = std::max(1, c->prm.itp_max_iter);
  const bool want_e = prm->want_energy != 0;
  double dt = prm->dt;
  const double eps = prm->eps;
  if (!(N1 > 0) || !(N2 > 0)) return fail(c, GPE_ERR_INVALID, "groundstate_itp (2comp): N1 and N2 must be positive");
  if (!(M1 > 0) || !(M2 > 0)) return fail(c, GPE_ERR_INVALID, "groundstate_itp (2comp): M1 and M2 must be positive");
  if (want_e && !(c->prm.Ntotal > 0))
    return fail(c, GPE_ERR_INVALID, "groundstate_itp (2comp): EE divides by Ntotal, which must be positive");
  if (c->spin.coupling_re != 0.0 || c->spin.coupling_im != 0.0 || c->spin.nlincpl != 0.0)
    return fail(c, GPE_ERR_INVALID, "groundstate_itp (2comp): an incoherent mixture has coupling = nlincpl = 0");
  if (!f.aux) CU(cudaMalloc(&f.aux, (size_t)c->PS * sizeof(R)));
  const size_t hlen = 3 * (size_t)maxit;
  if (c->d_hist_len < hlen) {
    cudaFree(c->d_hist);
    c->d_hist = nullptr;
    CU(cudaMalloc(&c->d_hist, hlen * sizeof(double)));
    c->d_hist_len = hlen;
  }
  double* dMU1 = c->d_hist;
  double* dMU2 = c->d_hist + maxit;
  double* dEE = c->d_hist + 2 * (size_t)maxit;
  CHECK(materialize<R>(c));  // also resets scale2
  launch_reset_scalars(c->sc, c->stream);
  const bool same_mass = M1 == M2;
  // Rotating frame (2D, :31-36, 61-80): x then y half steps before the
  // nonlinear factor, y then x after it, each with exp(-(k^2/2 -+ k c omega)
  // dt/2/M_j); energies use lap(phi, omega) (GPEtask2comp.m:60).
  const bool rot = c->prm.omega != 0.0;
  auto set_tables = [&](double h) -> gpe_status {
    if (rot) {
      CHECK(rot_half_tables<R>(c, f, 0.5 * h / M1, f.rth[0]));
      if (!same_mass) CHECK(rot_half_tables<R>(c, f, 0.5 * h / M2, f.rth[1]));
      return GPE_OK;
    }
    CHECK(set_kinop<R>(c, f, h / M1, 0.0));  // php2 = exp(-kk h/2/M1)
    if (!same_mass)
      for (int ax = 0; ax < c->ndims; ++ax) CHECK(half_table<R>(c, f, ax, h / M2, 0.0, f.php2b[ax]));
    return GPE_OK;
  };
  CHECK(set_tables(dt));
  SpinorNL<R> q = spinor_nl_consts<R>(c, dt, 0.0);  // coupling 0: cosom = 1, sinomm = sinomp = 0
  std::vector<AxisPass> both = axis_passes(c), one = axis_passes(c, 0.0, true), two = one;
  for (auto& ap : both) ap.half = 1;
  for (auto& ap : one) ap.half = 1;
  for (auto& ap : two) ap.half = 2;
  cx<R>* psi2 = (cx<R>*)f.psi + P;
  const std::vector<AxisPass> rboth = rot ? rot_xy_passes(c, false) : std::vector<AxisPass>();
  const std::vector<AxisPass> rone = rot ? rot_xy_passes(c, true) : std::vector<AxisPass>();
  bool second = false;  // the half step after the nonlinear factor (y first)
  auto kinetic = [&]() -> gpe_status {
    if (rot) {
      const int o0 = second ? 1 : 0, o1 = 1 - o0;
      if (same_mass) {
        Field fr = rot_view(f, f.rth[0]);
        for (int k : {o0, o1}) CHECK(run_pass<R>(c, fr, rboth[k], KIND_STEP, PRO_NONE, EPI_NONE, 0, dt, 0.0, nullptr));
      } else {
        for (int j = 0; j < 2; ++j) {
          Field fr = rot_view(f, f.rth[j]);
          void* pj = j == 0 ? f.psi : (void*)psi2;
          for (int k : {o0, o1})
            CHECK(run_pass<R>(c, fr, rone[k], KIND_STEP, PRO_NONE, EPI_NONE, 0, dt, 0.0, nullptr, pj));
        }
      }
      return GPE_OK;
    }
    if (same_mass) {
      for (const auto& ap : both) CHECK(run_pass<R>(c, f, ap, KIND_STEP, PRO_NONE, EPI_NONE, 0, dt, 0.0, nullptr));
      return GPE_OK;
    }
    for (const auto& ap : one) CHECK(run_pass<R>(c, f, ap, KIND_STEP, PRO_NONE, EPI_NONE, 0, dt, 0.0, nullptr, f.psi));
    for (const auto& ap : two) CHECK(run_pass<R>(c, f, ap, KIND_STEP, PRO_NONE, EPI_NONE, 0, dt, 0.0, nullptr, psi2));
    return GPE_OK;
  };
  int i = 1, iswitch = 20;
  bool converged = false, pending = false;
  double last_delta = NAN;
  std::vector<double> win(10);
  for (;; ++i) {
    {
      Launch L(c, PC_NL_PHASE, (double)c->PS * (2 * sizeof(R) + 2 * sizeof(R)));
      launch_spinor_itp_factors<R>((const cx<R>*)f.psi, (const R*)f.V, P, c->sc, q, (R*)f.aux, 1, c->stream);
    }
    second = false;
    CHECK(kinetic());
    {
      Launch L(c, PC_NL_PHASE, (double)c->PS * (4 * sizeof(R) + sizeof(R)));
      launch_spinor_itp_couple<R>((cx<R>*)f.psi, (const R*)f.aux, P, c->sc, q, 1, c->stream);
      launch_set_scale_one(c->sc, c->stream);
    }
    second = true;
    CHECK(kinetic());
    MixFinalArgs a{};
    {
      Launch L(c, PC_NORM, (double)c->PS * 2 * sizeof(R));
      a.nblk1 = launch_norm<R>((const cx<R>*)f.psi, P, c->sc, c->partials, c->cap, c->stream);
      a.nblk2 = launch_norm<R>(psi2, P, c->sc, c->partials + c->cap, c->cap, c->stream);
    }
    a.part1 = c->partials + (size_t)S_N * c->cap;
    a.part2 = c->partials + (size_t)(S_N + 1) * c->cap;
    a.weight = c->weight;
    a.dt = dt;
    a.N1 = N1;
    a.N2 = N2;
    a.iter = i;
    a.MU1 = dMU1;
    a.MU2 = dMU2;
    {
      Launch L(c, PC_FINALIZE, 0);
      launch_finalize_mix(a, c->sc, c->stream);
    }
    pending = true;
    if (want_e) {
      {
        Launch L(c, PC_ELEMENTWISE, (double)c->PS * 4 * sizeof(R));
        launch_mix_apply_scales<R>((cx<R>*)f.psi, P, c->sc, c->stream);
        launch_set_scale_one(c->sc, c->stream);
      }
      pending = false;
      CHECK(spinor_finalize<R>(c, f, (const R*)f.V, 3, 0.0, nullptr, false, dEE + (i - 1)));
    }
    CU(cudaGetLastError());
    if ((i - iswitch) > 10 && i % 10 == 0) {
      const double* src = want_e ? dEE : dMU2;
      CU(cudaMemcpyAsync(win.data(), src + (i - 10), 10 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      DevScalars h;
      CHECK(read_scalars(c, &h));  // synchronises
      if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "groundstate_itp (2comp): non-finite norm");
      // win[k] = EE(i-9+k): EE(i) = win[9], EE(i-1) = win[8], EE(i-9) = win[0]
      const double delta = (std::abs(win[9] - win[0]) / 9 + std::abs(win[9] - win[8])) / dt;
      last_delta = delta;
      if (delta < eps) {
        if (dt < eps || dt < 5e-6) {
          converged = true;
          break;
        }
        dt = dt / 1.5;
        CHECK(set_tables(dt));
        q = spinor_nl_consts<R>(c, dt, 0.0);
        iswitch = i;
      }
    }
    if (i >= maxit) break;  // the reference warns (:136-139)
  }
  if (pending) {
    Launch L(c, PC_ELEMENTWISE, (double)c->PS * 4 * sizeof(R));
    launch_mix_apply_scales<R>((cx<R>*)f.psi, P, c->sc, c->stream);
    launch_set_scale_one(c->sc, c->stream);
  }
  DevScalars h;
  CHECK(read_scalars(c, &h));
  if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "groundstate_itp (2comp): non-finite norm");
  const int n_out = i - 1;  // MU1(1:i-1) (:143-154)
  const int k = std::min(n_out, cap);
  if (k > 0) {
    std::vector<double> h1(k), h2(k), he(k);
    CU(cudaMemcpy(h1.data(), dMU1, k * sizeof(double), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(h2.data(), dMU2, k * sizeof(double), cudaMemcpyDeviceToHost));
    if (want_e) CU(cudaMemcpy(he.data(), dEE, k * sizeof(double), cudaMemcpyDeviceToHost));
    else he = h2;
    if (MU1) std::copy(h1.begin(), h1.end(), MU1);
    if (MU2) std::copy(h2.begin(), h2.end(), MU2);
    if (EE) std::copy(he.begin(), he.end(), EE);
  }
  if (res) {
    res->iters = n_out;
    res->converged = converged;
    res->fp32_iters = 0;
    res->final_dt = dt;
    res->last_delta = last_delta;
    res->ms_main = 0.0;  // not timed on this path
    res->ms_fp64 = 0.0;
  }
  if (!converged) c->err = "groundstate_itp: Convergence not reached";
  return GPE_OK;
}

// observables_driver.cuh - host side of the on-device observables
// (observables.cu): vortex-core detection on a slice of the state
// (lib/util/detect_core.m of GPE-MATLAB) and the Thomas-Fermi guess
// (lib/@GPEtask/groundstate_tf.m).  Included by gpe_api.cu.
#pragma once

// Scratch of the observables, cached in the context (grown on demand).
static gpe_status obs_scratch(gpe_ctx* c, size_t bytes, void** out) {
  if (c->obs_len < bytes) {
    cudaFree(c->obs_buf);
    c->obs_buf = nullptr;
    c->obs_len = 0;
    CU(cudaMalloc(&c->obs_buf, bytes));
    c->obs_len = bytes;
  }
  *out = c->obs_buf;
  return GPE_OK;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

template <typename R>
gpe_status detect_core_impl(gpe_ctx* c, int comp, int z, int refine, double* pos, int cap_pos, int* n_pos,
                            double* neg, int cap_neg, int* n_neg) {
  const int nx = c->n[0], ny = c->n[1];
  const long long n = (long long)nx * ny;
  const int nb = elem_grid(n, 256), nch = core_chunks(n);
  const size_t b_max = align256((size_t)nb * sizeof(double)), b_thr = align256(sizeof(double));
  const size_t b_q = align256((size_t)n), b_cnt = align256((size_t)2 * nch * sizeof(int));
  const size_t b_off = align256(((size_t)2 * nch + 2) * sizeof(int));
  const size_t b_pos = align256((size_t)2 * std::max(cap_pos, 1) * sizeof(double));
  const size_t b_neg = align256((size_t)2 * std::max(cap_neg, 1) * sizeof(double));
  void* buf = nullptr;
  CHECK(obs_scratch(c, b_max + b_thr + b_q + b_cnt + b_off + b_pos + b_neg, &buf));
  char* p = static_cast<char*>(buf);
  CoreScratch w;
  w.blockmax = reinterpret_cast<double*>(p);
  w.thr = reinterpret_cast<double*>(p + b_max);
  w.q = reinterpret_cast<signed char*>(p + b_max + b_thr);
  w.cnt = reinterpret_cast<int*>(p + b_max + b_thr + b_q);
  w.off = reinterpret_cast<int*>(p + b_max + b_thr + b_q + b_cnt);
  double* dpos = reinterpret_cast<double*>(p + b_max + b_thr + b_q + b_cnt + b_off);
  double* dneg = reinterpret_cast<double*>(p + b_max + b_thr + b_q + b_cnt + b_off + b_pos);
  CoreGeom geo;
  geo.x0 = coord(c, 0, 0);
  geo.y0 = coord(c, 1, 0);
  geo.hxg = c->dx[0];
  geo.hyg = c->dx[1];
  // detect_core.m:13-14: dx = rx(1,end/2+1) - rx(1,end/2), dy likewise
  geo.hx = coord(c, 0, nx / 2) - coord(c, 0, nx / 2 - 1);
  geo.hy = coord(c, 1, ny / 2) - coord(c, 1, ny / 2 - 1);
  geo.refine = refine > 0;
  const cx<R>* slice = (const cx<R>*)c->main.psi + (long long)comp * c->P + (long long)z * n;
  {
    Launch L(c, PC_ELEMENTWISE, (double)n * 2 * sizeof(R));
    CU(launch_detect_core<R>(slice, nx, ny, geo, w, dpos, cap_pos, dneg, cap_neg, c->stream));
  }
  int tot[2];
  CU(cudaMemcpyAsync(tot, w.off + 2 * nch, sizeof(tot), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  *n_pos = tot[0];
  *n_neg = tot[1];
  const int kp = std::min(tot[0], cap_pos), km = std::min(tot[1], cap_neg);
  if (kp > 0) CU(cudaMemcpy(pos, dpos, (size_t)2 * kp * sizeof(double), cudaMemcpyDeviceToHost));
  if (km > 0) CU(cudaMemcpy(neg, dneg, (size_t)2 * km * sizeof(double), cudaMemcpyDeviceToHost));
  return GPE_OK;
}

// Sum of nb per-CTA partials on the host in CTA order.
static double host_sum(const std::vector<double>& v, int nb) {
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += v[i];
  return s;
}

template <typename R>
gpe_status groundstate_tf_impl(gpe_ctx* c, double eps, double N, const double* bounds, double* mu_out) {
  const long long P = c->P;
  const double* V = c->V64;  // the FP64 potential last set (both precisions keep it)
  std::vector<double> h(2 * 8 * (size_t)c->sms + 16);
  double mul, mur;
  if (bounds) {
    mul = bounds[0];
    mur = bounds[1];
  } else {  // groundstate_tf.m:22-23
    const int nb = launch_minmax(V, P, c->partials, c->stream);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(h.data(), c->partials, (size_t)2 * nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    mul = INFINITY;
    mur = -INFINITY;
    for (int i = 0; i < nb; ++i) {
      mul = std::min(mul, h[2 * i]);
      mur = std::max(mur, h[2 * i + 1]);
    }
  }
  const double g = c->prm.g;
  const double NC = N * g;  // :25
  double mu = (mul + mur) / 2, mu_eval = mu;
  for (int it = 0; (mur - mul) / mu > eps; ++it) {  // :27-36
    if (it >= 4096) return fail(c, GPE_ERR_INVALID, "groundstate_tf: bisection did not reach eps");
    mu_eval = mu;
    const int nb = launch_tf_sum(V, P, mu, c->partials, c->stream);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(h.data(), c->partials, (size_t)nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    const double NN = host_sum(h, nb) * c->weight;
    if (NN > NC) mur = mu;
    else mul = mu;
    mu = (mul + mur) / 2;
  }
  // phi = sqrt(vvv/g(1)) with vvv of the last evaluated mu (:37)
  launch_tf_state<R>((cx<R>*)c->main.psi, V, P, mu_eval, g, c->stream);
  launch_set_scale_one(c->sc, c->stream);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(c->stream));
  c->have_state = true;
  *mu_out = mu;
  return GPE_OK;
}

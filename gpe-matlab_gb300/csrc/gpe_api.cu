// gpe_api.cu - C ABI of libgpe (include/gpe.h): context, data movement and
// the host drivers of GPEtask.groundstate_itp / GPEtask.solve_split.
//
// The drivers enqueue every kernel of a run on the context stream and keep
// the reference's scalar bookkeeping (norms, mu, the ITP residual) in device
// memory, so the host only synchronises where the reference's semantics need
// a host decision: at ITP convergence checks (one check interval behind the
// device, the kernels of speculatively enqueued iterations return at once
// once a finalizer has stopped the run), at outer-step callbacks, and when a
// time-dependent potential is evaluated on the host.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "cluster2d.h"
#include "ctx.h"
#include "grid2d.h"
#include "pass_x2.cuh"

using namespace gpe;

namespace {

thread_local std::string g_create_err;

gpe_status fail(gpe_ctx* c, gpe_status st, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_err = msg;
  return st;
}

#define CU(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(c, GPE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CHECK(st)                  \
  do {                             \
    gpe_status s_ = (st);          \
    if (s_ != GPE_OK) return s_;   \
  } while (0)

// The bounds-checked build's report (common.cuh BoundsSite).
std::string bounds_message(const char* where, const DevScalars& h) {
  static const char* names[] = {"none", "state load", "state store", "side-array load", "ITP-factor store",
                                "shared-memory exchange", "partial-sum slot", "cluster shared memory"};
  const int s = h.bounds_site;
  return std::string(where) + ": index out of range at " + (s >= 0 && s < 8 ? names[s] : "an unknown site") +
         " (index " + std::to_string(h.bounds_index) + ")";
}

bool supported_n(int n) {
  switch (n) {
#define X(v) case v:
    GPE_FOR_EACH_N(X)
#undef X
    return true;
    default:
      return false;
  }
}

// Axis lengths with an alternative plan (FP32 direct passes).
bool has_alt_plan(int n) {
  switch (n) {
#define X(v) case v:
    GPE_FOR_EACH_ALT(X)
#undef X
    return true;
    default:
      return false;
  }
}

// Axis lengths whose default plan has a paired pass (E = 16).
bool has_x2d_plan(int n) { return n == 128 || n == 256 || n == 512; }

// var: plan variant (0 = Plan<N>; 1 = PlanAlt<N>, FP32 and has_alt_plan(N) only;
// 2 = PlanAlt<N> with the paired step pass (pass_x2.cuh) for the plain step
// passes it applies to, the scalar PlanAlt<N> kernels for the others;
// 3 = the same on Plan<N>, has_x2d_plan(N) only).
bool x2_pass(int var, const PassArgs<float>& a, bool strided) {
  return (var == 2 || var == 3) && x2_applies(a, strided);
}
// The scalar plan variant behind a paired one (its tables and fallback kernels).
int scalar_var(int var) { return var == 2 ? 1 : var == 3 ? 0 : var; }

template <typename R>
cudaError_t dispatch_pass(int N, int var, const PassArgs<R>& a, bool strided, cudaStream_t s) {
  if constexpr (sizeof(R) == 4) {
    if (x2_pass(var, a, strided)) {
      if (var == 3) {
        switch (N) {
          case 128: return launch_pass_x2<128, 0>(a, strided, s);
          case 256: return launch_pass_x2<256, 0>(a, strided, s);
          case 512: return launch_pass_x2<512, 0>(a, strided, s);
        }
        return cudaErrorInvalidValue;
      }
      switch (N) {
#define X(v) \
  case v:    \
    return launch_pass_x2<v, 1>(a, strided, s);
        GPE_FOR_EACH_ALT(X)
#undef X
      }
      return cudaErrorInvalidValue;
    }
    if (var == 1 || var == 2) {
      switch (N) {
#define X(v) \
  case v:    \
    return launch_pass<float, v, 1>(a, strided, s);
        GPE_FOR_EACH_ALT(X)
#undef X
      }
      return cudaErrorInvalidValue;
    }
  }
  switch (N) {
#define X(v) \
  case v:    \
    return launch_pass<R, v>(a, strided, s);
    GPE_FOR_EACH_N(X)
#undef X
  }
  return cudaErrorInvalidValue;
}

PassGeom dispatch_x2_geom(int N, int var, bool strided) {
  if (var == 3) {
    switch (N) {
      case 128: return pass_x2_geom<128, 0>(strided);
      case 256: return pass_x2_geom<256, 0>(strided);
      case 512: return pass_x2_geom<512, 0>(strided);
    }
    return PassGeom{0, 1, 0};
  }
  switch (N) {
#define X(v) \
  case v:    \
    return pass_x2_geom<v, 1>(strided);
    GPE_FOR_EACH_ALT(X)
#undef X
  }
  return PassGeom{0, 1, 0};
}

template <typename R>
PassGeom dispatch_geom(int N, int var, bool strided) {
  if constexpr (sizeof(R) == 4) {
    if (var == 1 || var == 2) {
      switch (N) {
#define X(v) \
  case v:    \
    return pass_geom<float, v, 1>(strided);
        GPE_FOR_EACH_ALT(X)
#undef X
      }
      return PassGeom{0, 1, 0};
    }
  }
  switch (N) {
#define X(v) \
  case v:    \
    return pass_geom<R, v>(strided);
    GPE_FOR_EACH_N(X)
#undef X
  }
  return PassGeom{0, 1, 0};
}

// The scalar omega of the rotating-frame kinetic factors (set_kinop.m:5-7,
// ssft_kin_step.m:12-15, lap.m:8-10); 0 while a rotating SGPE runs, whose
// omega enters only through its Lz Crank-Nicolson update.
double adi_omega(const gpe_ctx* c) { return c->adi_off ? 0.0 : c->prm.omega; }

enum { SPLIT_FULL = 0, SPLIT_FWD = 1, SPLIT_INV = 2, SPLIT_MASKED = 3 };

struct AxisPass {
  int axis;  // 0 = x, 1 = y, 2 = z
  int N;
  bool strided;
  long long n_batch, stride, inner, outer;
  int rot = 0;  // rotating frame: 1 = x pass with exp(+kx y omega dt/2), 2 = y pass with exp(-ky x omega dt)
  int split = SPLIT_FULL;  // energy cut-off chain: forward half only, inverse half only, or the masked pass
  double ecut = 0.0;
  int half = 0;  // spinor contexts: the half-step kinetic factors exp(-k^2/2 dt/2); 2: component 2's (php2b)
  int one_comp = 0;  // the pencils of one component only (psi_buf points at it)
};

// Pass order: y (contiguous, carries the prologue), x, then z (3D).  The
// last pass carries the epilogue.  Rotating frame (scalar omega,
// ssft_kin_step.m:12-15): x half step, y (and z), x half step again.
//
// Energy cut-off (ecut > 0, SGPEtask/solve_split.m:40-42): the mask kk < ecut
// does not factor over the axes, so the kinetic step becomes y and x forward
// halves (spectra stored in slot order), the last axis whole with the mask
// between its halves, then the x and y inverse halves: 2D y x~ y, 3D y x z~ x y.
//
// Spinor contexts: the components lie one after the other, so the pencils of
// every component are one batch (pencil index b = pencil + component * count;
// for z pencils outer = P steps to the next component).
std::vector<AxisPass> axis_passes(const gpe_ctx* c, double ecut = 0.0, bool one_comp = false) {
  const long long nx = c->n[0], ny = c->n[1], nz = c->ndims == 3 ? c->n[2] : 1, nc = one_comp ? 1 : c->ncomp;
  const AxisPass py{1, (int)ny, false, nx * nz * nc, 1, 1, 0};
  const AxisPass px{0, (int)nx, true, ny * nz * nc, ny, ny, nx * ny};
  const AxisPass pz{2, (int)nz, true, nx * ny * nc, nx * ny, nx * ny, c->P};
  std::vector<AxisPass> v;
  if (ecut > 0.0) {
    std::vector<AxisPass> fw{py, px};
    if (c->ndims == 3) fw.push_back(pz);
    for (size_t k = 0; k + 1 < fw.size(); ++k) {
      v.push_back(fw[k]);
      v.back().split = SPLIT_FWD;
    }
    v.push_back(fw.back());
    v.back().split = SPLIT_MASKED;
    v.back().ecut = ecut;
    for (size_t k = fw.size() - 1; k-- > 0;) {
      v.push_back(fw[k]);
      v.back().split = SPLIT_INV;
    }
    return v;
  }
  if (adi_omega(c) != 0.0) {
    AxisPass rx = px, ry = py;
    rx.rot = 1;
    ry.rot = 2;
    v.push_back(rx);
    v.push_back(ry);
    if (c->ndims == 3) v.push_back(pz);
    v.push_back(rx);
    return v;
  }
  v.push_back(py);
  v.push_back(px);
  if (c->ndims == 3) v.push_back(pz);
  for (auto& ap : v) ap.one_comp = one_comp;
  return v;
}

// The passes of one kinetic step.  Array omega (ssft_kin_step.m:3-11): the
// half-step passes, the Crank-Nicolson Lz update (an entry with axis = -1),
// the half-step passes again; otherwise axis_passes.
std::vector<AxisPass> step_passes(const gpe_ctx* c, double ecut = 0.0) {
  if (!c->omega_field) return axis_passes(c, ecut);
  std::vector<AxisPass> h = axis_passes(c);
  for (auto& ap : h) ap.half = 1;
  std::vector<AxisPass> v = h;
  AxisPass cn = h[0];
  cn.axis = -1;
  v.push_back(cn);
  v.insert(v.end(), h.begin(), h.end());
  return v;
}

// One pass per axis (energy sums): the axis passes without the second x half.
std::vector<AxisPass> energy_axes(const gpe_ctx* c) {
  std::vector<AxisPass> v = axis_passes(c);
  if (adi_omega(c) != 0.0) v.pop_back();
  return v;
}

template <typename R>
cudaError_t dispatch_tma(int N, const PassArgs<R>& a, bool strided, cudaStream_t s, int sms) {
  switch (N) {
#define X(v) \
  case v:    \
    return launch_pass_tma<R, v>(a, strided, s, sms, nullptr);
    GPE_FOR_EACH_N(X)
#undef X
  }
  return cudaErrorInvalidValue;
}

template <typename R>
int dispatch_tma_grid(int N, const PassArgs<R>& a, bool strided, int sms) {
  switch (N) {
#define X(v) \
  case v:    \
    return pass_tma_grid<R, v>(a, strided, sms);
    GPE_FOR_EACH_N(X)
#undef X
  }
  return 0;
}

template <typename R>
int dispatch_tma_ffts(int N, bool strided) {
  switch (N) {
#define X(v) \
  case v:    \
    return pass_tma_ffts<R, v>(strided);
    GPE_FOR_EACH_N(X)
#undef X
  }
  return 0;
}

PlanInfo dispatch_plan(int N);

// The TMA pass applies when every tile is one contiguous range (contiguous
// axis) or N rows of FFTS contiguous, 16-byte aligned elements (strided
// axes), and a CTA is at least two warps.  pass_variant: 0 = the direct
// pass everywhere, with L2 prefetch of the next wave's tiles (measured
// fastest on GB300 for the 256^3 and 512^3 workloads), 1 = the TMA pass
// where it applies, 2 = the direct pass without prefetch.
template <typename R>
size_t dispatch_tma_smem(int N, bool strided) {
  switch (N) {
#define X(v) \
  case v:    \
    return pass_tma_smem<R, v>(strided);
    GPE_FOR_EACH_N(X)
#undef X
  }
  return ~(size_t)0;
}

template <typename R>
bool use_tma(const gpe_ctx* c, const Field& f, const AxisPass& ap) {
  if (c->pass_variant != 1) return false;
  if (f.plan_var[ap.axis] != 0) return false;  // TMA passes are built on Plan<N> only
  if (ap.rot != 0) return false;                // and without the rotating-frame terms
  if (ap.split != SPLIT_FULL) return false;     // or the energy cut-off chain
  if (ap.half != 0) return false;               // or the spinor's half steps
  if (dispatch_tma_smem<R>(ap.N, ap.strided) > 200 * 1024) return false;
  const int ffts = dispatch_tma_ffts<R>(ap.N, ap.strided);
  if (!ap.strided) return true;
  const PlanInfo pi = dispatch_plan(ap.N);
  return ap.inner % ffts == 0 && ap.stride % ffts == 0 && ffts * pi.T >= 64 && (ffts * pi.T) % 32 == 0;
}

PlanInfo dispatch_plan(int N, int var) {
  if (var == 1 || var == 2) {  // the paired pass reads PlanAlt<N>'s tables
    switch (N) {
#define X(v) \
  case v:    \
    return plan_info<v, 1>();
      GPE_FOR_EACH_ALT(X)
#undef X
    }
    return PlanInfo{};
  }
  switch (N) {
#define X(v) \
  case v:    \
    return plan_info<v>();
    GPE_FOR_EACH_N(X)
#undef X
  }
  return PlanInfo{};
}
PlanInfo dispatch_plan(int N) { return dispatch_plan(N, 0); }

template <typename R>
long long pass_blocks(const AxisPass& p, int var) {
  PassGeom g = dispatch_geom<R>(p.N, var, p.strided);
  return (p.n_batch + g.ffts - 1) / g.ffts;
}

template <typename R>
size_t rsize() {
  return sizeof(R);
}

// ---- profiling --------------------------------------------------------------
enum ProfCls {
  PC_PASS_Y, PC_PASS_X, PC_PASS_Z, PC_ENERGY_Y, PC_ENERGY_X, PC_ENERGY_Z, PC_FINALIZE, PC_ITP_CHECK,
  PC_NORM, PC_ELEMENTWISE, PC_NL_PHASE, PC_ADJ_NL, PC_COPY, PC_CLUSTER, PC_FOLD_Y, PC_FOLD_X, PC_FOLD_Z, PC_COUNT
};
const char* kProfNames[PC_COUNT] = {"pass_y",   "pass_x",    "pass_z",      "energy_y",  "energy_x",
                                    "energy_z", "finalize",  "itp_check",   "norm",      "elementwise",
                                    "nl_phase", "adjoint_nl", "state_copy", "cluster_step", "pass_yy",
                                    "pass_xx",  "pass_zz"};

cudaEvent_t pool_event(gpe_ctx* c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

struct Launch {
  gpe_ctx* c;
  int cls;
  double bytes;
  cudaEvent_t a = nullptr;
  Launch(gpe_ctx* c_, int cls_, double bytes_) : c(c_), cls(cls_), bytes(bytes_) {
    c->launches++;
    if (c->nvtx) nvtxRangePushA(kProfNames[cls]);
    if (c->prof) {
      a = pool_event(c);
      cudaEventRecord(a, c->stream);
    }
  }
  ~Launch() {
    if (c->nvtx) nvtxRangePop();
    if (c->prof) {
      cudaEvent_t b = pool_event(c);
      cudaEventRecord(b, c->stream);
      c->prof_pending.push_back({cls, a, b});
      c->prof_classes[cls].bytes += bytes;
    }
  }
};

// ---- tables -------------------------------------------------------------------
double kval(const gpe_ctx* c, int axis, int p) {
  const int N = c->n[axis];
  const int q = (p <= N / 2) ? p : p - N;  // [0:n/2, -(n/2-1):-1], init.m:27
  return q * 2.0 * M_PI / (c->span[axis] + c->dx[axis]);
}

// FP32 rounding of a table entry z that keeps |z| as exact as the format
// allows: among the float pairs within 2 ulps of (Re z, Im z) whose angle is
// within about an ulp of arg z, take the one whose squared modulus is
// closest to |z|^2.  Independent rounding of both parts leaves |z| off by up
// to ~1e-7 with a fixed sign per entry, which a kinetic factor applied every
// step turns into a norm drift.
void round_pair_f32(std::complex<double> z, float* a, float* b) {
  const float a0 = (float)z.real(), b0 = (float)z.imag();
  const double m2 = std::norm(z), ang = std::arg(z);
  const double amax = 1.5e-7;
  double best = INFINITY;
  *a = a0;
  *b = b0;
  float ca = a0;
  for (int i = 0; i < 2; ++i) ca = std::nextafter(ca, -INFINITY);
  for (int i = -2; i <= 2; ++i, ca = std::nextafter(ca, INFINITY)) {
    float cb = b0;
    for (int j = 0; j < 2; ++j) cb = std::nextafter(cb, -INFINITY);
    for (int j = -2; j <= 2; ++j, cb = std::nextafter(cb, INFINITY)) {
      const double da = (double)ca, db = (double)cb;
      if (m2 > 0 && std::fabs(std::remainder(std::atan2(db, da) - ang, 2 * M_PI)) > amax) continue;
      const double err = std::fabs(da * da + db * db - m2);
      if (err < best) {
        best = err;
        *a = ca;
        *b = cb;
      }
    }
  }
}

template <typename R>
gpe_status upload_cx(gpe_ctx* c, void* dst, const std::vector<std::complex<double>>& v) {
  std::vector<R> h(2 * v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    if constexpr (sizeof(R) == 4) {
      float a, b;
      round_pair_f32(v[i], &a, &b);
      h[2 * i] = a;
      h[2 * i + 1] = b;
    } else {
      h[2 * i] = (R)v[i].real();
      h[2 * i + 1] = (R)v[i].imag();
    }
  }
  CU(cudaMemcpy(dst, h.data(), h.size() * sizeof(R), cudaMemcpyHostToDevice));
  return GPE_OK;
}

// Table layouts read by the pass kernels (fft.cuh apply_row, pass.cuh
// apply_phase): k- or thread-fastest, FP32 entries paired for 16-byte loads.
template <typename R>
int tw_index(int off, int Ns, int RAD, int k, int r) {
  if (sizeof(R) == 4 && RAD % 2 == 0) return off + 2 * ((r / 2) * Ns + k) + (r % 2);
  return off + r * Ns + k;
}
template <typename R>
int slot_index(int T, int t, int m) {
  if (sizeof(R) == 4) return 2 * ((m / 2) * T + t) + (m % 2);
  return m * T + t;
}

// Tables of one axis: stage twiddle rows and k^2/2/N in spectrum-slot order.
// Tables of axis ax for the plan variant f.plan_var[ax] (rebuilt when the
// autotuner changes the variant; the kinetic factors follow in set_kinop).
template <typename R>
gpe_status build_axis_tables(gpe_ctx* c, Field& f, int ax) {
  {
    const int N = c->n[ax];
    const PlanInfo pi = dispatch_plan(N, f.plan_var[ax]);
    if (f.tws[ax]) {
      cudaFree(f.tws[ax]);
      f.tws[ax] = nullptr;
    }
    int total = 0, Ns = pi.radix[0];
    for (int s = 1; s < pi.nstages; ++s) {
      total += (Ns * pi.radix[s] + 1) & ~1;
      Ns *= pi.radix[s];
    }
    std::vector<std::complex<double>> rows(std::max(total, 2), std::complex<double>(0.0, 0.0));
    Ns = pi.radix[0];
    for (int s = 1; s < pi.nstages; ++s) {
      const int RAD = pi.radix[s];
      const int off = stage_rows_offset(pi, s);
      for (int k = 0; k < Ns; ++k)
        for (int r = 0; r < RAD; ++r) {
          const double ang = -2.0 * M_PI * (double)(r * k) / (double)(Ns * RAD);
          rows[tw_index<R>(off, Ns, RAD, k, r)] = std::complex<double>(std::cos(ang), std::sin(ang));
        }
      Ns *= RAD;
    }
    CU(cudaMalloc(&f.tws[ax], rows.size() * 2 * sizeof(R)));
    CHECK(upload_cx<R>(c, f.tws[ax], rows));
    if (!f.php[ax]) CU(cudaMalloc(&f.php[ax], N * 2 * sizeof(R)));
    if (!f.k2p[ax]) CU(cudaMalloc(&f.k2p[ax], N * sizeof(R)));
    if (!f.kp[ax]) CU(cudaMalloc(&f.kp[ax], N * sizeof(R)));
    if (!f.kks[ax]) CU(cudaMalloc(&f.kks[ax], N * sizeof(R)));
    std::vector<R> k2(N), k1(N), kk(N);
    for (int t = 0; t < pi.T; ++t)
      for (int m = 0; m < pi.E; ++m) {
        const double k = kval(c, ax, plan_spec_pos(pi, t, m));
        k2[m * pi.T + t] = (R)(k * k / 2.0 / N);
        k1[m * pi.T + t] = (R)(k / N);
        kk[m * pi.T + t] = (R)(k * k / 2.0);
      }
    CU(cudaMemcpy(f.k2p[ax], k2.data(), N * sizeof(R), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(f.kp[ax], k1.data(), N * sizeof(R), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(f.kks[ax], kk.data(), N * sizeof(R), cudaMemcpyHostToDevice));
  }
  f.phase_valid = false;
  return GPE_OK;
}

// Coordinate of grid index i along axis ax: linspace(-xmax, xmax, n)
// (grid2d/init.m:12-13), xmax = span/2.
double coord(const gpe_ctx* c, int ax, int i) { return -0.5 * c->span[ax] + i * c->dx[ax]; }

// Rotating-frame weights of the energy sums (lap.m:8-10): the x pass adds
// -omega*y*kx, the y pass +omega*x*ky, y and x being the pencil's transverse
// coordinate: rotw[0][iy] = -omega*y(iy), rotw[1][ix] = +omega*x(ix).
template <typename R>
gpe_status ensure_rot_weights(gpe_ctx* c, Field& f) {
  const double om = adi_omega(c);
  if (om == 0.0 || (f.rotw[0] && f.rotw_omega == om)) return GPE_OK;
  for (int r = 0; r < 2; ++r) {
    const int tax = r == 0 ? 1 : 0;  // transverse axis: y for x pencils, x for y pencils
    std::vector<R> w(c->n[tax]);
    for (int i = 0; i < c->n[tax]; ++i) w[i] = (R)((r == 0 ? -om : om) * coord(c, tax, i));
    if (!f.rotw[r]) CU(cudaMalloc(&f.rotw[r], w.size() * sizeof(R)));
    CU(cudaMemcpy(f.rotw[r], w.data(), w.size() * sizeof(R), cudaMemcpyHostToDevice));
  }
  f.rotw_omega = om;
  return GPE_OK;
}

template <typename R>
gpe_status build_static_tables(gpe_ctx* c, Field& f) {
  for (int ax = 0; ax < c->ndims; ++ax) CHECK(build_axis_tables<R>(c, f, ax));
  return GPE_OK;
}

// kinop = exp(-kk*dt) (set_kinop.m:9), as one factor per axis with the 1/N of
// ifft folded in: exp(-k^2/2*dt)/N, dt = dre + i*dim, evaluated in FP64 and
// stored in the threads' spectrum-slot order.
//
// Rotating frame (scalar omega, set_kinop.m:5-7): the x factor is taken over
// half a step, exp(-(kx^2/2 - kx y omega) dt/2) (applied twice per step), the
// y factor exp(-(ky^2/2 + ky x omega) dt) and z as without rotation.  The
// k^2 part stays in the per-axis table; the cross term, which depends on the
// pencil's transverse coordinate, is a second table rot[ax][i][slot] =
// exp(+kx y(i) omega dt/2) (x) or exp(-ky x(i) omega dt) (y).
// exp(-k^2/4 dt)/N of axis ax in slot order (the per-axis factor of
// exp(-kk dt/2)), dt = dre + i dim, into dst (allocated on first use).
template <typename R>
gpe_status half_table(gpe_ctx* c, const Field& f, int ax, double dre, double dim, void*& dst) {
  const int N = c->n[ax];
  const PlanInfo pi = dispatch_plan(N, f.plan_var[ax]);
  std::vector<std::complex<double>> ph(N);
  for (int t = 0; t < pi.T; ++t)
    for (int m = 0; m < pi.E; ++m) {
      const double k = kval(c, ax, plan_spec_pos(pi, t, m));
      const double kk = k * k / 4.0;
      const double mag = std::exp(-kk * dre) / N;
      ph[slot_index<R>(pi.T, t, m)] = std::complex<double>(mag * std::cos(kk * dim), -mag * std::sin(kk * dim));
    }
  if (!dst) CU(cudaMalloc(&dst, N * 2 * sizeof(R)));
  return upload_cx<R>(c, dst, ph);
}

// Rotating two-component ITPs (GPEtaskSpinor/groundstate_itp.m:30-33,
// GPEtask2comp/groundstate_itp.m:31-36, 2D): the x factor
// exp(-(kx^2/2 - kx y omega) tau) and the y factor exp(-(ky^2/2 + ky x omega) tau),
// tau = dt/(2M), each as the per-axis table exp(-k^2/2 tau)/N (set[0], set[1])
// and the rotation table over the pencil's transverse coordinate c,
// exp(+kx y omega tau) / exp(-ky x omega tau) (set[2], set[3]).
template <typename R>
gpe_status rot_half_tables(gpe_ctx* c, const Field& f, double tau, void* set[4]) {
  const double om = c->prm.omega;
  for (int ax = 0; ax < 2; ++ax) {
    CHECK(half_table<R>(c, f, ax, 2.0 * tau, 0.0, set[ax]));
    const int N = c->n[ax];
    const PlanInfo pi = dispatch_plan(N, f.plan_var[ax]);
    const int tax = ax == 0 ? 1 : 0;
    const int nt = c->n[tax];
    const double s = (ax == 0 ? om : -om) * tau;
    std::vector<std::complex<double>> rt((size_t)nt * N);
    for (int i = 0; i < nt; ++i) {
      const double xc = coord(c, tax, i);
      for (int t = 0; t < pi.T; ++t)
        for (int m = 0; m < pi.E; ++m)
          rt[(size_t)i * N + slot_index<R>(pi.T, t, m)] = std::exp(s * kval(c, ax, plan_spec_pos(pi, t, m)) * xc);
    }
    if (!set[2 + ax]) CU(cudaMalloc(&set[2 + ax], rt.size() * 2 * sizeof(R)));
    CHECK(upload_cx<R>(c, set[2 + ax], rt));
  }
  return GPE_OK;
}

// The x (rot = 1) and y (rot = 2) passes of a rotating half step on a 2D
// grid, over every component or (one_comp) one.
std::vector<AxisPass> rot_xy_passes(const gpe_ctx* c, bool one_comp) {
  const long long nx = c->n[0], ny = c->n[1], nc = one_comp ? 1 : c->ncomp;
  AxisPass px{0, (int)nx, true, ny * nc, ny, ny, nx * ny};
  AxisPass py{1, (int)ny, false, nx * nc, 1, 1, 0};
  px.rot = 1;
  py.rot = 2;
  px.one_comp = py.one_comp = one_comp;
  return {px, py};
}

// A view of f whose x/y kinetic and rotation tables are one rot_half_tables set.
Field rot_view(const Field& f, void* const set[4]) {
  Field r = f;
  r.php[0] = set[0];
  r.php[1] = set[1];
  r.rot[0] = set[2];
  r.rot[1] = set[3];
  return r;
}

template <typename R>
gpe_status set_kinop(gpe_ctx* c, Field& f, double dre, double dim) {
  if (f.phase_valid && f.phase_dt[0] == dre && f.phase_dt[1] == dim) return GPE_OK;
  const double om = adi_omega(c);
  for (int ax = 0; ax < c->ndims; ++ax) {
    const int N = c->n[ax];
    const PlanInfo pi = dispatch_plan(N, f.plan_var[ax]);
    const double h = (om != 0.0 && ax == 0) ? 0.5 : 1.0;  // x takes half steps in the rotating frame
    std::vector<std::complex<double>> ph(N);
    for (int t = 0; t < pi.T; ++t)
      for (int m = 0; m < pi.E; ++m) {
        const double k = kval(c, ax, plan_spec_pos(pi, t, m));
        const double kk = k * k / 2.0;
        const double mag = std::exp(-kk * dre * h) / N;
        ph[slot_index<R>(pi.T, t, m)] =
            std::complex<double>(mag * std::cos(kk * dim * h), -mag * std::sin(kk * dim * h));
      }
    CHECK(upload_cx<R>(c, f.php[ax], ph));
    // GPEtaskSpinor/solve_split.m:44-45: ekkp = exp(-kk dt/2) at block starts;
    // set_kinop.m:3-4 for array omega: kinop = exp(-kk dt/2)
    // the last step's ekk times ekkm = exp(+kk dt/2) is exp(-kk dt/2) too
    if (c->ncomp == 2 || c->omega_field) CHECK(half_table<R>(c, f, ax, dre, dim, f.php2[ax]));
    if (om != 0.0 && ax < 2) {
      const int tax = ax == 0 ? 1 : 0;  // transverse axis of the pencils
      const int nt = c->n[tax];
      const double s = ax == 0 ? 0.5 * om : -om;
      std::vector<std::complex<double>> rt((size_t)nt * N);
      for (int i = 0; i < nt; ++i) {
        const double xc = coord(c, tax, i);
        for (int t = 0; t < pi.T; ++t)
          for (int m = 0; m < pi.E; ++m) {
            const double a = s * kval(c, ax, plan_spec_pos(pi, t, m)) * xc;  // exp(a*(dre + i dim))
            const double mag = std::exp(a * dre);
            rt[(size_t)i * N + slot_index<R>(pi.T, t, m)] =
                std::complex<double>(mag * std::cos(a * dim), mag * std::sin(a * dim));
          }
      }
      if (!f.rot[ax]) CU(cudaMalloc(&f.rot[ax], rt.size() * 2 * sizeof(R)));
      CHECK(upload_cx<R>(c, f.rot[ax], rt));
    }
  }
  f.phase_dt[0] = dre;
  f.phase_dt[1] = dim;
  f.phase_valid = true;
  return GPE_OK;
}

// ---- field allocation -----------------------------------------------------------
template <typename R>
gpe_status alloc_field(gpe_ctx* c, Field& f, int prec, bool share_V64) {
  f.prec = prec;
  CU(cudaMalloc(&f.psi, (size_t)c->PS * 2 * sizeof(R)));
  if (share_V64) {
    f.V = c->V64;
  } else {
    CU(cudaMalloc(&f.V, (size_t)c->PS * sizeof(R)));
  }
  return build_static_tables<R>(c, f);
}

template <typename R>
gpe_status ensure_itp_buffers(gpe_ctx* c, Field& f) {
  if (!f.aux) CU(cudaMalloc(&f.aux, (size_t)c->P * sizeof(R)));
  if (!f.absprev) CU(cudaMalloc(&f.absprev, (size_t)c->P * sizeof(R)));
  return GPE_OK;
}

void free_field(Field& f, const double* V64) {
  cudaFree(f.psi);
  if (f.V != (void*)V64) cudaFree(f.V);
  cudaFree(f.aux);
  cudaFree(f.absprev);
  for (int i = 0; i < 3; ++i) {
    cudaFree(f.tws[i]);
    cudaFree(f.php[i]);
    cudaFree(f.k2p[i]);
    cudaFree(f.kp[i]);
    cudaFree(f.kks[i]);
    cudaFree(f.php2[i]);
    cudaFree(f.php2b[i]);
  }
  for (auto& set : f.rth)
    for (void* p : set) cudaFree(p);
  for (int i = 0; i < 2; ++i) cudaFree(f.cn[i]);
  for (int i = 0; i < 2; ++i) {
    cudaFree(f.rot[i]);
    cudaFree(f.rotw[i]);
  }
  f = Field();
}

// FP64 polish field of an FP32 context (shares V64 as its potential).
gpe_status ensure_polish(gpe_ctx* c) {
  if (c->polish.psi) return GPE_OK;
  CHECK(alloc_field<double>(c, c->polish, GPE_FP64, true));
  c->polish.V_valid = true;
  return ensure_itp_buffers<double>(c, c->polish);
}

// ---- scalar helpers ---------------------------------------------------------------
gpe_status read_scalars(gpe_ctx* c, DevScalars* out) {
  CU(cudaMemcpyAsync(&c->sc_host[0], c->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  *out = c->sc_host[0];
  return GPE_OK;
}

gpe_status write_scalars(gpe_ctx* c, const DevScalars& v) {
  c->sc_host[1] = v;
  CU(cudaMemcpyAsync(c->sc, &c->sc_host[1], sizeof(DevScalars), cudaMemcpyHostToDevice, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return GPE_OK;
}

// ---- passes ---------------------------------------------------------------------
// fold = 1: a folded step pass (PassArgs::fold), scalar kernels only.
template <typename R>
gpe_status run_pass(gpe_ctx* c, Field& f, const AxisPass& ap, int kind, int pro, int epi, int energy_pot,
                    double dre, double dim, int* nblk, void* psi_buf = nullptr, int fold = 0) {
  PassArgs<R> a;
  a.psi = (cx<R>*)(psi_buf ? psi_buf : f.psi);  // psi_buf: another array of the grid's shape
  a.V = (const R*)f.V;
  a.aux = (R*)f.aux;
  a.php = (const cx<R>*)(ap.half == 2 ? f.php2b[ap.axis] : ap.half ? f.php2[ap.axis] : f.php[ap.axis]);
  if (!a.php) return fail(c, GPE_ERR_STATE, "kinetic factors not set");
  a.tws = (const cx<R>*)f.tws[ap.axis];
  a.k2p = (const R*)f.k2p[ap.axis];
  a.partials = c->partials;
  a.sc = c->sc;
  a.n_batch = ap.n_batch;
  a.stride = ap.stride;
  a.inner = ap.inner;
  a.outer = ap.outer;
  a.npts = ap.n_batch * (long long)ap.N;  // the pencils of a pass tile the array it covers
  a.cap = c->cap;
  // rotating-frame terms and the cut-off chain run in the extended step kernel
  // (and the folded passes)
  a.kind = (kind == KIND_STEP && (ap.rot != 0 || ap.split != SPLIT_FULL || fold)) ? KIND_STEP_EXT : kind;
  a.pro = pro;
  a.epi = epi;
  a.kin_slot = S_KX + ap.axis;
  a.energy_pot = energy_pot;
  a.g = c->prm.g;
  a.dre = dre;
  a.dim = dim;
  a.gr = (R)a.g;
  a.drer = (R)dre;
  a.dimr = (R)dim;
  a.prefetch = c->pass_variant == 0;
  a.pdl = c->pdl;
  if (ap.rot != 0) {
    const int r = ap.rot - 1;  // 0: x pencils (transverse y), 1: y pencils (transverse x)
    a.rot_period = c->n[r == 0 ? 1 : 0];
    if (kind == KIND_STEP) {
      a.rot = (const cx<R>*)f.rot[r];
      if (!a.rot) return fail(c, GPE_ERR_STATE, "rotating frame: kinetic factors not set");
    } else {
      a.rotw = (const R*)f.rotw[r];
      a.kp = (const R*)f.kp[ap.axis];
      if (!a.rotw) return fail(c, GPE_ERR_STATE, "rotating frame: energy weights not set");
    }
  }
  if (ap.split == SPLIT_FWD) a.skip_inv = 1;
  if (ap.split == SPLIT_INV) a.skip_fwd = 1;
  if (ap.split == SPLIT_MASKED) {
    // transverse axes of the last axis' pencils: y (b % ny) and, in 3D, x (b / ny)
    a.mask_a = (const R*)f.kks[1];
    a.mask_b = c->ndims == 3 ? (const R*)f.kks[0] : nullptr;
    a.mask_c = (const R*)f.kks[ap.axis];
    a.mask_pa = c->n[1];
    a.ecut = (R)ap.ecut;
  }
  const double P = (double)(ap.one_comp ? c->P : c->PS);  // points the pass covers
  double bytes = (kind == KIND_ENERGY ? 1.0 : 2.0) * P * 2 * sizeof(R);
  const bool useV = pro == PRO_RT_HALF || pro == PRO_RT_FULL || pro == PRO_ITP || epi == EPI_RT_END ||
                    (kind == KIND_ENERGY && energy_pot);
  if (useV || fold) bytes += P * sizeof(R);
  if (pro == PRO_ITP || epi == EPI_ITP) bytes += P * sizeof(R);
  int cls = (kind == KIND_ENERGY ? PC_ENERGY_Y : fold ? PC_FOLD_Y : PC_PASS_Y);
  cls += (ap.axis == 1 ? 0 : ap.axis == 0 ? 1 : 2);
  a.fold = fold;
  // The array staged with each tile by the TMA pass.
  a.side = (pro == PRO_RT_HALF || pro == PRO_RT_FULL || pro == PRO_ITP || epi == EPI_RT_END ||
            (kind == KIND_ENERGY && energy_pot))
               ? 1
               : (epi == EPI_ITP ? 2 : 0);
  if (fold) a.side = 1;
  if (!fold && use_tma<R>(c, f, ap)) {
    // Test knob of the timeout path (off unless GPE_TEST_TMA_STALL is set):
    // the TMA pass arms its barriers for copies it never issues and polls
    // them GPE_TEST_TMA_STALL times, so its bounded wait runs out with no
    // copy in flight.
    if (const char* e = getenv("GPE_TEST_TMA_STALL")) a.tma_stall = std::max(0, atoi(e));
    // strided tiles as tensor boxes (GPE_TMA_TENSOR=0: one bulk copy per row)
    const char* tt = getenv("GPE_TMA_TENSOR");
    a.tma_tensor = !(tt && atoi(tt) == 0);
    a.tdim[0] = c->n[1];
    a.tdim[1] = c->n[0];
    a.tdim[2] = c->ndims == 3 ? c->n[2] : 1;
    a.tdim[3] = ap.one_comp ? 1 : c->ncomp;
    const int grid = dispatch_tma_grid<R>(ap.N, a, ap.strided, c->sms);
    if (nblk) *nblk = grid;
    Launch L(c, cls, bytes);
    CU(dispatch_tma<R>(ap.N, a, ap.strided, c->stream, c->sms));
  } else {
    const int var = f.plan_var[ap.axis];
    if (nblk) {
      bool x2 = false;
      if constexpr (sizeof(R) == 4) x2 = x2_pass(var, a, ap.strided);
      if (x2) {
        const PassGeom g = dispatch_x2_geom(ap.N, var, ap.strided);
        *nblk = (int)((ap.n_batch + g.ffts - 1) / g.ffts);
      } else {
        *nblk = (int)pass_blocks<R>(ap, var);
      }
    }
    Launch L(c, cls, bytes);
    CU(dispatch_pass<R>(ap.N, var, a, ap.strided, c->stream));
  }
  return GPE_OK;
}

// Kinetic-energy passes (one forward FFT per axis); with `pot`, the y pass
// also sums n, Vn, n^2 and every pass applies the pending scale.
// ---- array omega: the Crank-Nicolson Lz update and its energy ----------------
LzGeom lz_geom(const gpe_ctx* c) {
  LzGeom g;
  g.nx = c->n[0];
  g.ny = c->n[1];
  g.h = c->dx[0];  // derivy.m passes obj.dx as well
  g.x0 = coord(c, 0, 0);
  g.y0 = coord(c, 1, 0);
  g.hxg = c->dx[0];
  g.hyg = c->dx[1];
  return g;
}

template <typename R>
const R* omega_field_ptr(const gpe_ctx* c) {
  return sizeof(R) == 8 ? (const R*)c->omf64 : (const R*)c->omfR;
}

template <typename R>
gpe_status ensure_cn_buffers(gpe_ctx* c, Field& f) {
  for (int k = 0; k < 2; ++k)
    if (!f.cn[k]) CU(cudaMalloc(&f.cn[k], (size_t)c->P * 2 * sizeof(R)));
  return GPE_OK;
}

// ssft_kin_step.m:5-10 between the two half kinetic steps, dt = dre + i dim:
//   lphi = phi; n_crank times: lphi = phi + dt/2 omega lz(lphi); phi += dt omega lz(lphi)
// with the omega array, or (the rotating SGPE, @SGPEtask/solve_split.m:58-64)
// the scalar omega when no array is set.
template <typename R>
gpe_status cn_step(gpe_ctx* c, Field& f, double dre, double dim) {
  CHECK(ensure_cn_buffers<R>(c, f));
  const LzGeom g = lz_geom(c);
  const R* om = c->omega_field ? omega_field_ptr<R>(c) : nullptr;
  const double oms = c->prm.omega;
  cx<R>* phi = (cx<R>*)f.psi;
  const cx<R>* src = phi;
  int k = 0;
  for (int it = 0; it < c->n_crank; ++it) {
    cx<R>* out = (cx<R>*)f.cn[k];
    Launch L(c, PC_ELEMENTWISE, (double)c->P * 6 * sizeof(R));
    launch_lz_cn<R>(out, phi, src, om, oms, c->P, g, 0.5 * dre, 0.5 * dim, c->stream);
    src = out;
    k ^= 1;
  }
  Launch L(c, PC_ELEMENTWISE, (double)c->P * 6 * sizeof(R));
  if (c->n_crank > 0) {
    launch_lz_cn<R>(phi, phi, src, om, oms, c->P, g, dre, dim, c->stream);  // reads src's neighbours only
  } else {
    launch_lz_cn<R>((cx<R>*)f.cn[0], phi, phi, om, oms, c->P, g, dre, dim, c->stream);
    CU(cudaMemcpyAsync(phi, f.cn[0], (size_t)c->P * 2 * sizeof(R), cudaMemcpyDeviceToDevice, c->stream));
  }
  CU(cudaGetLastError());
  return GPE_OK;
}

template <typename R>
gpe_status energy_passes(gpe_ctx* c, Field& f, bool pot, int nblk_kin[3], int* nblk_pot) {
  CHECK(ensure_rot_weights<R>(c, f));
  auto passes = energy_axes(c);
  nblk_kin[0] = nblk_kin[1] = nblk_kin[2] = 0;
  // The axes' sums are independent (each pass reads the state and writes
  // its own partial slots): the second and third pass run on side streams,
  // concurrently with the first (each is latency-bound on its own).  Not
  // while per-kernel profiling (its events live on the context stream) or
  // stream capture is on, or with GPE_ENERGY_CONCURRENT=0.
  bool conc = !c->prof && passes.size() > 1 && passes.size() <= 3;
  if (conc) {
    const char* e = getenv("GPE_ENERGY_CONCURRENT");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    conc = !(e && atoi(e) == 0) && cudaStreamIsCapturing(c->stream, &cap) == cudaSuccess &&
           cap == cudaStreamCaptureStatusNone;
  }
  if (conc) {
    for (int k = 0; k < 2; ++k) {
      if (!c->aux[k]) CU(cudaStreamCreateWithFlags(&c->aux[k], cudaStreamNonBlocking));
      if (!c->ev_join[k]) CU(cudaEventCreateWithFlags(&c->ev_join[k], cudaEventDisableTiming));
    }
    if (!c->ev_fork) CU(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CU(cudaEventRecord(c->ev_fork, c->stream));
    for (size_t k = 1; k < passes.size(); ++k) CU(cudaStreamWaitEvent(c->aux[k - 1], c->ev_fork, 0));
  }
  for (size_t i = 0; i < passes.size(); ++i) {
    const AxisPass& ap = passes[i];
    int nb = 0;
    const bool ep = pot && ap.axis == 1;
    const cudaStream_t main_stream = c->stream;
    if (conc && i > 0) c->stream = c->aux[i - 1];
    const gpe_status st =
        run_pass<R>(c, f, ap, KIND_ENERGY, pot ? PRO_SCALE : PRO_NONE, EPI_NONE, ep ? 1 : 0, 0.0, 0.0, &nb);
    c->stream = main_stream;
    CHECK(st);
    nblk_kin[ap.axis] = nb;
    if (ep && nblk_pot) *nblk_pot = nb;
  }
  if (conc) {
    for (size_t k = 1; k < passes.size(); ++k) {
      CU(cudaEventRecord(c->ev_join[k - 1], c->aux[k - 1]));
      CU(cudaStreamWaitEvent(c->stream, c->ev_join[k - 1], 0));
    }
  }
  if (c->omega_field || c->lz_scalar) {
    // the -omega Lz term of applyh0 (GPEtask.m:92-94; GPEtaskSpinor.m:72-74
    // per component with scalar omega), appended to the x pass's kinetic
    // partials so every finalizer adds it to the kinetic sum
    Launch L(c, PC_NORM, (double)c->PS * (2 * sizeof(R) + sizeof(R)));
    const R* om = c->omega_field ? omega_field_ptr<R>(c) : nullptr;
    const int nb = launch_lz_energy<R>((const cx<R>*)f.psi, om, c->prm.omega, c->PS, lz_geom(c), c->sc, pot,
                                       c->partials + (size_t)S_KX * c->cap + nblk_kin[0], c->stream);
    CU(cudaGetLastError());
    nblk_kin[0] += nb;
  }
  return GPE_OK;
}

template <typename R>
gpe_status observables_impl(gpe_ctx* c, Field& f, double div, int set_mu, DevScalars* out) {
  int nk[3], np = 0;
  CHECK(energy_passes<R>(c, f, true, nk, &np));
  ObsFinalArgs a{c->partials, c->cap, np, {nk[0], nk[1], nk[2]}, c->weight, c->prm.g, div, set_mu,
                 c->prm.mu_init};
  {
    Launch L(c, PC_FINALIZE, 0);
    launch_finalize_obs(a, c->sc, c->stream);
    CU(cudaGetLastError());
  }
  if (out) CHECK(read_scalars(c, out));
  return GPE_OK;
}

template <typename R>
gpe_status norm_impl(gpe_ctx* c, Field& f, double Ntotal) {
  int nb;
  {
    Launch L(c, PC_NORM, (double)c->P * 2 * sizeof(R));
    nb = launch_norm<R>((const cx<R>*)f.psi, c->P, c->sc, c->partials, c->cap, c->stream);
    CU(cudaGetLastError());
  }
  {
    Launch L(c, PC_FINALIZE, 0);
    launch_finalize_norm0(c->partials, c->cap, nb, c->weight, Ntotal, c->sc, c->stream);
    CU(cudaGetLastError());
  }
  return GPE_OK;
}

// ---- groundstate_itp ------------------------------------------------------------
struct ItpState {
  double dt;
  int i;  // iterations completed
};

template <typename R>
gpe_status itp_iteration(gpe_ctx* c, Field& f, double dt, int i) {
  auto passes = step_passes(c);
  int nb = 0;
  for (size_t k = 0; k < passes.size(); ++k) {
    const bool first = k == 0, last = k + 1 == passes.size();
    if (passes[k].axis < 0) {  // array omega: Crank-Nicolson Lz with the real ITP dt
      CHECK(cn_step<R>(c, f, dt, 0.0));
      continue;
    }
    CHECK(run_pass<R>(c, f, passes[k], KIND_STEP, first ? PRO_ITP : PRO_NONE, last ? EPI_ITP : EPI_NONE, 0,
                      dt, 0.0, last ? &nb : nullptr));
  }
  ItpFinalArgs a{c->partials, c->cap, nb, c->weight, dt, c->prm.Ntotal, c->prm.mu_init, i, c->d_hist};
  Launch L(c, PC_FINALIZE, 0);
  launch_finalize_itp(a, c->sc, c->stream);
  CU(cudaGetLastError());
  return GPE_OK;
}

template <typename R>
gpe_status itp_check(gpe_ctx* c, Field& f, const gpe_itp_params* prm, double dt, int i, bool fp32_phase) {
  const bool want = prm->want_mu2 || prm->want_energy;
  int nk[3] = {0, 0, 0}, np = 0;
  if (want) CHECK(energy_passes<R>(c, f, true, nk, &np));
  int nbc;
  {
    Launch L(c, PC_ITP_CHECK, (double)c->P * (2 * sizeof(R) + 2 * sizeof(R)));
    nbc = launch_itp_check<R>((const cx<R>*)f.psi, (R*)f.absprev, c->P, c->sc, c->partials, c->cap,
                              c->stream);
    CU(cudaGetLastError());
  }
  const int maxit = c->prm.itp_max_iter;
  CheckFinalArgs a;
  a.partials = c->partials;
  a.cap = c->cap;
  a.nblk_check = nbc;
  a.nblk_pot = want ? np : 0;
  a.nblk_kin[0] = nk[0];
  a.nblk_kin[1] = nk[1];
  a.nblk_kin[2] = nk[2];
  a.weight = c->weight;
  a.g = c->prm.g;
  a.dt = dt;
  a.eps = prm->eps;
  a.nnn = c->prm.Ntotal > 0 ? c->prm.Ntotal : 1.0;
  a.iter = i;
  a.want_mu2 = prm->want_mu2;
  a.adjust = c->prm.itp_adjust_stepsize;
  a.fp32_phase = fp32_phase ? 1 : 0;
  a.switch_delta = prm->switch_delta > 0 ? prm->switch_delta : 2e-4;
  a.MU = c->d_hist;
  a.MU2 = c->d_hist + maxit;
  a.EE = c->d_hist + 2 * (size_t)maxit;
  Launch L(c, PC_FINALIZE, 0);
  launch_finalize_check(a, c->sc, c->stream);
  CU(cudaGetLastError());
  return GPE_OK;
}

// Runs iterations in one precision until a finalizer stops the run or
// itp_max_iter is reached.  Returns the stop reason in *reason.
template <typename R>
gpe_status itp_phase(gpe_ctx* c, Field& f, const gpe_itp_params* prm, ItpState& st, bool fp32_phase,
                     int* reason) {
  CHECK(set_kinop<R>(c, f, st.dt, 0.0));
  const int maxit = c->prm.itp_max_iter, minit = c->prm.itp_min_iter;
  const bool adjust = c->prm.itp_adjust_stepsize != 0;
  int slot = 0, prev = -1;
  int i = st.i;
  *reason = RUNNING;
  bool stopped = false;
  while (i < maxit && !stopped) {
    ++i;
    CHECK(itp_iteration<R>(c, f, st.dt, i));
    if (i > minit && i % 10 == 0) {
      CHECK(itp_check<R>(c, f, prm, st.dt, i, fp32_phase));
      CU(cudaMemcpyAsync(&c->sc_host[slot], c->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
      CU(cudaEventRecord(c->ev_sc[slot], c->stream));
      if (adjust) {
        CU(cudaEventSynchronize(c->ev_sc[slot]));
        const DevScalars& h = c->sc_host[slot];
        if (h.stop) {
          if (h.status == HALVE_DT) {  // groundstate_itp.m:68-71
            st.dt /= 2;
            CHECK(set_kinop<R>(c, f, st.dt, 0.0));
            DevScalars v = h;
            v.stop = 0;
            v.status = RUNNING;
            CHECK(write_scalars(c, v));
          } else {
            stopped = true;
          }
        }
      } else {
        // Look one check interval behind: the GPU keeps running meanwhile.
        if (prev >= 0) {
          CU(cudaEventSynchronize(c->ev_sc[prev]));
          if (c->sc_host[prev].stop) stopped = true;
        }
        prev = slot;
        slot ^= 1;
      }
    }
  }
  DevScalars h;
  CHECK(read_scalars(c, &h));
  st.i = h.iter;
  *reason = h.stop ? h.status : RUNNING;
  if (h.timeout) return fail(c, GPE_ERR_TIMEOUT, "groundstate_itp: a device-side wait for staged data expired");
  if (h.bounds_site) return fail(c, GPE_ERR_BOUNDS, bounds_message("groundstate_itp", h));
  if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "groundstate_itp: non-finite norm or residual");
  return GPE_OK;
}

template <typename R>
gpe_status itp_impl(gpe_ctx* c, const gpe_itp_params* prm, double* MU, double* MU2, double* EE, int cap,
                    gpe_itp_result* res) {
  Field& f = c->main;
  const int maxit = c->prm.itp_max_iter;
  CHECK(ensure_itp_buffers<R>(c, f));
  if (c->d_hist_len < 3 * (size_t)maxit) {
    cudaFree(c->d_hist);
    c->d_hist = nullptr;
    CU(cudaMalloc(&c->d_hist, 3 * (size_t)maxit * sizeof(double)));
    c->d_hist_len = 3 * (size_t)maxit;
  }
  CU(cudaMemsetAsync(c->d_hist, 0, 3 * (size_t)maxit * sizeof(double), c->stream));
  // Reset the run scalars; dtmin = sqrt(eps) (groundstate_itp.m:35).
  DevScalars s0;
  CHECK(read_scalars(c, &s0));
  s0.stop = 0;
  s0.status = RUNNING;
  s0.nonfinite = 0;
  s0.timeout = 0;  // a timed-out earlier call does not fail this one
  s0.bounds_site = 0;
  s0.bounds_index = 0;
  s0.iter = 0;
  s0.stall = 0;
  s0.best_delta = INFINITY;
  s0.dtmin = std::sqrt(prm->eps);
  CHECK(write_scalars(c, s0));
  // process_init_state (GPEtask.m:159-160) and current_state = phi (:28).
  CHECK(norm_impl<R>(c, f, c->prm.Ntotal));
  {
    Launch L(c, PC_ELEMENTWISE, (double)c->P * 3 * sizeof(R));
    launch_abs_init<R>((const cx<R>*)f.psi, (R*)f.absprev, c->P, c->sc, c->stream);
    CU(cudaGetLastError());
  }
  ItpState st{prm->dt, 0};
  int reason = RUNNING;
  int fp32_iters = 0;
  const bool polish = (c->prec == GPE_FP32) && prm->fp64_polish;
  // device time of the two phases (events on the context stream)
  cudaEvent_t tev[3] = {nullptr, nullptr, nullptr};
  struct EvFree {
    cudaEvent_t* e;
    ~EvFree() {
      for (int k = 0; k < 3; ++k)
        if (e[k]) cudaEventDestroy(e[k]);
    }
  } tev_free{tev};
  for (int k = 0; k < 3; ++k) CU(cudaEventCreate(&tev[k]));
  CU(cudaEventRecord(tev[0], c->stream));
  CHECK(itp_phase<R>(c, f, prm, st, polish, &reason));
  CU(cudaEventRecord(tev[1], c->stream));
  CU(cudaEventRecord(tev[2], c->stream));
  if (polish && reason == SWITCH_FP64 && st.i < maxit) {
    fp32_iters = st.i;
    CHECK(ensure_polish(c));
    Field& p = c->polish;
    {
      Launch L(c, PC_ELEMENTWISE, (double)c->P * 24);
      launch_convert_cx<R, double>((const cx<R>*)f.psi, (cx<double>*)p.psi, c->P, c->sc, c->stream);
      launch_convert_re<R, double>((const R*)f.absprev, (double*)p.absprev, c->P, c->stream);
      launch_set_scale_one(c->sc, c->stream);
      launch_reset_scalars(c->sc, c->stream);
      CU(cudaGetLastError());
    }
    CHECK(itp_phase<double>(c, p, prm, st, false, &reason));
    {
      Launch L(c, PC_ELEMENTWISE, (double)c->P * 24);
      launch_convert_cx<double, R>((const cx<double>*)p.psi, (cx<R>*)f.psi, c->P, c->sc, c->stream);
      launch_set_scale_one(c->sc, c->stream);
      CU(cudaGetLastError());
    }
    CU(cudaEventRecord(tev[2], c->stream));
  } else if (polish) {
    fp32_iters = st.i;
  }
  DevScalars h;
  CHECK(read_scalars(c, &h));
  launch_reset_scalars(c->sc, c->stream);
  CU(cudaGetLastError());
  const int iters = st.i;
  std::vector<double> hist(3 * (size_t)maxit);
  CU(cudaMemcpy(hist.data(), c->d_hist, hist.size() * sizeof(double), cudaMemcpyDeviceToHost));
  const double* hMU = hist.data();
  const double* hMU2 = hist.data() + maxit;
  const double* hEE = hist.data() + 2 * (size_t)maxit;
  const int ncopy = std::min(iters, cap);
  const bool pos = c->prm.Ntotal > 0;
  for (int k = 0; k < ncopy; ++k) {
    if (MU) MU[k] = hMU[k];
    if (MU2) MU2[k] = pos ? hMU2[k] / c->prm.Ntotal : hMU2[k] / hMU[k];
    if (EE) EE[k] = pos ? hEE[k] / c->prm.Ntotal : hEE[k] / hMU[k];
  }
  if (iters > 0) {  // groundstate_itp.m:84-109
    if (pos) {
      c->cur.current_mu = hMU[iters - 1];
      c->cur.current_n = c->prm.Ntotal;
    } else if (prm->want_mu2) {
      c->cur.current_mu = hMU2[iters - 1] / hMU[iters - 1];
      c->cur.current_n = hMU[iters - 1];
    }
  }
  if (res) {
    res->iters = iters;
    res->converged = reason == CONVERGED;
    res->fp32_iters = fp32_iters;
    res->final_dt = st.dt;
    res->last_delta = h.delta;
    float m0 = 0.f, m1 = 0.f;
    CU(cudaEventSynchronize(tev[2]));
    CU(cudaEventElapsedTime(&m0, tev[0], tev[1]));
    CU(cudaEventElapsedTime(&m1, tev[1], tev[2]));
    res->ms_main = m0;
    res->ms_fp64 = m1;
  }
  if (reason == RUNNING && iters >= maxit)
    c->err = "groundstate_itp: Convergence not reached";  // groundstate_itp.m:79 (a warning)
  return GPE_OK;
}

// ---- solve_split -----------------------------------------------------------------
template <typename R>
gpe_status upload_V_double(gpe_ctx* c, const double* hostV, bool async_pinned) {
  const size_t bytes = (size_t)c->PS * sizeof(double);
  CU(cudaMemcpyAsync(c->V64, hostV, bytes, cudaMemcpyHostToDevice, c->stream));
  if (c->prec == GPE_FP32) {
    Launch L(c, PC_ELEMENTWISE, (double)c->PS * 12);
    launch_convert_re<double, float>(c->V64, (float*)c->main.V, c->PS, c->stream);
    CU(cudaGetLastError());
  }
  if (!async_pinned) CU(cudaStreamSynchronize(c->stream));
  c->main.V_valid = true;
  return GPE_OK;
}

template <typename R>
gpe_status vtd_upload(gpe_ctx* c, const gpe_split_params* prm, double time, int& k) {
  const size_t bytes = (size_t)c->PS * sizeof(double);
  if (!c->pinned_V[k]) CU(cudaMallocHost(&c->pinned_V[k], bytes));
  CU(cudaEventSynchronize(c->ev_V[k]));  // the previous copy out of this buffer is done
  if (prm->vtd(prm->vtd_user, time, c->pinned_V[k]) != 0)
    return fail(c, GPE_ERR_CALLBACK, "solve_split: potential callback failed");
  CHECK(upload_V_double<R>(c, c->pinned_V[k], true));
  CU(cudaEventRecord(c->ev_V[k], c->stream));
  k ^= 1;
  return GPE_OK;
}

// One solve_split run of one context: the values fixed at its start.
struct SplitRun {
  int n_rec = 1, start = 0, nout = 0, nb = 1;
  double ddt = 0, dre = 0, dim = 0, dt_outer = 0;
  bool feedback = false;
  std::vector<AxisPass> passes;
  size_t hist_off = 0;  // history slot of outer step j: d_hist + hist_off + 3*(j - start - 1)
  // Stochastic GPE (SGPEtask.solve_split): mu fixed at mu_init, no
  // renormalisation, noise sigma * (n1 + i n2) before every kinetic step.
  bool sgpe = false;
  bool sgpe_cn = false;        // rotating SGPE: Lz Crank-Nicolson after each kinetic step (solve_split.m:58-64)
  double sigma = 0.0;          // sqrt(T gamma ddt / weight), solve_split.m:49
  unsigned long long seed = 0;
  int niter_inner = 1;         // for the global step index of the noise counter
};

// solve_split.m:13-47: NN0, n_rec, complex dt, kinetic factors, initial mu.
template <typename R>
gpe_status split_setup(gpe_ctx* c, const gpe_split_params* prm, SplitRun& run, int& vk, size_t hist_extra,
                       const gpe_sgpe_params* sg = nullptr) {
  Field& f = c->main;
  const double ddt = prm->ddt;
  const double gam = c->prm.gamma;
  int n_rec = c->prm.n_recalc;
  if (n_rec < 1) return fail(c, GPE_ERR_INVALID, "n_recalc must be >= 1");
  if (prm->niter_inner < 1) return fail(c, GPE_ERR_INVALID, "niter_inner must be >= 1");
  if (prm->niter_inner % n_rec != 0) {
    // GPEtask: n_rec = 1 (solve_split.m:25-27).  SGPEtask keeps n_rec and runs
    // floor(niter_inner/n_rec) blocks (its loop 1:niter_inner/n_rec,
    // @SGPEtask/solve_split.m:54), none at all (an error there) below n_rec.
    if (!sg) n_rec = 1;
    else if (prm->niter_inner < n_rec)
      return fail(c, GPE_ERR_INVALID, "solve_sgpe: niter_inner < n_recalc runs no block (solve_split.m:54)");
  }
  const int start = c->cur.current_iter;
  const int nout = prm->niter_outer;
  // dt = ddt*1i/(1+1i*gam) (solve_split.m:31)
  const std::complex<double> dtc = ddt * std::complex<double>(0.0, 1.0) / std::complex<double>(1.0, gam);
  const double dre = dtc.real(), dim = dtc.imag();
  CHECK(set_kinop<R>(c, f, dre, dim));
  DevScalars s0;
  CHECK(read_scalars(c, &s0));
  // NN0 (solve_split.m:17-21)
  double NN0 = c->prm.Ntotal;
  if (!(NN0 > 0)) {
    CHECK(norm_impl<R>(c, f, 0.0));
    DevScalars h;
    CHECK(read_scalars(c, &h));
    NN0 = h.ncur;
    s0 = h;
  }
  s0.stop = 0;
  s0.status = RUNNING;
  s0.nonfinite = 0;
  s0.timeout = 0;  // a timed-out earlier call does not fail this one
  s0.bounds_site = 0;
  s0.bounds_index = 0;
  s0.outer = 0;
  s0.NN0 = NN0;
  s0.NNN = NN0;
  if (sg) s0.mu = c->prm.mu_init;  // SGPE: mu = mu_init throughout (SGPEtask solve_split.m:52)
  CHECK(write_scalars(c, s0));
  // muc/mu at the start (solve_split.m:40-46): applyham at current_time.
  if (prm->vtd) CHECK(vtd_upload<R>(c, prm, c->cur.current_time, vk));
  if (!sg) CHECK(observables_impl<R>(c, f, NN0, 1, nullptr));
  run.n_rec = n_rec;
  run.start = start;
  run.nout = nout;
  run.ddt = ddt;
  run.dre = dre;
  run.dim = dim;
  run.feedback = gam > 0 && c->prm.mu_init == 0 && !sg;
  run.niter_inner = prm->niter_inner;
  if (sg) {
    run.sgpe = true;
    run.sgpe_cn = c->prm.omega != 0.0;
    if (run.sgpe_cn) CHECK(ensure_cn_buffers<R>(c, f));
    run.sigma = std::sqrt(sg->T * gam * ddt / c->weight);
    run.seed = sg->seed;
  }
  run.dt_outer = ddt * prm->niter_inner;
  run.nb = prm->niter_inner / n_rec;
  // the cut-off mask applies only with noise (SGPEtask/solve_split.m:40)
  run.passes = step_passes(c, (sg && sg->T > 0 && sg->ecut > 0) ? sg->ecut : 0.0);
  if (c->omega_field) CHECK(ensure_cn_buffers<R>(c, f));  // before any graph capture
  run.hist_off = hist_extra;
  const int nsteps_out = std::max(0, nout - start);
  const size_t hlen = hist_extra + 3 * (size_t)std::max(1, nsteps_out);
  if (c->d_hist_len < hlen) {
    cudaFree(c->d_hist);
    c->d_hist = nullptr;
    CU(cudaMalloc(&c->d_hist, hlen * sizeof(double)));
    c->d_hist_len = hlen;
  }
  CU(cudaMemsetAsync(c->d_hist, 0, hlen * sizeof(double), c->stream));
  return GPE_OK;
}

// One block of n_rec steps, solve_split.m:51-79 (VV refresh is the caller's).
// hist: where the block-end finalizer stores (muc, ncur), or nullptr.
// Folded steps (one component, plain axis passes; GPE_FOLD=0 turns them
// off): the odd steps of a block take the axes in the order y x z (2D: y x),
// the even steps z x y (x y), so that the last pass of a step and the first
// of the next are on one axis; those two run as one folded pass (transform,
// full nonlinear step, transform).  A block of n steps is 2n + 1 passes
// instead of 3n (2D: n + 1 instead of 2n).  The kinetic factors of the axes
// commute (ssft_kin_step.m:17 applies them together in Fourier space), so
// the reordering changes only the rounding.
bool fold_env() {
  const char* e = getenv("GPE_FOLD");
  return !(e && atoi(e) == 0);
}
bool fold_steps(const gpe_ctx* c, const SplitRun& run) {
  if (c->ncomp != 1 || run.sgpe || run.sgpe_cn || c->omega_field || (int)run.passes.size() != c->ndims) return false;
  for (const auto& ap : run.passes)
    if (ap.axis < 0 || ap.rot != 0 || ap.split != SPLIT_FULL || ap.half != 0 || ap.one_comp) return false;
  return fold_env();
}

template <typename R>
gpe_status enqueue_block(gpe_ctx* c, const SplitRun& run, double time2, bool last_block, double* hist,
                         unsigned long long step0 = 0) {
  Field& f = c->main;
  int nb_epi = 0;
  const bool folded = fold_steps(c, run);
  if (folded) {
    const int np = (int)run.passes.size();
    // the axis order of step i (1-based): y x z for odd i, z x y for even i
    auto order = [&](int i, int j) -> const AxisPass& {
      return run.passes[i % 2 == 0 ? np - 1 - j : j];
    };
    auto folds = [&](int i) {  // the last pass of step i folds with the first of step i+1
      return i < run.n_rec && order(i, np - 1).axis == order(i + 1, 0).axis;
    };
    for (int i = 1; i <= run.n_rec; ++i) {
      for (int j = 0; j < np; ++j) {
        if (j == 0 && i > 1 && folds(i - 1)) continue;  // run by the previous step's last pass
        const AxisPass& ap = order(i, j);
        const bool lastp = j == np - 1;
        // solve_split.m:55-56 (block start) / 60-61 (between unfolded steps)
        const int pro = j == 0 ? (i == 1 ? PRO_RT_HALF : PRO_RT_FULL) : PRO_NONE;
        const bool end = lastp && i == run.n_rec;
        const int fold = (lastp && folds(i)) ? 1 : 0;  // solve_split.m:60-61 between the transforms
        CHECK(run_pass<R>(c, f, ap, KIND_STEP, pro, end ? EPI_RT_END : EPI_NONE, 0, run.dre, run.dim,
                          end ? &nb_epi : nullptr, nullptr, fold));
      }
    }
  }
  for (int i = 1; i <= run.n_rec && !folded; ++i) {
    if (run.sgpe) {
      // SGPE (solve_split.m:57-66): the nonlinear factor (half at the block
      // start, else the full one of the previous step) and the noise of step
      // step0 + i - 1 come before the kinetic passes, in one elementwise pass
      Launch L(c, PC_NL_PHASE, (double)c->P * (4 * sizeof(R) + sizeof(R)));
      launch_sgpe_nl_noise<R>((cx<R>*)f.psi, (const R*)f.V, c->P, c->sc, c->prm.g, run.dre, run.dim, i == 1,
                              run.sigma, run.seed, step0 + (unsigned long long)(i - 1), c->stream);
    }
    for (size_t k = 0; k < run.passes.size(); ++k) {
      const bool first = k == 0, last = k + 1 == run.passes.size();
      if (run.passes[k].axis < 0) {  // array omega: Crank-Nicolson Lz (ssft_kin_step.m:5-10)
        CHECK(cn_step<R>(c, f, run.dre, run.dim));
        continue;
      }
      const int pro = (first && !run.sgpe) ? (i == 1 ? PRO_RT_HALF : PRO_RT_FULL) : PRO_NONE;
      const bool end = last && i == run.n_rec && !run.sgpe_cn;
      CHECK(run_pass<R>(c, f, run.passes[k], KIND_STEP, pro, end ? EPI_RT_END : EPI_NONE, 0, run.dre, run.dim,
                        end ? &nb_epi : nullptr));
    }
    if (run.sgpe_cn) {
      // rotating SGPE: the Lz update follows the kinetic step, the nonlinear
      // factor follows it (the next step's first kernel, or the block end)
      CHECK(cn_step<R>(c, f, run.dre, run.dim));
      if (i == run.n_rec) {
        Launch L(c, PC_NL_PHASE, (double)c->P * (4 * sizeof(R) + sizeof(R)));
        nb_epi = launch_rt_block_end<R>((cx<R>*)f.psi, (const R*)f.V, c->P, c->sc, c->prm.g, run.dre, run.dim,
                                        c->partials, c->cap, c->stream);
        CU(cudaGetLastError());
      }
    }
  }
  const bool need_mu = (run.feedback || last_block) && !run.sgpe;
  int nk[3] = {0, 0, 0};
  if (need_mu) CHECK(energy_passes<R>(c, f, false, nk, nullptr));
  BlockFinalArgs a;
  a.partials = c->partials;
  a.cap = c->cap;
  a.nblk_epi = nb_epi;
  a.nblk_kin[0] = nk[0];
  a.nblk_kin[1] = nk[1];
  a.nblk_kin[2] = nk[2];
  a.weight = c->weight;
  a.g = c->prm.g;
  a.feedback = run.feedback;
  a.tau = c->prm.decay_rate;
  a.time2 = time2;
  a.hist_mu = hist;
  a.hist_n = hist ? hist + 1 : nullptr;
  a.hist_ok = nullptr;
  a.hist_e = hist ? hist + 2 : nullptr;
  a.pdl = c->pdl;
  a.fixed_mu = run.sgpe;  // SGPE reports mu = mu_init (solve_split.m:78)
  Launch L(c, PC_FINALIZE, 0);
  launch_finalize_block(a, c->sc, c->stream);
  CU(cudaGetLastError());
  return GPE_OK;
}

// End of a run: status checks, history and current_* from the device.
template <typename R>
gpe_status split_finish(gpe_ctx* c, const SplitRun& run, int last_j, double last_time2) {
  DevScalars h;
  CHECK(read_scalars(c, &h));
  if (h.timeout) return fail(c, GPE_ERR_TIMEOUT, "solve_split: a device-side wait for staged data expired");
  if (h.bounds_site) return fail(c, GPE_ERR_BOUNDS, bounds_message("solve_split", h));
  if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "solve_split: non-finite norm or chemical potential");
  const int start = run.start;
  if (last_j > start) {
    std::vector<double> dh(3 * (size_t)(last_j - start));
    CU(cudaMemcpy(dh.data(), c->d_hist + run.hist_off, dh.size() * sizeof(double), cudaMemcpyDeviceToHost));
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
    c->cur.current_time = last_time2;
    c->cur.current_mu = h.muc;
    c->cur.current_n = h.ncur;
  }
  return GPE_OK;
}

template <typename R>
gpe_status split_impl(gpe_ctx* c, const gpe_split_params* prm, const gpe_sgpe_params* sg = nullptr) {
  SplitRun run;
  int vk = 0;
  CHECK(split_setup<R>(c, prm, run, vk, 0, sg));
  const int start = run.start, nout = run.nout, nb = run.nb, n_rec = run.n_rec;
  const double ddt = run.ddt, dt_outer = run.dt_outer;
  int last_j = start;
  double last_time2 = c->cur.current_time;
  bool stop_req = false;
  for (int j = start + 1; j <= nout && !stop_req; ++j) {
    const double time = (j - 1) * dt_outer;
    double time2 = time;
    for (int jj = 1; jj <= nb; ++jj) {
      time2 = time + (jj - 1) * ddt * n_rec;  // solve_split.m:53
      if (prm->vtd) CHECK(vtd_upload<R>(c, prm, time2, vk));
      const size_t hj = (size_t)(j - start - 1);
      // global index of the block's first step: distinct noise for every step of every run
      const unsigned long long step0 =
          (unsigned long long)(j - 1) * (unsigned long long)run.niter_inner + (unsigned long long)(jj - 1) * n_rec;
      CHECK(enqueue_block<R>(c, run, time2, jj == nb, (jj == nb) ? c->d_hist + 3 * hj : nullptr, step0));
    }
    last_j = j;
    last_time2 = time2;
    if (prm->on_step) {  // ext_callback (solve_split.m:80)
      DevScalars h;
      CHECK(read_scalars(c, &h));
      if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "solve_split: non-finite norm or chemical potential");
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
      c->hist_e[j - 1] = run.sgpe ? NAN : h.energy;
      if (prm->on_step(prm->step_user, j, time2, h.muc, h.ncur) != 0) stop_req = true;
    }
  }
  return split_finish<R>(c, run, last_j, last_time2);
}

// ---- adjoint: dL/dV of L = 1 - |<target|psi(T)>|^2 / (|target|^2 |psi0|^2) ------
// Forward: M steps S = N K N from the current state (the gamma = 0 form of
// solve_split.m:55-64, adjoint_kernels.cu).  States are kept every K steps
// (checkpoints); the backward sweep recomputes each segment's K step-start
// states from its checkpoint, then walks the steps in reverse:
//   phi2 = K N x0;  lam <- adjN(lam; phi2);  lam <- K^H lam;  lam <- adjN(lam; x0).
gpe_status io_buffer(gpe_ctx* c, void** out);

template <typename R>
gpe_status kinetic_on(gpe_ctx* c, Field& f, void* buf, double ddt) {
  for (auto& ap : axis_passes(c)) CHECK(run_pass<R>(c, f, ap, KIND_STEP, PRO_NONE, EPI_NONE, 0, 0.0, ddt, nullptr, buf));
  return GPE_OK;
}

template <typename R>
gpe_status strang_step(gpe_ctx* c, Field& f, cx<R>* x, double ddt) {
  const double h = 0.5 * ddt;
  {
    Launch L(c, PC_NL_PHASE, (double)c->P * (4 * sizeof(R) + sizeof(R)));
    launch_nl_phase<R>(x, (const R*)f.V, c->P, c->prm.g, h, c->stream);
  }
  CHECK(kinetic_on<R>(c, f, x, ddt));
  {
    Launch L(c, PC_NL_PHASE, (double)c->P * (4 * sizeof(R) + sizeof(R)));
    launch_nl_phase<R>(x, (const R*)f.V, c->P, c->prm.g, h, c->stream);
  }
  CU(cudaGetLastError());
  return GPE_OK;
}

template <typename R>
gpe_status inner_impl(gpe_ctx* c, const cx<R>* a, const cx<R>* b, std::complex<double>* out) {
  const int nb = launch_inner<R>(a, b, c->P, c->partials, c->stream);
  c->launches++;
  std::vector<double> h(2 * (size_t)nb);
  CU(cudaMemcpyAsync(h.data(), c->partials, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  double re = 0.0, im = 0.0;
  for (int i = 0; i < nb; ++i) {
    re += h[2 * i];
    im += h[2 * i + 1];
  }
  *out = std::complex<double>(re, im) * c->weight;
  return GPE_OK;
}

template <typename R>
gpe_status adjoint_impl(gpe_ctx* c, Field& f, const gpe_adjoint_params* prm, const double* target,
                        double* dLdV_out, double* loss_out) {
  // f: the context's own field, or the FP64 field of an FP32 context.  The
  // start state is read from the context state (with its pending scale),
  // which is left as it is.
  launch_reset_scalars(c->sc, c->stream);  // passes skip their work while sc->stop is set
  const long long P = c->P;
  const size_t S = (size_t)P * 2 * sizeof(R);
  const int M = prm->nsteps;
  const double budget = prm->mem_budget > 0 ? prm->mem_budget : 60e9;
  // checkpoint interval: the caller's, or the one minimising stored states.
  // Stored: ceil(M/K)+1 checkpoints (the last is psi(T)), K-1 recomputed
  // states of one segment (K slots), x, lam, target, and dL/dV in FP64.
  int K = prm->checkpoint_every;
  auto bytes_for = [&](int k) { return ((double)((M + k - 1) / k + k + 4)) * S + (double)P * 8.0; };
  if (K <= 0) {
    K = 1;
    for (int k = 1; k <= M; ++k)
      if (bytes_for(k) < bytes_for(K)) K = k;
  }
  if (K > M) K = M;
  if (bytes_for(K) > budget)
    return fail(c, GPE_ERR_ALLOC, "adjoint: " + std::to_string(bytes_for(K) / 1e9) +
                                      " GB of states exceed the memory budget; raise mem_budget or change checkpoint_every");
  const int nck = (M + K - 1) / K;
  std::vector<void*> bufs;
  auto cleanup = [&]() {
    for (void* p : bufs) cudaFree(p);
  };
  auto alloc = [&](void** p, size_t bytes) -> bool {
    if (cudaMalloc(p, bytes) != cudaSuccess) return false;
    bufs.push_back(*p);
    return true;
  };
  void *ck = nullptr, *seg = nullptr, *x = nullptr, *lam = nullptr, *tgt = nullptr, *fwd32 = nullptr;
  double* dV = nullptr;
  if (!alloc(&ck, (size_t)(nck + 1) * S) || !alloc(&seg, (size_t)K * S) || !alloc(&x, S) || !alloc(&lam, S) ||
      !alloc(&tgt, S) || !alloc((void**)&dV, (size_t)P * sizeof(double))) {
    cleanup();
    return fail(c, GPE_ERR_ALLOC, "adjoint: device allocation of the checkpoint store failed");
  }
  auto st_at = [&](void* base, int i) { return (cx<R>*)((char*)base + (size_t)i * S); };
  // Error attribution of the FP64 sweep of an FP32 context (diagnostic,
  // GPE_ADJ_FORWARD): "fp32" runs every forward step (and recompute) in the
  // FP32 kernels, so the sweep sees an FP32 trajectory; "round32" keeps FP64
  // arithmetic and rounds each step's state to FP32, the storage error of an
  // FP32 trajectory alone; "kin32" runs only the kinetic passes in FP32 (the
  // nonlinear phases in FP64), "nl32" only the nonlinear phases.  Unset: the
  // FP64 forward.
  int fwd_mode = 0;
  if constexpr (sizeof(R) == 8) {
    if (const char* e = getenv("GPE_ADJ_FORWARD"))
      if (c->prec == GPE_FP32 && &f == &c->polish)
        fwd_mode = strcmp(e, "fp32") == 0      ? 1
                   : strcmp(e, "round32") == 0 ? 2
                   : strcmp(e, "kin32") == 0   ? 3
                   : strcmp(e, "nl32") == 0    ? 4
                                               : 0;
    if (fwd_mode != 0 && !alloc(&fwd32, (size_t)P * sizeof(cx<float>))) {
      cleanup();
      return fail(c, GPE_ERR_ALLOC, "adjoint: device allocation of the FP32 forward buffer failed");
    }
  }
  auto forward_step = [&](cx<R>* xs) -> gpe_status {
    if constexpr (sizeof(R) == 8) {
      if (fwd_mode == 1) {
        launch_convert_cx<double, float>(xs, (cx<float>*)fwd32, P, nullptr, c->stream);
        CHECK(strang_step<float>(c, c->main, (cx<float>*)fwd32, prm->ddt));
        launch_convert_cx<float, double>((const cx<float>*)fwd32, xs, P, nullptr, c->stream);
        c->launches += 2;
        return GPE_OK;
      }
      if (fwd_mode == 3 || fwd_mode == 4) {
        const double h = 0.5 * prm->ddt;
        auto nl = [&]() {
          if (fwd_mode == 3) {
            launch_nl_phase<double>(xs, (const double*)f.V, P, c->prm.g, h, c->stream);
          } else {
            launch_convert_cx<double, float>(xs, (cx<float>*)fwd32, P, nullptr, c->stream);
            launch_nl_phase<float>((cx<float>*)fwd32, (const float*)c->main.V, P, c->prm.g, h, c->stream);
            launch_convert_cx<float, double>((const cx<float>*)fwd32, xs, P, nullptr, c->stream);
          }
        };
        nl();
        if (fwd_mode == 3) {
          launch_convert_cx<double, float>(xs, (cx<float>*)fwd32, P, nullptr, c->stream);
          CHECK(kinetic_on<float>(c, c->main, fwd32, prm->ddt));
          launch_convert_cx<float, double>((const cx<float>*)fwd32, xs, P, nullptr, c->stream);
        } else {
          CHECK(kinetic_on<R>(c, f, xs, prm->ddt));
        }
        nl();
        CU(cudaGetLastError());
        return GPE_OK;
      }
      CHECK(strang_step<R>(c, f, xs, prm->ddt));
      if (fwd_mode == 2) {
        launch_convert_cx<double, float>(xs, (cx<float>*)fwd32, P, nullptr, c->stream);
        launch_convert_cx<float, double>((const cx<float>*)fwd32, xs, P, nullptr, c->stream);
        c->launches += 2;
      }
      return GPE_OK;
    } else {
      return strang_step<R>(c, f, xs, prm->ddt);
    }
  };
  gpe_status st = GPE_OK;
  auto run = [&]() -> gpe_status {
    CHECK(set_kinop<R>(c, f, 0.0, prm->ddt));
    if (fwd_mode == 1 || fwd_mode == 3) CHECK(set_kinop<float>(c, c->main, 0.0, prm->ddt));
    // target in the field's precision
    if constexpr (sizeof(R) == 8) {
      CU(cudaMemcpyAsync(tgt, target, (size_t)P * 16, cudaMemcpyHostToDevice, c->stream));
    } else {
      void* io = nullptr;
      CHECK(io_buffer(c, &io));
      CU(cudaMemcpyAsync(io, target, (size_t)P * 16, cudaMemcpyHostToDevice, c->stream));
      launch_convert_cx<double, R>((const cx<double>*)io, (cx<R>*)tgt, P, nullptr, c->stream);
      CU(cudaStreamSynchronize(c->stream));
      if (io != c->polish.psi) cudaFree(io);
    }
    // forward with checkpoints, from the context state times its pending scale
    if (c->prec == GPE_FP32)
      launch_convert_cx<float, R>((const cx<float>*)c->main.psi, (cx<R>*)x, P, c->sc, c->stream);
    else
      launch_convert_cx<double, R>((const cx<double>*)c->main.psi, (cx<R>*)x, P, c->sc, c->stream);
    c->launches++;
    for (int m = 0; m < M; ++m) {
      if (m % K == 0) {
        Launch L(c, PC_COPY, 2.0 * S);
        CU(cudaMemcpyAsync(st_at(ck, m / K), x, S, cudaMemcpyDeviceToDevice, c->stream));
      }
      CHECK(forward_step((cx<R>*)x));
    }
    {
      Launch L(c, PC_COPY, 2.0 * S);
      CU(cudaMemcpyAsync(st_at(ck, nck), x, S, cudaMemcpyDeviceToDevice, c->stream));  // x_M
    }
    // loss
    std::complex<double> ov, n0c, ntc;
    CHECK(inner_impl<R>(c, (const cx<R>*)tgt, (const cx<R>*)x, &ov));
    CHECK(inner_impl<R>(c, st_at(ck, 0), st_at(ck, 0), &n0c));
    CHECK(inner_impl<R>(c, (const cx<R>*)tgt, (const cx<R>*)tgt, &ntc));
    const double denom = std::sqrt(n0c.real() * ntc.real());
    const std::complex<double> cc = ov / denom;
    if (loss_out) *loss_out = 1.0 - std::norm(cc);
    // lam_T = dL/dpsi(T)* = -c * target * w / denom
    const std::complex<double> coef = -cc * (c->weight / denom);
    launch_cscale<R>((cx<R>*)lam, (const cx<R>*)tgt, P, coef.real(), coef.imag(), c->stream);
    CU(cudaMemsetAsync(dV, 0, (size_t)P * sizeof(double), c->stream));
    const double h = 0.5 * prm->ddt;
    const double adj_bytes = (double)P * (4.0 * sizeof(R) + sizeof(R) + 16.0);
    auto adj_nl = [&](const cx<R>* xm, int first, int second, int conj_in, int conj_out) {
      Launch L(c, PC_ADJ_NL, adj_bytes);
      launch_adj_nl<R>((cx<R>*)lam, xm, (const R*)f.V, dV, P, c->prm.g, h, first, second, conj_in, conj_out,
                       c->stream);
    };
    // adjoint of the last step's closing half: its output is x_M (slot nck)
    adj_nl(st_at(ck, nck), 0, 1, 0, 1);
    for (int s = nck - 1; s >= 0; --s) {
      const int m0 = s * K, m1 = std::min(M, m0 + K);
      // step-start states x_m0 .. x_{m1-1}; x_m1 is checkpoint s+1
      CU(cudaMemcpyAsync(x, st_at(ck, s), S, cudaMemcpyDeviceToDevice, c->stream));
      for (int m = m0 + 1; m < m1; ++m) {
        CHECK(forward_step((cx<R>*)x));
        Launch L(c, PC_COPY, 2.0 * S);
        CU(cudaMemcpyAsync(st_at(seg, m - m0), x, S, cudaMemcpyDeviceToDevice, c->stream));
      }
      for (int m = m1 - 1; m >= m0; --m) {
        CHECK(kinetic_on<R>(c, f, lam, prm->ddt));  // conj(K^H lam), lam held conjugated
        const cx<R>* xm = m == m0 ? st_at(ck, s) : st_at(seg, m - m0);
        // opening half of step m and, for m > 0, closing half of step m-1:
        // both are phases of |x_m|^2, applied in one pass
        adj_nl(xm, 1, m > 0, 1, m > 0);
        CU(cudaGetLastError());
      }
    }
    CU(cudaMemcpyAsync(dLdV_out, dV, (size_t)P * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return GPE_OK;
  };
  st = run();
  cudaStreamSynchronize(c->stream);
  cleanup();
  return st;
}

// ---- batched solve_split -------------------------------------------------------
// Many independent contexts (grids of any sizes) advance together: one block
// of n_rec steps of every context is captured once into a CUDA graph whose
// per-context chains hang off a fork/join pair of events, so the chains run
// concurrently on the GPU; the graph is then replayed block after block.
// A second graph holds the last block of an outer step (with the kinetic-
// energy passes and the history record).  Per-block host work (callbacks,
// time-dependent V, the decay target exp(-t/tau)) cannot live in a replayed
// graph, so those features are rejected here.
struct BatchGraph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t x = nullptr;
  ~BatchGraph() {
    if (x) cudaGraphExecDestroy(x);
    if (g) cudaGraphDestroy(g);
  }
};

gpe_status capture_blocks(gpe_ctx* c0, std::vector<gpe_ctx*>& cs, std::vector<SplitRun>& runs, bool last_block,
                          cudaStream_t master, std::vector<cudaEvent_t>& evs, BatchGraph& out) {
  gpe_ctx* c = c0;
  CU(cudaStreamBeginCapture(master, cudaStreamCaptureModeThreadLocal));
  gpe_status st = GPE_OK;
  cudaError_t e = cudaEventRecord(evs[0], master);
  for (size_t i = 0; i < cs.size() && st == GPE_OK && e == cudaSuccess; ++i) {
    gpe_ctx* ci = cs[i];
    e = cudaStreamWaitEvent(ci->stream, evs[0], 0);
    if (e != cudaSuccess) break;
    const bool prof = ci->prof;
    const long long launches = ci->launches;
    ci->prof = false;  // no profiling events inside a graph
    if (ci->prec == GPE_FP32) st = enqueue_block<float>(ci, runs[i], 0.0, last_block, last_block ? ci->d_hist : nullptr);
    else st = enqueue_block<double>(ci, runs[i], 0.0, last_block, last_block ? ci->d_hist : nullptr);
    ci->prof = prof;
    ci->launches = launches;  // counted per replay instead
    if (st != GPE_OK) break;
    e = cudaEventRecord(evs[1 + i], ci->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(master, evs[1 + i], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(master, &g);
  if (st != GPE_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(c, GPE_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  out.g = g;
  CU(cudaGraphInstantiate(&out.x, g, 0));
  return GPE_OK;
}

gpe_status batch_impl(std::vector<gpe_ctx*>& cs, const gpe_split_params* prm) {
  gpe_ctx* c = cs[0];
  const size_t n = cs.size();
  std::vector<SplitRun> runs(n);
  for (size_t i = 0; i < n; ++i) {
    int vk = 0;
    gpe_ctx* ci = cs[i];
    ci->err.clear();
    gpe_status st = ci->prec == GPE_FP32 ? split_setup<float>(ci, prm, runs[i], vk, 3)
                                         : split_setup<double>(ci, prm, runs[i], vk, 3);
    if (st != GPE_OK) return fail(c, st, "batch: context " + std::to_string(i) + ": " + ci->err);
    CU(cudaStreamSynchronize(ci->stream));
  }
  const SplitRun& r0 = runs[0];
  for (size_t i = 1; i < n; ++i)
    if (runs[i].n_rec != r0.n_rec || runs[i].start != r0.start)
      return fail(c, GPE_ERR_INVALID, "batch: all contexts need the same n_recalc and current_iter");
  // The graphs are launched on the first context's stream, so that context's
  // timer (gpe_timer_start/stop) brackets a batched run.
  cudaStream_t master = cs[0]->stream;
  std::vector<cudaEvent_t> evs(n + 1, nullptr);
  for (auto& ev : evs) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  auto cleanup = [&]() {
    for (auto ev : evs)
      if (ev) cudaEventDestroy(ev);
  };
  BatchGraph g_plain, g_last;
  gpe_status st = GPE_OK;
  // Several contexts' chains run side by side: programmatic dependent launch
  // would park each chain's next kernel on the SMs while it waits, which took
  // slots from the other chains' ready kernels (batch of 64 grids 7% slower),
  // so it is kept for one-context graphs only.
  std::vector<int> pdl_saved(n);
  for (size_t i = 0; i < n; ++i) {
    pdl_saved[i] = cs[i]->pdl;
    if (n > 1) cs[i]->pdl = 0;
  }
  if (r0.nb > 1) st = capture_blocks(c, cs, runs, false, master, evs, g_plain);
  if (st == GPE_OK) st = capture_blocks(c, cs, runs, true, master, evs, g_last);
  for (size_t i = 0; i < n; ++i) cs[i]->pdl = pdl_saved[i];
  if (st != GPE_OK) {
    cleanup();
    return st;
  }
  // kernels per replay, for the launch counters
  std::vector<long long> k_plain(n), k_last(n);
  for (size_t i = 0; i < n; ++i) {
    const long long steps = (long long)runs[i].n_rec * (long long)runs[i].passes.size();
    k_plain[i] = steps + (runs[i].feedback ? (long long)runs[i].passes.size() : 0) + 1;
    k_last[i] = steps + (long long)runs[i].passes.size() + 1;
  }
  int last_j = r0.start;
  cudaError_t e = cudaSuccess;
  for (int j = r0.start + 1; j <= r0.nout && e == cudaSuccess; ++j) {
    for (int jj = 1; jj < r0.nb && e == cudaSuccess; ++jj) e = cudaGraphLaunch(g_plain.x, master);
    if (e == cudaSuccess) e = cudaGraphLaunch(g_last.x, master);
    // the last block left (muc, ncur, energy) in each context's slot 0: file it
    const size_t hj = (size_t)(j - r0.start - 1);
    for (size_t i = 0; i < n && e == cudaSuccess; ++i)
      e = cudaMemcpyAsync(cs[i]->d_hist + 3 + 3 * hj, cs[i]->d_hist, 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                          master);
    for (size_t i = 0; i < n; ++i) cs[i]->launches += (long long)(r0.nb - 1) * k_plain[i] + k_last[i];
    last_j = j;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(master);
  cleanup();
  if (e != cudaSuccess) return fail(c, GPE_ERR_CUDA, std::string("batch replay: ") + cudaGetErrorString(e));
  for (size_t i = 0; i < n; ++i) {
    const double time2 = (last_j - 1) * runs[i].dt_outer + (runs[i].nb - 1) * runs[i].ddt * runs[i].n_rec;
    gpe_status st2 = cs[i]->prec == GPE_FP32 ? split_finish<float>(cs[i], runs[i], last_j, time2)
                                             : split_finish<double>(cs[i], runs[i], last_j, time2);
    if (st2 != GPE_OK) return fail(c, st2, "batch: context " + std::to_string(i) + ": " + cs[i]->err);
  }
  return GPE_OK;
}

// ---- persistent cluster path of small 2D grids (cluster2d.cuh) --------------------
// One k_cluster2d launch advances every context of a batch (or the single
// context of solve_split) by one outer step; the launch is captured once
// into a CUDA graph and replayed per outer step (it reads its outer-step
// index from each context's device scalars).  Used for 2D one-component
// grids with both axis lengths in GPE_C2_SIZES whose state fits the
// cluster's shared memory, with the default pass variant; anything else
// takes the per-pass paths.
bool c2_size_ok(int n) {
  switch (n) {
#define X(v) case v:
    GPE_C2_SIZES(X)
#undef X
    return true;
    default:
      return false;
  }
}

bool c2_eligible(const gpe_ctx* c) {
  return c->ndims == 2 && c->ncomp == 1 && !c->omega_field && c->prm.omega == 0.0 && c->pass_variant == 0 &&
         c2_size_ok(c->n[0]) && c2_size_ok(c->n[1]);
}

struct C2Plan {
  int cs = 0, nclusters = 0;
  int vsm = 0;  // V columns in shared memory
  size_t smem = 0;
};

// GPE_CLUSTER_SIZE=8|16 forces a cluster size (measurement); GPE_CLUSTER=0
// turns the path off.
int c2_env(const char* name, int dflt) {
  const char* e = getenv(name);
  return e ? atoi(e) : dflt;
}

// Cluster size and resident clusters: the candidate that keeps the most CTAs
// busy (clusters in use x size), 16 first so that a tie gives each grid more
// SMs.  cs = 0: no cluster shape fits.
template <typename R>
C2Plan c2_plan(const std::vector<gpe_ctx*>& cs) {
  C2Plan best;
  const int forced = c2_env("GPE_CLUSTER_SIZE", 0);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, cs[0]->device);
  long long best_score = -1;
  for (int cand : {16, 8}) {
    if (forced && cand != forced) continue;
    size_t smem = 0, smem_v = 0;
    bool ok = true;
    for (auto* c : cs) {
      if (c->n[0] % cand || c->n[1] % cand) ok = false;
      smem = std::max(smem, c2_geom(c->n[0], c->n[1], cand, (int)sizeof(cx<R>)).bytes);
      smem_v = std::max(smem_v, c2_geom(c->n[0], c->n[1], cand, (int)sizeof(cx<R>), 1).bytes);
    }
    if (!ok || smem > (size_t)optin) continue;
    const int maxc = cluster2d_max_clusters<R>(cand, smem);
    if (maxc <= 0) continue;
    // V columns in shared memory where they fit without losing clusters
    // (GPE_C2_VSM=0 turns this off)
    int vsm = 0;
    if (c2_env("GPE_C2_VSM", 1) != 0 && smem_v <= (size_t)optin &&
        cluster2d_max_clusters<R>(cand, smem_v) >= std::min<int>((int)cs.size(), maxc)) {
      vsm = 1;
      smem = smem_v;
    }
    const int ncl = std::min<int>((int)cs.size(), maxc);
    const long long score = (long long)ncl * cand;
    if (score > best_score) {
      best_score = score;
      best.cs = cand;
      best.nclusters = ncl;
      best.smem = smem;
      best.vsm = vsm;
    }
  }
  return best;
}

// Axis tables of the plans the cluster kernel is built on (C2Plan: the
// alternative plan where the length has one), for both axes.
template <typename R>
gpe_status cluster_plans(gpe_ctx* c) {
  for (int ax = 0; ax < 2; ++ax) {
    const int v = c2_plan_var(c->n[ax], (int)sizeof(cx<R>));
    if (c->main.plan_var[ax] != v) {
      c->main.plan_var[ax] = v;
      CHECK(build_axis_tables<R>(c, c->main, ax));
    }
  }
  return GPE_OK;
}

template <typename R>
gpe_status cluster_impl(std::vector<gpe_ctx*>& cs, const gpe_split_params* prm, const C2Plan& pl) {
  gpe_ctx* c = cs[0];
  const size_t n = cs.size();
  std::vector<SplitRun> runs(n);
  for (size_t i = 0; i < n; ++i) {
    int vk = 0;
    gpe_ctx* ci = cs[i];
    ci->err.clear();
    gpe_status st = cluster_plans<R>(ci);
    if (st == GPE_OK) st = split_setup<R>(ci, prm, runs[i], vk, 3);
    if (st != GPE_OK) return n > 1 ? fail(c, st, "batch: context " + std::to_string(i) + ": " + ci->err) : st;
    CU(cudaStreamSynchronize(ci->stream));
  }
  const SplitRun& r0 = runs[0];
  for (size_t i = 1; i < n; ++i)
    if (runs[i].n_rec != r0.n_rec || runs[i].start != r0.start)
      return fail(c, GPE_ERR_INVALID, "batch: all contexts need the same n_recalc and current_iter");
  // work table: one entry per context
  std::vector<C2Grid> grids(n);
  double bytes = 0.0;
  for (size_t i = 0; i < n; ++i) {
    gpe_ctx* ci = cs[i];
    Field& f = ci->main;
    C2Grid& G = grids[i];
    G.psi = f.psi;
    G.V = f.V;
    for (int ax = 0; ax < 2; ++ax) {
      G.tws[ax] = f.tws[ax];
      G.php[ax] = f.php[ax];
      G.k2p[ax] = f.k2p[ax];
    }
    G.sc = ci->sc;
    G.hist = ci->d_hist + runs[i].hist_off;
    G.nx = ci->n[0];
    G.ny = ci->n[1];
    G.feedback = runs[i].feedback ? 1 : 0;
    G.start = runs[i].start;
    G.weight = ci->weight;
    G.g = ci->prm.g;
    G.tau = ci->prm.decay_rate;
    G.dre = runs[i].dre;
    G.dim = runs[i].dim;
    bytes += (double)ci->P * (4 * sizeof(R) + sizeof(R));  // state in and out, V once
  }
  // Longest-processing-time assignment of the grids to the clusters (cost of
  // a grid: P log2 P, the FFT work of a step).
  std::vector<int> idx(n);
  for (size_t i = 0; i < n; ++i) idx[i] = (int)i;
  auto cost = [&](int i) { return (double)cs[i]->P * std::log2((double)cs[i]->P); };
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost(a) > cost(b); });
  const int ncl = pl.nclusters;
  std::vector<std::vector<int>> lists(ncl);
  std::vector<double> load(ncl, 0.0);
  for (int i : idx) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    lists[k].push_back(i);
    load[k] += cost(i);
  }
  std::vector<int> order, offs{0};
  for (auto& l : lists) {
    order.insert(order.end(), l.begin(), l.end());
    offs.push_back((int)order.size());
  }
  const size_t gb = n * sizeof(C2Grid), ob = order.size() * sizeof(int), fb = offs.size() * sizeof(int);
  char* dbuf = nullptr;
  CU(cudaMalloc(&dbuf, gb + ob + fb));
  struct Free {
    char* p;
    ~Free() { cudaFree(p); }
  } free_dbuf{dbuf};
  CU(cudaMemcpy(dbuf, grids.data(), gb, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(dbuf + gb, order.data(), ob, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(dbuf + gb + ob, offs.data(), fb, cudaMemcpyHostToDevice));
  C2Args a;
  a.grids = reinterpret_cast<const C2Grid*>(dbuf);
  a.order = reinterpret_cast<const int*>(dbuf + gb);
  a.offs = reinterpret_cast<const int*>(dbuf + gb + ob);
  a.n_rec = r0.n_rec;
  a.nb = r0.nb;
  a.nouter = 1;
  a.vsm = pl.vsm;
  a.fold = fold_env() ? 1 : 0;
  a.ddt = r0.ddt;
  a.dt_outer = r0.dt_outer;
  cudaStream_t master = c->stream;
  int last_j = r0.start;
  bool stop_req = false;
  const bool direct = c->prof || prm->on_step;
  BatchGraph gr;
  if (!direct && r0.nout > r0.start) {
    CU(cudaStreamBeginCapture(master, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e = launch_cluster2d<R>(a, ncl, pl.cs, pl.smem, master);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(master, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail(c, GPE_ERR_CUDA, std::string("cluster graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    gr.g = g;
    CU(cudaGraphInstantiate(&gr.x, g, 0));
  }
  for (int j = r0.start + 1; j <= r0.nout && !stop_req; ++j) {
    if (direct) {
      Launch L(c, PC_CLUSTER, bytes);
      CU(launch_cluster2d<R>(a, ncl, pl.cs, pl.smem, master));
    } else {
      c->launches++;
      CU(cudaGraphLaunch(gr.x, master));
    }
    last_j = j;
    if (prm->on_step) {  // ext_callback (solve_split.m:80); one context only
      DevScalars h;
      CHECK(read_scalars(c, &h));
      if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "solve_split: non-finite norm or chemical potential");
      const double time2 = (j - 1) * r0.dt_outer + (r0.nb - 1) * r0.ddt * r0.n_rec;
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
      if (prm->on_step(prm->step_user, j, time2, h.muc, h.ncur) != 0) stop_req = true;
    }
  }
  CU(cudaStreamSynchronize(master));
  for (size_t i = 0; i < n; ++i) {
    const double time2 = (last_j - 1) * runs[i].dt_outer + (runs[i].nb - 1) * runs[i].ddt * runs[i].n_rec;
    const gpe_status st2 = split_finish<R>(cs[i], runs[i], last_j, time2);
    if (st2 != GPE_OK) return n > 1 ? fail(c, st2, "batch: context " + std::to_string(i) + ": " + cs[i]->err) : st2;
  }
  return GPE_OK;
}

// ---- grid-wide persistent path of small 2D grids (grid2d.cu, FP32) -------------
// Tables: both axes on the default plans (the pass bodies the persistent
// kernel runs).
gpe_status grid2d_plans(gpe_ctx* c) {
  const int want[2] = {0, 0};
  for (int ax = 0; ax < 2; ++ax)
    if (c->main.plan_var[ax] != want[ax]) {
      c->main.plan_var[ax] = want[ax];
      CHECK(build_axis_tables<float>(c, c->main, ax));
    }
  return GPE_OK;
}

// nctas > 0: the grid-wide cooperative kernel on nctas CTAs; nctas == 0:
// the multi-grid pass kernels, one group of grids per shape, each group on
// its own stream.
gpe_status grid2d_impl(std::vector<gpe_ctx*>& cs, const gpe_split_params* prm, int nctas) {
  gpe_ctx* c = cs[0];
  const size_t n = cs.size();
  std::vector<SplitRun> runs(n);
  for (size_t i = 0; i < n; ++i) {
    int vk = 0;
    gpe_ctx* ci = cs[i];
    ci->err.clear();
    gpe_status st = grid2d_plans(ci);
    if (st == GPE_OK) st = split_setup<float>(ci, prm, runs[i], vk, 3);
    if (st != GPE_OK) return n > 1 ? fail(c, st, "batch: context " + std::to_string(i) + ": " + ci->err) : st;
    CU(cudaStreamSynchronize(ci->stream));
  }
  const SplitRun& r0 = runs[0];
  for (size_t i = 1; i < n; ++i)
    if (runs[i].n_rec != r0.n_rec || runs[i].start != r0.start)
      return fail(c, GPE_ERR_INVALID, "batch: all contexts need the same n_recalc and current_iter");
  std::vector<G2Grid> grids(n);
  std::vector<int> yoff{0}, xoff{0};
  double bytes = 0.0;
  for (size_t i = 0; i < n; ++i) {
    gpe_ctx* ci = cs[i];
    Field& f = ci->main;
    G2Grid& G = grids[i];
    G.psi = f.psi;
    G.V = f.V;
    for (int ax = 0; ax < 2; ++ax) {
      G.tws[ax] = f.tws[ax];
      G.php[ax] = f.php[ax];
      G.k2p[ax] = f.k2p[ax];
    }
    G.sc = ci->sc;
    G.partials = ci->partials;
    G.cap = ci->cap;
    G.hist = ci->d_hist + runs[i].hist_off;
    G.nx = ci->n[0];
    G.ny = ci->n[1];
    const int py = grid2d_tile_pencils(G.ny, false), px = grid2d_tile_pencils(G.nx, true);
    G.ytiles = (G.nx + py - 1) / py;
    G.xtiles = (G.ny + px - 1) / px;
    if (G.ytiles > G.cap || G.xtiles > G.cap) return fail(c, GPE_ERR_INVALID, "grid2d: partial-sum buffer too small");
    G.feedback = runs[i].feedback ? 1 : 0;
    G.start = runs[i].start;
    G.weight = ci->weight;
    G.g = ci->prm.g;
    G.tau = ci->prm.decay_rate;
    G.dre = runs[i].dre;
    G.dim = runs[i].dim;
    yoff.push_back(yoff.back() + G.ytiles);
    xoff.push_back(xoff.back() + G.xtiles);
    bytes += (double)ci->P * (4 * sizeof(float) + sizeof(float)) * r0.n_rec * r0.nb;  // state r/w per pass, V
  }
  const size_t gb = n * sizeof(G2Grid), ob = (n + 1) * sizeof(int);
  char* dbuf = nullptr;
  CU(cudaMalloc(&dbuf, gb + 2 * ob + 32));
  struct Free {
    char* p;
    ~Free() { cudaFree(p); }
  } free_dbuf{dbuf};
  CU(cudaMemcpy(dbuf, grids.data(), gb, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(dbuf + gb, yoff.data(), ob, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(dbuf + gb + ob, xoff.data(), ob, cudaMemcpyHostToDevice));
  unsigned* bar = reinterpret_cast<unsigned*>(dbuf + ((gb + 2 * ob + 15) & ~(size_t)15));
  int* failf = reinterpret_cast<int*>(bar + 2);
  CU(cudaMemset(bar, 0, 12));
  G2Args a;
  a.grids = reinterpret_cast<const G2Grid*>(dbuf);
  a.ngrids = (int)n;
  a.yoff = reinterpret_cast<const int*>(dbuf + gb);
  a.xoff = reinterpret_cast<const int*>(dbuf + gb + ob);
  a.n_rec = r0.n_rec;
  a.nb = r0.nb;
  a.nouter = 1;
  a.ddt = r0.ddt;
  a.dt_outer = r0.dt_outer;
  a.bar = bar;
  a.fail = failf;
  cudaStream_t master = c->stream;
  // multi-grid pass kernels: the grids grouped by shape, a group's grid
  // table and item offsets in a buffer of its own, a stream per group
  struct Group {
    G2Args a;
    int ny, nx, ny_items, nx_items;
    bool feedback;
    cudaStream_t s;
    cudaEvent_t done;
  };
  std::vector<Group> groups;
  struct GroupRes {
    std::vector<void*> bufs;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    ~GroupRes() {
      for (auto* p : bufs) cudaFree(p);
      for (auto st : streams) cudaStreamDestroy(st);
      for (auto ev : events) cudaEventDestroy(ev);
    }
  } gres;
  cudaEvent_t fork_ev = nullptr;
  if (nctas == 0) {
    // groups: the grids of one shape (splitting a shape that holds most of
    // the points over several streams measured no faster)
    std::vector<std::vector<int>> members;
    {
      std::vector<std::pair<int, int>> shapes;
      for (size_t i = 0; i < grids.size(); ++i) {
        const auto sh = std::make_pair(grids[i].ny, grids[i].nx);
        const size_t k = std::find(shapes.begin(), shapes.end(), sh) - shapes.begin();
        if (k == shapes.size()) {
          shapes.push_back(sh);
          members.emplace_back();
        }
        members[k].push_back((int)i);
      }
    }
    CU(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    gres.events.push_back(fork_ev);
    for (const auto& mem : members) {
      std::vector<G2Grid> gg;
      std::vector<int> yo{0}, xo{0};
      bool fb = false;
      for (int i : mem) {
        const G2Grid& G = grids[i];
        gg.push_back(G);
        yo.push_back(yo.back() + G.ytiles);
        xo.push_back(xo.back() + G.xtiles);
        fb = fb || G.feedback;
      }
      const size_t ggb = gg.size() * sizeof(G2Grid), gob = (gg.size() + 1) * sizeof(int);
      char* buf = nullptr;
      CU(cudaMalloc(&buf, ggb + 2 * gob));
      gres.bufs.push_back(buf);
      CU(cudaMemcpy(buf, gg.data(), ggb, cudaMemcpyHostToDevice));
      CU(cudaMemcpy(buf + ggb, yo.data(), gob, cudaMemcpyHostToDevice));
      CU(cudaMemcpy(buf + ggb + gob, xo.data(), gob, cudaMemcpyHostToDevice));
      Group grp;
      grp.a = a;
      grp.a.grids = reinterpret_cast<const G2Grid*>(buf);
      grp.a.ngrids = (int)gg.size();
      grp.a.yoff = reinterpret_cast<const int*>(buf + ggb);
      grp.a.xoff = reinterpret_cast<const int*>(buf + ggb + gob);
      grp.ny = gg[0].ny;
      grp.nx = gg[0].nx;
      grp.ny_items = yo.back();
      grp.nx_items = xo.back();
      grp.feedback = fb;
      if (groups.empty()) {
        grp.s = master;
      } else {
        CU(cudaStreamCreateWithFlags(&grp.s, cudaStreamNonBlocking));
        gres.streams.push_back(grp.s);
      }
      CU(cudaEventCreateWithFlags(&grp.done, cudaEventDisableTiming));
      gres.events.push_back(grp.done);
      groups.push_back(grp);
    }
  }
  // kernels of one outer step (the launch count the context reports)
  long long kernels = 1;
  if (nctas == 0) {
    kernels = 0;
    const bool fold = fold_env();
    for (const Group& grp : groups)
      for (int jj = 1; jj <= r0.nb; ++jj)
        kernels += (fold ? 1 + r0.n_rec : 2 * r0.n_rec) + ((grp.feedback || jj == r0.nb) ? 2 : 0) + 1;
  }
  int last_j = r0.start;
  bool stop_req = false;
  const bool direct = c->prof || prm->on_step;
  BatchGraph gr;
  auto enqueue = [&]() -> cudaError_t {
    if (nctas > 0) {
      cudaError_t e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), master);  // the failure flag stays once set
      if (e == cudaSuccess) e = launch_grid2d(a, nctas, master);
      return e;
    }
    cudaError_t e = cudaEventRecord(fork_ev, master);
    for (size_t k = 1; k < groups.size() && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(groups[k].s, fork_ev, 0);
    for (const Group& grp : groups)
      for (int jj = 1; jj <= r0.nb && e == cudaSuccess; ++jj) {
        const bool last = jj == r0.nb;
        e = launch_multi2d_block(grp.a, grp.ny, grp.nx, grp.ny_items, grp.nx_items, jj, last, grp.feedback || last,
                                 fold_env(), grp.s);
      }
    for (size_t k = 1; k < groups.size() && e == cudaSuccess; ++k) {
      e = cudaEventRecord(groups[k].done, groups[k].s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(master, groups[k].done, 0);
    }
    return e;
  };
  if (!direct && r0.nout > r0.start) {
    CU(cudaStreamBeginCapture(master, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e = enqueue();
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(master, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail(c, GPE_ERR_CUDA, std::string("grid2d graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    gr.g = g;
    CU(cudaGraphInstantiate(&gr.x, g, 0));
  }
  for (int j = r0.start + 1; j <= r0.nout && !stop_req; ++j) {
    if (direct) {
      Launch L(c, PC_CLUSTER, bytes);
      c->launches += kernels - 1;
      CU(enqueue());
    } else {
      c->launches += kernels;
      CU(cudaGraphLaunch(gr.x, master));
    }
    last_j = j;
    if (prm->on_step) {  // ext_callback (solve_split.m:80); one context only
      DevScalars h;
      CHECK(read_scalars(c, &h));
      if (h.nonfinite) return fail(c, GPE_ERR_NONFINITE, "solve_split: non-finite norm or chemical potential");
      const double time2 = (j - 1) * r0.dt_outer + (r0.nb - 1) * r0.ddt * r0.n_rec;
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
      if (prm->on_step(prm->step_user, j, time2, h.muc, h.ncur) != 0) stop_req = true;
    }
  }
  CU(cudaStreamSynchronize(master));
  int failed = 0;
  CU(cudaMemcpy(&failed, failf, sizeof(int), cudaMemcpyDeviceToHost));
  if (failed) {
    for (auto* ci : cs) {
      DevScalars h;
      CHECK(read_scalars(ci, &h));
      h.timeout = 1;
      h.stop = 1;
      CHECK(write_scalars(ci, h));
    }
  }
  for (size_t i = 0; i < n; ++i) {
    const double time2 = (last_j - 1) * runs[i].dt_outer + (runs[i].nb - 1) * runs[i].ddt * runs[i].n_rec;
    const gpe_status st2 = split_finish<float>(cs[i], runs[i], last_j, time2);
    if (st2 != GPE_OK) return n > 1 ? fail(c, st2, "batch: context " + std::to_string(i) + ": " + cs[i]->err) : st2;
  }
  return GPE_OK;
}

// Runs solve_split on cs through a persistent kernel of small 2D grids when
// every context is eligible (same precision, a shape that fits): the
// multi-grid pass kernels (FP32 batches), the grid-wide kernel (FP32,
// GPE_SMALL2D=grid) or the cluster kernel (the default rule below).  *used = false leaves the call to the per-pass paths.
gpe_status cluster_run(std::vector<gpe_ctx*>& cs, const gpe_split_params* prm, bool* used) {
  *used = false;
  if (c2_env("GPE_CLUSTER", 1) == 0) return GPE_OK;
  for (auto* ci : cs)
    if (!c2_eligible(ci) || ci->prec != cs[0]->prec) return GPE_OK;
  // Default: the multi-grid pass kernels for FP32 batches (every SM busy on
  // the tiles of many grids, each pass kernel at the per-pass kernels'
  // occupancy: 64 uneven grids 5.7e10 grid-pt-steps/s against 4.9e10 for the
  // grid-wide kernel and 3.9e10 for the cluster kernel), the cluster kernel
  // for a single grid (a few tiles per pass: 256^2 5.7e9 against 4.2e9 for
  // either of the others).  GPE_SMALL2D=multi|grid|cluster forces one.
  const char* mode = getenv("GPE_SMALL2D");
  const bool fp32 = cs[0]->prec == GPE_FP32;
  if (fp32 && (mode ? strcmp(mode, "multi") == 0 : cs.size() > 1)) {
    *used = true;
    return grid2d_impl(cs, prm, 0);
  }
  if (fp32 && mode && strcmp(mode, "grid") == 0) {
    // GPE_G2_CTAS caps the CTAs of the grid-wide kernel (measurement: fewer
    // CTAs make each grid barrier cheaper)
    int nctas = grid2d_max_ctas();
    const int cap_ctas = c2_env("GPE_G2_CTAS", 0);
    if (cap_ctas > 0 && cap_ctas < nctas) nctas = cap_ctas;
    if (nctas > 0) {
      *used = true;
      return grid2d_impl(cs, prm, nctas);
    }
  }
  const C2Plan pl = cs[0]->prec == GPE_FP32 ? c2_plan<float>(cs) : c2_plan<double>(cs);
  if (pl.cs == 0) return GPE_OK;
  *used = true;
  return cs[0]->prec == GPE_FP32 ? cluster_impl<float>(cs, prm, pl) : cluster_impl<double>(cs, prm, pl);
}

template <typename R>
gpe_status materialize(gpe_ctx* c) {
  Launch L(c, PC_ELEMENTWISE, (double)c->PS * 4 * sizeof(R));
  launch_apply_scale<R>((cx<R>*)c->main.psi, c->PS, c->sc, c->stream);
  launch_set_scale_one(c->sc, c->stream);
  CU(cudaGetLastError());
  return GPE_OK;
}

gpe_status check_ctx(gpe_ctx* c) {
  if (!c) return fail(nullptr, GPE_ERR_INVALID, "null context");
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(c, GPE_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  return GPE_OK;
}

gpe_status need_state(gpe_ctx* c) {
  if (!c->have_state) return fail(c, GPE_ERR_STATE, "no state: call gpe_set_state first");
  return GPE_OK;
}
gpe_status need_V(gpe_ctx* c) {
  if (!c->have_V) return fail(c, GPE_ERR_STATE, "no potential: call gpe_set_potential first");
  return GPE_OK;
}

// io staging (P complex doubles) for precision conversions of state copies.
// The FP64 polish field's psi is idle outside groundstate_itp and is reused;
// otherwise a temporary buffer is allocated (the caller frees it).
gpe_status io_buffer(gpe_ctx* c, void** out) {
  if (c->prec == GPE_FP32 && c->polish.psi) {
    *out = c->polish.psi;
    return GPE_OK;
  }
  void* p = nullptr;
  CU(cudaMalloc(&p, (size_t)c->PS * 16));
  *out = p;
  return GPE_OK;
}

// ---- FFT plan autotuner ------------------------------------------------------
// For every FP32 axis pass whose length has two plans (plans.cuh Plan /
// PlanAlt), time both on a scratch array shaped like the state and keep the
// faster; the alternative must win by 5% so near-ties keep the default plan
// (and the choice does not flip between runs).  Choices are cached per
// device and pass geometry for the process, so contexts of one shape are
// timed once.
struct TuneKey {
  int dev, N, strided;
  long long n_batch, stride, inner, outer;
  bool operator==(const TuneKey& o) const {
    return dev == o.dev && N == o.N && strided == o.strided && n_batch == o.n_batch && stride == o.stride &&
           inner == o.inner && outer == o.outer;
  }
};
std::mutex g_tune_mu;
std::vector<std::pair<TuneKey, int>> g_tune_cache;

// Best of 3 launches of one axis pass on buf, in ms.  The contiguous pass
// runs with the real-time phase prologue it carries in every split step
// (when the context has a potential); the others run bare.
gpe_status time_axis_pass(gpe_ctx* c, Field& f, const AxisPass& ap, void* buf, float* ms) {
  const int pro = (!ap.strided && c->have_V && f.V) ? PRO_RT_FULL : PRO_NONE;
  cudaEvent_t e0 = pool_event(c), e1 = pool_event(c);
  float best = 1e30f;
  CHECK(run_pass<float>(c, f, ap, KIND_STEP, pro, EPI_NONE, 0, 0.0, 1e-3, nullptr, buf));  // warm-up
  for (int r = 0; r < 3; ++r) {
    CU(cudaEventRecord(e0, c->stream));
    CHECK(run_pass<float>(c, f, ap, KIND_STEP, pro, EPI_NONE, 0, 0.0, 1e-3, nullptr, buf));
    CU(cudaEventRecord(e1, c->stream));
    CU(cudaEventSynchronize(e1));
    float t = 0.0f;
    CU(cudaEventElapsedTime(&t, e0, e1));
    best = std::min(best, t);
  }
  c->ev_pool.push_back(e0);
  c->ev_pool.push_back(e1);
  *ms = best;
  return GPE_OK;
}

// chosen[ax]: the variant of axis ax, -1 where the length has one plan.
gpe_status autotune_main(gpe_ctx* c, int chosen[3]) {
  for (int ax = 0; ax < 3; ++ax) chosen[ax] = -1;
  c->tuned = true;
  if (c->prec != GPE_FP32) return GPE_OK;  // FP64 passes use Plan<N>
  Field& f = c->main;
  std::vector<AxisPass> todo;
  for (auto& ap : axis_passes(c))
    if (has_alt_plan(ap.N)) todo.push_back(ap);
  if (todo.empty()) return GPE_OK;
  void* buf = nullptr;
  CU(cudaMalloc(&buf, (size_t)c->P * 2 * sizeof(float)));
  gpe_status st = GPE_OK;
  auto tune = [&]() -> gpe_status {
    CU(cudaMemsetAsync(buf, 0, (size_t)c->P * 2 * sizeof(float), c->stream));
    launch_reset_scalars(c->sc, c->stream);  // passes skip their work while sc->stop is set
    for (auto& ap : todo) {
      const TuneKey key{c->device, ap.N, ap.strided ? 1 : 0, ap.n_batch, ap.stride, ap.inner, ap.outer};
      int var = -1;
      {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        for (auto& e : g_tune_cache)
          if (e.first == key) var = e.second;
      }
      if (var < 0) {
        // the default plan, the alternative, the paired passes on the
        // alternative and on the default plan; a non-default one must be 5%
        // faster than the default
        float t[4] = {0.f, 1e30f, 1e30f, 1e30f};
        const int nv = has_x2d_plan(ap.N) ? 4 : 3;
        for (int v = 0; v < nv; ++v) {
          f.plan_var[ap.axis] = v;
          CHECK(build_axis_tables<float>(c, f, ap.axis));
          CHECK(set_kinop<float>(c, f, 0.0, 1e-3));  // any unit-modulus factor: timing only
          CHECK(time_axis_pass(c, f, ap, buf, &t[v]));
        }
        int best = 1;
        for (int v = 2; v < nv; ++v)
          if (t[v] < t[best]) best = v;
        var = t[best] < 0.95f * t[0] ? best : 0;
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache.push_back({key, var});
      }
      f.plan_var[ap.axis] = var;
      CHECK(build_axis_tables<float>(c, f, ap.axis));
      chosen[ap.axis] = var;
    }
    f.phase_valid = false;  // the next run builds its own kinetic factors
    return GPE_OK;
  };
  st = tune();
  cudaStreamSynchronize(c->stream);
  cudaFree(buf);
  return st;
}

// Automatic tuning on the first hot-path call of a large FP32 context.
gpe_status maybe_autotune(gpe_ctx* c) {
  if (c->tuned || c->tune_mode != 2 || c->prec != GPE_FP32 || c->pass_variant == 1 || c->ncomp != 1) return GPE_OK;
  if (c->P < (1LL << 20)) return GPE_OK;
  int chosen[3];
  return autotune_main(c, chosen);
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
#include "spinor_driver.cuh"
#include "observables_driver.cuh"

extern "C" {

int gpe_abi_version(void) { return GPE_ABI_VERSION; }

int gpe_device_available(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return 0;
  for (int d = 0; d < n; ++d) {
    int maj = 0, min = 0;
    cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, d);
    cudaDeviceGetAttribute(&min, cudaDevAttrComputeCapabilityMinor, d);
    if (maj == 10 && min == 3) return 1;
  }
  return 0;
}

const char* gpe_last_error(const gpe_ctx* ctx) {
  if (!ctx) return g_create_err.c_str();
  return ctx->err.c_str();
}

void gpe_default_params(gpe_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->n_recalc = 10;
  p->itp_max_iter = 5000;
  p->itp_min_iter = 50;
}

static gpe_status create_impl(const gpe_grid_desc* d, gpe_ctx** out, int ncomp) {
  gpe_ctx* c = nullptr;
  if (!d || !out) return fail(nullptr, GPE_ERR_INVALID, "gpe_create: null argument");
  *out = nullptr;
  if (d->ndims != 2 && d->ndims != 3) return fail(nullptr, GPE_ERR_INVALID, "ndims must be 2 or 3");
  if (d->precision != GPE_FP32 && d->precision != GPE_FP64)
    return fail(nullptr, GPE_ERR_INVALID, "precision must be GPE_FP32 or GPE_FP64");
  for (int a = 0; a < d->ndims; ++a) {
    if (!supported_n(d->n[a]))
      return fail(nullptr, GPE_ERR_UNSUPPORTED,
                  "axis length " + std::to_string(d->n[a]) +
                      " has no FFT plan (supported: even 2^a*3^b in 8..1024: 8 12 16 24 32 48 64 96 128 192 "
                      "256 384 512 768 1024)");
    if (!(d->dx[a] > 0) || !std::isfinite(d->dx[a]) || !std::isfinite(d->span[a]))
      return fail(nullptr, GPE_ERR_INVALID, "dx must be positive and finite");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return fail(nullptr, GPE_ERR_NO_DEVICE, "no CUDA device");
  if (d->device < 0 || d->device >= ndev) return fail(nullptr, GPE_ERR_INVALID, "device ordinal out of range");
  int maj = 0, min = 0;
  cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, d->device);
  cudaDeviceGetAttribute(&min, cudaDevAttrComputeCapabilityMinor, d->device);
  if (!(maj == 10 && min == 3))
    return fail(nullptr, GPE_ERR_NO_DEVICE,
                "libgpe is built for sm_103a (GB300); device is sm_" + std::to_string(maj * 10 + min));
  c = new gpe_ctx();
  c->ncomp = ncomp;
  c->device = d->device;
  c->ndims = d->ndims;
  for (int a = 0; a < 3; ++a) {
    c->n[a] = (a < d->ndims) ? d->n[a] : 1;
    c->dx[a] = (a < d->ndims) ? d->dx[a] : 1.0;
    c->span[a] = (a < d->ndims) ? d->span[a] : 0.0;
  }
  c->P = (long long)c->n[0] * c->n[1] * c->n[2];
  c->PS = c->P * c->ncomp;
  c->weight = c->dx[0] * c->dx[1] * (d->ndims == 3 ? c->dx[2] : 1.0);  // init.m:36, grid3d/init.m:83
  c->prec = d->precision;
  gpe_default_params(&c->prm);
  c->main.prec = c->prec;
  auto cleanup = [&](gpe_status st) {
    std::string m = c->err;
    gpe_destroy(c);
    return fail(nullptr, st, m);
  };
  if (cudaSetDevice(c->device) != cudaSuccess) return cleanup(GPE_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    c->err = "cudaStreamCreate failed";
    return cleanup(GPE_ERR_CUDA);
  }
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
  if (c->sms <= 0) c->sms = 152;
  // GPE_PDL=0|1: launch the direct passes with programmatic dependent launch.
  if (const char* e = getenv("GPE_PDL")) c->pdl = atoi(e) != 0;
  // GPE_NVTX=1: a host NVTX range (named by the kernel class) around every launch.
  if (const char* e = getenv("GPE_NVTX")) c->nvtx = atoi(e) != 0;
  // GPE_AUTOTUNE=0|1|2 sets the initial autotuner mode (gpe_autotune) of new contexts.
  if (const char* e = getenv("GPE_AUTOTUNE")) {
    const int m = atoi(e);
    if (m >= 0 && m <= 2) c->tune_mode = m;
  }
  // partial-sum capacity: the largest grid of any pass in either precision
  // and any plan variant
  long long cap = 8LL * 1024;  // (+ room for the Lz energy partials after the x pass's, array omega)
  for (auto& ap : axis_passes(c)) {
    cap = std::max(cap, pass_blocks<float>(ap, 0));
    if (has_alt_plan(ap.N)) cap = std::max(cap, pass_blocks<float>(ap, 1));
    cap = std::max(cap, pass_blocks<double>(ap, 0));
  }
  c->cap = (int)cap + 8 * c->sms;
  gpe_status st = GPE_OK;
  if (cudaMalloc(&c->partials, (size_t)(NSLOTS + 1) * c->cap * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->sc, sizeof(DevScalars)) != cudaSuccess ||
      cudaMallocHost(&c->sc_host, 2 * sizeof(DevScalars)) != cudaSuccess ||
      cudaMalloc(&c->V64, (size_t)c->PS * sizeof(double)) != cudaSuccess ||
      (ncomp == 2 && cudaMalloc(&c->spin_part, ((size_t)SP_NSUMS * 8 * c->sms + 8) * sizeof(double)) != cudaSuccess)) {
    c->err = "device allocation failed";
    return cleanup(GPE_ERR_ALLOC);
  }
  DevScalars z;
  memset(&z, 0, sizeof(z));
  z.scale = 1.0;
  z.scale2 = 1.0;
  z.best_delta = INFINITY;
  cudaMemcpy(c->sc, &z, sizeof(z), cudaMemcpyHostToDevice);
  if (c->prec == GPE_FP32) st = alloc_field<float>(c, c->main, GPE_FP32, false);
  else st = alloc_field<double>(c, c->main, GPE_FP64, true);
  if (st != GPE_OK) return cleanup(st);
  for (int k = 0; k < 2; ++k) {
    cudaEventCreateWithFlags(&c->ev_V[k], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_sc[k], cudaEventDisableTiming);
    cudaEventRecord(c->ev_V[k], c->stream);
  }
  cudaEventCreate(&c->t0);
  cudaEventCreate(&c->t1);
  c->prof_classes.resize(PC_COUNT);
  for (int k = 0; k < PC_COUNT; ++k) c->prof_classes[k].name = kProfNames[k];
  if (cudaGetLastError() != cudaSuccess) {
    c->err = "CUDA error during context creation";
    return cleanup(GPE_ERR_CUDA);
  }
  *out = c;
  return GPE_OK;
}

gpe_status gpe_create(const gpe_grid_desc* d, gpe_ctx** out) { return create_impl(d, out, 1); }

gpe_status gpe_create_spinor(const gpe_grid_desc* d, gpe_ctx** out) {
  const gpe_status st = create_impl(d, out, 2);
  if (st == GPE_OK) {
    gpe_ctx* c = *out;
    c->spin.g[0] = c->spin.g[1] = c->spin.g[2] = c->spin.g[3] = 0.0;
    c->spin.coupling_re = c->spin.coupling_im = c->spin.nlincpl = 0.0;
  }
  return st;
}

gpe_status gpe_set_spinor_params(gpe_ctx* c, const gpe_spinor_params* p) {
  CHECK(check_ctx(c));
  if (c->ncomp != 2) return fail(c, GPE_ERR_STATE, "gpe_set_spinor_params: not a spinor context");
  if (!p) return fail(c, GPE_ERR_INVALID, "null spinor params");
  for (double v : {p->g[0], p->g[1], p->g[2], p->g[3], p->coupling_re, p->coupling_im, p->nlincpl})
    if (!std::isfinite(v)) return fail(c, GPE_ERR_INVALID, "spinor params must be finite");
  c->spin = *p;
  return GPE_OK;
}

gpe_status gpe_set_omega_field(gpe_ctx* c, const double* omega, int n_crank) {
  CHECK(check_ctx(c));
  if (n_crank < 0) return fail(c, GPE_ERR_INVALID, "set_omega_field: n_crank must be >= 0");
  c->n_crank = n_crank;  // also the rotating SGPE's Crank-Nicolson count
  if (!omega) {
    if (c->omega_field) {
      c->main.phase_valid = false;  // the half-step tables follow the mode
      c->polish.phase_valid = false;
    }
    c->omega_field = false;
    return GPE_OK;
  }
  if (c->ncomp != 1) return fail(c, GPE_ERR_UNSUPPORTED, "set_omega_field: not available on a spinor context");
  c->main.phase_valid = false;
  c->polish.phase_valid = false;
  for (long long i = 0; i < c->P; ++i)
    if (!std::isfinite(omega[i])) return fail(c, GPE_ERR_INVALID, "set_omega_field: omega must be finite");
  if (!c->omf64) CU(cudaMalloc(&c->omf64, (size_t)c->P * sizeof(double)));
  CU(cudaMemcpy(c->omf64, omega, (size_t)c->P * sizeof(double), cudaMemcpyHostToDevice));
  if (c->prec == GPE_FP32) {
    if (!c->omfR) CU(cudaMalloc(&c->omfR, (size_t)c->P * sizeof(float)));
    launch_convert_re<double, float>(c->omf64, (float*)c->omfR, c->P, c->stream);
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(c->stream));
  }
  c->omega_field = true;
  c->n_crank = n_crank;
  return GPE_OK;
}

gpe_status gpe_get_spinor_params(const gpe_ctx* c, gpe_spinor_params* p) {
  if (!c || !p) return fail(nullptr, GPE_ERR_INVALID, "null argument");
  if (c->ncomp != 2) return GPE_ERR_STATE;
  *p = c->spin;
  return GPE_OK;
}

void gpe_destroy(gpe_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_field(c->main, c->V64);
  free_field(c->polish, c->V64);
  cudaFree(c->V64);
  cudaFree(c->Vmu);
  cudaFree(c->VmuR);
  cudaFree(c->spin_part);
  cudaFree(c->obs_buf);
  cudaFree(c->omf64);
  cudaFree(c->omfR);
  cudaFree(c->partials);
  cudaFree(c->sc);
  cudaFree(c->d_hist);
  if (c->sc_host) cudaFreeHost(c->sc_host);
  for (int k = 0; k < 2; ++k) {
    if (c->pinned_V[k]) cudaFreeHost(c->pinned_V[k]);
    if (c->ev_V[k]) cudaEventDestroy(c->ev_V[k]);
    if (c->ev_sc[k]) cudaEventDestroy(c->ev_sc[k]);
  }
  for (auto& r : c->prof_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  for (int k = 0; k < 2; ++k) {
    if (c->aux[k]) cudaStreamDestroy(c->aux[k]);
    if (c->ev_join[k]) cudaEventDestroy(c->ev_join[k]);
  }
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

gpe_status gpe_set_params(gpe_ctx* c, const gpe_params* p) {
  CHECK(check_ctx(c));
  if (!p) return fail(c, GPE_ERR_INVALID, "null params");
  if (p->n_recalc < 1) return fail(c, GPE_ERR_INVALID, "n_recalc must be >= 1");
  if (p->itp_max_iter < 1) return fail(c, GPE_ERR_INVALID, "itp_max_iter must be >= 1");
  if (p->itp_min_iter < 0) return fail(c, GPE_ERR_INVALID, "itp_min_iter must be >= 0");
  if (!std::isfinite(p->g) || !std::isfinite(p->gamma) || !std::isfinite(p->Ntotal) ||
      !std::isfinite(p->mu_init) || !std::isfinite(p->decay_rate) || p->gamma < 0 || !std::isfinite(p->omega))
    return fail(c, GPE_ERR_INVALID, "parameters must be finite, gamma >= 0");
  if (p->omega != c->prm.omega) {  // the kinetic factors and rotation tables depend on omega
    c->main.phase_valid = false;
    c->polish.phase_valid = false;
  }
  c->prm = *p;
  return GPE_OK;
}

gpe_status gpe_get_params(const gpe_ctx* c, gpe_params* p) {
  if (!c || !p) return GPE_ERR_INVALID;
  *p = c->prm;
  return GPE_OK;
}

gpe_status gpe_get_current(const gpe_ctx* c, gpe_current* cur) {
  if (!c || !cur) return GPE_ERR_INVALID;
  *cur = c->cur;
  return GPE_OK;
}

gpe_status gpe_set_current(gpe_ctx* c, const gpe_current* cur) {
  CHECK(check_ctx(c));
  if (!cur || cur->current_iter < 0) return fail(c, GPE_ERR_INVALID, "invalid current");
  c->cur = *cur;
  return GPE_OK;
}

gpe_status gpe_get_history(const gpe_ctx* c, double* mu, double* n, int cap, int* len) {
  if (!c) return GPE_ERR_INVALID;
  const int L = (int)c->hist_mu.size();
  if (len) *len = L;
  for (int k = 0; k < std::min(L, cap); ++k) {
    if (mu) mu[k] = c->hist_mu[k];
    if (n) n[k] = c->hist_n[k];
  }
  return GPE_OK;
}

gpe_status gpe_get_history_energy(const gpe_ctx* c, double* E, int cap, int* len) {
  if (!c) return GPE_ERR_INVALID;
  const int L = (int)c->hist_mu.size();
  if (len) *len = L;
  for (int k = 0; k < std::min(L, cap); ++k)
    if (E) E[k] = k < (int)c->hist_e.size() ? c->hist_e[k] : NAN;
  return GPE_OK;
}

gpe_status gpe_clear_history(gpe_ctx* c) {
  CHECK(check_ctx(c));
  c->hist_mu.clear();
  c->hist_n.clear();
  c->hist_e.clear();
  return GPE_OK;
}

gpe_status gpe_set_potential(gpe_ctx* c, const double* V) {
  CHECK(check_ctx(c));
  if (!V) return fail(c, GPE_ERR_INVALID, "null potential");
  if (c->prec == GPE_FP32) CHECK(upload_V_double<float>(c, V, false));
  else CHECK(upload_V_double<double>(c, V, false));
  c->have_V = true;
  return GPE_OK;
}

gpe_status gpe_set_potential_f32(gpe_ctx* c, const float* V) {
  CHECK(check_ctx(c));
  if (!V) return fail(c, GPE_ERR_INVALID, "null potential");
  std::vector<double> tmp(V, V + c->PS);
  return gpe_set_potential(c, tmp.data());
}

static gpe_status set_state_any(gpe_ctx* c, const void* src, int src_prec, cudaMemcpyKind kind) {
  CHECK(check_ctx(c));
  if (!src) return fail(c, GPE_ERR_INVALID, "null state");
  const size_t n = (size_t)c->PS;
  if (src_prec == c->prec) {
    CU(cudaMemcpyAsync(c->main.psi, src, n * 2 * (src_prec == GPE_FP32 ? 4 : 8), kind, c->stream));
  } else {
    void* io = nullptr;
    CHECK(io_buffer(c, &io));
    CU(cudaMemcpyAsync(io, src, n * 2 * (src_prec == GPE_FP32 ? 4 : 8), kind, c->stream));
    if (src_prec == GPE_FP64)
      launch_convert_cx<double, float>((const cx<double>*)io, (cx<float>*)c->main.psi, c->PS, nullptr, c->stream);
    else
      launch_convert_cx<float, double>((const cx<float>*)io, (cx<double>*)c->main.psi, c->PS, nullptr, c->stream);
    c->launches++;
    CU(cudaStreamSynchronize(c->stream));
    if (io != c->polish.psi) cudaFree(io);
  }
  launch_set_scale_one(c->sc, c->stream);
  c->launches++;
  CU(cudaStreamSynchronize(c->stream));
  c->have_state = true;
  return GPE_OK;
}

static gpe_status get_state_any(gpe_ctx* c, void* dst, int dst_prec, cudaMemcpyKind kind) {
  CHECK(check_ctx(c));
  CHECK(need_state(c));
  if (!dst) return fail(c, GPE_ERR_INVALID, "null output");
  const size_t n = (size_t)c->PS;
  if (c->prec == GPE_FP32) CHECK(materialize<float>(c));
  else CHECK(materialize<double>(c));
  if (dst_prec == c->prec) {
    CU(cudaMemcpyAsync(dst, c->main.psi, n * 2 * (dst_prec == GPE_FP32 ? 4 : 8), kind, c->stream));
    CU(cudaStreamSynchronize(c->stream));
  } else {
    void* io = nullptr;
    CHECK(io_buffer(c, &io));
    if (dst_prec == GPE_FP64)
      launch_convert_cx<float, double>((const cx<float>*)c->main.psi, (cx<double>*)io, c->PS, nullptr, c->stream);
    else
      launch_convert_cx<double, float>((const cx<double>*)c->main.psi, (cx<float>*)io, c->PS, nullptr, c->stream);
    c->launches++;
    CU(cudaMemcpyAsync(dst, io, n * 2 * (dst_prec == GPE_FP32 ? 4 : 8), kind, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (io != c->polish.psi) cudaFree(io);
  }
  return GPE_OK;
}

gpe_status gpe_set_state(gpe_ctx* c, const double* psi) {
  return set_state_any(c, psi, GPE_FP64, cudaMemcpyHostToDevice);
}
gpe_status gpe_set_state_f32(gpe_ctx* c, const float* psi) {
  return set_state_any(c, psi, GPE_FP32, cudaMemcpyHostToDevice);
}
gpe_status gpe_get_state(gpe_ctx* c, double* psi) {
  return get_state_any(c, psi, GPE_FP64, cudaMemcpyDeviceToHost);
}
gpe_status gpe_get_state_f32(gpe_ctx* c, float* psi) {
  return get_state_any(c, psi, GPE_FP32, cudaMemcpyDeviceToHost);
}
gpe_status gpe_set_state_device(gpe_ctx* c, const void* d, int precision) {
  if (precision != GPE_FP32 && precision != GPE_FP64) return fail(c, GPE_ERR_INVALID, "bad precision");
  return set_state_any(c, d, precision, cudaMemcpyDeviceToDevice);
}
gpe_status gpe_get_state_device(gpe_ctx* c, void* d, int precision) {
  if (precision != GPE_FP32 && precision != GPE_FP64) return fail(c, GPE_ERR_INVALID, "bad precision");
  return get_state_any(c, d, precision, cudaMemcpyDeviceToDevice);
}

gpe_status gpe_groundstate_itp(gpe_ctx* c, const gpe_itp_params* prm, double* MU, double* MU2, double* EE,
                               int cap, gpe_itp_result* res) {
  CHECK(check_ctx(c));
  CHECK(need_state(c));
  CHECK(need_V(c));
  if (!prm || !(prm->dt > 0) || !std::isfinite(prm->dt) || !(prm->eps > 0))
    return fail(c, GPE_ERR_INVALID, "groundstate_itp: dt and eps must be positive");
  if (cap < 0) return fail(c, GPE_ERR_INVALID, "negative cap");
  if (c->ncomp == 2) {
    if (c->prm.omega != 0.0 && c->ndims != 2)
      return fail(c, GPE_ERR_UNSUPPORTED,
                  "groundstate_itp (spinor): omega != 0 in 3D (the reference's rotating branch has no z kinetic factor)");
    c->err.clear();
    if (c->prec == GPE_FP32) return spinor_itp_impl<float>(c, prm, MU, MU2, EE, cap, res);
    return spinor_itp_impl<double>(c, prm, MU, MU2, EE, cap, res);
  }
  if (c->omega_field && c->prm.omega != 0.0)
    return fail(c, GPE_ERR_INVALID, "omega is either a scalar (gpe_params.omega) or an array (gpe_set_omega_field)");
  c->err.clear();
  CHECK(maybe_autotune(c));
  if (c->prec == GPE_FP32) return itp_impl<float>(c, prm, MU, MU2, EE, cap, res);
  return itp_impl<double>(c, prm, MU, MU2, EE, cap, res);
}

gpe_status gpe_groundstate_itp_2comp(gpe_ctx* c, const gpe_itp_params* prm, double N1, double N2, double M1,
                                     double M2, double* MU1, double* MU2, double* EE, int cap,
                                     gpe_itp_result* res) {
  CHECK(check_ctx(c));
  if (c->ncomp != 2) return fail(c, GPE_ERR_UNSUPPORTED, "groundstate_itp (2comp): needs a two-component context");
  CHECK(need_state(c));
  CHECK(need_V(c));
  if (!prm || !(prm->dt > 0) || !std::isfinite(prm->dt) || !(prm->eps > 0))
    return fail(c, GPE_ERR_INVALID, "groundstate_itp: dt and eps must be positive");
  if (cap < 0) return fail(c, GPE_ERR_INVALID, "negative cap");
  if (c->prm.omega != 0.0 && c->ndims != 2)
    return fail(c, GPE_ERR_UNSUPPORTED,
                "groundstate_itp (2comp): omega != 0 in 3D (the reference's rotating branch has no z kinetic factor)");
  c->err.clear();
  if (c->prec == GPE_FP32) return mix_itp_impl<float>(c, prm, N1, N2, M1, M2, MU1, MU2, EE, cap, res);
  return mix_itp_impl<double>(c, prm, N1, N2, M1, M2, MU1, MU2, EE, cap, res);
}

gpe_status gpe_solve_split(gpe_ctx* c, const gpe_split_params* prm) {
  CHECK(check_ctx(c));
  CHECK(need_state(c));
  if (!prm || !(prm->ddt > 0) || !std::isfinite(prm->ddt))
    return fail(c, GPE_ERR_INVALID, "solve_split: ddt must be positive");
  if (!prm->vtd) CHECK(need_V(c));
  if (c->omega_field && c->prm.omega != 0.0)
    return fail(c, GPE_ERR_INVALID, "omega is either a scalar (gpe_params.omega) or an array (gpe_set_omega_field)");
  c->err.clear();
  if (c->ncomp == 2) {
    if (c->prec == GPE_FP32) return spinor_split_impl<float>(c, prm);
    return spinor_split_impl<double>(c, prm);
  }
  CHECK(maybe_autotune(c));
  // Small 2D grids: the persistent cluster kernel (any callbacks but Vtd).
  if (!prm->vtd) {
    std::vector<gpe_ctx*> one{c};
    bool used = false;
    const gpe_status st = cluster_run(one, prm, &used);
    if (used) return st;
  }
  // Small grids are launch-bound: run their blocks as replayed CUDA graphs
  // (the batched path with one context) when no per-block host work is
  // needed (no Vtd or outer-step callback, no decay target) and no per-launch
  // profiling events are requested.
  if (!prm->vtd && !prm->on_step && !(c->prm.decay_rate > 0) && !c->prof && c->P <= (1LL << 20)) {
    std::vector<gpe_ctx*> one{c};
    return batch_impl(one, prm);
  }
  if (c->prec == GPE_FP32) return split_impl<float>(c, prm);
  return split_impl<double>(c, prm);
}

gpe_status gpe_adjoint_grad(gpe_ctx* c, const gpe_adjoint_params* prm, const double* psi_target, double* dLdV,
                            double* loss) {
  CHECK(check_ctx(c));
  if (c->ncomp != 1) return fail(c, GPE_ERR_UNSUPPORTED, "adjoint_grad: not available on a spinor context");
  CHECK(need_state(c));
  CHECK(need_V(c));
  if (!prm || !psi_target || !dLdV) return fail(c, GPE_ERR_INVALID, "adjoint: null argument");
  if (!(prm->ddt > 0) || prm->nsteps < 1) return fail(c, GPE_ERR_INVALID, "adjoint: ddt > 0 and nsteps >= 1 needed");
  if (c->prm.gamma != 0.0 || c->prm.decay_rate > 0)
    return fail(c, GPE_ERR_UNSUPPORTED,
                "adjoint: only gamma = 0 and decay_rate = 0 (conservative dynamics) are differentiated");
  if (c->prm.omega != 0.0 || c->omega_field)
    return fail(c, GPE_ERR_UNSUPPORTED, "adjoint: the rotating frame is not differentiated");
  const int prec = prm->precision ? prm->precision : c->prec;
  if (prec != GPE_FP32 && prec != GPE_FP64) return fail(c, GPE_ERR_INVALID, "adjoint: precision must be 0, GPE_FP32 or GPE_FP64");
  if (prec == GPE_FP32 && c->prec == GPE_FP64)
    return fail(c, GPE_ERR_UNSUPPORTED, "adjoint: an FP64 context has no FP32 tables; use precision 0");
  c->err.clear();
  CHECK(maybe_autotune(c));
  if (prec == GPE_FP32) return adjoint_impl<float>(c, c->main, prm, psi_target, dLdV, loss);
  if (c->prec == GPE_FP32) {
    CHECK(ensure_polish(c));
    return adjoint_impl<double>(c, c->polish, prm, psi_target, dLdV, loss);
  }
  return adjoint_impl<double>(c, c->main, prm, psi_target, dLdV, loss);
}

gpe_status gpe_solve_split_batch(gpe_ctx** ctxs, int count, const gpe_split_params* prm) {
  if (!ctxs || count < 1 || !ctxs[0]) return fail(nullptr, GPE_ERR_INVALID, "solve_split_batch: no contexts");
  gpe_ctx* c = ctxs[0];
  CHECK(check_ctx(c));
  if (!prm || !(prm->ddt > 0) || !std::isfinite(prm->ddt))
    return fail(c, GPE_ERR_INVALID, "solve_split_batch: ddt must be positive");
  if (prm->vtd || prm->on_step)
    return fail(c, GPE_ERR_INVALID, "solve_split_batch: per-block host callbacks are not supported in batches");
  std::vector<gpe_ctx*> cs;
  for (int i = 0; i < count; ++i) {
    gpe_ctx* ci = ctxs[i];
    if (!ci) return fail(c, GPE_ERR_INVALID, "solve_split_batch: null context");
    if (ci->device != c->device) return fail(c, GPE_ERR_INVALID, "solve_split_batch: contexts on different devices");
    if (!ci->have_state || !ci->have_V) return fail(c, GPE_ERR_STATE, "solve_split_batch: a context lacks state or V");
    if (ci->ncomp != 1) return fail(c, GPE_ERR_UNSUPPORTED, "solve_split_batch: spinor contexts are not batched");
    if (ci->prm.decay_rate > 0)
      return fail(c, GPE_ERR_INVALID, "solve_split_batch: decay_rate > 0 needs per-block host times");
    for (auto* cj : cs)
      if (cj == ci) return fail(c, GPE_ERR_INVALID, "solve_split_batch: a context appears twice");
    cs.push_back(ci);
  }
  c->err.clear();
  {
    bool used = false;
    const gpe_status st = cluster_run(cs, prm, &used);
    if (used) return st;
  }
  // Batched contexts are tuned whatever their size (one timing per distinct
  // grid shape), before any graph is captured.
  for (auto* ci : cs) {
    if (ci->tuned || ci->tune_mode != 2 || ci->prec != GPE_FP32 || ci->pass_variant == 1) continue;
    int chosen[3];
    if (autotune_main(ci, chosen) != GPE_OK) return fail(c, GPE_ERR_CUDA, "solve_split_batch: autotune: " + ci->err);
  }
  return batch_impl(cs, prm);
}

gpe_status gpe_autotune(gpe_ctx* c, int mode, int* chosen) {
  CHECK(check_ctx(c));
  if (c->ncomp != 1) return fail(c, GPE_ERR_UNSUPPORTED, "autotune: not available on a spinor context");
  if (mode < 0 || (mode > 5 && (mode < 16 || mode > 23) && (mode < 32 || mode > 39) && (mode < 48 || mode > 55)))
    return fail(c, GPE_ERR_INVALID,
                "autotune mode must be 0 (off), 1 (now), 2 (auto), 3 (alternative plans), 4 (paired passes on the "
                "alternative plans), 5 (paired passes on the default plans), or 16 / 32 / 48 + axis mask");
  int ch[3] = {-1, -1, -1};
  if (mode == 0 || mode == 3 || mode == 4 || mode == 5 || mode >= 16) {
    // fixed plans: the defaults, the alternative wherever one exists (3),
    // the paired passes on the alternative (4) or on the default plan (5)
    // wherever they exist, or the alternative (16 + mask), paired on the
    // alternative (32 + mask), paired on the default (48 + mask) on the
    // axes of the bit mask (bit 0 = x) (FP32)
    const int mask = (mode >= 3 && mode <= 5) ? 7 : (mode & 15) & 7;
    const int var = (mode == 5 || mode >= 48) ? 3 : (mode == 4 || mode >= 32) ? 2 : 1;
    c->tune_mode = mode == 0 ? 0 : 1;
    c->tuned = mode != 0;
    for (int ax = 0; ax < c->ndims; ++ax) {
      const bool has = var == 3 ? has_x2d_plan(c->n[ax]) : has_alt_plan(c->n[ax]);
      const int v = ((mask >> ax) & 1) && c->prec == GPE_FP32 && has ? var : 0;
      if (c->main.plan_var[ax] == v) continue;
      c->main.plan_var[ax] = v;
      if (c->prec == GPE_FP32) CHECK(build_axis_tables<float>(c, c->main, ax));
      else CHECK(build_axis_tables<double>(c, c->main, ax));
    }
    c->main.phase_valid = false;
  } else if (mode == 1) {
    c->tune_mode = 1;
    CHECK(autotune_main(c, ch));
  } else {
    c->tune_mode = 2;
  }
  if (chosen)
    for (int ax = 0; ax < 3; ++ax)
      chosen[ax] = (mode == 1) ? ch[ax] : (ax < c->ndims && has_alt_plan(c->n[ax]) ? c->main.plan_var[ax] : -1);
  return GPE_OK;
}

gpe_status gpe_observables(gpe_ctx* c, gpe_obs* o) {
  CHECK(check_ctx(c));
  CHECK(need_state(c));
  CHECK(need_V(c));
  if (!o) return fail(c, GPE_ERR_INVALID, "null output");
  o->ecpl = 0.0;
  if (c->ncomp == 2) {
    if (c->prec == GPE_FP32) return spinor_observables<float>(c, o);
    return spinor_observables<double>(c, o);
  }
  CHECK(maybe_autotune(c));
  DevScalars h;
  if (c->prec == GPE_FP32) CHECK(observables_impl<float>(c, c->main, 0.0, 0, &h));
  else CHECK(observables_impl<double>(c, c->main, 0.0, 0, &h));
  o->norm = h.sums[S_N];
  o->ekin = h.sums[S_KX] + h.sums[S_KY] + h.sums[S_KZ];
  o->epot = h.sums[S_VN];
  o->eint = c->prm.g * h.sums[S_N2];
  o->mu_integral = o->ekin + o->epot + o->eint;
  o->energy = o->ekin + o->epot + 0.5 * o->eint;
  return GPE_OK;
}

gpe_status gpe_detect_core(gpe_ctx* c, int component, int z_index, int refine, double* pos, int cap_pos,
                           int* n_pos, double* neg, int cap_neg, int* n_neg) {
  CHECK(check_ctx(c));
  CHECK(need_state(c));
  if (!n_pos || !n_neg || cap_pos < 0 || cap_neg < 0 || (cap_pos > 0 && !pos) || (cap_neg > 0 && !neg))
    return fail(c, GPE_ERR_INVALID, "detect_core: bad output arguments");
  if (component < 0 || component >= c->ncomp) return fail(c, GPE_ERR_INVALID, "detect_core: bad component");
  const int nz = c->ndims == 3 ? c->n[2] : 1;
  if (z_index < 0 || z_index >= nz) return fail(c, GPE_ERR_INVALID, "detect_core: z_index out of range");
  if (c->prec == GPE_FP32)
    return detect_core_impl<float>(c, component, z_index, refine, pos, cap_pos, n_pos, neg, cap_neg, n_neg);
  return detect_core_impl<double>(c, component, z_index, refine, pos, cap_pos, n_pos, neg, cap_neg, n_neg);
}

gpe_status gpe_groundstate_tf(gpe_ctx* c, double eps, double N, const double* bounds, double* mu) {
  CHECK(check_ctx(c));
  if (c->ncomp != 1) return fail(c, GPE_ERR_UNSUPPORTED, "groundstate_tf: not available on a spinor context");
  CHECK(need_V(c));
  if (!mu || !(eps > 0) || !std::isfinite(N)) return fail(c, GPE_ERR_INVALID, "groundstate_tf: bad arguments");
  if (!(c->prm.g > 0)) return fail(c, GPE_ERR_INVALID, "groundstate_tf: g must be positive (phi = sqrt(vvv/g))");
  if (bounds && !(bounds[0] < bounds[1])) return fail(c, GPE_ERR_INVALID, "groundstate_tf: need mul < mur");
  c->err.clear();
  if (c->prec == GPE_FP32) return groundstate_tf_impl<float>(c, eps, N, bounds, mu);
  return groundstate_tf_impl<double>(c, eps, N, bounds, mu);
}

gpe_status gpe_synchronize(gpe_ctx* c) {
  CHECK(check_ctx(c));
  CU(cudaStreamSynchronize(c->stream));
  return GPE_OK;
}

gpe_status gpe_timer_start(gpe_ctx* c) {
  CHECK(check_ctx(c));
  CU(cudaStreamSynchronize(c->stream));
  CU(cudaEventRecord(c->t0, c->stream));
  return GPE_OK;
}

gpe_status gpe_timer_stop(gpe_ctx* c, double* ms) {
  CHECK(check_ctx(c));
  CU(cudaEventRecord(c->t1, c->stream));
  CU(cudaEventSynchronize(c->t1));
  float f = 0;
  CU(cudaEventElapsedTime(&f, c->t0, c->t1));
  if (ms) *ms = f;
  return GPE_OK;
}

gpe_status gpe_profile_enable(gpe_ctx* c, int on) {
  CHECK(check_ctx(c));
  c->prof = on != 0;
  return GPE_OK;
}

gpe_status gpe_profile_read(gpe_ctx* c, gpe_kernel_stat* out, int cap, int* n) {
  CHECK(check_ctx(c));
  CU(cudaStreamSynchronize(c->stream));
  for (auto& r : c->prof_pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, r.a, r.b);
    c->prof_classes[r.cls].launches++;
    c->prof_classes[r.cls].total_ms += ms;
    c->ev_pool.push_back(r.a);
    c->ev_pool.push_back(r.b);
  }
  c->prof_pending.clear();
  int k = 0;
  for (auto& pc : c->prof_classes) {
    if (pc.launches == 0) continue;
    if (out && k < cap) {
      memset(&out[k], 0, sizeof(gpe_kernel_stat));
      snprintf(out[k].name, sizeof(out[k].name), "%s", pc.name.c_str());
      out[k].launches = pc.launches;
      out[k].total_ms = pc.total_ms;
      out[k].bytes_per_launch = pc.bytes / (double)pc.launches;
    }
    ++k;
  }
  if (n) *n = k;
  return GPE_OK;
}

long long gpe_kernel_launches(const gpe_ctx* c) { return c ? c->launches : 0; }

gpe_status gpe_selftest_trig(const float* x, float* s, float* co, long long n) {
  gpe_ctx* c = nullptr;
  if (!x || !s || !co || n <= 0) return fail(c, GPE_ERR_INVALID, "gpe_selftest_trig: bad arguments");
  float* d = nullptr;
  CU(cudaMalloc(&d, 3 * (size_t)n * sizeof(float)));
  cudaError_t e = cudaMemcpy(d, x, n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_selftest_trig(d, d + n, d + 2 * n, n, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(s, d + n, n * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(co, d + 2 * n, n * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(c, GPE_ERR_CUDA, std::string("gpe_selftest_trig: ") + cudaGetErrorString(e));
  return GPE_OK;
}

gpe_status gpe_selftest_noise(unsigned long long seed, unsigned long long step, long long n, float* out) {
  gpe_ctx* c = nullptr;
  if (!out || n <= 0) return fail(c, GPE_ERR_INVALID, "gpe_selftest_noise: bad arguments");
  float* d = nullptr;
  CU(cudaMalloc(&d, 2 * (size_t)n * sizeof(float)));
  cudaError_t e = launch_selftest_noise(d, n, seed, step, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(out, d, 2 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(c, GPE_ERR_CUDA, std::string("gpe_selftest_noise: ") + cudaGetErrorString(e));
  return GPE_OK;
}

gpe_status gpe_solve_sgpe(gpe_ctx* c, const gpe_split_params* prm, const gpe_sgpe_params* sg) {
  CHECK(check_ctx(c));
  if (c->ncomp != 1) return fail(c, GPE_ERR_UNSUPPORTED, "solve_sgpe: not available on a spinor context");
  CHECK(need_state(c));
  if (!prm || !sg || !(prm->ddt > 0) || !std::isfinite(prm->ddt))
    return fail(c, GPE_ERR_INVALID, "solve_sgpe: ddt must be positive");
  if (!(sg->T >= 0) || !std::isfinite(sg->T) || !(sg->ecut >= 0))
    return fail(c, GPE_ERR_INVALID, "solve_sgpe: T and ecut must be >= 0");
  if (c->omega_field)
    return fail(c, GPE_ERR_UNSUPPORTED, "solve_sgpe: an omega array (the reference's SGPE takes a scalar omega)");
  if (!prm->vtd) CHECK(need_V(c));
  c->err.clear();
  CHECK(maybe_autotune(c));
  // The SGPE's kinetic factor is exp(-kk dt) whatever omega is (solve_split.m:
  // 40-45); a scalar omega acts through the Lz step only.  The kinetic tables
  // are rebuilt on entry and exit when the rotating-frame ones differ.
  struct AdiOff {
    gpe_ctx* c;
    bool on;
    AdiOff(gpe_ctx* cc) : c(cc), on(cc->prm.omega != 0.0) {
      if (on) {
        c->adi_off = true;
        c->main.phase_valid = false;
      }
    }
    ~AdiOff() {
      if (on) {
        c->adi_off = false;
        c->main.phase_valid = false;
      }
    }
  } guard(c);
  if (c->prec == GPE_FP32) return split_impl<float>(c, prm, sg);
  return split_impl<double>(c, prm, sg);
}

gpe_status gpe_set_pass_variant(gpe_ctx* c, int variant) {
  CHECK(check_ctx(c));
  if (variant < 0 || variant > 2)
    return fail(c, GPE_ERR_INVALID, "pass variant must be 0 (direct + L2 prefetch), 1 (TMA) or 2 (direct)");
  c->pass_variant = variant;
  return GPE_OK;
}

gpe_status gpe_host_register(void* ptr, size_t bytes) {
  gpe_ctx* c = nullptr;
  if (!ptr || bytes == 0) return fail(c, GPE_ERR_INVALID, "gpe_host_register: null or empty buffer");
  CU(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return GPE_OK;
}

gpe_status gpe_host_unregister(void* ptr) {
  gpe_ctx* c = nullptr;
  if (!ptr) return fail(c, GPE_ERR_INVALID, "gpe_host_unregister: null buffer");
  CU(cudaHostUnregister(ptr));
  return GPE_OK;
}

}  // extern "C"

namespace gpe {
// Lets the context-free entry point (noalloc.cu) report through
// gpe_last_error(NULL).
void set_thread_error(const std::string& msg) { g_create_err = msg; }
}  // namespace gpe

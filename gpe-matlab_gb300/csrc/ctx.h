// ctx.h - the solver context behind the gpe_ctx handle of include/gpe.h.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gpe.h"
#include "aux_kernels.cuh"
#include "pass.cuh"

namespace gpe {

// Device arrays of one precision (the context's own, or the FP64 polish
// copy of an FP32 context).
struct Field {
  int prec = 0;             // GPE_FP32 / GPE_FP64
  void* psi = nullptr;      // P complex
  void* V = nullptr;        // P real
  void* aux = nullptr;      // P real: ITP nonlinear factor
  void* absprev = nullptr;  // P real: |psi| at the previous ITP check
  void* tws[3] = {nullptr, nullptr, nullptr};    // per axis: stage twiddle rows
  void* php[3] = {nullptr, nullptr, nullptr};    // per axis: permuted kinetic factor, N complex
  void* k2p[3] = {nullptr, nullptr, nullptr};    // per axis: permuted k^2/2/N, N real
  double phase_dt[2] = {0.0, 0.0};               // dt the phase tables hold
  bool phase_valid = false;
  bool V_valid = false;
  int plan_var[3] = {0, 0, 0};                   // per axis: FFT plan variant (plans.cuh PlanSel)
  // Rotating frame (scalar omega): per axis x (0) and y (1)
  void* kp[3] = {nullptr, nullptr, nullptr};     // permuted k/N, N real (energy weights)
  void* rot[2] = {nullptr, nullptr};             // [transverse index][slot] complex factors of the step
  void* rotw[2] = {nullptr, nullptr};            // per transverse index: -omega*y (x) / +omega*x (y)
  double rotw_omega = 0.0;                       // omega the rotw arrays hold
  void* kks[3] = {nullptr, nullptr, nullptr};    // per axis: permuted k^2/2, N real (energy cut-off)
  void* php2[3] = {nullptr, nullptr, nullptr};   // spinor, array omega: the kinetic factors of half a step
  void* php2b[3] = {nullptr, nullptr, nullptr};  // two-component ITP with M2 != M1: component 2's half-step factors
  // Rotating two-component ITPs: per table set (component mass) the x and y
  // half-step factors and their rotation tables (x: [y][slot], y: [x][slot]).
  void* rth[2][4] = {{nullptr, nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr, nullptr}};
  void* cn[2] = {nullptr, nullptr};              // array omega: Crank-Nicolson iterates (P complex each)
};

struct ProfRec {
  int cls;
  cudaEvent_t a, b;
};

struct ProfClass {
  std::string name;
  long long launches = 0;
  double total_ms = 0.0;
  double bytes = 0.0;
};

}  // namespace gpe

struct gpe_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int ndims = 2;
  int n[3] = {1, 1, 1};  // nx, ny, nz
  double dx[3] = {1, 1, 1}, span[3] = {1, 1, 1};
  long long P = 0;
  // Components of the state (1; 2 for a spinor context).  State, potential
  // and their staging buffers hold PS = ncomp*P points, component after
  // component; the axis passes run over all components in one launch.
  int ncomp = 1;
  long long PS = 0;
  gpe_spinor_params spin{};
  double* Vmu = nullptr;  // spinor with a time-dependent V: getVtotal(current_time) (FP64 copy)
  void* VmuR = nullptr;   // the same in the context precision
  double* spin_part = nullptr;  // spinor sums: [SP_NSUMS][grid] partials, then 8 observables
  void* obs_buf = nullptr;      // scratch of the on-device observables (vortex-core detection)
  // Array omega (ssft_kin_step.m:3-11): omega per grid point, FP64 and the
  // context precision, and the Crank-Nicolson iteration count n_crank.
  bool omega_field = false;
  bool adi_off = false;   // rotating SGPE run: scalar omega drives only its Lz step, not the ADI kinetic factors
  bool lz_scalar = false; // rotating spinor ITP: energies add -omega <psi|lz psi> with grid1d's stencil lz
  double* omf64 = nullptr;
  void* omfR = nullptr;
  int n_crank = 3;
  size_t obs_len = 0;
  double weight = 1.0;
  int prec = GPE_FP64;
  gpe_params prm{};
  gpe_current cur{};
  std::vector<double> hist_mu, hist_n, hist_e;

  gpe::Field main, polish;  // polish: FP64 field of an FP32 context
  double* V64 = nullptr;    // FP64 copy of V (upload staging; polish potential)
  bool have_V = false, have_state = false;
  double* partials = nullptr;
  int cap = 0;
  gpe::DevScalars* sc = nullptr;      // device
  gpe::DevScalars* sc_host = nullptr; // pinned, 2 slots
  double* d_hist = nullptr;           // device history scratch
  size_t d_hist_len = 0;
  double* pinned_V[2] = {nullptr, nullptr};
  cudaEvent_t ev_V[2] = {nullptr, nullptr};
  cudaEvent_t ev_sc[2] = {nullptr, nullptr};
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  // Side streams of the block-end energy passes (the three axes' sums run
  // concurrently), created on first use, and their fork/join events.
  cudaStream_t aux[2] = {nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[2] = {nullptr, nullptr};
  std::string err;

  int sms = 152;          // SM count of the device
  int pass_variant = 0;   // 0: direct passes + L2 prefetch, 1: TMA-staged where they apply, 2: direct
  int pdl = 1;            // direct passes: programmatic dependent launch (GPE_PDL=0 turns it off)
  int tune_mode = 2;      // FFT plan autotuner: 0 off, 1 explicit only, 2 on the first hot-path call
  bool tuned = false;     // the autotuner has set main.plan_var
  bool prof = false;
  bool nvtx = false;      // GPE_NVTX=1: an NVTX range around every kernel launch, named by its class
  std::vector<gpe::ProfRec> prof_pending;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<gpe::ProfClass> prof_classes;
  long long launches = 0;
};

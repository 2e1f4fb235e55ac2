// Internal: the C ABI's context (one system on one GPU) and the device
// FIRE2 engine's state, shared by cdft_api.cu and cdft_fire_dev.cu.
#pragma once
#include <array>
#include <cmath>
#include <memory>
#include <string>
#include <vector>
#include "../../include/cdft.h"
#include "cdft_internal.h"

// FMT_Species alias maps (src/FMT_Species.cpp:29-93): rho = dmin + c y^2/(1+y^2).
struct Alias {
  double dmin, c;
};

struct FireDevEngine;  // cdft_fire_dev.cu
struct NewtonWork;     // cdft_newton.cu

// ------------------------------------------------------------- context ---
struct cdft_ctx {
  cdft_params p{};
  cdft_info info{};
  std::string err;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::shared_ptr<cdft::FFTTable> tx, ty, tz;
  std::unique_ptr<cdft::Evaluator<double>> e64;
  std::unique_ptr<cdft::Evaluator<float>> e32;
  int precision = CDFT_FP64;
  double mu = 0, fixed_mass = -1;
  int fixed_bg = 0, homo_bd = 0;  // Species::setFixedBackground / setHomogeneousBoundary
  double* rho = nullptr;
  double* dF = nullptr;
  double* vext = nullptr;
  double* red_part = nullptr;  // map-reduce partials
  double* red_out = nullptr;   // finished values
  double* host_out = nullptr;  // pinned copy of red_out
  // FIRE state (fireMinimizer2 members)
  bool fire_ready = false;
  cdft_fire_params fp{};
  double* fx[2] = {nullptr, nullptr};
  double* fv[2] = {nullptr, nullptr};
  double* fg[2] = {nullptr, nullptr};
  int cur = 0;
  double F = 0, dt = 0, dt_max = 0, alpha = 0, vv = 1, dt_best = 0, fmax = -1, resid = 0, vdotf = 0;
  int Npos = 0, Nneg = 0, backtracks = 0;
  unsigned it = 0;
  long fire_steps = 0, calls = 0;
  // DDFT state
  bool ddft_ready = false;
  double ddft_dt = 0, ddft_dt_max = 1, ddft_tol = 1e-4, ddft_time = 0, ddft_rhs = 1;
  double ddft_mass0 = 0;  // sum rho of the run's start (FP32 mode restores it after each propagation)
  bool ddft_restore = true;   // FP32 mode: shift each propagated density back to ddft_mass0
  double ddft_max_dev = 0;    // FP32 mode: largest |sum rho - mass0| / mass0 of a propagation, before any restore
  bool ddft_have_factors = false;
  int ddft_successes = 0;
  double *dd0 = nullptr, *dd1 = nullptr, *ddn = nullptr, *dR = nullptr, *dfac = nullptr;
  void *rk0 = nullptr, *R0k = nullptr, *R1k = nullptr, *work = nullptr;
  std::vector<double> Lx, Ly, Lz;
  // Graph of the whole grand-canonical evaluation (passes, reductions, copies
  // of the sums to pinned memory), captured on cap_stream and replayed on
  // stream; re-captured when its inputs change (precision, only_fex, the
  // external-field pointer, mu, the transform plans).
  cudaStream_t cap_stream = nullptr;
  // captured evaluation graphs, one per bulk precision (index: precision == CDFT_FP64),
  // with the settings each was captured under
  cudaGraphExec_t eval_exec[2] = {nullptr, nullptr};
  int eg_only_fex[2] = {-1, -1};
  const double* eg_vext[2] = {nullptr, nullptr};
  double eg_mu[2] = {0, 0};
  unsigned plan_gen = 0, eg_plan_gen[2] = {~0u, ~0u};
  double* eg_mirror[2] = {nullptr, nullptr};  // the host dF the graph's final pass also writes
  unsigned* host_status = nullptr;  // pinned
  double last_dF_l2 = 0;            // ||dF||_2 / dV of the last evaluation
  // Hessian-vector product buffers (device, N doubles each; allocated on first use)
  double *hv_v = nullptr, *hv_out = nullptr;
  // device FIRE2 engine (graph-captured steps)
  FireDevEngine* fire_dev = nullptr;
  // Newton-Krylov refinement work arrays
  NewtonWork* newton = nullptr;

  Alias alias() const {
    Alias a;
    a.dmin = 1e-18;  // SMALL_VALUE (include/Density.h:24)
    const double etamin = a.dmin * (4 * M_PI * info.hsd * info.hsd * info.hsd / 3);
    a.c = (1.0 - etamin) / info.dV;
    return a;
  }
};


// helpers shared with cdft_fire_dev.cu
int cdft_internal_fail(cdft_ctx* c, int code, const std::string& m);
int cdft_internal_eval(cdft_ctx* c, double* terms8, int only_fex);
int cdft_internal_fire_accept(cdft_ctx* c, int s_idx);
void cdft_internal_fire_dev_free(cdft_ctx* c);
void cdft_internal_newton_free(cdft_ctx* c);
int cdft_internal_newton_ensure(cdft_ctx* c);
void cdft_internal_newton_save(cdft_ctx* c);
void cdft_internal_newton_restore(cdft_ctx* c);
// FIRE2 state re-derived from the current density: x = alias(rho), v = 0, one evaluation
int cdft_internal_fire_resync(cdft_ctx* c);
// Lattice::is_boundary_point (include/Lattice.h:184-196): the planes i = 0, j = 0, k = 0
__host__ __device__ inline bool cdft_on_boundary(long p, int ny, int nz) {
  const long t = p / nz;
  return p % nz == 0 || t % ny == 0 || t / ny == 0;
}
inline long cdft_n_boundary(int nx, int ny, int nz) { return (long)nx * ny + (long)nx * nz + (long)ny * nz - nx - ny - nz + 1; }
// a[p] = value on the boundary points (device, asynchronous on the context's stream)
void cdft_internal_boundary_set(cdft_ctx* c, double* a, double value);
// y = M x on the device (M: 0 the Hessian, 1 the DDFT matrix g . H; cdft_api.cu)
int cdft_internal_matvec(cdft_ctx* c, int matrix, const double* x, double* y, bool prepare);
// plans cdft_autotune chose for the context's shape, model and precision (cdft_tune.cu)
bool cdft_internal_tuned_plans(const cdft_ctx* c, int precision, std::array<std::vector<int>, 3>* plans);
std::vector<std::vector<int>> cdft_internal_radix_candidates(int n);

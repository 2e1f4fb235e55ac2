// Mixed-precision Newton-Krylov refinement of a minimum (no counterpart in the
// reference, whose minimisers are FIRE2 and DDFT). The residual is an FP64
// evaluation (DFT::calculateFreeEnergyAndDerivatives); each Newton correction
// solves H d = -dF with preconditioned conjugate gradients whose
// Hessian-vector products (DFT::matrix_dot_v_intern, src/DFT.cpp:435-488) run
// in the FP32 bulk precision: the correction only has to be accurate
// relative to itself, so FP32 products suffice, while every accepted state is
// judged by FP64. At fixed mass the system is solved on sum(d) = 0 (the
// constraint Species::setFixedMass imposes) by projecting the operator, the
// right-hand side and the preconditioned residuals. The preconditioner is the
// inverse of the ideal-gas block of H, rho/dV.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "cdft_ctx.h"
#include "cdft_kernels.cuh"

using namespace cdft;

namespace {
constexpr int kT = 256;
unsigned grid_of(long n) { return (unsigned)std::max<long>(1, std::min<long>((n + kT - 1) / kT, 152 * 4)); }

// Block sums of up to 3 values, FP64, one slot per block.
template <int NV>
__device__ void block_store(double* v, double* part) {
  __shared__ double sh[NV][kT / 32];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double x = v[j];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) sh[j][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0;
      for (int w = 0; w < kT / 32; ++w) s += sh[j][w];
      part[blockIdx.x * NV + j] = s;
    }
}

// The CG sums accumulate in FP64: the projections onto sum(d) = 0 subtract
// means of nearly cancelling sums, and FP32 partial sums there left the hardest
// state points of a sweep unconverged. Conversions run on the integer pipes.
__global__ void __launch_bounds__(kT) k_nk_init(const double* dF, float* r, float* dl, long n, double* part) {
  double s = 0;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    const float x = -conv<float>(dF[i]);
    r[i] = x;
    dl[i] = 0.f;
    s += conv<double>(x);
  }
  double v[1] = {s};
  block_store<1>(v, part);
}
__global__ void k_nk_shift(float* x, long n, float c) {
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) x[i] -= c;
}
// z = (rho/dV) r; sums: z
__global__ void __launch_bounds__(kT) k_nk_precond(const float* r, const double* rho, float* z, long n, float idV, double* part) {
  double s = 0;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    const float x = r[i] * conv<float>(rho[i]) * idV;
    z[i] = x;
    s += conv<double>(x);
  }
  double v[1] = {s};
  block_store<1>(v, part);
}
// z -= zshift; sums: r.z, r.r
__global__ void __launch_bounds__(kT) k_nk_rz(const float* r, float* z, long n, float zshift, double* part) {
  double a = 0, b = 0;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    const float zz = z[i] - zshift;
    z[i] = zz;
    const double rd = conv<double>(r[i]);
    a = fma(rd, conv<double>(zz), a);
    b = fma(rd, rd, b);
  }
  double v[2] = {a, b};
  block_store<2>(v, part);
}
__global__ void k_nk_p(float* p, const float* z, long n, float beta) {
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) p[i] = z[i] + beta * p[i];
}
// sums: q, p.q
__global__ void __launch_bounds__(kT) k_nk_pq(const float* p, const float* q, long n, double* part) {
  double a = 0, b = 0;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    const double qd = conv<double>(q[i]);
    a += qd;
    b = fma(conv<double>(p[i]), qd, b);
  }
  double v[2] = {a, b};
  block_store<2>(v, part);
}
__global__ void k_nk_update(float* dl, float* r, const float* p, const float* q, long n, float alpha, float qshift) {
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    dl[i] += alpha * p[i];
    r[i] -= alpha * (q[i] - qshift);
  }
}
// largest fraction of rho any point loses: max(-d/rho); sums slot holds the max
__global__ void __launch_bounds__(kT) k_nk_loss(const double* rho, const float* dl, long n, double* part) {
  float m = 0.f;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) m = fmaxf(m, -dl[i] / conv<float>(rho[i]));
  __shared__ float sh[kT / 32];
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float x = 0.f;
    for (int w = 0; w < kT / 32; ++w) x = fmaxf(x, sh[w]);
    part[blockIdx.x] = (double)x;
  }
}
// a fixed background holds the boundary planes (Species::setFixedBackground): the
// correction lives on the interior, so each Hessian product's boundary rows are zeroed
__global__ void k_nk_zero_boundary(float* q, long n, int ny, int nz) {
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT)
    if (cdft_on_boundary(i, ny, nz)) q[i] = 0.f;
}
__global__ void k_nk_step(double* rho, const double* rho0, const float* dl, long n, double s) {
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) rho[i] = rho0[i] + s * (double)dl[i];
}
}  // namespace

// ---- device-driven conjugate gradients: one CUDA graph whose WHILE node runs
// the CG iterations with every scalar (alpha, beta, projections, the stopping
// test) kept on the device, so an iteration has no host round trip. Each pass of
// the body increments a counter that ends the loop after max_it + 2 passes
// whatever the state, so the loop is bounded by construction.
struct CgDev {
  double rz, r0, eta, alpha, qshift, zshift, beta;
  int it, done, upd, max_it, fixed, passes;
  long N;
};

namespace {
// FP64 tree over the NV block partials part[b * NV + j]; thread 0 gets the totals
template <int NV>
__device__ void fin_sums(const double* part, int nblk, double* tot) {
  __shared__ double sh[NV][256];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double a = 0;
    for (int b = threadIdx.x; b < nblk; b += 256) a += part[b * NV + j];
    sh[j][threadIdx.x] = a;
  }
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
#pragma unroll
      for (int j = 0; j < NV; ++j) sh[j][threadIdx.x] += sh[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) tot[j] = sh[j][0];
}

__global__ void __launch_bounds__(256) k_cg_fin_pq(const double* part, int nblk, CgDev* st) {
  if (st->done) return;
  double t[2];
  fin_sums<2>(part, nblk, t);
  if (threadIdx.x) return;
  const double qsum = t[0], pq = t[1];
  if (!(pq > 0)) {  // not positive along p: stop; at the first iteration step along p itself
    st->upd = st->it == 0 ? 1 : 0;
    st->alpha = st->rz / fmax(fabs(pq), 1e-300);
    st->qshift = 0;
    if (st->upd) st->it = 1;
    st->done = 1;
  } else {
    st->upd = 1;
    st->alpha = st->rz / pq;
    st->qshift = st->fixed ? qsum / (double)st->N : 0.0;
  }
}
__global__ void k_cg_update(float* dl, float* r, const float* p, const float* q, long n, const CgDev* st) {
  if (!st->upd) return;
  const float alpha = (float)st->alpha, qs = (float)st->qshift;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    dl[i] += alpha * p[i];
    r[i] -= alpha * (q[i] - qs);
  }
}
__global__ void __launch_bounds__(kT) k_cg_precond(const float* r, const double* rho, float* z, long n, float idV, double* part, const CgDev* st) {
  if (st->done) return;
  double s = 0;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    const float x = r[i] * conv<float>(rho[i]) * idV;
    z[i] = x;
    s += conv<double>(x);
  }
  double v[1] = {s};
  block_store<1>(v, part);
}
__global__ void __launch_bounds__(256) k_cg_fin_z(const double* part, int nblk, CgDev* st) {
  if (st->done) return;
  double t[1];
  fin_sums<1>(part, nblk, t);
  if (threadIdx.x == 0) st->zshift = st->fixed ? t[0] / (double)st->N : 0.0;
}
__global__ void __launch_bounds__(kT) k_cg_rz(const float* r, float* z, long n, double* part, const CgDev* st) {
  if (st->done) return;
  const float zshift = (float)st->zshift;
  double a = 0, b = 0;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) {
    const float zz = z[i] - zshift;
    z[i] = zz;
    const double rd = conv<double>(r[i]);
    a = fma(rd, conv<double>(zz), a);
    b = fma(rd, rd, b);
  }
  double v[2] = {a, b};
  block_store<2>(v, part);
}
__global__ void __launch_bounds__(256) k_cg_fin_rz(const double* part, int nblk, CgDev* st) {
  if (st->done) return;
  double t[2];
  fin_sums<2>(part, nblk, t);
  if (threadIdx.x) return;
  st->it += 1;
  if (sqrt(t[1]) <= st->eta * st->r0 || st->it >= st->max_it) {
    st->done = 1;
  } else {
    st->beta = t[0] / st->rz;
    st->rz = t[0];
  }
}
__global__ void k_cg_p(float* p, const float* z, long n, const CgDev* st) {
  if (st->done) return;
  const float beta = (float)st->beta;
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)gridDim.x * kT) p[i] = z[i] + beta * p[i];
}
__global__ void k_cg_tail(CgDev* st, cudaGraphConditionalHandle h) {
  st->passes += 1;
  cudaGraphSetConditional(h, (!st->done && st->passes < st->max_it + 2) ? 1u : 0u);
}
}  // namespace

struct NewtonWork {
  float *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dl = nullptr;
  double* rho0 = nullptr;
  double* start = nullptr;  // a saved starting density (cdft_internal_newton_save / _restore)
  double* part = nullptr;   // device, 3 x grid
  double* hpart = nullptr;  // pinned
  CgDev* cg = nullptr;      // device CG state
  CgDev* hcg = nullptr;     // pinned copy
  cudaGraphExec_t cg_exec = nullptr;
  unsigned cg_plan_gen = ~0u;
  int cg_fixed_bg = -1;  // the boundary mode the graph was built for
  cudaStream_t cg_stream = nullptr;  // capture stream of the CG graph
  bool cg_ok = true;                 // false: the graph could not be built; host-driven CG
  ~NewtonWork() {
    if (cg_exec) cudaGraphExecDestroy(cg_exec);
    if (cg_stream) cudaStreamDestroy(cg_stream);
    cudaFree(cg);
    cudaFreeHost(hcg);
    cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q); cudaFree(dl); cudaFree(rho0); cudaFree(start); cudaFree(part);
    cudaFreeHost(hpart);
  }
};

void cdft_internal_newton_free(cdft_ctx* c) {
  delete c->newton;
  c->newton = nullptr;
}

// Work arrays (and the FP32 evaluator the Hessian products use), allocated once.
int cdft_internal_newton_ensure(cdft_ctx* c) {
  const int prec = c->precision;
  int rc = cdft_set_precision(c, CDFT_FP32);
  if (!rc) rc = cdft_set_precision(c, prec);
  if (rc) return rc;
  if (c->newton) return CDFT_OK;
  const long N = c->info.N;
  const unsigned g = grid_of(N);
  NewtonWork* W = new NewtonWork();
  c->newton = W;
  const size_t fb = N * sizeof(float);
  if (cudaMalloc(&W->r, fb) != cudaSuccess || cudaMalloc(&W->z, fb) != cudaSuccess || cudaMalloc(&W->p, fb) != cudaSuccess ||
      cudaMalloc(&W->q, fb) != cudaSuccess || cudaMalloc(&W->dl, fb) != cudaSuccess ||
      cudaMalloc(&W->rho0, N * sizeof(double)) != cudaSuccess || cudaMalloc(&W->start, N * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&W->part, (size_t)g * 3 * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&W->hpart, (size_t)g * 3 * sizeof(double)) != cudaSuccess || cudaMalloc(&W->cg, sizeof(CgDev)) != cudaSuccess ||
      cudaMallocHost(&W->hcg, sizeof(CgDev)) != cudaSuccess || cudaStreamCreateWithFlags(&W->cg_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cdft_internal_newton_free(c);
    return cdft_internal_fail(c, CDFT_ERR_CUDA, "Newton work arrays");
  }
  if (!c->e32->hess_ready() && c->e32->hess_prepare(c->rho, c->stream)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "Hessian buffers");
  return CDFT_OK;
}

// Builds (once per set of transform plans) the graph of the device-driven CG loop.
static bool build_cg_graph(cdft_ctx* c) {
  NewtonWork* W = c->newton;
  if (W->cg_exec && W->cg_plan_gen == c->plan_gen && W->cg_fixed_bg == c->fixed_bg) return true;
  if (W->cg_exec) cudaGraphExecDestroy(W->cg_exec);
  W->cg_exec = nullptr;
  const long N = c->info.N;
  const double dV = c->info.dV;
  const unsigned g = grid_of(N);
  cudaGraph_t graph = nullptr;
  if (cudaGraphCreate(&graph, 0) != cudaSuccess) return false;
  cudaGraphConditionalHandle h;
  bool ok = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  alignas(cudaGraphNodeParams) unsigned char npb[sizeof(cudaGraphNodeParams)];  // zero-initialised, as the API requires
  std::memset(npb, 0, sizeof(npb));
  cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(npb);
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  ok = ok && cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np) == cudaSuccess;
  if (ok) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    cudaStream_t s = W->cg_stream;
    ok = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      bool launch_ok = c->e32->hess_apply<float>(W->p, c->rho, W->q, dV, s) == 0;
      if (c->fixed_bg) k_nk_zero_boundary<<<g, kT, 0, s>>>(W->q, N, c->p.ny, c->p.nz);
      k_nk_pq<<<g, kT, 0, s>>>(W->p, W->q, N, W->part);
      k_cg_fin_pq<<<1, 256, 0, s>>>(W->part, (int)g, W->cg);
      k_cg_update<<<g, kT, 0, s>>>(W->dl, W->r, W->p, W->q, N, W->cg);
      k_cg_precond<<<g, kT, 0, s>>>(W->r, c->rho, W->z, N, (float)(1.0 / dV), W->part, W->cg);
      k_cg_fin_z<<<1, 256, 0, s>>>(W->part, (int)g, W->cg);
      k_cg_rz<<<g, kT, 0, s>>>(W->r, W->z, N, W->part, W->cg);
      k_cg_fin_rz<<<1, 256, 0, s>>>(W->part, (int)g, W->cg);
      k_cg_p<<<g, kT, 0, s>>>(W->p, W->z, N, W->cg);
      k_cg_tail<<<1, 1, 0, s>>>(W->cg, h);
      cudaGraph_t captured = nullptr;
      ok = cudaStreamEndCapture(s, &captured) == cudaSuccess && launch_ok;
    }
  }
  ok = ok && cudaGraphInstantiate(&W->cg_exec, graph, 0) == cudaSuccess;
  cudaGraphDestroy(graph);
  cudaGetLastError();  // a failed build falls back to host-driven CG; clear its error
  if (!ok) {
    W->cg_exec = nullptr;
    return false;
  }
  W->cg_plan_gen = c->plan_gen;
  W->cg_fixed_bg = c->fixed_bg;
  return true;
}

// Saves / restores the context's density (a Newton run that stalls is retried from the same start).
void cdft_internal_newton_save(cdft_ctx* c) {
  cudaMemcpyAsync(c->newton->start, c->rho, c->info.N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
}
void cdft_internal_newton_restore(cdft_ctx* c) {
  cudaMemcpyAsync(c->rho, c->newton->start, c->info.N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
}

// Sums the NV block partials of the last reduction (synchronises the stream).
template <int NV>
static bool sums(cdft_ctx* c, unsigned g, double* out) {
  NewtonWork* W = c->newton;
  if (cudaMemcpyAsync(W->hpart, W->part, (size_t)g * NV * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return false;
  for (int j = 0; j < NV; ++j) out[j] = 0;
  for (unsigned b = 0; b < g; ++b)
    for (int j = 0; j < NV; ++j) out[j] += W->hpart[b * NV + j];
  return true;
}

extern "C" int cdft_newton_refine(cdft_ctx* c, double tol, int max_newton, int max_cg, double cg_rtol, cdft_newton_report* rep) {
  cdft_newton_params p;
  p.max_newton = max_newton;
  p.max_cg = max_cg;
  p.cg_rtol = cg_rtol;
  p.eta_max = 0.1;
  p.fp32_above = 1e-4;
  p.host_cg = 0;
  return cdft_newton_refine_ex(c, tol, &p, rep);
}

extern "C" int cdft_newton_refine_ex(cdft_ctx* c, double tol, const cdft_newton_params* prm, cdft_newton_report* rep) {
  if (!c || !prm) return CDFT_ERR_ARG;
  // the reference's Hessian of an FMT_AO_Species system (src/FMT.cpp:437-567) leaves out the
  // AO free energy, so it is not the Jacobian of the AO force that Newton-Krylov would need
  if (c->p.ao_rp > 0) return cdft_internal_fail(c, CDFT_ERR_ARG, "Newton-Krylov is not built for the AO model (its Hessian omits the AO term)");
  if (c->homo_bd) return cdft_internal_fail(c, CDFT_ERR_ARG, "Newton-Krylov is not built for the homogeneous boundary");
  const int max_newton = prm->max_newton, max_cg = prm->max_cg;
  const double cg_rtol = prm->cg_rtol, eta_max = prm->eta_max, fp32_above = prm->fp32_above;
  if (!(tol > 0) || max_newton <= 0 || max_cg <= 0 || !(cg_rtol > 0) || !(eta_max >= 0) || !(fp32_above >= 0)) return CDFT_ERR_ARG;
  const long N = c->info.N;
  const double dV = c->info.dV;
  const bool fixed = c->fixed_mass > 0;
  int rc = cdft_set_precision(c, CDFT_FP32);  // the Hessian products' evaluator
  if (!rc) rc = cdft_set_precision(c, CDFT_FP64);
  if (rc) return rc;
  const unsigned g = grid_of(N);
  rc = cdft_internal_newton_ensure(c);
  if (rc) return rc;
  NewtonWork* W = c->newton;
  cudaStream_t s = c->stream;
  cdft_newton_report R{};
  double t[8];
  // Residuals far from the solution come from FP32 evaluations (their noise,
  // ~1e-6, is far below the residual); from kFp64Below on, and for every
  // residual that can end the run, from FP64.
  const double kFp64Below = fp32_above;
  bool fp64 = fp32_above <= 0;
  auto evaluate = [&](bool use64) -> int {
    int e = cdft_set_precision(c, use64 ? CDFT_FP64 : CDFT_FP32);
    if (!e) e = cdft_internal_eval(c, t, 0);
    ++R.evals;
    return e;
  };
  rc = evaluate(fp64);
  if (rc && rc != CDFT_ERR_ETA) return rc;
  if (!fp64 && (rc || t[6] <= kFp64Below)) {
    fp64 = true;
    rc = evaluate(true);
    if (rc) return rc;
  }
  double resid = t[6];
  double l2 = c->last_dF_l2;
  R.F = t[0];
  int stop = 0;
  for (int k = 0; k < max_newton && resid > tol; ++k) {
    // Hessian at the current state; right-hand side -dF, projected at fixed mass
    if (c->e32->hess_prepare(c->rho, s)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "Hessian prepare failed");
    double sm[3];
    k_nk_init<<<g, kT, 0, s>>>(c->dF, W->r, W->dl, N, W->part);
    if (!sums<1>(c, g, sm)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "Newton reduction");
    if (fixed) k_nk_shift<<<g, kT, 0, s>>>(W->r, N, (float)(sm[0] / N));
    auto precond = [&](double* rz_rr) -> bool {
      k_nk_precond<<<g, kT, 0, s>>>(W->r, c->rho, W->z, N, (float)(1.0 / dV), W->part);
      double zs[1];
      if (!sums<1>(c, g, zs)) return false;
      k_nk_rz<<<g, kT, 0, s>>>(W->r, W->z, N, fixed ? (float)(zs[0] / N) : 0.f, W->part);
      return sums<2>(c, g, rz_rr);
    };
    double rz_rr[2];
    if (!precond(rz_rr)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "Newton reduction");
    cudaMemcpyAsync(W->p, W->z, N * sizeof(float), cudaMemcpyDeviceToDevice, s);
    double rz = rz_rr[0];
    const double r0 = std::sqrt(rz_rr[1]);
    bool max_cg_done = false;  // the device-driven loop ran the CG iterations
    // forcing term: a loose linear solve while the residual is large (inexact Newton)
    const double eta = eta_max > 0 ? std::max(cg_rtol, std::min(eta_max, resid)) : cg_rtol;
    int it = 0;
    const bool use_graph = !prm->host_cg && W->cg_ok && (build_cg_graph(c) || (W->cg_ok = false));
    if (use_graph) {
      CgDev& hc = *W->hcg;
      std::memset(&hc, 0, sizeof(CgDev));
      hc.rz = rz;
      hc.r0 = r0;
      hc.eta = eta;
      hc.max_it = max_cg;
      hc.fixed = fixed ? 1 : 0;
      hc.N = N;
      cudaMemcpyAsync(W->cg, W->hcg, sizeof(CgDev), cudaMemcpyHostToDevice, s);
      if (cudaGraphLaunch(W->cg_exec, s) != cudaSuccess) return cdft_internal_fail(c, CDFT_ERR_CUDA, "CG graph launch failed");
      cudaMemcpyAsync(W->hcg, W->cg, sizeof(CgDev), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cdft_internal_fail(c, CDFT_ERR_CUDA, "CG graph failed");
      it = W->hcg->it;
      max_cg_done = true;
    }
    for (; !max_cg_done && it < max_cg; ++it) {
      if (c->e32->hess_apply<float>(W->p, c->rho, W->q, dV, s)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "Hessian product failed");
      if (c->fixed_bg) k_nk_zero_boundary<<<g, kT, 0, s>>>(W->q, N, c->p.ny, c->p.nz);
      k_nk_pq<<<g, kT, 0, s>>>(W->p, W->q, N, W->part);
      double pq[2];
      if (!sums<2>(c, g, pq)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "Newton reduction");
      if (!(pq[1] > 0)) {  // not positive along p: keep the correction built so far
        if (it == 0) {
          // negative curvature along the preconditioned gradient itself: step along that
          // descent direction instead (the line search below sizes it on Omega)
          k_nk_update<<<g, kT, 0, s>>>(W->dl, W->r, W->p, W->q, N, (float)(rz / std::max(std::fabs(pq[1]), 1e-300)), 0.f);
          ++it;
        }
        break;
      }
      const double alpha = rz / pq[1];
      k_nk_update<<<g, kT, 0, s>>>(W->dl, W->r, W->p, W->q, N, (float)alpha, fixed ? (float)(pq[0] / N) : 0.f);
      double nz[2];
      if (!precond(nz)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "Newton reduction");
      if (std::sqrt(nz[1]) <= eta * r0) { ++it; break; }
      const double beta = nz[0] / rz;
      rz = nz[0];
      k_nk_p<<<g, kT, 0, s>>>(W->p, W->z, N, (float)beta);
    }
    R.cg_iters += it;
    // step: at most half of any point's density, then halve until the FP64 residual drops
    k_nk_loss<<<g, kT, 0, s>>>(c->rho, W->dl, N, W->part);
    if (cudaMemcpyAsync(W->hpart, W->part, g * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return cdft_internal_fail(c, CDFT_ERR_CUDA, "Newton reduction");
    double loss = 0;
    for (unsigned b = 0; b < g; ++b) loss = std::max(loss, W->hpart[b]);
    double step = loss > 0.5 ? 0.5 / loss : 1.0;
    cudaMemcpyAsync(W->rho0, c->rho, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
    bool accepted = false;
    for (int ls = 0; ls < 6 && !accepted; ++ls, step *= 0.5) {
      k_nk_step<<<g, kT, 0, s>>>(c->rho, W->rho0, W->dl, N, step);
      rc = evaluate(fp64);
      if (rc && rc != CDFT_ERR_ETA) return rc;
      // accept a lower residual (max or 2-norm), or (far from the minimum) a real decrease of Omega
      if (!rc && (t[6] < resid || c->last_dF_l2 < l2 || t[0] < R.F - (fp64 ? 1e-13 : 1e-6) * std::fabs(R.F))) {
        accepted = true;
        resid = t[6];
        l2 = c->last_dF_l2;
        R.F = t[0];
      }
    }
    ++R.newton;
    if (!accepted) {  // no decrease along the correction: back to the last state
      cudaMemcpyAsync(c->rho, W->rho0, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
      rc = evaluate(true);
      if (rc) return rc;
      fp64 = true;
      resid = t[6];
      R.F = t[0];
      stop = 3;
      break;
    }
    if (!fp64 && resid <= kFp64Below) {  // close enough: FP64 residuals from here on
      fp64 = true;
      rc = evaluate(true);
      if (rc) return rc;
      resid = t[6];
      l2 = c->last_dF_l2;
      R.F = t[0];
    }
  }
  if (!fp64) {  // the run ends on an FP64 residual
    rc = evaluate(true);
    if (rc) return rc;
    resid = t[6];
    R.F = t[0];
  }
  if (resid <= tol) stop = 2;
  R.resid = resid;
  R.stop = stop;
  if (rep) *rep = R;
  // keep the FIRE2 state consistent with the refined density
  if (c->fire_ready) {
    rc = cdft_internal_fire_resync(c);
    if (rc) return rc;
  }
  return CDFT_OK;
}

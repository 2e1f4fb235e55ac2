// Device-resident FIRE2 (fireMinimizer2::step, src/Minimizer.cpp:160-327) for
// runs to a residual target: the step's scalar logic runs in one-thread
// control kernels over a FireState in device memory, the vector work in
// grid kernels, and one whole step (control, vector passes, the F+dF
// evaluation with its Species constraints, the alias conversion) is captured
// once as a CUDA graph. The host launches the graph and reads the state every
// few steps; no host round trip sits inside a step.
//
// The vectors (x, v, alias derivative, density, dF) are stored in the
// arithmetic type S of the phase: FP32 for the bulk phase (GB300 runs FP64 at
// a small fraction of its FP32 rate, and the alias maps are division-heavy),
// FP64 for the refinement phase. The residual max|dOmega/drho| that ends a run
// is always taken from an FP64 evaluation.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <thread>
#include <vector>
#include "cdft_ctx.h"
#include "cdft_kernels.cuh"
#include "cdft_tma.cuh"

using namespace cdft;

struct FireConsts {
  double dmin, c;  // alias map
  double dV, volume;
  double f_inc, f_dec, f_alf, alpha_start, dt_min;
  int n_delay, n_neg_max, initial_delay;
  double tol;  // residual target
  double fixed_mass;
  long N;
};

struct FireState {
  double F, fold, dt, dt_max, alpha, vv, dt_best, fmax, resid, vdotf, vscale, coef, mu;
  double omega, f_id, f_hs, f_mf, f_ext, natoms;
  int Npos, Nneg, backtracks, cur, uphill, status, done, skip, failed;
  unsigned it;
  long steps, calls;
  double red[8];
};

namespace {

constexpr int kThreads = 256;
unsigned grid_n(long n) { return (unsigned)std::max<long>(1, std::min<long>((n + kThreads - 1) / kThreads, 152 * 8)); }

// step start: fireMinimizer2::step up to SemiImplicitEuler (src/Minimizer.cpp:160-217)
__global__ void k_fc_pre(FireState* st, FireConsts k) {
  if (st->done) {
    st->skip = 1;
    return;
  }
  st->skip = 0;
  st->it++;
  const double P = -st->vdotf;
  st->fold = st->F;
  st->uphill = 0;
  if (P > 0) {
    st->Npos++;
    st->Nneg = 0;
    if (st->Npos > k.n_delay) {
      st->dt = fmin(st->dt * k.f_inc, st->dt_max);
      st->alpha = st->alpha * k.f_alf;
    }
  } else {
    st->Npos = 0;
    st->Nneg++;
    if (st->Nneg > k.n_neg_max) {
      st->status = CDFT_ERR_UPHILL;
      st->done = 1;
      st->skip = 1;
      return;
    }
    if (!(k.initial_delay && st->it < (unsigned)k.n_delay)) {
      if (st->dt * k.f_dec >= k.dt_min) st->dt *= k.f_dec;
      st->alpha = k.alpha_start;
    }
    st->uphill = 1;
    st->backtracks++;
  }
}

template <class S>
__device__ __forceinline__ void block_sums_to(double* v, int nv, double* part) {
  // per-block plain FP64 tree of nv per-thread partials
  __shared__ double red[32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < nv; ++k) {
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0) red[warp][k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
    part[blockIdx.x * 8 + threadIdx.x] = t;
  }
}
template <class S>
__device__ __forceinline__ void block_max_to(double* v, int nv, int off, double* part) {
  __shared__ double red[32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  for (int k = 0; k < nv; ++k) {
    for (int o = 16; o > 0; o >>= 1) v[k] = fmax(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
    if (lane == 0) red[warp][k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w][threadIdx.x]);
    part[blockIdx.x * 8 + off + threadIdx.x] = t;
  }
}

// SemiImplicitEuler first half (src/Minimizer.cpp:279-289) with the uphill
// restart of step(): x' = x - dt/2 v (uphill), v' = (0.1 v if uphill else v) - dt g.
template <class S>
__global__ void __launch_bounds__(kThreads) k_fire_pre(S* x0, S* x1, S* v0, S* v1, const S* g0, const S* g1, const FireState* st, long n,
                                                       double* part) {
  if (st->skip) return;
  const int cur = st->cur;
  const S* x = cur ? x1 : x0;
  const S* v = cur ? v1 : v0;
  const S* g = cur ? g1 : g0;
  S* xo = cur ? x0 : x1;
  S* vo = cur ? v0 : v1;
  const S dt = (S)st->dt, vs = (S)st->vscale;
  const int up = st->uphill;
  double acc[2] = {0, 0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    S xi = x[i], vi = v[i] * vs;
    if (up) {
      xi += vi * (S)(-0.5 * st->dt);
      vi *= (S)0.1;
    }
    const S gi = g[i];
    vi += gi * (-dt);
    xo[i] = xi;
    vo[i] = vi;
    acc[0] += (double)(vi * vi);
    acc[1] += (double)(gi * gi);
  }
  block_sums_to<S>(acc, 2, part);
}

// One block merges the per-block partials: 256-way strided sums (maxima),
// then a fixed-order tree; the result goes to st->red[dst + k].
__global__ void __launch_bounds__(256) k_fire_sum_finish(const double* part, int nblk, int off, int nv, FireState* st, int dst) {
  __shared__ double ss[256], sc[256];
  for (int k = 0; k < nv; ++k) {
    Acc a;
    a.init();
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) a.add(part[b * 8 + off + k]);
    ss[threadIdx.x] = a.s;
    sc[threadIdx.x] = a.c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) {
        Acc t;
        t.s = ss[threadIdx.x];
        t.c = sc[threadIdx.x];
        t.merge(ss[threadIdx.x + o], sc[threadIdx.x + o]);
        ss[threadIdx.x] = t.s;
        sc[threadIdx.x] = t.c;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) st->red[dst + k] = ss[0] + sc[0];
    __syncthreads();
  }
}
__global__ void __launch_bounds__(256) k_fire_max_finish(const double* part, int nblk, int off, int nv, FireState* st, int dst) {
  __shared__ double sm[256];
  for (int k = 0; k < nv; ++k) {
    double m = 0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) m = fmax(m, part[b * 8 + off + k]);
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
      __syncthreads();
    }
    if (threadIdx.x == 0) st->red[dst + k] = sm[0];
    __syncthreads();
  }
}

// mixing coefficient sqrt(vnorm/fnorm), norms taken as the reference does (:283-293)
__global__ void k_fc_mid(FireState* st) {
  if (st->skip) return;
  const double nv = sqrt(st->red[0]), nf = sqrt(st->red[1]);
  st->coef = sqrt((nv * nv) / (nf * nf));
}

// v = (1-a) v - a c g; x += dt v; rho = alias(x) (:292-297, src/FMT_Species.cpp:29-45)
template <class S>
__global__ void __launch_bounds__(kThreads) k_fire_mix(S* x0, S* x1, S* v0, S* v1, const S* g0, const S* g1, S* rho, const FireState* st,
                                                       long n, FireConsts k) {
  if (st->skip) return;
  const int cur = st->cur;
  S* x = cur ? x0 : x1;  // the pending state
  S* v = cur ? v0 : v1;
  const S* g = cur ? g1 : g0;
  const S a = (S)st->alpha, coef = (S)(st->alpha * st->coef), dt = (S)st->dt;
  const S dmin = (S)k.dmin, c = (S)k.c;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    S vi = v[i] * ((S)1 - a);
    vi += g[i] * (-coef);
    const S xi = x[i] + vi * dt;
    v[i] = vi;
    x[i] = xi;
    rho[i] = dmin + c * xi * xi / ((S)1 + xi * xi);
  }
}

// Species::beginForceCalculation under fixed mass (src/Species.cpp:64-71)
template <class S>
__global__ void __launch_bounds__(kThreads) k_sum_rho(const S* rho, long n, const FireState* st, double* part) {
  if (st->skip) return;
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) acc[0] += (double)rho[i];
  block_sums_to<S>(acc, 1, part);
}
template <class S>
__global__ void k_scale_rho(S* rho, long n, const FireState* st, FireConsts k) {
  if (st->skip) return;
  const S f = (S)(k.fixed_mass / (st->red[6] * k.dV));
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) rho[i] *= f;
}

// Terms of DFT::calculateFreeEnergyAndDerivatives from the evaluator's sums;
// fixed mass: mu = sum dF rho / M (src/Species.cpp:97-109).
__global__ void k_eval_finish(const double* terms, const unsigned* status, FireState* st, FireConsts k, double mu, int has_fmt, int has_mf) {
  if (st->skip) return;
  const double dV = k.dV;
  const double f_hs = has_fmt ? terms[0] * dV : 0.0;
  const double f_mf = has_mf ? 0.5 * dV * terms[1] : 0.0;
  const double f_id = terms[2];
  const double f_ext = terms[4] * dV - (terms[3] * dV) * mu;
  st->f_hs = f_hs;
  st->f_mf = f_mf;
  st->f_id = f_id;
  st->f_ext = f_ext;
  st->natoms = terms[3] * dV;
  st->omega = ((f_id + f_hs) + f_mf) + f_ext;
  st->failed = (*status & 1u) ? 1 : 0;
  if (*status & kStatusTimeout) {
    st->status = CDFT_ERR_TIMEOUT;
    st->done = 1;
  }
  st->mu = (k.fixed_mass > 0) ? terms[5] / k.fixed_mass : mu;
}
template <class S>
__global__ void k_sub_mu(S* dF, long n, const FireState* st, FireConsts k) {
  if (st->skip || st->failed) return;
  const S m = (S)(st->mu * k.dV);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) dF[i] = dF[i] - m;
}

// Species::endForceCalculation with a fixed background (src/Species.cpp:78-82): dF = 0 on
// the boundary planes
template <class S>
__global__ void k_zero_boundary(S* dF, long n, int ny, int nz, const FireState* st) {
  if (st->skip || st->failed) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    if (cdft_on_boundary(i, ny, nz)) dF[i] = (S)0;
}

// Species::endForceCalculation with a homogeneous boundary (src/Species.cpp:84-95): dF on
// the boundary planes replaced by its mean over them (k_boundary_dF_sum, then the finished
// sum in red[7], k_boundary_dF_fill); with fixed mass the sum dF . rho is then taken again
// over the averaged dF (k_dF_rho_sum, red[7], k_mu_from_sum), as the host path does.
template <class S>
__global__ void __launch_bounds__(kThreads) k_boundary_dF_sum(const S* dF, long n, int ny, int nz, const FireState* st, double* part) {
  if (st->skip || st->failed) return;
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    if (cdft_on_boundary(i, ny, nz)) acc[0] += (double)dF[i];
  block_sums_to<S>(acc, 1, part);
}
template <class S>
__global__ void k_boundary_dF_fill(S* dF, long n, int ny, int nz, const FireState* st, double inv_nb) {
  if (st->skip || st->failed) return;
  const S m = (S)(st->red[7] * inv_nb);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    if (cdft_on_boundary(i, ny, nz)) dF[i] = m;
}
template <class S>
__global__ void __launch_bounds__(kThreads) k_dF_rho_sum(const S* dF, const S* rho, long n, const FireState* st, double* part) {
  if (st->skip || st->failed) return;
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) acc[0] += (double)dF[i] * (double)rho[i];
  block_sums_to<S>(acc, 1, part);
}
__global__ void k_mu_from_sum(FireState* st, FireConsts k) {
  if (st->skip || st->failed) return;
  st->mu = st->red[7] / k.fixed_mass;
}

// Minimizer::getDF_DX after the evaluation (src/Minimizer.cpp:90-115): alias
// derivative into g of the pending state; sums v.g; maxima |dF|, |g|.
template <class S>
__global__ void __launch_bounds__(kThreads) k_fire_post(const S* dF, const S* x0, const S* x1, const S* v0, const S* v1, S* g0, S* g1,
                                                        const FireState* st, long n, FireConsts k, double* part) {
  if (st->skip || st->failed) return;
  const int nxt = 1 - st->cur;
  const S* x = nxt ? x1 : x0;
  const S* v = nxt ? v1 : v0;
  S* g = nxt ? g1 : g0;
  const S c2 = (S)(2 * k.c);
  double acc[1] = {0}, mx[2] = {0, 0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const S y = x[i], d = dF[i];
    const S q = (S)1 + y * y;
    const S ga = d * (c2 * y / (q * q));
    g[i] = ga;
    acc[0] += (double)(v[i] * ga);
    mx[0] = fmax(mx[0], (double)fabs(d));
    mx[1] = fmax(mx[1], (double)fabs(ga));
  }
  block_sums_to<S>(acc, 1, part);
  block_max_to<S>(mx, 2, 1, part);
}

// step end: accept or back track (src/Minimizer.cpp:218-257)
__global__ void k_fc_post(FireState* st, FireConsts k) {
  if (st->skip) return;
  st->calls++;
  if (st->failed) {
    st->vscale *= 0.5;
    st->vdotf *= 0.5;
    st->dt /= 2;
    st->fmax = 1000;
    st->backtracks++;
  } else {
    st->F = st->omega;
    st->cur = 1 - st->cur;
    st->vscale = 1.0;
    st->vdotf = st->red[3];
    st->resid = st->red[4] / k.dV;
    st->fmax = st->red[5] / k.dV;
    st->vv = st->vv * 0.9 + 0.1 * (fabs(st->F - st->fold) / st->dt);
    st->dt_best = fmax(st->dt, st->dt_best);
  }
  if (st->backtracks >= 10) {
    st->dt_max = fmin(st->dt_best, 0.9 * st->dt_max);
    st->dt_best = 0;
    st->backtracks = 0;
  }
  st->steps++;
  if (!st->failed && k.tol > 0 && st->resid <= k.tol) st->done = 1;
}

template <class S>
__global__ void k_convert(const double* a, S* b, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = (S)a[i];
}
template <class S>
__global__ void k_convert_back(const S* a, double* b, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = (double)a[i];
}

}  // namespace

// --------------------------------------------------------------- engine ---
struct FireDevEngine {
  cudaStream_t stream = nullptr;
  FireState* st = nullptr;      // device
  FireState* host = nullptr;    // pinned
  double* part = nullptr;       // 8 doubles per block
  // FP32 phase arrays
  float *x32[2] = {nullptr, nullptr}, *v32[2] = {nullptr, nullptr}, *g32[2] = {nullptr, nullptr}, *rho32 = nullptr, *dF32 = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;  // recorded after each batch's state read
  int exec_prec = -1;
  ~FireDevEngine() {
    if (exec) cudaGraphExecDestroy(exec);
    if (done) cudaEventDestroy(done);
    cudaFree(st); cudaFreeHost(host); cudaFree(part);
    for (int i = 0; i < 2; ++i) { cudaFree(x32[i]); cudaFree(v32[i]); cudaFree(g32[i]); }
    cudaFree(rho32); cudaFree(dF32);
    if (stream) cudaStreamDestroy(stream);
  }
};

void cdft_internal_fire_dev_free(cdft_ctx* c) {
  delete c->fire_dev;
  c->fire_dev = nullptr;
}

static FireConsts consts_of(const cdft_ctx* c, double tol) {
  FireConsts k;
  const Alias a = c->alias();
  k.dmin = a.dmin;
  k.c = a.c;
  k.dV = c->info.dV;
  k.volume = c->info.volume;
  k.f_inc = c->fp.f_inc;
  k.f_dec = c->fp.f_dec;
  k.f_alf = c->fp.f_alf;
  k.alpha_start = c->fp.alpha_start;
  k.dt_min = c->fp.dt_min;
  k.n_delay = c->fp.n_delay;
  k.n_neg_max = c->fp.n_p_negative_max;
  k.initial_delay = c->fp.initial_delay;
  k.tol = tol;
  k.fixed_mass = c->fixed_mass;
  k.N = c->info.N;
  return k;
}

static void state_from_ctx(const cdft_ctx* c, FireState* h) {
  std::memset(h, 0, sizeof(FireState));
  h->F = c->F; h->dt = c->dt; h->dt_max = c->dt_max; h->alpha = c->alpha; h->vv = c->vv; h->dt_best = c->dt_best;
  h->fmax = c->fmax; h->resid = c->resid; h->vdotf = c->vdotf; h->vscale = 1.0; h->mu = c->mu;
  h->Npos = c->Npos; h->Nneg = c->Nneg; h->backtracks = c->backtracks; h->cur = c->cur; h->it = c->it;
  h->steps = c->fire_steps; h->calls = c->calls;
}
static void ctx_from_state(cdft_ctx* c, const FireState* h) {
  c->F = h->F; c->dt = h->dt; c->dt_max = h->dt_max; c->alpha = h->alpha; c->vv = h->vv; c->dt_best = h->dt_best;
  c->fmax = h->fmax; c->resid = h->resid; c->vdotf = h->vdotf;
  c->Npos = h->Npos; c->Nneg = h->Nneg; c->backtracks = h->backtracks; c->cur = h->cur; c->it = h->it;
  c->fire_steps = h->steps; c->calls = h->calls;
  if (c->fixed_mass > 0) c->mu = h->mu;
}

// Records one FIRE2 step on the engine's stream (to be captured).
template <class S, class T>
static void record_step(cdft_ctx* c, FireDevEngine* E, Evaluator<T>* ev, S* x[2], S* v[2], S* g[2], S* rho, S* dF, double tol) {
  const long N = c->info.N;
  const unsigned gn = grid_n(N);
  const FireConsts k = consts_of(c, tol);
  cudaStream_t s = E->stream;
  k_fc_pre<<<1, 1, 0, s>>>(E->st, k);
  k_fire_pre<S><<<gn, kThreads, 0, s>>>(x[0], x[1], v[0], v[1], g[0], g[1], E->st, N, E->part);
  k_fire_sum_finish<<<1, 256, 0, s>>>(E->part, (int)gn, 0, 2, E->st, 0);
  k_fc_mid<<<1, 1, 0, s>>>(E->st);
  k_fire_mix<S><<<gn, kThreads, 0, s>>>(x[0], x[1], v[0], v[1], g[0], g[1], rho, E->st, N, k);
  const double mu_eval = c->fixed_mass > 0 ? 0.0 : c->mu;
  if (c->fixed_mass > 0) {
    k_sum_rho<S><<<gn, kThreads, 0, s>>>(rho, N, E->st, E->part);
    k_fire_sum_finish<<<1, 256, 0, s>>>(E->part, (int)gn, 0, 1, E->st, 6);
    k_scale_rho<S><<<gn, kThreads, 0, s>>>(rho, N, E->st, k);
  }
  ev->template launch<S>(rho, c->vext, dF, c->info.dV, mu_eval, 1, s, nullptr);
  k_eval_finish<<<1, 1, 0, s>>>(ev->dev_terms(), ev->dev_status(), E->st, k, mu_eval, ev->M() > 0 ? 1 : 0, ev->has_mf() ? 1 : 0);
  if (c->homo_bd) {
    k_boundary_dF_sum<S><<<gn, kThreads, 0, s>>>(dF, N, c->p.ny, c->p.nz, E->st, E->part);
    k_fire_sum_finish<<<1, 256, 0, s>>>(E->part, (int)gn, 0, 1, E->st, 7);
    k_boundary_dF_fill<S><<<gn, kThreads, 0, s>>>(dF, N, c->p.ny, c->p.nz, E->st, 1.0 / (double)cdft_n_boundary(c->p.nx, c->p.ny, c->p.nz));
    if (c->fixed_mass > 0) {
      k_dF_rho_sum<S><<<gn, kThreads, 0, s>>>(dF, rho, N, E->st, E->part);
      k_fire_sum_finish<<<1, 256, 0, s>>>(E->part, (int)gn, 0, 1, E->st, 7);
      k_mu_from_sum<<<1, 1, 0, s>>>(E->st, k);
    }
  }
  if (c->fixed_mass > 0) k_sub_mu<S><<<gn, kThreads, 0, s>>>(dF, N, E->st, k);
  if (c->fixed_bg) k_zero_boundary<S><<<gn, kThreads, 0, s>>>(dF, N, c->p.ny, c->p.nz, E->st);
  k_fire_post<S><<<gn, kThreads, 0, s>>>(dF, x[0], x[1], v[0], v[1], g[0], g[1], E->st, N, k, E->part);
  k_fire_sum_finish<<<1, 256, 0, s>>>(E->part, (int)gn, 0, 1, E->st, 3);
  k_fire_max_finish<<<1, 256, 0, s>>>(E->part, (int)gn, 1, 2, E->st, 4);
  k_fc_post<<<1, 1, 0, s>>>(E->st, k);
}

static int ensure_engine(cdft_ctx* c) {
  if (c->fire_dev) return CDFT_OK;
  FireDevEngine* E = new FireDevEngine();
  c->fire_dev = E;
  const long N = c->info.N;
  if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) != cudaSuccess || cudaMalloc(&E->st, sizeof(FireState)) != cudaSuccess ||
      cudaMallocHost(&E->host, sizeof(FireState)) != cudaSuccess || cudaMalloc(&E->part, (size_t)152 * 8 * 8 * sizeof(double)) != cudaSuccess ||
      cudaEventCreateWithFlags(&E->done, cudaEventDisableTiming) != cudaSuccess)
    return cdft_internal_fail(c, CDFT_ERR_CUDA, "device FIRE engine allocation failed");
  (void)N;
  return CDFT_OK;
}

static int ensure_fp32_arrays(cdft_ctx* c) {
  FireDevEngine* E = c->fire_dev;
  if (E->rho32) return CDFT_OK;
  const size_t b = c->info.N * sizeof(float);
  for (int i = 0; i < 2; ++i)
    if (cudaMalloc(&E->x32[i], b) != cudaSuccess || cudaMalloc(&E->v32[i], b) != cudaSuccess || cudaMalloc(&E->g32[i], b) != cudaSuccess)
      return cdft_internal_fail(c, CDFT_ERR_CUDA, "FP32 FIRE arrays");
  if (cudaMalloc(&E->rho32, b) != cudaSuccess || cudaMalloc(&E->dF32, b) != cudaSuccess)
    return cdft_internal_fail(c, CDFT_ERR_CUDA, "FP32 FIRE arrays");
  return CDFT_OK;
}

// A phase runs graph-captured steps in one precision. It is split into
// begin (upload the state, convert the vectors, capture one step), launch
// (queue a batch of steps and an asynchronous read of the state), poll (read
// the state after the batch and decide whether the phase is over) and end
// (download the state, convert the vectors back), so that one host thread can
// drive many contexts, each on its own stream.
struct PhaseRun {
  int prec = CDFT_FP64;
  double tol = 0, switch_tol = 0;
  long max_steps = -1, k = 0, best_at = 0, base = 0;
  double best = 1e300;
  int stop = 0;
};

static int phase_begin(cdft_ctx* c, PhaseRun* ph, int prec, double tol, double switch_tol, long max_steps) {
  FireDevEngine* E = c->fire_dev;
  const long N = c->info.N;
  const unsigned gn = grid_n(N);
  cudaStream_t s = E->stream;
  *ph = PhaseRun();
  ph->prec = prec;
  ph->tol = tol;
  ph->switch_tol = switch_tol;
  ph->max_steps = max_steps;
  ph->base = c->fire_steps;
  state_from_ctx(c, E->host);
  cudaMemcpyAsync(E->st, E->host, sizeof(FireState), cudaMemcpyHostToDevice, s);
  if (prec == CDFT_FP32) {
    int rc = ensure_fp32_arrays(c);
    if (rc) return rc;
    for (int i = 0; i < 2; ++i) {
      k_convert<float><<<gn, kThreads, 0, s>>>(c->fx[i], E->x32[i], N);
      k_convert<float><<<gn, kThreads, 0, s>>>(c->fv[i], E->v32[i], N);
      k_convert<float><<<gn, kThreads, 0, s>>>(c->fg[i], E->g32[i], N);
    }
  }
  cudaGraph_t graph;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return cdft_internal_fail(c, CDFT_ERR_CUDA, "capture");
  if (prec == CDFT_FP32) {
    float* x[2] = {E->x32[0], E->x32[1]};
    float* v[2] = {E->v32[0], E->v32[1]};
    float* g[2] = {E->g32[0], E->g32[1]};
    record_step<float, float>(c, E, c->e32.get(), x, v, g, E->rho32, E->dF32, 0.0);
  } else {
    record_step<double, double>(c, E, c->e64.get(), c->fx, c->fv, c->fg, c->rho, c->dF, tol);
  }
  if (cudaStreamEndCapture(s, &graph) != cudaSuccess) return cdft_internal_fail(c, CDFT_ERR_CUDA, "capture end");
  if (E->exec) cudaGraphExecDestroy(E->exec);
  E->exec = nullptr;
  if (cudaGraphInstantiate(&E->exec, graph, 0) != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cdft_internal_fail(c, CDFT_ERR_CUDA, "graph instantiate");
  }
  cudaGraphDestroy(graph);
  return CDFT_OK;
}

// Queues up to `batch` steps and the state read; returns the number queued (0: step budget spent).
static long phase_launch(cdft_ctx* c, PhaseRun* ph, int batch) {
  FireDevEngine* E = c->fire_dev;
  const long nb = (ph->max_steps > 0) ? std::min<long>(batch, ph->max_steps - ph->k) : batch;
  if (nb <= 0) return 0;
  for (long j = 0; j < nb; ++j) cudaGraphLaunch(E->exec, E->stream);
  cudaMemcpyAsync(E->host, E->st, sizeof(FireState), cudaMemcpyDeviceToHost, E->stream);
  cudaEventRecord(E->done, E->stream);
  return nb;
}

// After the queued batch has completed: 1 if the phase is over, 0 to go on, < 0 never;
// a device status (uphill, timeout) is returned through *rc.
static int phase_poll(cdft_ctx* c, PhaseRun* ph, int* rc) {
  FireDevEngine* E = c->fire_dev;
  *rc = CDFT_OK;
  if (cudaEventSynchronize(E->done) != cudaSuccess) {
    *rc = cdft_internal_fail(c, CDFT_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    return 1;
  }
  const FireState& h = *E->host;
  ph->k = h.steps - ph->base;
  if (h.status) {
    ctx_from_state(c, E->host);
    *rc = cdft_internal_fail(c, h.status, h.status == CDFT_ERR_UPHILL ? "Cannot stop going uphill in Fire2" : "device wait timed out");
    return 1;
  }
  if (h.done) { ph->stop = 2; return 1; }
  if (ph->prec == CDFT_FP32) {
    if (h.resid < ph->best * 0.98) { ph->best = h.resid; ph->best_at = ph->k; }
    if (h.resid <= ph->switch_tol) { ph->stop = 3; return 1; }
    if (ph->k - ph->best_at > 96) { ph->stop = 4; return 1; }  // the FP32 residual has stalled (its noise floor)
  }
  if (ph->max_steps > 0 && ph->k >= ph->max_steps) return 1;
  return 0;
}

// Downloads the scalars and moves the FP32 phase's vectors back into FP64 storage (asynchronous).
static void phase_end(cdft_ctx* c, PhaseRun* ph) {
  FireDevEngine* E = c->fire_dev;
  const long N = c->info.N;
  const unsigned gn = grid_n(N);
  cudaStream_t s = E->stream;
  ctx_from_state(c, E->host);
  if (ph->prec == CDFT_FP32) {
    for (int i = 0; i < 2; ++i) {
      k_convert_back<float><<<gn, kThreads, 0, s>>>(E->x32[i], c->fx[i], N);
      k_convert_back<float><<<gn, kThreads, 0, s>>>(E->v32[i], c->fv[i], N);
      k_convert_back<float><<<gn, kThreads, 0, s>>>(E->g32[i], c->fg[i], N);
    }
    k_convert_back<float><<<gn, kThreads, 0, s>>>(E->rho32, c->rho, N);
    k_convert_back<float><<<gn, kThreads, 0, s>>>(E->dF32, c->dF, N);
  }
}

constexpr int kStepsPerRead = 16;
// Newton-Krylov refinement of the mixed = 2 policy: corrections, CG iterations per correction, CG tolerance
constexpr int kNewtonMax = 12, kNewtonCg = 200;
constexpr int kNewtonMax3 = 40;  // Newton from an arbitrary start (mixed = 3)
constexpr double kNewtonRtol = 1e-3;

// Runs one phase to its end on one context.
static int run_phase(cdft_ctx* c, int prec, double tol, double switch_tol, long max_steps, long* taken, int* stop) {
  PhaseRun ph;
  int rc = phase_begin(c, &ph, prec, tol, switch_tol, max_steps);
  if (rc) return rc;
  while (phase_launch(c, &ph, kStepsPerRead) > 0) {
    if (phase_poll(c, &ph, &rc)) break;
  }
  *taken = ph.k;
  *stop = ph.stop;
  if (rc) return rc;
  phase_end(c, &ph);
  cudaStreamSynchronize(c->fire_dev->stream);
  return CDFT_OK;
}

static void report_of(const cdft_ctx* c, long steps, int stop, cdft_fire_report* r, long steps32 = 0) {
  if (!r) return;
  r->steps_fp32 = steps32;
  r->newton = 0;
  r->cg_iters = 0;
  r->steps = steps;
  r->total_steps = c->fire_steps;
  r->calls = c->calls;
  r->F = c->F;
  r->dt = c->dt;
  r->dt_max = c->dt_max;
  r->alpha = c->alpha;
  r->vv = c->vv;
  r->fmax = c->fmax;
  r->resid = c->resid;
  r->backtracks = 0;
  r->stop = stop;
}

__global__ void k_rho_from_alias_pub(const double* x, double* rho, long n, Alias a) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double y = x[i];
    rho[i] = a.dmin + a.c * y * y / (1 + y * y);
  }
}

// Re-evaluates in FP64 at the current alias state (the refinement phase's
// first gradient): rho = alias(x[cur]), F, dF, g[cur], v.g, residual.
static int refresh_fp64(cdft_ctx* c) {
  int rc = cdft_set_precision(c, CDFT_FP64);
  if (rc) return rc;
  cudaStreamSynchronize(c->fire_dev->stream);
  const long N = c->info.N;
  k_rho_from_alias_pub<<<grid_n(N), kThreads, 0, c->stream>>>(c->fx[c->cur], c->rho, N, c->alias());
  double t[8];
  rc = cdft_internal_eval(c, t, 0);
  if (rc) return rc;
  c->F = t[0];
  return cdft_internal_fire_accept(c, c->cur);
}

extern "C" int cdft_fire_run_device(cdft_ctx* c, double resid_tol, double switch_tol, long max_steps, int mixed, cdft_fire_report* rep) {
  if (!c) return CDFT_ERR_ARG;
  if (!c->fire_ready) return cdft_internal_fail(c, CDFT_ERR_STATE, "cdft_fire_init has not been called");
  if (mixed < 0 || mixed > 3) return cdft_internal_fail(c, CDFT_ERR_ARG, "mixed must be 0, 1, 2 or 3");
  if (mixed >= 2 && c->p.ao_rp > 0) mixed = 1;  // no Newton-Krylov for the AO model: the FIRE2 policy
  if (mixed >= 2 && c->homo_bd) mixed = 1;  // Newton-Krylov is not built for the homogeneous boundary: the FIRE2 policy
  int rc = ensure_engine(c);
  if (rc) return rc;
  long total = 0, taken = 0, steps32 = 0;
  int stop = 0;
  long nk = 0, ncg = 0;
  if (mixed == 3) {
    // Newton-Krylov from the current state: first the fast settings (loose CG while the
    // residual is large, FP32 residuals above 1e-4); if that stalls, again from the same
    // start with FP64 residuals throughout (a path whose last corrections stalled in the
    // FP32-to-FP64 hand-over near 1e-7 converges this way), then with CG to 1e-3
    // throughout as well; then the mixed = 2 path.
    cdft_newton_params fast{kNewtonMax3, kNewtonCg, kNewtonRtol, 0.1, 1e-4, 0};
    cdft_newton_params fp64{2 * kNewtonMax3, kNewtonCg, kNewtonRtol, 0.1, 0.0, 0};
    cdft_newton_params safe{2 * kNewtonMax3, kNewtonCg, kNewtonRtol, 0.0, 0.0, 0};  // slow, steady: allow more corrections
    rc = cdft_internal_newton_ensure(c);
    if (rc) return rc;
    cdft_internal_newton_save(c);
    for (const cdft_newton_params* p : {&fast, &fp64, &safe}) {
      if (p != &fast) cdft_internal_newton_restore(c);
      cdft_newton_report nr;
      rc = cdft_newton_refine_ex(c, resid_tol, p, &nr);
      if (rc) return rc;
      nk += nr.newton;
      ncg += nr.cg_iters;
      if (nr.stop == 2) {
        report_of(c, 0, 2, rep, 0);
        if (rep) rep->newton = nk, rep->cg_iters = ncg;
        return CDFT_OK;
      }
    }
    mixed = 2;
  }
  if (mixed) {
    rc = cdft_set_precision(c, CDFT_FP32);
    if (rc) return rc;
    rc = run_phase(c, CDFT_FP32, resid_tol, switch_tol, max_steps, &taken, &stop);
    total += taken;
    steps32 = taken;
    if (rc) {
      report_of(c, total, stop, rep, steps32);
      return rc;
    }
    rc = refresh_fp64(c);
    if (rc) return rc;
    if (max_steps > 0 && total >= max_steps) {
      report_of(c, total, 0, rep, steps32);
      return CDFT_OK;
    }
    if (c->resid <= resid_tol) {
      report_of(c, total, 2, rep, steps32);
      return CDFT_OK;
    }
    if (mixed == 2) {  // Newton-Krylov refinement; FP64 FIRE2 only if it stalls
      cdft_newton_report nr;
      rc = cdft_newton_refine(c, resid_tol, kNewtonMax, kNewtonCg, kNewtonRtol, &nr);
      if (rc) return rc;
      nk += nr.newton;
      ncg += nr.cg_iters;
      if (nr.stop == 2) {
        report_of(c, total, 2, rep, steps32);
        if (rep) rep->newton = nk, rep->cg_iters = ncg;
        return CDFT_OK;
      }
    }
  }
  rc = run_phase(c, CDFT_FP64, resid_tol, 0.0, max_steps > 0 ? max_steps - total : -1, &taken, &stop);
  total += taken;
  report_of(c, total, stop, rep, steps32);
  if (rep) rep->newton = nk, rep->cg_iters = ncg;
  return rc;
}

// ------------------------------------------------------------ batches ---
// Many independent systems (state points, possibly on different grids) run
// their device FIRE2 concurrently: each context's graph-captured steps go to
// its own stream, and one host thread polls every context's batch-end event,
// queueing the next batch of a context as soon as its previous one has
// finished. Small grids that cannot fill 152 SMs alone overlap on the GPU.
namespace {
struct BatchItem {
  cdft_ctx* c = nullptr;
  cudaStream_t saved_stream = nullptr;
  PhaseRun ph;
  int stage = 0;  // 0 FP32 bulk phase, 1 FP64 phase, 2 finished
  long total = 0, steps32 = 0, newton = 0, cg = 0;
  int rc = CDFT_OK;
};
}  // namespace

static void batch_finish(BatchItem& b, cdft_fire_report* rep, int stop) {
  report_of(b.c, b.total, stop, rep, b.steps32);
  if (rep) {
    rep->newton = b.newton;
    rep->cg_iters = b.cg;
  }
  b.stage = 2;
}

// Starts the FP64 phase of an item, or finishes it when nothing is left to do.
static void batch_start_fp64(BatchItem& b, double tol, long max_steps, cdft_fire_report* rep) {
  if ((max_steps > 0 && b.total >= max_steps) || b.c->resid <= tol) {
    batch_finish(b, rep, b.c->resid <= tol ? 2 : 0);
    return;
  }
  b.rc = phase_begin(b.c, &b.ph, CDFT_FP64, tol, 0.0, max_steps > 0 ? max_steps - b.total : -1);
  if (b.rc) { batch_finish(b, rep, 0); return; }
  b.stage = 1;
  if (phase_launch(b.c, &b.ph, kStepsPerRead) == 0) batch_finish(b, rep, 0);
}

// Host threads of a Newton-Krylov batch: CDFT_BATCH_THREADS (1-64) when set, else 8.
static int batch_threads() {
  const char* e = std::getenv("CDFT_BATCH_THREADS");
  const int v = e ? std::atoi(e) : 0;
  return v >= 1 && v <= 64 ? v : 8;
}

// mixed = 3: Newton-Krylov per context is host-driven (a synchronisation per CG
// iteration), so contexts are spread over host threads, each context on its own
// stream, and the GPU interleaves their kernels.
static int batch_newton(cdft_ctx* const* ctx, int n, double resid_tol, double switch_tol, long max_steps, cdft_fire_report* reps,
                        int* rcs) {
  std::vector<cudaStream_t> saved(n);
  for (int i = 0; i < n; ++i) {
    cdft_ctx* c = ctx[i];
    int rc = ensure_engine(c);
    if (!rc) rc = cdft_set_precision(c, CDFT_FP32);
    if (!rc) rc = ensure_fp32_arrays(c);
    if (!rc) rc = cdft_set_precision(c, CDFT_FP64);
    if (!rc) rc = cdft_internal_newton_ensure(c);
    if (rc) return rc;
    cudaStreamSynchronize(c->stream);
    saved[i] = c->stream;
    c->stream = c->fire_dev->stream;
  }
  std::atomic<int> next(0);
  std::vector<int> st(n, CDFT_OK);
  int dev = 0;
  cudaGetDevice(&dev);
  auto work = [&]() {
    cudaSetDevice(dev);
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= n) break;
      cdft_fire_report r{};
      st[i] = cdft_fire_run_device(ctx[i], resid_tol, switch_tol, max_steps, 3, &r);
      if (reps) reps[i] = r;
    }
  };
  const int nt = std::min(n, batch_threads());
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t) pool.emplace_back(work);
  for (auto& t : pool) t.join();
  int first = CDFT_OK;
  for (int i = 0; i < n; ++i) {
    cudaStreamSynchronize(ctx[i]->stream);
    ctx[i]->stream = saved[i];
    if (rcs) rcs[i] = st[i];
    if (st[i] && !first) first = st[i];
  }
  return first;
}

extern "C" int cdft_fire_run_batch(cdft_ctx* const* ctx, int n, double resid_tol, double switch_tol, long max_steps, int mixed,
                                   cdft_fire_report* reps, int* rcs) {
  if (!ctx || n <= 0 || mixed < 0 || mixed > 3) return CDFT_ERR_ARG;
  std::vector<BatchItem> items(n);
  for (int i = 0; i < n; ++i) {
    if (!ctx[i]) return CDFT_ERR_ARG;
    for (int j = 0; j < i; ++j)
      if (ctx[j] == ctx[i]) return cdft_internal_fail(ctx[i], CDFT_ERR_ARG, "a context appears twice in the batch");
    if (!ctx[i]->fire_ready) return cdft_internal_fail(ctx[i], CDFT_ERR_STATE, "cdft_fire_init has not been called");
    // Newton-Krylov is not built for the homogeneous boundary: such a batch takes the FIRE2 policy
    if (mixed >= 2 && ctx[i]->homo_bd) mixed = 1;
  }
  if (mixed == 3) return batch_newton(ctx, n, resid_tol, switch_tol, max_steps, reps, rcs);
  // allocation first (nothing may allocate while a stream is captured), and
  // every context's own work on its engine's stream
  for (int i = 0; i < n; ++i) {
    BatchItem& b = items[i];
    b.c = ctx[i];
    int rc = ensure_engine(b.c);
    if (!rc && mixed) rc = cdft_set_precision(b.c, CDFT_FP32);
    if (!rc && mixed) rc = ensure_fp32_arrays(b.c);
    if (!rc) rc = cdft_set_precision(b.c, CDFT_FP64);
    if (!rc && mixed == 2) rc = cdft_internal_newton_ensure(b.c);
    if (rc) return rc;
    cudaStreamSynchronize(b.c->stream);
    b.saved_stream = b.c->stream;
    b.c->stream = b.c->fire_dev->stream;
  }
  for (int i = 0; i < n; ++i) {
    BatchItem& b = items[i];
    cdft_fire_report* rep = reps ? &reps[i] : nullptr;
    if (mixed) {
      b.rc = cdft_set_precision(b.c, CDFT_FP32);
      if (!b.rc) b.rc = phase_begin(b.c, &b.ph, CDFT_FP32, resid_tol, switch_tol, max_steps);
      if (b.rc) { batch_finish(b, rep, 0); continue; }
      b.stage = 0;
      if (phase_launch(b.c, &b.ph, kStepsPerRead) == 0) { batch_finish(b, rep, 0); continue; }
    } else {
      batch_start_fp64(b, resid_tol, max_steps, rep);
    }
  }
  for (;;) {
    int active = 0, progressed = 0;
    for (int i = 0; i < n; ++i) {
      BatchItem& b = items[i];
      if (b.stage == 2) continue;
      ++active;
      if (cudaEventQuery(b.c->fire_dev->done) == cudaErrorNotReady) continue;
      ++progressed;
      cdft_fire_report* rep = reps ? &reps[i] : nullptr;
      int rc = CDFT_OK;
      bool over = phase_poll(b.c, &b.ph, &rc) != 0;
      if (!over && phase_launch(b.c, &b.ph, kStepsPerRead) == 0) over = true;
      if (!over) continue;
      b.total += b.ph.k;
      if (rc) {
        b.rc = rc;
        batch_finish(b, rep, b.ph.stop);
        continue;
      }
      phase_end(b.c, &b.ph);
      if (b.stage == 0) {
        b.steps32 = b.ph.k;
        b.rc = refresh_fp64(b.c);
        if (b.rc) { batch_finish(b, rep, 0); continue; }
        if (mixed == 2 && b.c->resid > resid_tol) {  // Newton-Krylov refinement on this context's stream
          cdft_newton_report nr;
          b.rc = cdft_newton_refine(b.c, resid_tol, kNewtonMax, kNewtonCg, kNewtonRtol, &nr);
          if (b.rc) { batch_finish(b, rep, 0); continue; }
          b.newton = nr.newton;
          b.cg = nr.cg_iters;
        }
        batch_start_fp64(b, resid_tol, max_steps, rep);
      } else {
        cudaStreamSynchronize(b.c->fire_dev->stream);
        batch_finish(b, rep, b.ph.stop);
      }
    }
    if (!active) break;
    if (!progressed) std::this_thread::yield();
  }
  int first = CDFT_OK;
  for (int i = 0; i < n; ++i) {
    BatchItem& b = items[i];
    cudaStreamSynchronize(b.c->stream);
    b.c->stream = b.saved_stream;
    if (rcs) rcs[i] = b.rc;
    if (b.rc && !first) first = b.rc;
  }
  return first;
}

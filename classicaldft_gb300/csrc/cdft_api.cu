// C ABI of the GB300 engine (include/cdft.h): context management, the F+dF
// evaluation with the Species begin/end force constraints, bulk
// thermodynamics, and the FIRE2 and DDFT drivers. The drivers keep the
// reference's step logic on the host (scalars only) and run every N-sized
// operation on the device, with fused FP64 compensated reductions.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>
#include "../../include/cdft.h"
#include "cdft_internal.h"
#include "cdft_kernels.cuh"
#include "cdft_ctx.h"

using namespace cdft;

namespace {

// ------------------------------------------------------- map-reduce ---
// Each functor fills NS sums (compensated) and NM maxima for element i.
template <int NS, int NM, class F>
__global__ void __launch_bounds__(256) k_map_reduce(long n, F f, double* __restrict__ part) {
  Acc acc[NS > 0 ? NS : 1];
  double mx[NM > 0 ? NM : 1];
  for (int v = 0; v < NS; ++v) acc[v].init();
  for (int v = 0; v < NM; ++v) mx[v] = -INFINITY;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double s[NS > 0 ? NS : 1], m[NM > 0 ? NM : 1];
    f(i, s, m);
    for (int v = 0; v < NS; ++v) acc[v].add(s[v]);
    for (int v = 0; v < NM; ++v) mx[v] = fmax(mx[v], m[v]);
  }
  constexpr int kNS = (NS > 0) ? NS : 1;
  if (NS > 0) block_reduce_store<kNS>(acc, part, blockIdx.x);
  // maxima: warp then block
  __shared__ double red[32][NM > 0 ? NM : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int v = 0; v < NM; ++v) {
    for (int o = 16; o > 0; o >>= 1) mx[v] = fmax(mx[v], __shfl_down_sync(0xffffffffu, mx[v], o));
    if (lane == 0) red[warp][v] = mx[v];
  }
  __syncthreads();
  if (threadIdx.x == 0 && NM > 0) {
    double* pm = part + (long)gridDim.x * 2 * NS;
    for (int v = 0; v < NM; ++v) {
      double t = -INFINITY;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w][v]);
      pm[(long)blockIdx.x * NM + v] = t;
    }
  }
}

// Deterministic finish of the block partials, 256 threads: thread t merges blocks
// t, t + 256, ... in order, then a fixed-shape tree combines the threads. (A
// single thread merging ~1000 compensated pairs is a serial chain of FP64
// operations, which GB300's FP64 pipe makes slow.)
constexpr int kFinishThreads = 256;
__global__ void __launch_bounds__(kFinishThreads) k_finish_map_reduce(const double* __restrict__ part, int nblk, int ns, int nm,
                                                                      double* __restrict__ out) {
  __shared__ double sh_s[kFinishThreads], sh_c[kFinishThreads];
  const int tid = threadIdx.x;
  for (int v = 0; v < ns; ++v) {
    Acc a;
    a.init();
    for (int b = tid; b < nblk; b += kFinishThreads) a.merge(part[(b * ns + v) * 2], part[(b * ns + v) * 2 + 1]);
    sh_s[tid] = a.s;
    sh_c[tid] = a.c;
    __syncthreads();
    for (int o = kFinishThreads / 2; o > 0; o >>= 1) {
      if (tid < o) {
        Acc x;
        x.s = sh_s[tid];
        x.c = sh_c[tid];
        x.merge(sh_s[tid + o], sh_c[tid + o]);
        sh_s[tid] = x.s;
        sh_c[tid] = x.c;
      }
      __syncthreads();
    }
    if (tid == 0) out[v] = sh_s[0] + sh_c[0];
    __syncthreads();
  }
  const double* pm = part + (long)nblk * 2 * ns;
  for (int v = 0; v < nm; ++v) {
    double t = -INFINITY;
    for (int b = tid; b < nblk; b += kFinishThreads) t = fmax(t, pm[b * nm + v]);
    sh_s[tid] = t;
    __syncthreads();
    for (int o = kFinishThreads / 2; o > 0; o >>= 1) {
      if (tid < o) sh_s[tid] = fmax(sh_s[tid], sh_s[tid + o]);
      __syncthreads();
    }
    if (tid == 0) out[ns + v] = sh_s[0];
    __syncthreads();
  }
}

struct FSumRho {
  const double* r;
  __device__ void operator()(long i, double* s, double*) const { s[0] = r[i]; }
};
// Species::endForceCalculation's boundary sum (src/Species.cpp:88-91) and the fixed-mass
// sum dF . rho taken after it (:100-102)
struct FBoundarySum {
  const double* a;
  int ny, nz;
  __device__ void operator()(long i, double* s, double*) const { s[0] = cdft_on_boundary(i, ny, nz) ? a[i] : 0.0; }
};
struct FSumDot {
  const double *a, *b;
  __device__ void operator()(long i, double* s, double*) const { s[0] = a[i] * b[i]; }
};
struct FAbsMax {
  const double* a;
  __device__ void operator()(long i, double*, double* m) const { m[0] = fabs(a[i]); }
};
// max |dF| (the residual) and sum dF^2 (its 2-norm, for the Newton line search):
// plain FP64 sums, one multiply-add per point, deterministic block and tree order.
__global__ void __launch_bounds__(256) k_dF_norms(const double* __restrict__ a, long n, double* __restrict__ part) {
  double sq = 0, mx = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = a[i];
    sq = fma(v, v, sq);
    mx = fmax(mx, fabs(v));
  }
  __shared__ double s_sq[256], s_mx[256];
  s_sq[threadIdx.x] = sq;
  s_mx[threadIdx.x] = mx;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      s_sq[threadIdx.x] += s_sq[threadIdx.x + o];
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s_sq[0];
    part[2 * blockIdx.x + 1] = s_mx[0];
  }
}
// out[0] = sum dF^2, out[1] = max |dF|
__global__ void __launch_bounds__(256) k_dF_norms_finish(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  double sq = 0, mx = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    sq += part[2 * b];
    mx = fmax(mx, part[2 * b + 1]);
  }
  __shared__ double s_sq[256], s_mx[256];
  s_sq[threadIdx.x] = sq;
  s_mx[threadIdx.x] = mx;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      s_sq[threadIdx.x] += s_sq[threadIdx.x + o];
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s_sq[0];
    out[1] = s_mx[0];
  }
}

__device__ __forceinline__ double alias_rho(const Alias& a, double y) { return a.dmin + a.c * y * y / (1 + y * y); }

__global__ void k_alias_from_rho(const double* __restrict__ rho, double* __restrict__ x, long n, Alias a) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double z = (rho[i] - a.dmin) / a.c;
    x[i] = sqrt(fabs(z / (1 - z)));
  }
}
__global__ void k_rho_from_alias(const double* __restrict__ x, double* __restrict__ rho, long n, Alias a) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) rho[i] = alias_rho(a, x[i]);
}
__global__ void k_scale_vec(double* __restrict__ x, long n, double s) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] *= s;
}
__global__ void k_add_const(double* __restrict__ x, long n, double s) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] = x[i] - s;
}

// FIRE2 step, first half (fireMinimizer2::step uphill branch + SemiImplicitEuler
// first line, src/Minimizer.cpp:198-217, 279-289): xo = x - dt/2 v (uphill),
// vo = (0.1 v if uphill else v) - dt dF; sums |vo|^2, |dF|^2.
struct FFirePre {
  const double *x, *v, *dF;
  double *xo, *vo;
  double dt;
  int uphill;
  __device__ void operator()(long i, double* s, double*) const {
    double xi = x[i], vi = v[i];
    if (uphill) {
      xi += vi * (-0.5 * dt);
      vi *= 0.1;
    }
    const double g = dF[i];
    vi += g * (-dt);
    xo[i] = xi;
    vo[i] = vi;
    s[0] = vi * vi;
    s[1] = g * g;
  }
};
// Second half (src/Minimizer.cpp:292-297): v = (1-a) v - a c dF; x += dt v; rho = alias(x).
__global__ void k_fire_mix(double* __restrict__ x, double* __restrict__ v, const double* __restrict__ dF, double* __restrict__ rho, long n,
                           double dt, double alpha, double coef, Alias a) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double vi = v[i] * (1 - alpha);
    vi += dF[i] * (-alpha * coef);
    const double xi = x[i] + vi * dt;
    v[i] = vi;
    x[i] = xi;
    rho[i] = alias_rho(a, xi);
  }
}
// After an accepted evaluation (Minimizer::getDF_DX, src/Minimizer.cpp:90-115):
// dF_alias = dF 2 c y/(1+y^2)^2; sums v.dF_alias; maxima |dF|, |dF_alias|.
struct FFirePost {
  const double *dF, *x, *v;
  double* dFa;
  double c;
  __device__ void operator()(long i, double* s, double* m) const {
    const double y = x[i], g = dF[i];
    const double ga = g * (2 * c * y / ((1 + y * y) * (1 + y * y)));
    dFa[i] = ga;
    s[0] = v[i] * ga;
    m[0] = fabs(g);
    m[1] = fabs(ga);
  }
};

// DDFT right-hand side (DDFT::calculate_excess_RHS, g_dot_x, subtract_ideal_gas;
// src/DDFT.cpp:212-235, 320-351): R = g.dF / dV - Laplacian_h rho with
// g.x = sum_axes D [(rho+ + rho0)(x+ - x0) - (rho0 + rho-)(x0 - x-)], D = 1/(2 dx^2).
struct FDdftRhs {
  const double *rho, *dF;
  double* R;
  int nx, ny, nz;
  double dx, dV;
  int fixed;  // a fixed background: g.x = 0 on the boundary (src/DDFT.cpp:333-338)
  __device__ void operator()(long p, double*, double* m) const {
    const int k = (int)(p % nz);
    const long t = p / nz;
    const int j = (int)(t % ny), i = (int)(t / ny);
    auto at = [&](int a, int b, int c) -> long {
      a = (a + nx) % nx; b = (b + ny) % ny; c = (c + nz) % nz;
      return c + (long)nz * (b + (long)ny * a);
    };
    const long px = at(i + 1, j, k), mx = at(i - 1, j, k), py = at(i, j + 1, k), my = at(i, j - 1, k), pz = at(i, j, k + 1), mz = at(i, j, k - 1);
    const double D = 1.0 / (2 * dx * dx);
    const double x0 = dF[p], d0 = rho[p];
    double g = D * ((rho[px] + d0) * (dF[px] - x0) - (d0 + rho[mx]) * (x0 - dF[mx]));
    g += D * ((rho[py] + d0) * (dF[py] - x0) - (d0 + rho[my]) * (x0 - dF[my]));
    g += D * ((rho[pz] + d0) * (dF[pz] - x0) - (d0 + rho[mz]) * (x0 - dF[mz]));
    g *= 1.0 / dV;
    if (fixed && cdft_on_boundary(p, ny, nz)) g = 0.0;
    m[0] = fabs(g);
    const double L = 1.0 / (dx * dx);
    R[p] = g + (-L * (rho[px] + rho[mx] - 2 * d0) - L * (rho[py] + rho[my] - 2 * d0) - L * (rho[pz] + rho[mz] - 2 * d0));
  }
};
// DDFT::apply_diffusion_propogator k-space update (src/DDFT.cpp:239-273):
// work = U0 rho0~ + U1 R0~ + U2 (R1~ - R0~), U0 = e^{L dt}, U1 = (e^{L dt}-1)/L,
// U2 = (e^{L dt}-1-L dt)/(L^2 dt); at k = 0: U1 = dt, U2 = dt/2.
template <class T>
__global__ void k_ddft_prop(const typename Cx<T>::type* __restrict__ rk, const typename Cx<T>::type* __restrict__ R0,
                            const typename Cx<T>::type* __restrict__ R1, typename Cx<T>::type* __restrict__ out,
                            const double* __restrict__ fac, int nx, int ny, int nzc, int pz, double dt) {
  const long Nc = (long)nx * ny * pz;  // padded rows; columns kz >= nzc carry no data
  const double* Lx = fac;
  const double* Ly = Lx + nx;
  const double* Lz = Ly + ny;
  const double* fx = Lz + nzc;
  const double* fy = fx + nx;
  const double* fz = fy + ny;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Nc; p += (long)gridDim.x * blockDim.x) {
    const int iz = (int)(p % pz);
    const long t = p / pz;
    const int iy = (int)(t % ny), ix = (int)(t / ny);
    if (iz >= nzc) {
      out[p] = mk<T>(0, 0);
      continue;
    }
    const double Lam = Lx[ix] + Ly[iy] + Lz[iz];
    const double e = fx[ix] * fy[iy] * fz[iz];
    const double U0 = e;
    const double U1 = (p == 0 ? dt : (e - 1) / Lam);
    const double U2 = (p == 0 ? dt / 2 : (e - 1 - dt * Lam) / (Lam * Lam * dt));
    const typename Cx<T>::type x = rk[p], a = R0[p], b = R1[p];  // p == 0 is the k = 0 mode in either layout
    out[p] = mk<T>((T)(U0 * (double)x.x + U1 * (double)a.x + U2 * ((double)b.x - (double)a.x)),
                   (T)(U0 * (double)x.y + U1 * (double)a.y + U2 * ((double)b.y - (double)a.y)));
  }
}
struct FDdftDev {
  const double *d1, *dn;
  __device__ void operator()(long i, double*, double* m) const {
    m[0] = fabs(d1[i] - dn[i]);
    m[1] = -dn[i];  // max(-x) = -min(x)
  }
};

constexpr long kRedPartLen = 152 * 8 * 16;  // doubles in red_part: 16 per block of the largest grid_for grid
unsigned grid_for(long n) { return (unsigned)std::max<long>(1, std::min<long>((n + 255) / 256, 152 * 8)); }

}  // namespace

static int fail(cdft_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  return code;
}
#define CUDA_OR_FAIL(c, x)                                                                  \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) return fail(c, CDFT_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// FMT_AO_Species: the polymer weights (FMT_Species::generateWeights at diameter 2 Rp,
// src/FMT_Species.cpp:645-664) computed on the host and handed to an evaluator.
template <class T>
static int ensure_ao_host(cdft_ctx* c, Evaluator<T>* e, std::string* err) {
  std::vector<double> wp[11];
  try {
    fmt_weights_real(c->p.nx, c->p.ny, c->p.nz, c->p.dx, 2 * c->p.ao_rp, wp);
  } catch (std::exception& ex) {
    *err = ex.what();
    return CDFT_ERR_ARG;
  }
  return e->enable_ao(2 * c->p.ao_rp, c->p.ao_reservoir, wp, nullptr, c->stream, err);
}

static int ensure_evaluator(cdft_ctx* c, int precision) {
  const int nx = c->p.nx, ny = c->p.ny, nz = c->p.nz;
  if ((precision == CDFT_FP64 && c->e64) || (precision == CDFT_FP32 && c->e32)) return CDFT_OK;
  std::vector<double> w[11], watt;
  const bool fmt = c->p.model >= 0;
  std::string err;
  int rc;
  if (precision == CDFT_FP32 && c->e64) {  // round the FP64 evaluator's weight spectra instead of recomputing them
    c->e32.reset(new Evaluator<float>());
    rc = c->e32->init(nx, ny, nz, c->p.model, c->info.hsd, c->p.es_A, c->p.es_B, nullptr, nullptr, c->tx.get(), c->ty.get(),
                      c->tz.get(), c->stream, &err, fmt ? c->e64->weight_spectra() : nullptr,
                      c->p.lj ? c->e64->att_spectrum() : nullptr);
    if (!rc && c->p.ao_rp > 0)
      rc = c->e64->has_ao() ? c->e32->enable_ao(2 * c->p.ao_rp, c->p.ao_reservoir, nullptr, c->e64->ao_spectra(), c->stream, &err)
                            : ensure_ao_host(c, c->e32.get(), &err);
    if (rc) {
      c->e32.reset();
      return fail(c, rc, err);
    }
    return CDFT_OK;
  }
  try {
    if (fmt) fmt_weights_real(nx, ny, nz, c->p.dx, c->info.hsd, w);
    if (c->p.lj) {
      double a;
      qf_kernel_real(nx, ny, nz, c->p.dx, c->p.lj_sigma, c->p.lj_eps, c->p.lj_rc, c->p.kT, watt, a);
    }
  } catch (std::exception& e) {
    return fail(c, CDFT_ERR_ARG, e.what());
  }
  if (precision == CDFT_FP64) {
    c->e64.reset(new Evaluator<double>());
    rc = c->e64->init(nx, ny, nz, c->p.model, c->info.hsd, c->p.es_A, c->p.es_B, fmt ? w : nullptr, c->p.lj ? &watt : nullptr, c->tx.get(),
                      c->ty.get(), c->tz.get(), c->stream, &err);
    if (!rc && c->p.ao_rp > 0) rc = ensure_ao_host(c, c->e64.get(), &err);
    if (rc) c->e64.reset();
  } else {
    c->e32.reset(new Evaluator<float>());
    rc = c->e32->init(nx, ny, nz, c->p.model, c->info.hsd, c->p.es_A, c->p.es_B, fmt ? w : nullptr, c->p.lj ? &watt : nullptr, c->tx.get(),
                      c->ty.get(), c->tz.get(), c->stream, &err);
    if (!rc && c->p.ao_rp > 0) rc = ensure_ao_host(c, c->e32.get(), &err);
    if (rc) c->e32.reset();
  }
  if (rc) return fail(c, rc, err);
  return CDFT_OK;
}

template <int NS, int NM, class F>
static int map_reduce(cdft_ctx* c, long n, F f, double* host_out) {
  const unsigned g = grid_for(n);
  k_map_reduce<NS, NM, F><<<g, 256, 0, c->stream>>>(n, f, c->red_part);
  k_finish_map_reduce<<<1, kFinishThreads, 0, c->stream>>>(c->red_part, (int)g, NS, NM, c->red_out);
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->host_out, c->red_out, (NS + NM) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  std::memcpy(host_out, c->host_out, (NS + NM) * sizeof(double));
  return CDFT_OK;
}

// One evaluation on the context's density: Species::beginForceCalculation,
// DFT::calculateFreeEnergyAndDerivatives_internal_, Species::endForceCalculation.
// Grand-canonical evaluation as one graph launch and one synchronisation:
// the pass sequence, max|dF| and the copies of every sum to pinned memory.
static int eval_graph(cdft_ctx* c, double* terms8, int only_fex, double* mirror = nullptr) {
  const long N = c->info.N;
  const double dV = c->info.dV;
  const int gi = c->precision == CDFT_FP64 ? 1 : 0;
  cudaGraphExec_t& exec = c->eval_exec[gi];
  if (!exec || c->eg_only_fex[gi] != only_fex || c->eg_vext[gi] != c->vext || c->eg_mu[gi] != c->mu ||
      c->eg_plan_gen[gi] != c->plan_gen || c->eg_mirror[gi] != mirror) {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    if (!c->cap_stream) CUDA_OR_FAIL(c, cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    if (!c->host_status) CUDA_OR_FAIL(c, cudaMallocHost(&c->host_status, sizeof(unsigned)));
    cudaStream_t s = c->cap_stream;
    cudaGraph_t g;
    CUDA_OR_FAIL(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc;
    // the final row pass stores the dF-norm partials itself when they fit red_part
    const long fb = c->precision == CDFT_FP64 ? c->e64->final_blocks() : c->e32->final_blocks();
    double* nrm = 2 * fb <= kRedPartLen ? c->red_part : nullptr;
    if (c->precision == CDFT_FP64) rc = c->e64->launch(c->rho, c->vext, c->dF, dV, c->mu, only_fex ? 0 : 1, s, nullptr, nrm, mirror);
    else rc = c->e32->launch(c->rho, c->vext, c->dF, dV, c->mu, only_fex ? 0 : 1, s, nullptr, nrm, mirror);
    if (nrm) {
      k_dF_norms_finish<<<1, 256, 0, s>>>(c->red_part, (int)fb, c->red_out);
    } else {
      const unsigned gr = grid_for(N);
      k_dF_norms<<<gr, 256, 0, s>>>(c->dF, N, c->red_part);
      k_dF_norms_finish<<<1, 256, 0, s>>>(c->red_part, (int)gr, c->red_out);
    }
    const double* dterms = c->precision == CDFT_FP64 ? c->e64->dev_terms() : c->e32->dev_terms();
    const unsigned* dst = c->precision == CDFT_FP64 ? c->e64->dev_status() : c->e32->dev_status();
    cudaMemcpyAsync(c->host_out, dterms, 8 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(c->host_out + 8, c->red_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(c->host_status, dst, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (rc || ce != cudaSuccess) return fail(c, CDFT_ERR_CUDA, "evaluation graph capture failed");
    const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      exec = nullptr;
      return fail(c, CDFT_ERR_CUDA, "evaluation graph instantiate failed");
    }
    c->eg_only_fex[gi] = only_fex;
    c->eg_vext[gi] = c->vext;
    c->eg_mu[gi] = c->mu;
    c->eg_plan_gen[gi] = c->plan_gen;
    c->eg_mirror[gi] = mirror;
  }
  CUDA_OR_FAIL(c, cudaGraphLaunch(exec, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  EvalTerms t;
  int rc = c->precision == CDFT_FP64 ? c->e64->terms_from(c->host_out, *c->host_status, dV, c->mu, &t)
                                     : c->e32->terms_from(c->host_out, *c->host_status, dV, c->mu, &t);
  if (rc == 3) return fail(c, CDFT_ERR_TIMEOUT, "a tensor copy did not complete within its wait limit");
  if (rc) return fail(c, CDFT_ERR_CUDA, "evaluation failed");
  if (terms8) {
    terms8[0] = t.Omega;
    terms8[1] = t.F_id;
    terms8[2] = t.F_hs;
    terms8[3] = t.F_mf;
    terms8[4] = t.F_ext;
    terms8[5] = c->mu;
    terms8[6] = c->host_out[9] / dV;
    terms8[7] = t.sum_rho * dV;
  }
  c->last_dF_l2 = std::sqrt(c->host_out[8]) / dV;
  if (t.status & 1u) return fail(c, CDFT_ERR_ETA, "Eta too large in FMT::dPHI");
  return CDFT_OK;
}

__global__ void k_boundary_set(double* __restrict__ a, long N, int ny, int nz, double value) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < N; p += (long)gridDim.x * blockDim.x)
    if (cdft_on_boundary(p, ny, nz)) a[p] = value;
}
__global__ void k_boundary_copy(double* __restrict__ a, const double* __restrict__ b, long N, int ny, int nz) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < N; p += (long)gridDim.x * blockDim.x)
    if (cdft_on_boundary(p, ny, nz)) a[p] = b[p];
}
void cdft_internal_boundary_set(cdft_ctx* c, double* a, double value) {
  k_boundary_set<<<grid_for(c->info.N), 256, 0, c->stream>>>(a, c->info.N, c->p.ny, c->p.nz, value);
}

// mirror (optional, device-visible): the graph path's final pass also stores dF there;
// *mirrored tells whether it did.
static int eval_internal(cdft_ctx* c, double* terms8, int only_fex = 0, double* mirror = nullptr, bool* mirrored = nullptr) {
  const long N = c->info.N;
  const double dV = c->info.dV;
  int rc = ensure_evaluator(c, c->precision);
  if (rc) return rc;
  if (mirrored) *mirrored = false;
  if (c->fixed_mass <= 0 && !c->fixed_bg && !c->homo_bd) {
    if (mirrored) *mirrored = mirror != nullptr;
    return eval_graph(c, terms8, only_fex, mirror);
  }
  if (c->fixed_bg && c->fixed_mass > 0)  // src/Species.cpp:75-76
    return fail(c, CDFT_ERR_ARG, "Cannot have both fixed background and fixed mass .... aborting");
  if (c->fixed_mass > 0) {  // src/Species.cpp:64-71
    double s;
    rc = map_reduce<1, 0>(c, N, FSumRho{c->rho}, &s);
    if (rc) return rc;
    k_scale_vec<<<grid_for(N), 256, 0, c->stream>>>(c->rho, N, c->fixed_mass / (s * dV));
    c->mu = 0.0;
  }
  EvalTerms t;
  if (c->precision == CDFT_FP64) rc = c->e64->eval(c->rho, c->vext, c->dF, dV, c->mu, only_fex ? 0 : 1, &t, c->stream);
  else rc = c->e32->eval(c->rho, c->vext, c->dF, dV, c->mu, only_fex ? 0 : 1, &t, c->stream);
  if (rc == 3) return fail(c, CDFT_ERR_TIMEOUT, "a tensor copy did not complete within its wait limit");
  if (rc) return fail(c, CDFT_ERR_CUDA, std::string("evaluation launch failed: ") + cudaGetErrorString(cudaGetLastError()));
  if (c->fixed_bg) cdft_internal_boundary_set(c, c->dF, 0.0);  // src/Species.cpp:78-82
  if (c->homo_bd) {                                            // src/Species.cpp:84-95
    double sb;
    rc = map_reduce<1, 0>(c, N, FBoundarySum{c->dF, c->p.ny, c->p.nz}, &sb);
    if (rc) return rc;
    cdft_internal_boundary_set(c, c->dF, sb / (double)cdft_n_boundary(c->p.nx, c->p.ny, c->p.nz));
    if (c->fixed_mass > 0) {  // the fixed-mass sum sees the averaged boundary
      rc = map_reduce<1, 0>(c, N, FSumDot{c->dF, c->rho}, &t.sum_dF_rho);
      if (rc) return rc;
    }
  }
  if (c->fixed_mass > 0) {  // src/Species.cpp:97-109
    c->mu = t.sum_dF_rho / c->fixed_mass;
    k_add_const<<<grid_for(N), 256, 0, c->stream>>>(c->dF, N, c->mu * dV);
  }
  double sq_mx[2];
  {
    const unsigned gr = grid_for(N);
    k_dF_norms<<<gr, 256, 0, c->stream>>>(c->dF, N, c->red_part);
    k_dF_norms_finish<<<1, 256, 0, c->stream>>>(c->red_part, (int)gr, c->red_out);
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->host_out, c->red_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    sq_mx[0] = c->host_out[0];
    sq_mx[1] = c->host_out[1];
  }
  const double mx = sq_mx[1];
  c->last_dF_l2 = std::sqrt(sq_mx[0]) / dV;
  if (terms8) {
    terms8[0] = t.Omega;
    terms8[1] = t.F_id;
    terms8[2] = t.F_hs;
    terms8[3] = t.F_mf;
    terms8[4] = t.F_ext;
    terms8[5] = c->mu;
    terms8[6] = mx / dV;
    terms8[7] = t.sum_rho * dV;
  }
  if (t.status & 1u) return fail(c, CDFT_ERR_ETA, "Eta too large in FMT::dPHI");
  return CDFT_OK;
}

int cdft_internal_fail(cdft_ctx* c, int code, const std::string& m) { return fail(c, code, m); }
int cdft_internal_eval(cdft_ctx* c, double* terms8, int only_fex) { return eval_internal(c, terms8, only_fex); }

extern "C" {

int cdft_create(const cdft_params* p, cdft_ctx** out) {
  if (!p || !out) return CDFT_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<cdft_ctx> c(new cdft_ctx());
  c->p = *p;
  if (p->nx < 2 || p->ny < 2 || p->nz < 2 || !(p->dx > 0)) return fail(nullptr, CDFT_ERR_ARG, "bad lattice");
  if (p->precision != CDFT_FP64 && p->precision != CDFT_FP32) return CDFT_ERR_ARG;
  if (p->model < -1 || p->model > 4) return CDFT_ERR_ARG;
  cudaGetDevice(&c->device);
  c->stream = nullptr;
  c->precision = p->precision;
  c->mu = p->mu;
  c->fixed_mass = p->fixed_mass;
  if (p->fixed_mass > 0) c->mu = 0.0;
  c->info.nx = p->nx; c->info.ny = p->ny; c->info.nz = p->nz;
  c->info.N = (long)p->nx * p->ny * p->nz;
  c->info.Nc = (long)p->nx * p->ny * (p->nz / 2 + 1);
  c->info.dV = p->dx * p->dx * p->dx;
  c->info.volume = c->info.N * c->info.dV;
  c->info.hsd = p->hsd;
  if (p->lj && p->hsd <= 0) c->info.hsd = bh_diameter_lj(p->lj_sigma, p->lj_eps, p->lj_rc, p->kT);
  if (p->model >= 0 && !(c->info.hsd >= p->dx)) return CDFT_ERR_ARG;  // generateWeights throws for hsd < dx
  if (p->ao_rp > 0 && (p->model < 0 || !(2 * p->ao_rp >= p->dx) || !(p->ao_reservoir >= 0)))
    return fail(nullptr, CDFT_ERR_ARG, "the AO model needs an FMT model, polymer diameter >= dx and a reservoir density >= 0");
  if (p->lj) {
    std::vector<double> w;
    double a;
    qf_kernel_real(2, 2, 2, p->dx, p->lj_sigma, p->lj_eps, p->lj_rc, p->kT, w, a);  // a_vdw does not depend on the box
    c->info.a_vdw = a;
  }
  std::string err;
  c->tx = make_fft_table(p->nx, &err);
  c->ty = (p->ny == p->nx) ? c->tx : make_fft_table(p->ny, &err);
  c->tz = (p->nz == p->nx) ? c->tx : (p->nz == p->ny ? c->ty : make_fft_table(p->nz, &err));
  if (!c->tx || !c->ty || !c->tz) return CDFT_ERR_ARG;
  std::array<std::vector<int>, 3> tuned;
  if (cdft_internal_tuned_plans(c.get(), c->precision, &tuned)) {  // cdft_autotune ran for this shape
    c->tx = make_fft_table(p->nx, &err, &tuned[0]);
    c->ty = make_fft_table(p->ny, &err, &tuned[1]);
    c->tz = make_fft_table(p->nz, &err, &tuned[2]);
    if (!c->tx || !c->ty || !c->tz) return CDFT_ERR_ARG;
  }
  const long N = c->info.N;
  if (cudaMalloc(&c->rho, N * sizeof(double)) != cudaSuccess || cudaMalloc(&c->dF, N * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->red_part, (size_t)kRedPartLen * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->red_out, 16 * sizeof(double)) != cudaSuccess || cudaMallocHost(&c->host_out, 16 * sizeof(double)) != cudaSuccess)
    return CDFT_ERR_CUDA;
  cudaMemset(c->rho, 0, N * sizeof(double));
  cudaMemset(c->dF, 0, N * sizeof(double));
  int rc = ensure_evaluator(c.get(), c->precision);
  if (rc) return rc;
  *out = c.release();
  return CDFT_OK;
}

int cdft_destroy(cdft_ctx* c) {
  if (!c) return CDFT_OK;
  cudaStreamSynchronize(c->stream);
  cdft_internal_fire_dev_free(c);
  cdft_internal_newton_free(c);
  c->e64.reset();
  c->e32.reset();
  cudaFree(c->rho); cudaFree(c->dF); cudaFree(c->vext); cudaFree(c->red_part); cudaFree(c->red_out); cudaFreeHost(c->host_out);
  for (int i = 0; i < 2; ++i) { cudaFree(c->fx[i]); cudaFree(c->fv[i]); cudaFree(c->fg[i]); }
  cudaFree(c->dd0); cudaFree(c->dd1); cudaFree(c->ddn); cudaFree(c->dR); cudaFree(c->dfac);
  cudaFree(c->rk0); cudaFree(c->R0k); cudaFree(c->R1k); cudaFree(c->work);
  cudaFree(c->hv_v); cudaFree(c->hv_out);
  for (cudaGraphExec_t ge : c->eval_exec)
    if (ge) cudaGraphExecDestroy(ge);
  if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
  cudaFreeHost(c->host_status);
  delete c;
  return CDFT_OK;
}

const char* cdft_last_error(const cdft_ctx* c) { return c ? c->err.c_str() : "no context"; }

int cdft_set_stream(cdft_ctx* c, void* s) {
  if (!c) return CDFT_ERR_ARG;
  cudaStreamSynchronize(c->stream);
  c->stream = (cudaStream_t)s;
  return CDFT_OK;
}

int cdft_get_info(const cdft_ctx* c, cdft_info* out) {
  if (!c || !out) return CDFT_ERR_ARG;
  *out = c->info;
  return CDFT_OK;
}

int cdft_set_precision(cdft_ctx* c, int precision) {
  if (!c || (precision != CDFT_FP64 && precision != CDFT_FP32)) return CDFT_ERR_ARG;
  int rc = ensure_evaluator(c, precision);
  if (rc) return rc;
  c->precision = precision;
  return CDFT_OK;
}

int cdft_set_density(cdft_ctx* c, const double* rho, int on_device) {
  if (!c || !rho) return CDFT_ERR_ARG;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rho, rho, c->info.N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return CDFT_OK;
}

int cdft_get_density(const cdft_ctx* c, double* rho, int on_device) {
  if (!c || !rho) return CDFT_ERR_ARG;
  if (cudaMemcpyAsync(rho, c->rho, c->info.N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream) !=
      cudaSuccess)
    return CDFT_ERR_CUDA;
  return cudaStreamSynchronize(c->stream) == cudaSuccess ? CDFT_OK : CDFT_ERR_CUDA;
}

int cdft_set_external_field(cdft_ctx* c, const double* v, int on_device) {
  if (!c) return CDFT_ERR_ARG;
  if (!v) {
    cudaFree(c->vext);
    c->vext = nullptr;
    return CDFT_OK;
  }
  if (!c->vext) CUDA_OR_FAIL(c, cudaMalloc(&c->vext, c->info.N * sizeof(double)));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->vext, v, c->info.N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return CDFT_OK;
}

int cdft_set_chem_potential(cdft_ctx* c, double mu) {
  if (!c) return CDFT_ERR_ARG;
  c->mu = mu;
  c->fixed_mass = -1;
  return CDFT_OK;
}
int cdft_set_fixed_mass(cdft_ctx* c, double m) {
  if (!c) return CDFT_ERR_ARG;
  c->fixed_mass = m;
  if (m > 0.0) c->mu = 0.0;
  return CDFT_OK;
}
int cdft_get_chem_potential(const cdft_ctx* c, double* mu) {
  if (!c || !mu) return CDFT_ERR_ARG;
  *mu = c->mu;
  return CDFT_OK;
}
int cdft_set_boundary(cdft_ctx* c, int fixed_background, int homogeneous) {
  if (!c) return CDFT_ERR_ARG;
  c->fixed_bg = fixed_background ? 1 : 0;
  c->homo_bd = homogeneous ? 1 : 0;
  return CDFT_OK;
}

// DFT::matrix_dot_v1 with the full Hessian (src/Dynamical_Matrix.cpp,
// src/DFT.cpp:435-488; FMT::add_second_derivative src/FMT.cpp:437-567;
// Interaction_Base::add_second_derivative src/Interaction.cpp:119-147), at the
// context's current density.
// DDFT::g_dot_x (src/DDFT.cpp:320-351), forward differences: the DDFT mobility
// operator gx = sum_axes D [(rho+ + rho0)(x+ - x0) - (rho0 + rho-)(x0 - x-)], D = 1/(2 dx^2).
__global__ void k_g_dot_x(const double* __restrict__ rho, const double* __restrict__ x, double* __restrict__ gx, int nx, int ny, int nz,
                          double dx) {
  const long N = (long)nx * ny * nz;
  const double D = 1.0 / (2 * dx * dx);
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < N; p += (long)gridDim.x * blockDim.x) {
    const int k = (int)(p % nz);
    const long t = p / nz;
    const int j = (int)(t % ny), i = (int)(t / ny);
    auto at = [&](int a, int b, int c) -> long {
      a = (a + nx) % nx; b = (b + ny) % ny; c = (c + nz) % nz;
      return c + (long)nz * (b + (long)ny * a);
    };
    const long px = at(i + 1, j, k), mx = at(i - 1, j, k), py = at(i, j + 1, k), my = at(i, j - 1, k), pz = at(i, j, k + 1),
               mz = at(i, j, k - 1);
    const double x0 = x[p], d0 = rho[p];
    double g = D * ((rho[px] + d0) * (x[px] - x0) - (d0 + rho[mx]) * (x0 - x[mx]));
    g += D * ((rho[py] + d0) * (x[py] - x0) - (d0 + rho[my]) * (x0 - x[my]));
    g += D * ((rho[pz] + d0) * (x[pz] - x0) - (d0 + rho[mz]) * (x0 - x[mz]));
    gx[p] = g;
  }
}

// H v between device arrays on the context's stream (asynchronous).
static int hessian_device(cdft_ctx* c, const double* vd, double* od) {
  int rc = c->precision == CDFT_FP64 ? c->e64->hess_prepare(c->rho, c->stream) : c->e32->hess_prepare(c->rho, c->stream);
  if (!rc)
    rc = c->precision == CDFT_FP64 ? c->e64->hess_apply<double>(vd, c->rho, od, c->info.dV, c->stream)
                                   : c->e32->hess_apply<double>(vd, c->rho, od, c->info.dV, c->stream);
  return rc ? fail(c, CDFT_ERR_CUDA, "Hessian launch failed") : CDFT_OK;
}

static int hessian_buffers(cdft_ctx* c) {
  int rc = ensure_evaluator(c, c->precision);
  if (rc) return rc;
  const size_t nb = c->info.N * sizeof(double);
  if (!c->hv_v && (cudaMalloc(&c->hv_v, nb) != cudaSuccess || cudaMalloc(&c->hv_out, nb) != cudaSuccess))
    return fail(c, CDFT_ERR_CUDA, "Hessian buffers");
  return CDFT_OK;
}

// The product's input on the device: the caller's array, or hv_v holding a copy (from the
// host, or with its boundary entries zeroed under a fixed background, as
// Dynamical_Matrix::matrix_dot_v1 zeroes them, src/Dynamical_Matrix.cpp).
static int product_input(cdft_ctx* c, const double* v, int on_device, const double** vd) {
  *vd = v;
  if (on_device && !c->fixed_bg) return CDFT_OK;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->hv_v, v, c->info.N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  c->stream));
  if (c->fixed_bg) cdft_internal_boundary_set(c, c->hv_v, 0.0);
  *vd = c->hv_v;
  return CDFT_OK;
}

int cdft_hessian_dot_v(cdft_ctx* c, const double* v, double* out, int on_device) {
  if (!c || !v || !out) return CDFT_ERR_ARG;
  int rc = hessian_buffers(c);
  if (rc) return rc;
  const size_t nb = c->info.N * sizeof(double);
  const double* vd = v;
  double* od = on_device ? out : c->hv_out;
  rc = product_input(c, v, on_device, &vd);
  if (rc) return rc;
  rc = hessian_device(c, vd, od);
  if (rc) return rc;
  if (c->fixed_bg) cdft_internal_boundary_set(c, od, 0.0);  // src/DFT.cpp:480-487
  if (!on_device) CUDA_OR_FAIL(c, cudaMemcpyAsync(out, od, nb, cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return CDFT_OK;
}

// y = M x between device arrays, M the Hessian (matrix 0) or the DDFT matrix g . H
// (matrix 1), for the spectral drivers; prepare = true first stores the weighted
// densities of the current density. x and y must not be the context's hv_out.
// (C++ linkage: an internal helper between the ABI's entry points.)
}  // extern "C"
int cdft_internal_matvec(cdft_ctx* c, int matrix, const double* x, double* y, bool prepare) {
  int rc = hessian_buffers(c);
  if (rc) return rc;
  if (prepare) {
    rc = c->precision == CDFT_FP64 ? c->e64->hess_prepare(c->rho, c->stream) : c->e32->hess_prepare(c->rho, c->stream);
    if (rc) return fail(c, CDFT_ERR_CUDA, "Hessian prepare failed");
  }
  double* hv = matrix == 0 ? y : c->hv_out;
  if (c->fixed_bg) {  // zero boundary entries in, zero boundary entries out
    rc = product_input(c, x, 1, &x);
    if (rc) return rc;
  }
  rc = c->precision == CDFT_FP64 ? c->e64->hess_apply<double>(x, c->rho, hv, c->info.dV, c->stream)
                                 : c->e32->hess_apply<double>(x, c->rho, hv, c->info.dV, c->stream);
  if (rc) return fail(c, CDFT_ERR_CUDA, "Hessian launch failed");
  if (c->fixed_bg) cdft_internal_boundary_set(c, hv, 0.0);
  if (matrix != 0) {
    k_g_dot_x<<<grid_for(c->info.N), 256, 0, c->stream>>>(c->rho, hv, y, c->p.nx, c->p.ny, c->p.nz, c->p.dx);
    if (c->fixed_bg) cdft_internal_boundary_set(c, y, 0.0);
  }
  return cudaGetLastError() == cudaSuccess ? CDFT_OK : fail(c, CDFT_ERR_CUDA, "matrix product launch failed");
}
extern "C" {

// DDFT::matrix_dot_v_intern (src/DDFT.cpp:353-361): g . (H v) at the current density.
int cdft_ddft_matrix_dot_v(cdft_ctx* c, const double* v, double* out, int on_device) {
  if (!c || !v || !out) return CDFT_ERR_ARG;
  int rc = hessian_buffers(c);
  if (rc) return rc;
  const size_t nb = c->info.N * sizeof(double);
  // v -> H v in hv_out -> g . (H v) in hv_v (v is no longer needed) or the caller's array
  const double* vd = v;
  rc = product_input(c, v, on_device, &vd);
  if (rc) return rc;
  rc = hessian_device(c, vd, c->hv_out);
  if (rc) return rc;
  if (c->fixed_bg) cdft_internal_boundary_set(c, c->hv_out, 0.0);
  double* gd = on_device ? out : c->hv_v;
  k_g_dot_x<<<grid_for(c->info.N), 256, 0, c->stream>>>(c->rho, c->hv_out, gd, c->p.nx, c->p.ny, c->p.nz, c->p.dx);
  if (c->fixed_bg) cdft_internal_boundary_set(c, gd, 0.0);  // src/DDFT.cpp:333-338
  if (!on_device) CUDA_OR_FAIL(c, cudaMemcpyAsync(out, gd, nb, cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  return CDFT_OK;
}

int cdft_eval(cdft_ctx* c, int only_fex, double* terms, double* dF, int on_device) {
  if (!c) return CDFT_ERR_ARG;
  // a page-locked host dF: the final row pass writes it directly (over the host link while
  // the pass runs) instead of a copy after the evaluation
  double* mirror = nullptr;
  if (dF && !on_device) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, dF) == cudaSuccess) {
      if (a.type == cudaMemoryTypeHost && a.devicePointer) mirror = static_cast<double*>(a.devicePointer);
    } else {
      cudaGetLastError();  // not a CUDA-known pointer: the copy path below
    }
  }
  bool mirrored = false;
  int rc = eval_internal(c, terms, only_fex, mirror, &mirrored);
  if (dF && !mirrored && (rc == CDFT_OK || rc == CDFT_ERR_ETA)) {
    if (cudaMemcpyAsync(dF, c->dF, c->info.N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      return fail(c, CDFT_ERR_CUDA, "copy of dF failed");
  }
  return rc;
}

// ------------------------------------------------ bulk phase equilibria ---
// DFT::findSpinodal / find_density_from_mu / findCoex (src/DFT_Coex.cpp:53-196):
// golden-section search for the stationary points of the pressure p = -omega,
// bisection on mu, and bisection on the pressure difference along mu(x_vap) = mu(x_liq).
namespace {
struct Bulk {
  const cdft_ctx* c;
  double mu(double x) const { double o[3]; cdft_bulk(c, x, o); return o[0]; }
  double p(double x) const { double o[3]; cdft_bulk(c, x, o); return -o[1]; }
};
bool spinodal(const Bulk& B, double xmax, double dx, double& xs1, double& xs2, double tol) {
  double x = 2 * dx, p = B.p(2 * dx), dp = p - B.p(dx);
  if (dp < 0) return false;
  while (dp > 0 && x < xmax - dx) { dp = -p; x += dx; p = B.p(x); dp += p; }
  if (x >= xmax - dx) return false;
  const double r = (3 - std::sqrt(5.0)) / 2;
  double a = x - 2 * dx, b = x, u = a + r * (b - a), v = b - r * (b - a), fu = B.p(u), fv = B.p(v);
  do {
    if (fu > fv) { b = v; v = u; fv = fu; u = a + r * (b - a); fu = B.p(u); }
    else { a = u; u = v; fu = fv; v = b - r * (b - a); fv = B.p(v); }
  } while (b - a > 1e-8);
  xs1 = (a + b) / 2;
  x = xs1;
  p = B.p(x);
  do { dp = -p; x += dx; p = B.p(x); dp += p; } while (dp < 0 && x < xmax - dx);
  if (x >= xmax - dx) return false;
  a = x - 2 * dx; b = x; u = a + r * (b - a); v = b - r * (b - a); fu = B.p(u); fv = B.p(v);
  do {
    if (fu < fv) { b = v; v = u; fv = fu; u = a + r * (b - a); fu = B.p(u); }
    else { a = u; u = v; fu = fv; v = b - r * (b - a); fv = B.p(v); }
  } while (b - a > tol);
  xs2 = (a + b) / 2;
  return true;
}
bool density_from_mu(const Bulk& B, double mu, double xmin, double xmax, double tol, double& out) {
  double mu1 = B.mu(xmin), mu2 = B.mu(xmax);
  if (mu1 > mu2) { std::swap(xmin, xmax); std::swap(mu1, mu2); }
  if (mu2 < mu || mu1 > mu) return false;
  do {
    const double x = (xmin + xmax) / 2, m = B.mu(x);
    if (m > mu) { xmax = x; mu2 = m; }
    else { xmin = x; mu1 = m; }
  } while (mu2 - mu1 > tol);
  out = (xmin + xmax) / 2;
  return true;
}
}  // namespace

int cdft_find_coex(const cdft_ctx* c, double xmax, double dx, double tol, double* out) {
  if (!c || !out || !(xmax > 0) || !(dx > 0) || !(tol > 0)) return CDFT_ERR_ARG;
  const Bulk B{c};
  double xs1, xs2;
  if (!spinodal(B, xmax, dx, xs1, xs2, tol)) return CDFT_ERR_ARG;
  double xvap = xs1, xliq;
  if (!density_from_mu(B, B.mu(xvap), xs2, xmax - dx, tol, xliq)) return CDFT_ERR_ARG;
  double dp1 = B.p(xvap) - B.p(xliq), dp2;
  do {
    dp2 = dp1;
    xvap /= 1.1;
    if (!density_from_mu(B, B.mu(xvap), xs2, xmax - dx, tol, xliq)) return CDFT_ERR_ARG;
    dp1 = B.p(xvap) - B.p(xliq);
  } while (xvap > 1e-16 && ((dp1 < 0) == (dp2 < 0)));
  if (xvap < 1e-16) return CDFT_ERR_ARG;
  double y1 = xvap, y2 = xvap * 1.1;
  do {
    const double y = (y1 + y2) / 2;
    if (!density_from_mu(B, B.mu(y), xs2, xmax - dx, tol, xliq)) return CDFT_ERR_ARG;
    const double dp = B.p(y) - B.p(xliq);
    if ((dp < 0) == (dp1 < 0)) { y1 = y; dp1 = dp; }
    else { y2 = y; dp2 = dp; }
  } while (std::fabs(y2 - y1) > tol);
  out[0] = (y1 + y2) / 2;
  out[1] = xliq;
  out[2] = B.mu(out[0]);
  out[3] = xs1;
  out[4] = xs2;
  return CDFT_OK;
}

int cdft_time_passes(cdft_ctx* c, int reps, double* ms, double* bytes, int* npass) {
  if (!c || reps < 1) return CDFT_ERR_ARG;
  int rc = ensure_evaluator(c, c->precision);
  if (rc) return rc;
  cudaEvent_t ev[CDFT_NPASS + 1];
  for (auto& e : ev) cudaEventCreate(&e);
  std::vector<double> acc(CDFT_NPASS, 0.0);
  for (int r = 0; r < reps; ++r) {
    if (c->precision == CDFT_FP64) c->e64->launch(c->rho, c->vext, c->dF, c->info.dV, c->mu, 1, c->stream, ev);
    else c->e32->launch(c->rho, c->vext, c->dF, c->info.dV, c->mu, 1, c->stream, ev);
    CUDA_OR_FAIL(c, cudaEventSynchronize(ev[CDFT_NPASS]));
    for (int i = 0; i < CDFT_NPASS; ++i) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      acc[i] += t;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (ms)
    for (int i = 0; i < CDFT_NPASS; ++i) ms[i] = acc[i] / reps;
  if (bytes) {
    if (c->precision == CDFT_FP64) c->e64->pass_bytes(bytes);
    else c->e32->pass_bytes(bytes);
  }
  if (npass) *npass = CDFT_NPASS;
  return CDFT_OK;
}

int cdft_bulk(const cdft_ctx* c, double rho, double* out3) {
  if (!c || !out3 || !(rho > 0)) return CDFT_ERR_ARG;
  const int m = c->p.model;
  // DFT::mu_times_beta: compensated sum of ln rho, FMT BulkMuex, interaction Mu (src/DFT.cpp:58-71)
  double s = 0, cc = 0;
  auto add = [&](double v) {
    double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) cc += (s - t) + v;
    else cc += (v - t) + s;
    s = t;
  };
  add(std::log(rho));
  const bool ao = m >= 0 && c->p.ao_rp > 0;
  if (m >= 0)  // FMT::BulkMuex, with the AO term when the species is FMT_AO_Species (src/FMT.cpp:616-673)
    add(bulk_muex(m, c->p.es_A, c->p.es_B, c->info.hsd, rho) +
        (ao ? bulk_muex_ao(m, c->p.es_A, c->p.es_B, c->info.hsd, 2 * c->p.ao_rp, c->p.ao_reservoir, rho) : 0.0));
  if (c->p.lj) add(0.5 * c->info.a_vdw * rho + 0.5 * c->info.a_vdw * rho);
  const double mu = s + cc;
  double F = rho * std::log(rho) - rho;  // fhelmholtz_times_beta_over_volume (src/DFT.cpp:90-115)
  if (m >= 0)
    F += bulk_fex(m, c->p.es_A, c->p.es_B, c->info.hsd, rho) +
         (ao ? bulk_fex_ao(m, c->p.es_A, c->p.es_B, c->info.hsd, 2 * c->p.ao_rp, c->p.ao_reservoir, rho) : 0.0);
  if (c->p.lj) F += 0.5 * c->info.a_vdw * rho * rho;
  out3[0] = mu;
  out3[1] = F - rho * mu;
  out3[2] = F;
  return CDFT_OK;
}

int cdft_bh_diameter(double sigma, double eps, double rc, double kT, double* out) {
  if (!out || !(kT > 0) || !(rc > 0)) return CDFT_ERR_ARG;
  *out = bh_diameter_lj(sigma, eps, rc, kT);
  return CDFT_OK;
}

int cdft_fmt_weights(int nx, int ny, int nz, double dx, double hsd, double* w11) {
  if (!w11 || nx < 1 || ny < 1 || nz < 1 || !(dx > 0)) return CDFT_ERR_ARG;
  try {
    std::vector<double> w[11];
    fmt_weights_real(nx, ny, nz, dx, hsd, w);
    const long N = (long)nx * ny * nz;
    for (int a = 0; a < 11; ++a) std::memcpy(w11 + a * N, w[a].data(), N * sizeof(double));
  } catch (std::exception&) {
    return CDFT_ERR_ARG;
  }
  return CDFT_OK;
}

int cdft_get_weights(const cdft_ctx* c, double* w11, double* w_att) {
  if (!c) return CDFT_ERR_ARG;
  const long N = c->info.N;
  try {
    if (w11 && c->p.model >= 0) {
      std::vector<double> w[11];
      fmt_weights_real(c->p.nx, c->p.ny, c->p.nz, c->p.dx, c->info.hsd, w);
      for (int a = 0; a < 11; ++a) std::memcpy(w11 + a * N, w[a].data(), N * sizeof(double));
    }
    if (w_att && c->p.lj) {
      std::vector<double> w;
      double a;
      qf_kernel_real(c->p.nx, c->p.ny, c->p.nz, c->p.dx, c->p.lj_sigma, c->p.lj_eps, c->p.lj_rc, c->p.kT, w, a);
      std::memcpy(w_att, w.data(), N * sizeof(double));
    }
  } catch (std::exception&) {
    return CDFT_ERR_ARG;
  }
  return CDFT_OK;
}

// ------------------------------------------------------------------ FIRE ---
int cdft_fire_default_params(cdft_fire_params* p) {
  if (!p) return CDFT_ERR_ARG;
  // fireMinimizer2 constructor defaults (src/Minimizer.cpp:117-147), Minimizer forceLimit_ (:18)
  p->dt = 1e-3;
  p->dt_max = 1e-2;
  p->dt_min = 0.0;
  p->alpha_start = 0.1;
  p->f_alf = 0.99;
  p->f_dec = 0.5;
  p->f_inc = 1.1;
  p->force_limit = 0.1;
  p->n_delay = 5;
  p->n_p_negative_max = 20;
  p->initial_delay = 1;
  return CDFT_OK;
}

// Minimizer::getDF_DX on the pending alias state xs, vs (device): density from
// alias (already in c->rho), evaluate, convert dF to alias derivative into gs.
static int fire_accept(cdft_ctx* c, int s_idx) {
  double red[3];
  FFirePost f{c->dF, c->fx[s_idx], c->fv[s_idx], c->fg[s_idx], c->alias().c};
  int rc = map_reduce<1, 2>(c, c->info.N, f, red);
  if (rc) return rc;
  c->vdotf = red[0];
  c->resid = red[1] / c->info.dV;
  c->fmax = red[2] / c->info.dV;
  return CDFT_OK;
}

extern "C++" int cdft_internal_fire_accept(cdft_ctx* c, int s_idx) { return fire_accept(c, s_idx); }
extern "C++" int cdft_internal_fire_resync(cdft_ctx* c) {
  const long N = c->info.N;
  const Alias a = c->alias();
  const int k = c->cur;
  k_alias_from_rho<<<grid_for(N), 256, 0, c->stream>>>(c->rho, c->fx[k], N, a);
  k_rho_from_alias<<<grid_for(N), 256, 0, c->stream>>>(c->fx[k], c->rho, N, a);
  CUDA_OR_FAIL(c, cudaMemsetAsync(c->fv[k], 0, N * sizeof(double), c->stream));
  double t[8];
  int rc = eval_internal(c, t);
  if (rc) return rc;
  c->F = t[0];
  return fire_accept(c, k);
}

static int fire_buffers(cdft_ctx* c) {
  const long N = c->info.N;
  for (int i = 0; i < 2; ++i) {
    if (!c->fx[i]) CUDA_OR_FAIL(c, cudaMalloc(&c->fx[i], N * sizeof(double)));
    if (!c->fv[i]) CUDA_OR_FAIL(c, cudaMalloc(&c->fv[i], N * sizeof(double)));
    if (!c->fg[i]) CUDA_OR_FAIL(c, cudaMalloc(&c->fg[i], N * sizeof(double)));
  }
  return CDFT_OK;
}

int cdft_fire_init(cdft_ctx* c, const cdft_fire_params* p) {
  if (!c) return CDFT_ERR_ARG;
  cdft_fire_params d;
  cdft_fire_default_params(&d);
  c->fp = p ? *p : d;
  const long N = c->info.N;
  int rc0 = fire_buffers(c);
  if (rc0) return rc0;
  c->cur = 0;
  const Alias a = c->alias();
  // Minimizer::Minimizer: x = alias(rho); fireMinimizer2: F = getDF_DX(), v = 0
  k_alias_from_rho<<<grid_for(N), 256, 0, c->stream>>>(c->rho, c->fx[0], N, a);
  k_rho_from_alias<<<grid_for(N), 256, 0, c->stream>>>(c->fx[0], c->rho, N, a);
  CUDA_OR_FAIL(c, cudaMemsetAsync(c->fv[0], 0, N * sizeof(double), c->stream));
  double t[8];
  int rc = eval_internal(c, t);
  if (rc) return rc;
  c->calls = 1;
  c->F = t[0];
  rc = fire_accept(c, 0);
  if (rc) return rc;
  c->dt = c->fp.dt;
  c->dt_max = c->fp.dt_max;
  c->alpha = c->fp.alpha_start;
  c->vv = 1.0;
  c->dt_best = 1e-3;  // dt_best_ = the constructor's dt_ before setTimeStep
  c->Npos = c->Nneg = c->backtracks = 0;
  c->it = 0;
  c->fire_steps = 0;
  c->fire_ready = true;
  return CDFT_OK;
}

// FIRE2 state on disk: the minimizer the reference serialises with Boost
// (fireMinimizer2::serialize, include/Minimizer.h:145-180: the alias coordinates x of
// Minimizer, v, the step parameters and counters), here as raw native doubles behind a
// small header: "CDFTFIR1", int64 N, int32 nx ny nz 0, the parameters (8 doubles, 3 int32
// and one pad), the state (10 doubles: F dt dt_max alpha vv dt_best fmax resid vdotf mu;
// int32 Npos Nneg backtracks it; int64 steps calls), then rho, x, v (N doubles each).
namespace {
const char kFireMagic[8] = {'C', 'D', 'F', 'T', 'F', 'I', 'R', '1'};
struct FireFileHead {
  char magic[8];
  int64_t N;
  int32_t nx, ny, nz, pad0;
  double prm_d[8];  // dt dt_max dt_min alpha_start f_alf f_dec f_inc force_limit
  int32_t prm_i[4];  // n_delay n_p_negative_max initial_delay 0
  double st_d[10];
  int32_t st_i[4];
  int64_t st_l[2];
};
}  // namespace

int cdft_fire_save(cdft_ctx* c, const char* path) {
  if (!c || !path) return CDFT_ERR_ARG;
  if (!c->fire_ready) return fail(c, CDFT_ERR_STATE, "cdft_fire_init has not been called");
  const long N = c->info.N;
  FireFileHead h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kFireMagic, 8);
  h.N = N; h.nx = c->p.nx; h.ny = c->p.ny; h.nz = c->p.nz;
  const cdft_fire_params& q = c->fp;
  const double pd[8] = {q.dt, q.dt_max, q.dt_min, q.alpha_start, q.f_alf, q.f_dec, q.f_inc, q.force_limit};
  std::memcpy(h.prm_d, pd, sizeof(pd));
  h.prm_i[0] = q.n_delay; h.prm_i[1] = q.n_p_negative_max; h.prm_i[2] = q.initial_delay;
  const double sd[10] = {c->F, c->dt, c->dt_max, c->alpha, c->vv, c->dt_best, c->fmax, c->resid, c->vdotf, c->mu};
  std::memcpy(h.st_d, sd, sizeof(sd));
  h.st_i[0] = c->Npos; h.st_i[1] = c->Nneg; h.st_i[2] = c->backtracks; h.st_i[3] = (int32_t)c->it;
  h.st_l[0] = c->fire_steps; h.st_l[1] = c->calls;
  std::vector<double> buf(3 * (size_t)N);
  CUDA_OR_FAIL(c, cudaMemcpyAsync(buf.data(), c->rho, N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(buf.data() + N, c->fx[c->cur], N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(buf.data() + 2 * N, c->fv[c->cur], N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(c, CDFT_ERR_ARG, std::string("could not open ") + path);
  const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(buf.data(), sizeof(double), buf.size(), f) == buf.size();
  if (std::fclose(f) != 0 || !ok) return fail(c, CDFT_ERR_ARG, std::string("could not write ") + path);
  return CDFT_OK;
}

static int fire_buffers(cdft_ctx* c);

int cdft_fire_load(cdft_ctx* c, const char* path) {
  if (!c || !path) return CDFT_ERR_ARG;
  const long N = c->info.N;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(c, CDFT_ERR_ARG, std::string("could not open ") + path);
  FireFileHead h;
  std::vector<double> buf(3 * (size_t)N);
  const bool rd = std::fread(&h, sizeof(h), 1, f) == 1;
  const bool ok = rd && std::memcmp(h.magic, kFireMagic, 8) == 0 && h.N == N && h.nx == c->p.nx && h.ny == c->p.ny && h.nz == c->p.nz &&
                  std::fread(buf.data(), sizeof(double), buf.size(), f) == buf.size();
  std::fclose(f);
  if (!ok) return fail(c, CDFT_ERR_ARG, std::string(path) + " is not a FIRE2 state of this lattice");
  int rc = fire_buffers(c);
  if (rc) return rc;
  cdft_fire_params& q = c->fp;
  q.dt = h.prm_d[0]; q.dt_max = h.prm_d[1]; q.dt_min = h.prm_d[2]; q.alpha_start = h.prm_d[3];
  q.f_alf = h.prm_d[4]; q.f_dec = h.prm_d[5]; q.f_inc = h.prm_d[6]; q.force_limit = h.prm_d[7];
  q.n_delay = h.prm_i[0]; q.n_p_negative_max = h.prm_i[1]; q.initial_delay = h.prm_i[2];
  c->cur = 0;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rho, buf.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->fx[0], buf.data() + N, N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->fv[0], buf.data() + 2 * N, N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->fixed_mass <= 0) c->mu = h.st_d[9];
  // the derivative and alias gradient of the saved state, from one evaluation at its density
  double t[8];
  rc = eval_internal(c, t);
  if (rc) return rc;
  rc = fire_accept(c, 0);
  if (rc) return rc;
  c->F = h.st_d[0]; c->dt = h.st_d[1]; c->dt_max = h.st_d[2]; c->alpha = h.st_d[3]; c->vv = h.st_d[4]; c->dt_best = h.st_d[5];
  c->fmax = h.st_d[6];
  c->Npos = h.st_i[0]; c->Nneg = h.st_i[1]; c->backtracks = h.st_i[2]; c->it = (unsigned)h.st_i[3];
  c->fire_steps = h.st_l[0]; c->calls = h.st_l[1];
  c->fire_ready = true;
  return CDFT_OK;
}

// fireMinimizer2::step (src/Minimizer.cpp:160-271).
static int fire_one_step(cdft_ctx* c, int* backtracked) {
  const long N = c->info.N;
  const cdft_fire_params& fp = c->fp;
  c->it++;
  const double P = -c->vdotf;
  const double fold = c->F;
  bool uphill = false;
  if (P > 0) {
    c->Npos++;
    c->Nneg = 0;
    if (c->Npos > fp.n_delay) {
      c->dt = std::min(c->dt * fp.f_inc, c->dt_max);
      c->alpha = c->alpha * fp.f_alf;
    }
  } else {
    c->Npos = 0;
    c->Nneg++;
    if (c->Nneg > fp.n_p_negative_max) return fail(c, CDFT_ERR_UPHILL, "Cannot stop going uphill in Fire2");
    if (!(fp.initial_delay && c->it < (unsigned)fp.n_delay)) {
      if (c->dt * fp.f_dec >= fp.dt_min) c->dt *= fp.f_dec;
      c->alpha = fp.alpha_start;
    }
    uphill = true;
    c->backtracks++;
  }
  const int s = c->cur, n = 1 - c->cur;
  double red[2];
  FFirePre pre{c->fx[s], c->fv[s], c->fg[s], c->fx[n], c->fv[n], c->dt, uphill ? 1 : 0};
  int rc = map_reduce<2, 0>(c, N, pre, red);
  if (rc) return rc;
  const double nv = std::sqrt(red[0]), nf = std::sqrt(red[1]);
  const double vnorm = nv * nv, fnorm = nf * nf;
  k_fire_mix<<<grid_for(N), 256, 0, c->stream>>>(c->fx[n], c->fv[n], c->fg[s], c->rho, N, c->dt, c->alpha, std::sqrt(vnorm / fnorm), c->alias());
  double t[8];
  rc = eval_internal(c, t);
  c->calls++;
  if (rc == CDFT_ERR_ETA) {
    // restore x, v (x0.5), dF; halve dt (src/Minimizer.cpp:233-245)
    k_scale_vec<<<grid_for(N), 256, 0, c->stream>>>(c->fv[s], N, 0.5);
    c->vdotf *= 0.5;
    c->dt /= 2;
    c->fmax = 1000;
    c->backtracks++;
    if (backtracked) *backtracked = 1;
  } else if (rc) {
    return rc;
  } else {
    c->F = t[0];
    rc = fire_accept(c, n);
    if (rc) return rc;
    c->cur = n;
    c->vv = c->vv * 0.9 + 0.1 * (std::fabs(c->F - fold) / c->dt);
    c->dt_best = std::max(c->dt, c->dt_best);
  }
  if (c->backtracks >= 10) {
    c->dt_max = std::min(c->dt_best, 0.9 * c->dt_max);
    c->dt_best = 0;
    c->backtracks = 0;
  }
  c->fire_steps++;
  return CDFT_OK;
}

static void fire_report(const cdft_ctx* c, long steps, int bt, int stop, cdft_fire_report* r) {
  if (!r) return;
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
  r->backtracks = bt;
  r->stop = stop;
  r->steps_fp32 = 0;
}

static int fire_loop(cdft_ctx* c, long max_steps, double resid_tol, bool use_monitor, cdft_fire_report* rep) {
  if (!c) return CDFT_ERR_ARG;
  if (!c->fire_ready) return fail(c, CDFT_ERR_STATE, "cdft_fire_init has not been called");
  long k = 0;
  int bt = 0, stop = 0;
  while (true) {
    int b = 0;
    int rc = fire_one_step(c, &b);
    bt += b;
    if (rc) {
      fire_report(c, k, bt, stop, rep);
      return rc;
    }
    ++k;
    if (use_monitor && std::fabs(c->vv / c->info.volume) < c->fp.force_limit) { stop = 1; break; }
    if (!use_monitor && c->resid <= resid_tol && c->fmax < 1000) { stop = 2; break; }
    if (max_steps > 0 && k >= max_steps) break;
  }
  fire_report(c, k, bt, stop, rep);
  return CDFT_OK;
}

int cdft_fire_step(cdft_ctx* c, int nsteps, cdft_fire_report* rep) {
  if (!c) return CDFT_ERR_ARG;
  if (!c->fire_ready) return fail(c, CDFT_ERR_STATE, "cdft_fire_init has not been called");
  int bt = 0;
  for (int k = 0; k < nsteps; ++k) {
    int b = 0;
    int rc = fire_one_step(c, &b);
    bt += b;
    if (rc) {
      fire_report(c, k, bt, 0, rep);
      return rc;
    }
  }
  fire_report(c, nsteps, bt, 0, rep);
  return CDFT_OK;
}

int cdft_fire_run(cdft_ctx* c, long max_steps, cdft_fire_report* rep) { return fire_loop(c, max_steps, 0.0, true, rep); }
int cdft_fire_run_to_residual(cdft_ctx* c, double resid_tol, long max_steps, cdft_fire_report* rep) {
  return fire_loop(c, max_steps, resid_tol, false, rep);
}

// ------------------------------------------------------------------ DDFT ---
static int ddft_r2c(cdft_ctx* c, const double* real, void* spec) {
  if (c->precision == CDFT_FP64) c->e64->r2c(real, reinterpret_cast<double2*>(spec), c->stream);
  else c->e32->r2c(real, reinterpret_cast<float2*>(spec), c->stream);
  return CDFT_OK;
}

int cdft_ddft_init(cdft_ctx* c, double dt, double dt_max, double tol) {
  if (!c) return CDFT_ERR_ARG;
  if (c->p.model < 0 && !c->p.lj) return fail(c, CDFT_ERR_ARG, "DDFT needs an FMT model or an interaction");
  const long N = c->info.N;
  const long Nc = c->precision == CDFT_FP64 ? c->e64->spectrum_len() : c->e32->spectrum_len();  // padded rows
  const size_t cs = sizeof(double2);  // large enough for either precision
  if (!c->dd0) {
    CUDA_OR_FAIL(c, cudaMalloc(&c->dd0, N * sizeof(double)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->dd1, N * sizeof(double)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->ddn, N * sizeof(double)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->dR, N * sizeof(double)));
    CUDA_OR_FAIL(c, cudaMalloc(&c->rk0, Nc * cs));
    CUDA_OR_FAIL(c, cudaMalloc(&c->R0k, Nc * cs));
    CUDA_OR_FAIL(c, cudaMalloc(&c->R1k, Nc * cs));
    CUDA_OR_FAIL(c, cudaMalloc(&c->work, Nc * cs));
    CUDA_OR_FAIL(c, cudaMalloc(&c->dfac, 2 * (c->p.nx + c->p.ny + c->p.nz) * sizeof(double)));
  }
  const int nx = c->p.nx, ny = c->p.ny, nz = c->p.nz, nzc = nz / 2 + 1;
  const double D = 1.0 / (c->p.dx * c->p.dx);
  c->Lx.resize(nx); c->Ly.resize(ny); c->Lz.resize(nzc);
  for (int i = 0; i < nx; i++) c->Lx[i] = 2 * D * (std::cos((2 * M_PI * i) / nx) - 1);  // DDFT::DDFT, src/DDFT.cpp:66-92
  for (int i = 0; i < ny; i++) c->Ly[i] = 2 * D * (std::cos((2 * M_PI * i) / ny) - 1);
  for (int i = 0; i < nzc; i++) c->Lz[i] = 2 * D * (std::cos((2 * M_PI * i) / nz) - 1);
  double t[8];
  int rc = eval_internal(c, t);  // the constructor's evaluation (src/DDFT.cpp:52)
  if (rc) return rc;
  rc = map_reduce<1, 0>(c, N, FSumRho{c->rho}, &c->ddft_mass0);
  if (rc) return rc;
  c->ddft_dt = dt;
  c->ddft_dt_max = dt_max;
  c->ddft_tol = tol;
  c->ddft_time = 0;
  c->ddft_successes = 0;
  c->ddft_have_factors = false;
  c->ddft_max_dev = 0;
  c->ddft_ready = true;
  return CDFT_OK;
}

int cdft_ddft_set_mass_restore(cdft_ctx* c, int on) {
  if (!c) return CDFT_ERR_ARG;
  c->ddft_restore = on != 0;
  return CDFT_OK;
}

int cdft_ddft_mass_deviation(cdft_ctx* c, double* max_rel) {
  if (!c || !max_rel) return CDFT_ERR_ARG;
  *max_rel = c->ddft_max_dev;
  return CDFT_OK;
}

// DDFT::change_timestep (src/DDFT.cpp:194-215), with its early return.
static void ddft_change_timestep(cdft_ctx* c, double ndt) {
  if (std::fabs(c->ddft_dt - ndt) < 1e-10) return;
  c->ddft_dt = ndt;
  const int nx = c->p.nx, ny = c->p.ny, nzc = c->p.nz / 2 + 1;
  std::vector<double> h;
  h.insert(h.end(), c->Lx.begin(), c->Lx.end());
  h.insert(h.end(), c->Ly.begin(), c->Ly.end());
  h.insert(h.end(), c->Lz.begin(), c->Lz.end());
  for (int i = 0; i < nx; i++) h.push_back(std::exp(c->Lx[i] * ndt));
  for (int i = 0; i < ny; i++) h.push_back(std::exp(c->Ly[i] * ndt));
  for (int i = 0; i < nzc; i++) h.push_back(std::exp(c->Lz[i] * ndt));
  cudaMemcpyAsync(c->dfac, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  cudaStreamSynchronize(c->stream);
  c->ddft_have_factors = true;
}

static int ddft_rhs(cdft_ctx* c, const double* rho, void* spec, double* rmax) {
  double m;
  FDdftRhs f{rho, c->dF, c->dR, c->p.nx, c->p.ny, c->p.nz, c->p.dx, c->info.dV, c->fixed_bg};
  int rc = map_reduce<0, 1>(c, c->info.N, f, &m);
  if (rc) return rc;
  if (rmax) *rmax = m / c->info.dV;
  return ddft_r2c(c, c->dR, spec);
}

// DDFT::step (src/DDFT.cpp:113-182), single species, periodic boundaries.
// The reference evaluates at the step's start, at every fixed-point iterate and at
// the end. Two of those evaluations repeat one already made at the same density, and
// (without fixed mass, whose rescaling is not bit-idempotent) are reused bit for bit:
// the start of a step that follows another in the same call (dF_current: the last
// step's final evaluation is at this density), and the first iterate of every pass,
// which starts from d1 = d0, so its right-hand side is the step's first one.
static int ddft_one_step(cdft_ctx* c, int* restarts, bool dF_current) {
  const long N = c->info.N;
  const size_t nb = N * sizeof(double);
  const bool reuse = c->fixed_mass <= 0;
  if (!c->ddft_have_factors) {
    double tmp = c->ddft_dt;
    c->ddft_dt = 0;
    ddft_change_timestep(c, tmp);
  }
  double t[8];
  int rc = CDFT_OK;
  if (!(reuse && dF_current)) rc = eval_internal(c, t);
  if (rc) return rc;
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->dd0, c->rho, nb, cudaMemcpyDeviceToDevice, c->stream));
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->dd1, c->rho, nb, cudaMemcpyDeviceToDevice, c->stream));
  double rhs_max = 0;
  rc = ddft_rhs(c, c->dd0, c->R0k, &rhs_max);
  if (rc) return rc;
  c->ddft_rhs = rhs_max;
  ddft_r2c(c, c->dd0, c->rk0);
  bool decreased = false, restart;
  int tries = 0;
  do {
    if (++tries > 40) return fail(c, CDFT_ERR_TIMEOUT, "DDFT fixed point did not converge after 40 time-step reductions");
    double deviation = 1;
    restart = false;
    for (int i = 0; i < 100 && deviation > c->ddft_tol && !restart; i++) {
      const int nx = c->p.nx, ny = c->p.ny, nzc = c->p.nz / 2 + 1;
      const int pz = c->precision == CDFT_FP64 ? c->e64->pitch() : c->e32->pitch();
      if (i == 0 && reuse) {  // d1 = d0: the right-hand side of the step's start
        const size_t sb = (size_t)nx * ny * pz * (c->precision == CDFT_FP64 ? sizeof(double2) : sizeof(float2));
        CUDA_OR_FAIL(c, cudaMemcpyAsync(c->R1k, c->R0k, sb, cudaMemcpyDeviceToDevice, c->stream));
      } else {
        CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rho, c->dd1, nb, cudaMemcpyDeviceToDevice, c->stream));
        rc = eval_internal(c, t);
        if (rc) return rc;
        rc = ddft_rhs(c, c->dd1, c->R1k, nullptr);
        if (rc) return rc;
      }
      const unsigned g = grid_for((long)nx * ny * pz);
      if (c->precision == CDFT_FP64) {
        k_ddft_prop<double><<<g, 256, 0, c->stream>>>((const double2*)c->rk0, (const double2*)c->R0k, (const double2*)c->R1k, (double2*)c->work,
                                                       c->dfac, nx, ny, nzc, pz, c->ddft_dt);
        c->e64->c2r((const double2*)c->work, c->ddn, 1.0 / (double)N, c->stream);
      } else {
        k_ddft_prop<float><<<g, 256, 0, c->stream>>>((const float2*)c->rk0, (const float2*)c->R0k, (const float2*)c->R1k, (float2*)c->work,
                                                      c->dfac, nx, ny, nzc, pz, c->ddft_dt);
        c->e32->c2r((const float2*)c->work, c->ddn, 1.0f / (float)N, c->stream);
      }
      if (c->precision == CDFT_FP32) {
        // FP32 transforms keep the k = 0 mode only to FP32 rounding: restore
        // the run's mass with a uniform FP64 shift (compensated FP64 sum).
        // The deviation found before the shift is recorded either way.
        double m;
        rc = map_reduce<1, 0>(c, N, FSumRho{c->ddn}, &m);
        if (rc) return rc;
        if (c->ddft_mass0 != 0) c->ddft_max_dev = std::max(c->ddft_max_dev, std::fabs(m - c->ddft_mass0) / std::fabs(c->ddft_mass0));
        if (c->ddft_restore) k_add_const<<<grid_for(N), 256, 0, c->stream>>>(c->ddn, N, (m - c->ddft_mass0) / (double)N);
      }
      if (c->fixed_bg)  // the boundary keeps the iterate's densities (src/DDFT.cpp:280-281)
        k_boundary_copy<<<grid_for(N), 256, 0, c->stream>>>(c->ddn, c->dd1, N, c->p.ny, c->p.nz);
      double red[2];
      rc = map_reduce<0, 2>(c, N, FDdftDev{c->dd1, c->ddn}, red);
      if (rc) return rc;
      const double old = deviation;
      deviation = red[0];
      const double mn = -red[1];
      std::swap(c->dd1, c->ddn);
      if (mn < 0 || (i > 0 && old < deviation)) restart = true;
    }
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rho, c->dd0, nb, cudaMemcpyDeviceToDevice, c->stream));
    if (restart || deviation > c->ddft_tol) {
      ddft_change_timestep(c, c->ddft_dt / 10);
      CUDA_OR_FAIL(c, cudaMemcpyAsync(c->dd1, c->dd0, nb, cudaMemcpyDeviceToDevice, c->stream));
      decreased = true;
      restart = true;
      if (restarts) (*restarts)++;
    }
  } while (restart);
  c->ddft_time += c->ddft_dt;
  if (decreased) c->ddft_successes = 0;
  else c->ddft_successes++;
  if (c->ddft_successes >= 5 && c->ddft_dt < c->ddft_dt_max) {
    ddft_change_timestep(c, std::min(2 * c->ddft_dt, c->ddft_dt_max));
    c->ddft_successes = 0;
  }
  CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rho, c->dd1, nb, cudaMemcpyDeviceToDevice, c->stream));
  rc = eval_internal(c, t);
  if (rc) return rc;
  c->F = t[0];
  return CDFT_OK;
}

int cdft_ddft_step(cdft_ctx* c, int nsteps, cdft_ddft_report* rep) {
  if (!c) return CDFT_ERR_ARG;
  if (!c->ddft_ready) return fail(c, CDFT_ERR_STATE, "cdft_ddft_init has not been called");
  int restarts = 0;
  for (int k = 0; k < nsteps; ++k) {
    int rc = ddft_one_step(c, &restarts, k > 0);
    if (rc) return rc;
  }
  if (rep) {
    double s;
    int rc = map_reduce<1, 0>(c, c->info.N, FSumRho{c->rho}, &s);
    if (rc) return rc;
    rep->steps = nsteps;
    rep->F = c->F;
    rep->time = c->ddft_time;
    rep->dt = c->ddft_dt;
    rep->mass = s * c->info.dV;
    rep->rhs_max = c->ddft_rhs;
    rep->restarts = restarts;
  }
  return CDFT_OK;
}

}  // extern "C"

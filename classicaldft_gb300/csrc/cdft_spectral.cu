// Spectral drivers on the matrices of the path (consumers of the Hessian product):
//   Log_Det::calculate_log_det          (include/Log_Det.h, src/Log_Det.cpp:22-166)
//   Eigenvalues::calculate_eigenvector  (include/Eigenvalues.h, src/Eigenvalues.cpp)
//   Arnoldi::determine_largest_eigenpairs (include/Arnoldi.h, src/Arnoldi.cpp:72-283)
// Every vector lives on the device and every product is the context's Hessian pass;
// the host holds only scalars and the small projected matrices.
//
// Log_Det keeps the reference's estimator exactly: the Chebyshev coefficients of log,
// the three-term recurrence and Hutchinson's trace with the +-1 vectors that
// std::mt19937(seed) and uniform_int_distribution<>(0, 1) give, drawn in point order
// (on the device, k_mt_probe, sample i + 1's on a side stream while sample i's products
// run; with another standard library than libstdc++ 13, the host draws sample i + 1 while
// the device runs sample i's queued products).
// Eigenvalues and Arnoldi compute what the reference computes (the smallest eigenvalue of the signed, scaled and
// rank-one shifted Hessian; the k eigenpairs of H + shift of largest magnitude) with a
// thick-restart Lanczos iteration, fully re-orthogonalised, instead of nlopt's L-BFGS on
// the Rayleigh quotient and Armadillo's complex implicitly restarted Arnoldi: the
// Hessian is symmetric, so its Krylov projection is symmetric and real.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#include "cdft_ctx.h"

namespace {

constexpr int kDotBlocks = 512;  // partial sums per dot product (fixed: the sums are deterministic)
constexpr int kRitzChunk = 16;   // Ritz vectors formed per pass of the basis

// part[i * kDotBlocks + b] = block b's share of V_i . w for i < nv (V_i = V + i * N)
__global__ void __launch_bounds__(256) k_dots(const double* __restrict__ V, int nv, const double* __restrict__ w, long N,
                                              double* __restrict__ part) {
  __shared__ double red[8];
  const int i = blockIdx.y;
  const double* v = V + (long)i * N;
  double acc = 0;
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) acc += v[p] * w[p];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int k = 0; k < 8; ++k) s += red[k];
    part[(long)i * kDotBlocks + blockIdx.x] = s;
  }
  (void)nv;
}
// out[i] = sum of part[i * kDotBlocks ...] in a fixed tree order; one block per vector
__global__ void __launch_bounds__(256) k_dots_finish(const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double red[8];
  const double* q = part + (long)blockIdx.x * kDotBlocks;
  double acc = 0;
  for (int b = threadIdx.x; b < kDotBlocks; b += 256) acc += q[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int k = 0; k < 8; ++k) s += red[k];
    out[blockIdx.x] = s;
  }
}
// w -= sum_{i < nv} h_i V_i (h on the device)
__global__ void __launch_bounds__(256) k_sub_proj(const double* __restrict__ V, int nv, const double* __restrict__ h, double* __restrict__ w,
                                                  long N) {
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) {
    double s = 0;
    for (int i = 0; i < nv; ++i) s += h[i] * V[(long)i * N + p];
    w[p] -= s;
  }
}
// y <- a * y + b * (s . x) * s + c * x, with the dot s . x read from the device
// (Eigenvalues::calculate_gradients' vshift term, src/Eigenvalues.cpp:49-50, and the shift)
__global__ void __launch_bounds__(256) k_op_finish(double* __restrict__ y, const double* __restrict__ x, const double* __restrict__ s,
                                                   const double* __restrict__ sdotx, double a, double b, double c, long N) {
  const double bs = s ? b * sdotx[0] : 0.0;
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) {
    double v = a * y[p] + c * x[p];
    if (s) v += bs * s[p];
    y[p] = v;
  }
}
// dst = src / sqrt(nrm2[0])
__global__ void __launch_bounds__(256) k_normalise(const double* __restrict__ src, double* __restrict__ dst, const double* __restrict__ nrm2,
                                                   long N) {
  const double f = 1.0 / sqrt(nrm2[0]);
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) dst[p] = src[p] * f;
}
// out_q = sum_j V_j S[j * ldS + q] for q < nq (nq <= kRitzChunk), S in device memory
__global__ void __launch_bounds__(256) k_ritz(const double* __restrict__ V, int nj, const double* __restrict__ S, int ldS, int nq,
                                              double* __restrict__ out, long N) {
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) {
    double acc[kRitzChunk];
#pragma unroll
    for (int q = 0; q < kRitzChunk; ++q) acc[q] = 0;
    for (int j = 0; j < nj; ++j) {
      const double v = V[(long)j * N + p];
#pragma unroll
      for (int q = 0; q < kRitzChunk; ++q)
        if (q < nq) acc[q] += v * S[j * ldS + q];
    }
#pragma unroll
    for (int q = 0; q < kRitzChunk; ++q)
      if (q < nq) out[(long)q * N + p] = acc[q];
  }
}
// a seeded start vector: splitmix64 of (seed, point), uniform in [-1, 1)
__global__ void __launch_bounds__(256) k_seed_vector(double* __restrict__ x, long N, unsigned long long seed) {
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ULL * (unsigned long long)(p + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    x[p] = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
  }
}

// The DDFT mobility of DDFT::g_dot_x (src/DDFT.cpp:320-351, forward differences) is
// g = -C^T C, with C the edge-weighted difference operator on the 3N lattice edges
// (p, p + e_ax): (C x)_(ax, p) = c (x[p + e_ax] - x[p]), c = sqrt(D (rho[p] + rho[p + e_ax])),
// D = 1/(2 dx^2). Edge fields are stored axis-major, w[ax * N + p].
__device__ __forceinline__ long sp_nb(long p, int ax, int dir, int nx, int ny, int nz) {
  const int k = (int)(p % nz);
  const long t = p / nz;
  int j = (int)(t % ny), i = (int)(t / ny);
  int kk = k;
  if (ax == 0) i = (i + dir + nx) % nx;
  else if (ax == 1) j = (j + dir + ny) % ny;
  else kk = (k + dir + nz) % nz;
  return kk + (long)nz * (j + (long)ny * i);
}
// w = s C x
__global__ void __launch_bounds__(256) k_mob_c(const double* __restrict__ rho, const double* __restrict__ x, double* __restrict__ w, int nx,
                                               int ny, int nz, double D, double s) {
  const long N = (long)nx * ny * nz;
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256)
    for (int ax = 0; ax < 3; ++ax) {
      const long q = sp_nb(p, ax, 1, nx, ny, nz);
      w[ax * N + p] = s * sqrt(D * (rho[p] + rho[q])) * (x[q] - x[p]);
    }
}
// y = C^T w: y[p] = sum_ax c(p - e_ax, p) w[ax, p - e_ax] - c(p, p + e_ax) w[ax, p]
__global__ void __launch_bounds__(256) k_mob_ct(const double* __restrict__ rho, const double* __restrict__ w, double* __restrict__ y, int nx,
                                                int ny, int nz, double D) {
  const long N = (long)nx * ny * nz;
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) {
    double acc = 0;
    for (int ax = 0; ax < 3; ++ax) {
      const long q = sp_nb(p, ax, 1, nx, ny, nz), m = sp_nb(p, ax, -1, nx, ny, nz);
      acc += sqrt(D * (rho[m] + rho[p])) * w[ax * N + m] - sqrt(D * (rho[p] + rho[q])) * w[ax * N + p];
    }
    y[p] = acc;
  }
}
// y = a x + b y
__global__ void __launch_bounds__(256) k_axpby(double a, const double* __restrict__ x, double b, double* __restrict__ y, long N) {
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) y[p] = a * x[p] + b * y[p];
}
__global__ void __launch_bounds__(256) k_fill(double* __restrict__ y, double v, long N) {
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) y[p] = v;
}

// Chebyshev steps of Log_Det::calculate_log_det (src/Log_Det.cpp:113-144). r = M x
// from the matrix pass; the matrix the estimator expands is A x = sg r + z sum(x)
// (sg = -1 for a dynamic matrix, z = lam_mid / N when it has a zero eigenvalue).
// First term: w1 = al (A v) + be v; u = c0 v + c1 w1.
__global__ void __launch_bounds__(256) k_cheb_first(const double* __restrict__ r, const double* __restrict__ v, const double* __restrict__ sum_v,
                                                    double sg, double z, double al, double be, double c0, double c1, double* __restrict__ w1,
                                                    double* __restrict__ u, long N) {
  const double zs = z * sum_v[0];
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) {
    const double x = v[p];
    const double w = (sg * r[p] + zs) * al + be * x;
    w1[p] = w;
    u[p] = c0 * x + c1 * w;
  }
}
// Next term, in place over w0: w2 = al (A w1) + be w1 - w0; u += ck w2.
__global__ void __launch_bounds__(256) k_cheb_next(const double* __restrict__ r, const double* __restrict__ w1, const double* __restrict__ sum_w1,
                                                   double sg, double z, double al, double be, double ck, double* __restrict__ w0,
                                                   double* __restrict__ u, long N) {
  const double zs = z * sum_w1[0];
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) {
    const double w = (sg * r[p] + zs) * al + be * w1[p] - w0[p];
    w0[p] = w;
    u[p] += ck * w;
  }
}
// part[b] = block b's share of sum(x)
__global__ void __launch_bounds__(256) k_sum(const double* __restrict__ x, long N, double* __restrict__ part) {
  __shared__ double red[8];
  double acc = 0;
  for (long p = blockIdx.x * 256L + threadIdx.x; p < N; p += (long)gridDim.x * 256) acc += x[p];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int k = 0; k < 8; ++k) s += red[k];
    part[blockIdx.x] = s;
  }
}

}  // namespace

#define SP_CK(c, x)                                                                        \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess) return cdft_internal_fail(c, CDFT_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

namespace {

unsigned sp_grid(long n) { return (unsigned)std::max<long>(1, std::min<long>((n + 255) / 256, 152 * 8)); }

// Device work arrays of one driver call (freed on return).
// Log_Det's +-1 probes drawn on the device, bit for bit those of the host loop
//   std::mt19937 rng(seed); std::uniform_int_distribution<> d(0, 1); d(rng) > 0 ? 1 : -1
// One block keeps the generator's 624-word state in shared memory. A twist updates word i
// from words i, i + 1 and i + 397 (mod 624) in increasing i, so it runs as three parallel
// phases (i < 227 reads only old words; 227 <= i < 454 reads the words the first phase made;
// the rest reads the second phase's, word 623 also the new word 0) into a second copy of the
// state, and each new word is tempered into one draw. libstdc++ (release 13 here) maps a
// 32-bit draw to {0, 1} by Lemire's method with range 2, which is its top bit. The state
// and the position of the next unused word live in gst (625 words) between calls, as in
// the engine object.
__device__ __forceinline__ unsigned mt_next_word(unsigned xi, unsigned xi1, unsigned xm) {
  const unsigned y = (xi & 0x80000000u) | (xi1 & 0x7fffffffu);
  return xm ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}
__device__ __forceinline__ double mt_sign(unsigned y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return (y >> 31) ? 1.0 : -1.0;
}
__global__ void __launch_bounds__(256) k_mt_probe(unsigned* __restrict__ gst, double* __restrict__ out, long N) {
  __shared__ unsigned xs[2][624];
  const int t = threadIdx.x;
  for (int i = t; i < 624; i += 256) xs[0][i] = gst[i];
  int pos = (int)gst[624];
  __syncthreads();
  int cur = 0;
  long p = min((long)(624 - pos), N);  // the words left from the previous call
  for (int i = t; i < p; i += 256) out[i] = mt_sign(xs[0][pos + i]);
  pos += (int)p;
  while (p < N) {
    const unsigned* o = xs[cur];
    unsigned* n = xs[cur ^ 1];
    if (t < 227) n[t] = mt_next_word(o[t], o[t + 1], o[t + 397]);
    __syncthreads();
    if (t < 227) n[t + 227] = mt_next_word(o[t + 227], o[t + 228], n[t]);
    __syncthreads();
    if (t < 169) n[t + 454] = mt_next_word(o[t + 454], o[t + 455], n[t + 227]);
    else if (t == 169) n[623] = mt_next_word(o[623], n[0], n[396]);
    __syncthreads();  // n complete; o is read no more, so the next twist may overwrite it
    cur ^= 1;
    const long cnt = min(624L, N - p);
    for (int i = t; i < cnt; i += 256) out[p + i] = mt_sign(n[i]);
    p += cnt;
    pos = (int)cnt;
  }
  __syncthreads();
  for (int i = t; i < 624; i += 256) gst[i] = xs[cur][i];
  if (t == 0) gst[624] = (unsigned)pos;
}
#if defined(_GLIBCXX_RELEASE) && _GLIBCXX_RELEASE >= 13
constexpr bool kDeviceProbes = true;
#else
constexpr bool kDeviceProbes = false;  // another standard library's distribution: draw on the host
#endif

struct DevBuf {
  std::vector<void*> ptrs;
  ~DevBuf() {
    for (void* p : ptrs) cudaFree(p);
  }
  double* get(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return (double*)p;
  }
};

// out[0..nv) = V_i . w (device), through part (nv * kDotBlocks doubles)
void dots(const double* V, int nv, const double* w, long N, double* part, double* out, cudaStream_t s) {
  k_dots<<<dim3(kDotBlocks, nv), 256, 0, s>>>(V, nv, w, N, part);
  k_dots_finish<<<nv, 256, 0, s>>>(part, out);
}

// Symmetric eigen-decomposition of the n x n matrix A (row-major) by cyclic Jacobi
// rotations: eigenvalues in w, eigenvectors in the columns of Z (row-major, Z[i * n + k]).
void jacobi_eigen(std::vector<double> A, int n, std::vector<double>& w, std::vector<double>& Z) {
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, diag = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) (i == j ? diag : off) += A[(size_t)i * n + j] * A[(size_t)i * n + j];
    if (off <= 1e-30 * diag || off == 0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        if (apq == 0) continue;
        const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        const double theta = (aqq - app) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
        for (int k = 0; k < n; ++k) {  // A <- J^T A J
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = cs * akp - sn * akq;
          A[(size_t)k * n + q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = cs * apk - sn * aqk;
          A[(size_t)q * n + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double zkp = Z[(size_t)k * n + p], zkq = Z[(size_t)k * n + q];
          Z[(size_t)k * n + p] = cs * zkp - sn * zkq;
          Z[(size_t)k * n + q] = sn * zkp + cs * zkq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = A[(size_t)i * n + i];
}

// Log_Det::get_coefficients (src/Log_Det.cpp:34-57): the Chebyshev coefficients of
// log(0.5 (b - a) x + 0.5 (b + a)) on [-1, 1] at the order + 1 Chebyshev nodes.
std::vector<double> log_cheb_coefficients(int order, double a, double b) {
  std::vector<double> c(order + 1, 0.0);
  for (int k = 0; k <= order; ++k) {
    const double xk = std::cos(M_PI * (k + 0.5) / (order + 1));
    double Tm2 = 0, Tm1 = 0, T = 1;
    for (int j = 0; j <= order; ++j) {
      T = j == 0 ? 1.0 : j == 1 ? xk : 2 * xk * Tm1 - Tm2;
      c[j] += std::log(0.5 * (b - a) * xk + 0.5 * (b + a)) * T;
      Tm2 = Tm1;
      Tm1 = T;
    }
  }
  for (int j = 0; j <= order; ++j) c[j] *= (j == 0 ? 1.0 : 2.0) / (order + 1);
  return c;
}

}  // namespace

int cdft_log_det(cdft_ctx* c, int matrix, int order, double lam_max, double lam_min, long seed, int num_samples, int has_zero_eigenvalue,
                 double* log_det, double* variance) {
  if (!c || !log_det) return CDFT_ERR_ARG;
  if ((matrix != CDFT_MATRIX_HESSIAN && matrix != CDFT_MATRIX_DDFT) || order < 1 || num_samples < 1 || !(lam_max > lam_min) ||
      !(lam_min + lam_max > 0))
    return cdft_internal_fail(c, CDFT_ERR_ARG, "log_det: needs order >= 1, num_samples >= 1 and lam_max > lam_min with lam_min + lam_max > 0");
  const long N = c->info.N;
  const double scale = 1.0 / (lam_min + lam_max), a = lam_min * scale, b = lam_max * scale, lam_mid = 0.5 * (lam_max + lam_min);
  const std::vector<double> cf = log_cheb_coefficients(order, a, b);
  const double sg = matrix == CDFT_MATRIX_DDFT ? -1.0 : 1.0, z = has_zero_eigenvalue ? lam_mid / (double)N : 0.0;
  cudaStream_t s = c->stream;
  DevBuf buf;
  double *v = buf.get(N), *w0 = buf.get(N), *w1 = buf.get(N), *u = buf.get(N), *r = buf.get(N), *part = buf.get(kDotBlocks),
         *scal = buf.get(2 + (size_t)num_samples);
  if (!v || !w0 || !w1 || !u || !r || !part || !scal) return cdft_internal_fail(c, CDFT_ERR_CUDA, "log_det: out of device memory");
  SP_CK(c, cudaMemsetAsync(scal, 0, (2 + (size_t)num_samples) * sizeof(double), s));  // sum(x) stays 0 without a zero eigenvalue
  // two pinned +-1 vectors: the host draws the next sample while the device runs this one
  double* hv[2] = {nullptr, nullptr};
  for (auto& h : hv)
    if (cudaMallocHost(&h, N * sizeof(double)) != cudaSuccess) {
      for (auto& g : hv)
        if (g) cudaFreeHost(g);
      return cdft_internal_fail(c, CDFT_ERR_CUDA, "log_det: pinned buffers");
    }
  struct Pinned {
    double** p;
    ~Pinned() { cudaFreeHost(p[0]); cudaFreeHost(p[1]); }
  } pinned{hv};
  cudaEvent_t copied[2];
  cudaEventCreateWithFlags(&copied[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&copied[1], cudaEventDisableTiming);
  struct Ev {
    cudaEvent_t* e;
    ~Ev() { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
  } evs{copied};
  if (seed <= 0) seed = (long)std::random_device{}();
  std::mt19937 rng((unsigned long)seed);
  std::uniform_int_distribution<> distrib(0, 1);
  const int ny = c->p.ny, nz = c->p.nz;
  auto draw = [&](double* h) {
    for (long p = 0; p < N; ++p) h[p] = distrib(rng) > 0 ? 1.0 : -1.0;
    if (c->fixed_bg)  // Log_Det::set_boundary_points_to_zero (src/Log_Det.cpp:59-64, 111)
      for (long p = 0; p < N; ++p)
        if (cdft_on_boundary(p, ny, nz)) h[p] = 0.0;
  };
  unsigned* mt = nullptr;  // the device generator's state (kDeviceProbes)
  // Device probes: sample i's probe is in pb[i & 1]; probe i + 1 is drawn on a side stream
  // (one block) while sample i's products run, after probe i (the generator's state is
  // sequential) and after sample i - 1 has stopped reading the buffer it overwrites.
  double* pb[2] = {v, nullptr};
  struct Side {
    cudaStream_t st = nullptr;
    cudaEvent_t ready = nullptr, freed = nullptr;
    ~Side() {
      if (ready) cudaEventDestroy(ready);
      if (freed) cudaEventDestroy(freed);
      if (st) cudaStreamDestroy(st);
    }
  } side;
  if (kDeviceProbes) {
    mt = reinterpret_cast<unsigned*>(buf.get(313));  // 625 words
    if (!mt) return cdft_internal_fail(c, CDFT_ERR_CUDA, "log_det: out of device memory");
    std::vector<unsigned> x(625);  // std::mt19937's seeding; its first draw twists
    x[0] = (unsigned)(unsigned long)seed;
    for (int i = 1; i < 624; ++i) x[i] = 1812433253u * (x[i - 1] ^ (x[i - 1] >> 30)) + (unsigned)i;
    x[624] = 624;
    SP_CK(c, cudaMemcpyAsync(mt, x.data(), 625 * sizeof(unsigned), cudaMemcpyHostToDevice, s));
    SP_CK(c, cudaStreamSynchronize(s));
    if (num_samples > 1) {
      pb[1] = buf.get(N);
      if (!pb[1]) return cdft_internal_fail(c, CDFT_ERR_CUDA, "log_det: out of device memory");
      SP_CK(c, cudaStreamCreateWithFlags(&side.st, cudaStreamNonBlocking));
      SP_CK(c, cudaEventCreateWithFlags(&side.ready, cudaEventDisableTiming));
      SP_CK(c, cudaEventCreateWithFlags(&side.freed, cudaEventDisableTiming));
    }
    k_mt_probe<<<1, 256, 0, s>>>(mt, pb[0], N);
    if (num_samples > 1) SP_CK(c, cudaEventRecord(side.freed, s));  // the side stream's first draw follows probe 0
  } else {
    draw(hv[0]);
  }
  const unsigned g = sp_grid(N);
  bool prepared = false;
  auto matvec = [&](const double* x, double* y) -> int {
    int rc = cdft_internal_matvec(c, matrix, x, y, !prepared);
    prepared = true;
    return rc;
  };
  auto sum_of = [&](const double* x, double* out) {
    k_sum<<<kDotBlocks, 256, 0, s>>>(x, N, part);
    k_dots_finish<<<1, 256, 0, s>>>(part, out);
  };
  for (int i = 0; i < num_samples; ++i) {
    const int cur = i & 1;
    double* const v = kDeviceProbes ? pb[cur] : pb[0];  // this sample's probe
    if (kDeviceProbes) {
      if (i > 0) SP_CK(c, cudaStreamWaitEvent(s, side.ready, 0));  // probe i drawn
      if (i + 1 < num_samples) {
        SP_CK(c, cudaStreamWaitEvent(side.st, side.freed, 0));
        k_mt_probe<<<1, 256, 0, side.st>>>(mt, pb[cur ^ 1], N);
        SP_CK(c, cudaEventRecord(side.ready, side.st));
      }
      if (c->fixed_bg) cdft_internal_boundary_set(c, v, 0.0);  // Log_Det::set_boundary_points_to_zero
    } else {
      SP_CK(c, cudaMemcpyAsync(v, hv[cur], N * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    SP_CK(c, cudaEventRecord(copied[cur], s));
    int rc = matvec(v, r);
    if (rc) return rc;
    if (z != 0) sum_of(v, scal);
    k_cheb_first<<<g, 256, 0, s>>>(r, v, scal, sg, z, scale * 2.0 / (b - a), -(b + a) / (b - a), cf[0], cf[1], w1, u, N);
    double *p0 = w0, *p1 = w1;  // w0 holds the term before w1: v for k = 2
    SP_CK(c, cudaMemcpyAsync(p0, v, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    for (int k = 2; k <= order; ++k) {
      rc = matvec(p1, r);
      if (rc) return rc;
      if (z != 0) sum_of(p1, scal);
      k_cheb_next<<<g, 256, 0, s>>>(r, p1, scal, sg, z, scale * 4.0 / (b - a), -2.0 * (b + a) / (b - a), cf[k], p0, u, N);
      std::swap(p0, p1);
    }
    dots(v, 1, u, N, part, scal + 2 + i, s);
    SP_CK(c, cudaGetLastError());
    if (kDeviceProbes && i + 2 < num_samples) SP_CK(c, cudaEventRecord(side.freed, s));  // probe i + 2 may now overwrite v
    if (!kDeviceProbes && i + 1 < num_samples) {  // with this sample's products queued, draw the next probe into the other pinned buffer
      SP_CK(c, cudaEventSynchronize(copied[cur ^ 1]));  // (once the copy that last read it is done)
      draw(hv[cur ^ 1]);
    }
  }
  std::vector<double> vu(num_samples);
  SP_CK(c, cudaMemcpyAsync(vu.data(), scal + 2, num_samples * sizeof(double), cudaMemcpyDeviceToHost, s));
  SP_CK(c, cudaStreamSynchronize(s));
  // the reference's running sums (src/Log_Det.cpp:145-165)
  double acc = 0, acc2 = 0, var = 0;
  for (int i = 1; i <= num_samples; ++i) {
    acc += vu[i - 1];
    acc2 += vu[i - 1] * vu[i - 1];
    const double av = acc / i, av2 = acc2 / i;
    var = std::sqrt(std::fabs(av2 - av * av));
  }
  double ld = acc / num_samples;
  if (has_zero_eigenvalue) ld -= std::log(lam_mid);
  const long n_active = N - (c->fixed_bg ? cdft_n_boundary(c->p.nx, ny, nz) : 0);  // src/Log_Det.cpp:91
  ld -= (double)n_active * std::log(scale);
  *log_det = ld;
  if (variance) *variance = var;
  return CDFT_OK;
}

namespace {

// The symmetric operator the eigen drivers iterate on:
// y = a (H x + 0.5 (vshift . x) vshift) + shift x, H the context's Hessian.
struct SymOp {
  cdft_ctx* c;
  double a, shift;
  const double* vshift;  // device, or null
  double *part, *sdot;
  bool prepared;
  long matvecs;
  long n;  // vector length: N
  int apply(const double* x, double* y) {
    const long N = c->info.N;
    int rc = cdft_internal_matvec(c, CDFT_MATRIX_HESSIAN, x, y, !prepared);
    if (rc) return rc;
    prepared = true;
    ++matvecs;
    if (vshift) dots(vshift, 1, x, N, part, sdot, c->stream);
    k_op_finish<<<sp_grid(N), 256, 0, c->stream>>>(y, x, vshift, sdot, a, 0.5 * a, shift, N);
    return CDFT_OK;
  }
};

// The symmetric operator behind the DDFT dynamical matrix g.H = -C^T C H: on 3N-vectors,
// A w = -C H C^T w. For w in the range of C (where every Krylov vector started from C x0
// stays), A has exactly the non-zero eigenvalues of g.H; an eigenvector w of A gives the
// eigenvector C^T w of g.H. The shift is not applied here (components outside the range
// of C, left by rounding, are annihilated by A instead of kept at the shift).
struct MobOp {
  cdft_ctx* c;
  double shift;  // 0: the drivers rank by |theta + shift| outside the operator
  double *part, *sdot;
  bool prepared;
  long matvecs;
  long n;           // 3N
  double *tN, *uN;  // N-vector work arrays
  double D;
  int apply(const double* w, double* y) {
    const long N = c->info.N;
    const unsigned g = sp_grid(N);
    k_mob_ct<<<g, 256, 0, c->stream>>>(c->rho, w, tN, c->p.nx, c->p.ny, c->p.nz, D);
    if (c->fixed_bg) cdft_internal_boundary_set(c, tN, 0.0);
    int rc = cdft_internal_matvec(c, CDFT_MATRIX_HESSIAN, tN, uN, !prepared);
    if (rc) return rc;
    prepared = true;
    ++matvecs;
    k_mob_c<<<g, 256, 0, c->stream>>>(c->rho, uN, y, c->p.nx, c->p.ny, c->p.nz, D, -1.0);
    return CDFT_OK;
  }
};

enum class Want { Smallest, LargestMagnitude };

struct LanczosResult {
  std::vector<double> theta, resid;  // wanted Ritz values of the operator and their residual norms
  bool converged = false;
  int restarts = 0;
};

// Thick-restart Lanczos with full (twice-applied) re-orthogonalisation for the nev wanted
// eigenpairs of a symmetric operator; the basis V (ncv + 1 vectors) and the Ritz vectors
// stay on the device, the projected ncv x ncv matrix on the host. x0 is the (device)
// start vector. Converged when every wanted pair (only the first with all = false) has
// |residual| <= tol |theta - shift|, or (degenerate_rule) lies within tol of the first
// discarded Ritz value (the stopping rule of src/Arnoldi.cpp:247-263). vecs (nev * N, device) receives the
// Ritz vectors, unit norm.
// The eigenvalues are ranked by theta (Smallest) or by |theta + sel_shift| (LargestMagnitude).
// drop_zero ranks Ritz values with |theta| <= 1e-10 max|theta| last: for MobOp those are
// rounding residue outside the range of C (exact zeros of -C H C^T), not eigenvalues of g.H.
template <class Op>
int lanczos(cdft_ctx* c, Op& op, Want want, int nev, int ncv, double tol, bool all, bool degenerate_rule, long max_matvecs,
            int max_restarts, const double* x0, double* vecs, LanczosResult* out, double sel_shift = 0.0, bool drop_zero = false) {
  const long N = op.n;
  cudaStream_t s = c->stream;
  const unsigned g = sp_grid(N);
  DevBuf buf;
  double* V = buf.get((size_t)(ncv + 1) * N);
  double* Y = buf.get((size_t)ncv * N);
  double* w = buf.get(N);
  double* part = buf.get((size_t)(ncv + 1) * kDotBlocks);
  double* dh = buf.get(2 * (size_t)(ncv + 1) + 2);
  double* dS = buf.get((size_t)ncv * ncv);
  if (!V || !Y || !w || !part || !dh || !dS) return cdft_internal_fail(c, CDFT_ERR_CUDA, "eigen solver: out of device memory");
  op.part = part;
  op.sdot = dh + 2 * (ncv + 1) + 1;
  const int ob = ncv + 1, onrm = 2 * (ncv + 1);
  // v0 = x0 / |x0|
  dots(x0, 1, x0, N, part, dh + onrm, s);
  k_normalise<<<g, 256, 0, s>>>(x0, V, dh + onrm, N);
  std::vector<double> H((size_t)ncv * ncv, 0.0), hh(2 * (size_t)(ncv + 1) + 1), theta, Z;
  int nkeep = 0;
  for (;;) {
    int m = ncv;
    double beta = 0;
    for (int j = nkeep; j < ncv; ++j) {
      double* vj = V + (long)j * N;
      int rc = op.apply(vj, w);
      if (rc) return rc;
      dots(V, j + 1, w, N, part, dh, s);
      k_sub_proj<<<g, 256, 0, s>>>(V, j + 1, dh, w, N);
      dots(V, j + 1, w, N, part, dh + ob, s);
      k_sub_proj<<<g, 256, 0, s>>>(V, j + 1, dh + ob, w, N);
      dots(w, 1, w, N, part, dh + onrm, s);
      k_normalise<<<g, 256, 0, s>>>(w, V + (long)(j + 1) * N, dh + onrm, N);
      SP_CK(c, cudaMemcpyAsync(hh.data(), dh, hh.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      SP_CK(c, cudaStreamSynchronize(s));
      double hnorm = 0;
      for (int i = 0; i <= j; ++i) {
        const double h = hh[i] + hh[ob + i];
        H[(size_t)i * ncv + j] = H[(size_t)j * ncv + i] = h;
        hnorm = std::max(hnorm, std::fabs(h));
      }
      beta = std::sqrt(std::max(hh[onrm], 0.0));
      if (!std::isfinite(beta)) return cdft_internal_fail(c, CDFT_ERR_NONFINITE, "eigen solver: non-finite Krylov vector");
      if (beta <= 1e-14 * hnorm) {  // an invariant subspace: its Ritz pairs are exact
        m = j + 1;
        beta = 0;
        break;
      }
    }
    std::vector<double> Hm((size_t)m * m);
    for (int i = 0; i < m; ++i)
      for (int k = 0; k < m; ++k) Hm[(size_t)i * m + k] = H[(size_t)i * ncv + k];
    jacobi_eigen(Hm, m, theta, Z);
    std::vector<int> idx(m);
    for (int i = 0; i < m; ++i) idx[i] = i;
    double tmax = 0;
    for (int i = 0; i < m; ++i) tmax = std::max(tmax, std::fabs(theta[i]));
    auto key = [&](int x) { return (drop_zero && std::fabs(theta[x]) <= 1e-10 * tmax) ? -1.0 : std::fabs(theta[x] + sel_shift); };
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) {
      return want == Want::Smallest ? theta[x] < theta[y] : key(x) > key(y);
    });
    const int nw = std::min(nev, m);
    out->theta.assign(nw, 0.0);
    out->resid.assign(nw, 0.0);
    bool conv = true;
    for (int i = 0; i < nw; ++i) {
      const int q = idx[i];
      out->theta[i] = theta[q];
      out->resid[i] = beta * std::fabs(Z[(size_t)(m - 1) * m + q]);
      const bool degenerate = degenerate_rule && m > nw && std::fabs(theta[q] - theta[idx[nw]]) <= tol;
      if (out->resid[i] > tol * std::fabs(theta[q] - op.shift) && !degenerate && (all || i == 0)) conv = false;
    }
    out->converged = conv;
    const bool stop = conv || beta == 0 || op.matvecs >= max_matvecs || out->restarts >= max_restarts;
    // the Ritz vectors to keep: the wanted ones for output, or about half the basis to restart with
    const int nk = stop ? nw : std::min(m - 1, std::max(nw + (m - nw) / 2, nw));
    std::vector<double> Ssel((size_t)m * nk);
    for (int j = 0; j < m; ++j)
      for (int q = 0; q < nk; ++q) Ssel[(size_t)j * nk + q] = Z[(size_t)j * m + idx[q]];
    SP_CK(c, cudaMemcpyAsync(dS, Ssel.data(), Ssel.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    double* dst = stop ? vecs : Y;
    for (int q0 = 0; q0 < nk; q0 += kRitzChunk)
      k_ritz<<<g, 256, 0, s>>>(V, m, dS + q0, nk, std::min(kRitzChunk, nk - q0), dst + (long)q0 * N, N);
    if (stop) {
      for (int q = 0; q < nk; ++q) {
        dots(vecs + (long)q * N, 1, vecs + (long)q * N, N, part, dh + onrm, s);
        k_normalise<<<g, 256, 0, s>>>(vecs + (long)q * N, vecs + (long)q * N, dh + onrm, N);
      }
      SP_CK(c, cudaStreamSynchronize(s));  // dS is host-visible until here
      SP_CK(c, cudaGetLastError());
      return CDFT_OK;
    }
    // thick restart: V <- [Ritz vectors, the last Krylov direction]; H <- diag(theta) plus
    // the couplings the next column recomputes
    SP_CK(c, cudaMemcpyAsync(V, Y, (size_t)nk * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SP_CK(c, cudaMemcpyAsync(V + (long)nk * N, V + (long)m * N, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SP_CK(c, cudaStreamSynchronize(s));
    std::fill(H.begin(), H.end(), 0.0);
    for (int q = 0; q < nk; ++q) H[(size_t)q * ncv + q] = theta[idx[q]];
    nkeep = nk;
    ++out->restarts;
  }
}

// the start vector: the caller's guess (host or device) or the seeded one
int start_vector(cdft_ctx* c, const double* guess, int on_device, long seed, double* x0) {
  const long N = c->info.N;
  if (guess)
    SP_CK(c, cudaMemcpyAsync(x0, guess, N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  else
    k_seed_vector<<<sp_grid(N), 256, 0, c->stream>>>(x0, N, (unsigned long long)seed);
  if (c->fixed_bg) cdft_internal_boundary_set(c, x0, 0.0);  // src/Eigenvalues.cpp:75-83
  return CDFT_OK;
}

}  // namespace

// Eigenvalues::calculate_eigenvector (src/Eigenvalues.cpp:69-99; objective :44-66): the
// smallest eigenvalue of sg scale (H + vshift vshift^T / 2), sg = -1 with change_sign,
// reported as the reference reports it (divided by scale, sign restored).
int cdft_eigenvalue(cdft_ctx* c, double scale, double tol, int change_sign, const double* vshift, const double* guess, long max_matvecs,
                    double* eigval, double* eigvec, int on_device, cdft_eigen_report* rep) {
  if (!c || !eigval) return CDFT_ERR_ARG;
  const long N = c->info.N;
  if (!(scale > 0) || !(tol > 0) || max_matvecs < 1 || N < 2)
    return cdft_internal_fail(c, CDFT_ERR_ARG, "eigenvalue: needs scale > 0, tol > 0 and max_matvecs >= 1");
  DevBuf buf;
  double *x0 = buf.get(N), *vec = buf.get(N), *vs = vshift ? buf.get(N) : nullptr;
  if (!x0 || !vec || (vshift && !vs)) return cdft_internal_fail(c, CDFT_ERR_CUDA, "eigenvalue: out of device memory");
  if (vshift)
    SP_CK(c, cudaMemcpyAsync(vs, vshift, N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  int rc = start_vector(c, guess, on_device, 20240601, x0);
  if (rc) return rc;
  const double a = (change_sign ? -1.0 : 1.0) * scale;
  SymOp op{c, a, 0.0, vs, nullptr, nullptr, false, 0, N};
  const int ncv = (int)std::min<long>(24, N);
  LanczosResult r;
  rc = lanczos(c, op, Want::Smallest, 1, ncv, tol, true, false, max_matvecs, 1 << 30, x0, vec, &r);
  if (rc) return rc;
  *eigval = r.theta[0] / a;
  if (eigvec)
    SP_CK(c, cudaMemcpyAsync(eigvec, vec, N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
  SP_CK(c, cudaStreamSynchronize(c->stream));
  if (rep) {
    rep->matvecs = op.matvecs;
    rep->restarts = r.restarts;
    rep->converged = r.converged ? 1 : 0;
    rep->residual = r.resid[0] / std::fabs(a);
  }
  return CDFT_OK;
}

// Arnoldi::determine_largest_eigenpairs (src/Arnoldi.cpp:72-283): the k eigenpairs of
// H + shift of largest magnitude, from a k + p dimensional Krylov basis restarted at most
// max_steps times; eigenvalues reported without the shift, in that order.
int cdft_arnoldi_largest(cdft_ctx* c, double shift, int k, int p, int all_k, long max_steps, double tol, const double* guess,
                         double* eigvals, double* eigvecs, int on_device, cdft_eigen_report* rep) {
  if (!c || !eigvals) return CDFT_ERR_ARG;
  const long N = c->info.N;
  if (k < 1 || p < 1 || (long)k + p > N || max_steps < 1 || !(tol > 0))
    return cdft_internal_fail(c, CDFT_ERR_ARG, "arnoldi: needs k >= 1, p >= 1, k + p <= N, max_steps >= 1 and tol > 0");
  DevBuf buf;
  double *x0 = buf.get(N), *vecs = buf.get((size_t)k * N);
  if (!x0 || !vecs) return cdft_internal_fail(c, CDFT_ERR_CUDA, "arnoldi: out of device memory");
  int rc = start_vector(c, guess, on_device, 20240601, x0);
  if (rc) return rc;
  SymOp op{c, 1.0, shift, nullptr, nullptr, nullptr, false, 0, N};
  LanczosResult r;
  rc = lanczos(c, op, Want::LargestMagnitude, k, k + p, tol, all_k != 0, true, 1L << 62, (int)std::min<long>(max_steps, 1 << 30), x0,
               vecs, &r);
  if (rc) return rc;
  const int nw = (int)r.theta.size();
  for (int i = 0; i < k; ++i) eigvals[i] = i < nw ? r.theta[i] - shift : NAN;
  if (eigvecs)
    SP_CK(c, cudaMemcpyAsync(eigvecs, vecs, (size_t)nw * N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             c->stream));
  SP_CK(c, cudaStreamSynchronize(c->stream));
  if (rep) {
    rep->matvecs = op.matvecs;
    rep->restarts = r.restarts;
    rep->converged = r.converged ? 1 : 0;
    rep->residual = r.resid.empty() ? 0 : r.resid[0];
  }
  if (!r.converged) return cdft_internal_fail(c, CDFT_ERR_TIMEOUT, "IRArnoldi method: Exceeded max iterations");
  return CDFT_OK;
}

namespace {
// The eigenvector of the zero eigenvalue of g.H on a periodic lattice: g 1 = 0, so
// g.H x = 0 for H x = 1. Conjugate gradients on H (Hessian products; H is positive
// definite at a stable state), then x / |x|. Returns whether the residual reached
// 1e-10 |1|.
int zero_mode_vector(cdft_ctx* c, double* x, bool* converged) {
  const long N = c->info.N;
  const unsigned g = sp_grid(N);
  cudaStream_t s = c->stream;
  DevBuf buf;
  double *r = buf.get(N), *pv = buf.get(N), *q = buf.get(N), *part = buf.get(kDotBlocks), *dh = buf.get(2);
  if (!r || !pv || !q || !part || !dh) return cdft_internal_fail(c, CDFT_ERR_CUDA, "arnoldi: out of device memory");
  k_fill<<<g, 256, 0, s>>>(x, 0.0, N);
  k_fill<<<g, 256, 0, s>>>(r, 1.0, N);
  k_fill<<<g, 256, 0, s>>>(pv, 1.0, N);
  double rr = (double)N, h[2];
  const double stop = 1e-10 * std::sqrt((double)N);
  *converged = false;
  for (int it = 0; it < 4000; ++it) {
    int rc = cdft_internal_matvec(c, CDFT_MATRIX_HESSIAN, pv, q, false);
    if (rc) return rc;
    dots(pv, 1, q, N, part, dh, s);
    SP_CK(c, cudaMemcpyAsync(h, dh, sizeof(double), cudaMemcpyDeviceToHost, s));
    SP_CK(c, cudaStreamSynchronize(s));
    if (!(h[0] > 0)) break;  // H not positive definite along pv: leave the current iterate
    const double alpha = rr / h[0];
    k_axpby<<<g, 256, 0, s>>>(alpha, pv, 1.0, x, N);
    k_axpby<<<g, 256, 0, s>>>(-alpha, q, 1.0, r, N);
    dots(r, 1, r, N, part, dh + 1, s);
    SP_CK(c, cudaMemcpyAsync(h + 1, dh + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    SP_CK(c, cudaStreamSynchronize(s));
    const double rr_new = h[1];
    if (std::sqrt(rr_new) <= stop) {
      *converged = true;
      break;
    }
    k_axpby<<<g, 256, 0, s>>>(1.0, r, rr_new / rr, pv, N);
    rr = rr_new;
  }
  dots(x, 1, x, N, part, dh, s);
  k_normalise<<<g, 256, 0, s>>>(x, x, dh, N);
  return CDFT_OK;
}
}  // namespace

// Arnoldi::determine_largest_eigenpairs (src/Arnoldi.cpp:72-283) on either matrix of the
// path: the Hessian (as cdft_arnoldi_largest), or the DDFT dynamical matrix g.H (DDFT is a
// Dynamical_Matrix, include/Minimizer.h:189). For g.H the k eigenvalues of largest
// |lambda + shift| come from thick-restart Lanczos on -C H C^T over the range of C
// (MobOp), each eigenvector C^T w normalised, plus, on a periodic lattice, the zero
// eigenvalue of the conserved mass with eigenvector H^-1 1 (zero_mode_vector).
int cdft_arnoldi_largest_matrix(cdft_ctx* c, int matrix, double shift, int k, int p, int all_k, long max_steps, double tol,
                                const double* guess, double* eigvals, double* eigvecs, int on_device, cdft_eigen_report* rep) {
  if (matrix == CDFT_MATRIX_HESSIAN) return cdft_arnoldi_largest(c, shift, k, p, all_k, max_steps, tol, guess, eigvals, eigvecs, on_device, rep);
  if (!c || !eigvals) return CDFT_ERR_ARG;
  if (matrix != CDFT_MATRIX_DDFT) return cdft_internal_fail(c, CDFT_ERR_ARG, "arnoldi: matrix must be CDFT_MATRIX_HESSIAN or CDFT_MATRIX_DDFT");
  const long N = c->info.N, n3 = 3 * N;
  if (k < 1 || p < 1 || (long)k + p > N || max_steps < 1 || !(tol > 0))
    return cdft_internal_fail(c, CDFT_ERR_ARG, "arnoldi: needs k >= 1, p >= 1, k + p <= N, max_steps >= 1 and tol > 0");
  if (c->homo_bd) return cdft_internal_fail(c, CDFT_ERR_ARG, "arnoldi on the DDFT matrix: the homogeneous boundary is not built");
  DevBuf buf;
  double *x0 = buf.get(N), *w0 = buf.get(n3), *tN = buf.get(N), *uN = buf.get(N), *vecs3 = buf.get((size_t)k * n3),
         *out = buf.get((size_t)k * N), *part = buf.get(kDotBlocks), *dh = buf.get(1);
  if (!x0 || !w0 || !tN || !uN || !vecs3 || !out || !part || !dh) return cdft_internal_fail(c, CDFT_ERR_CUDA, "arnoldi: out of device memory");
  int rc = start_vector(c, guess, on_device, 20240601, x0);
  if (rc) return rc;
  const double D = 1.0 / (2.0 * c->p.dx * c->p.dx);
  const unsigned g = sp_grid(N);
  k_mob_c<<<g, 256, 0, c->stream>>>(c->rho, x0, w0, c->p.nx, c->p.ny, c->p.nz, D, 1.0);  // start in the range of C
  MobOp op{c, 0.0, nullptr, nullptr, false, 0, n3, tN, uN, D};
  LanczosResult r;
  rc = lanczos(c, op, Want::LargestMagnitude, k, k + p, tol, all_k != 0, true, 1L << 62, (int)std::min<long>(max_steps, 1 << 30), w0, vecs3,
               &r, shift, true);
  if (rc) return rc;
  struct Cand {
    double lam, res;
    int src;  // Ritz pair index, or -1 for the zero mode
  };
  std::vector<Cand> cand;
  double tmax = 0;
  for (double t : r.theta) tmax = std::max(tmax, std::fabs(t));
  for (int i = 0; i < (int)r.theta.size(); ++i)
    if (std::fabs(r.theta[i]) > 1e-10 * tmax) cand.push_back({r.theta[i], r.resid[i], i});  // not residue outside range(C)
  if (!c->fixed_bg) cand.push_back({0.0, 0.0, -1});
  std::stable_sort(cand.begin(), cand.end(), [&](const Cand& a, const Cand& b) { return std::fabs(a.lam + shift) > std::fabs(b.lam + shift); });
  bool zero_ok = true;
  for (int i = 0; i < k; ++i) {
    double* v = out + (long)i * N;
    if (i >= (int)cand.size()) {
      eigvals[i] = NAN;
      k_fill<<<g, 256, 0, c->stream>>>(v, 0.0, N);
      continue;
    }
    eigvals[i] = cand[i].lam;
    if (cand[i].src >= 0) {
      k_mob_ct<<<g, 256, 0, c->stream>>>(c->rho, vecs3 + (long)cand[i].src * n3, v, c->p.nx, c->p.ny, c->p.nz, D);
      if (c->fixed_bg) cdft_internal_boundary_set(c, v, 0.0);
      dots(v, 1, v, N, part, dh, c->stream);
      k_normalise<<<g, 256, 0, c->stream>>>(v, v, dh, N);
    } else {
      rc = zero_mode_vector(c, v, &zero_ok);
      if (rc) return rc;
    }
  }
  if (eigvecs)
    SP_CK(c, cudaMemcpyAsync(eigvecs, out, (size_t)k * N * sizeof(double), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             c->stream));
  SP_CK(c, cudaStreamSynchronize(c->stream));
  SP_CK(c, cudaGetLastError());
  if (rep) {
    rep->matvecs = op.matvecs;
    rep->restarts = r.restarts;
    rep->converged = (r.converged && zero_ok) ? 1 : 0;
    rep->residual = cand.empty() ? 0 : cand[0].res;
  }
  if (!r.converged) return cdft_internal_fail(c, CDFT_ERR_TIMEOUT, "IRArnoldi method: Exceeded max iterations");
  return CDFT_OK;
}

// FFT-plan autotuner. The evaluation's transforms are mixed-radix Stockham
// passes over shared-memory tiles; the order of the radices changes the
// stride pattern of every stage (bank conflicts, twiddle reuse) and the number
// of odd-radix stages, and the best order differs per axis because each axis
// is transformed by a different kernel (z: the row kernels and the fused Phi
// rows; y: the column tiles; x: the convolution tiles). The tuner times whole
// evaluations on the context's own stream for each candidate ordering of one
// axis at a time (z, then x, then y), keeps the fastest, and remembers the
// result for the grid, model and precision in a process-wide table that
// cdft_create consults, so that later contexts of the same shape start tuned.
#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include "cdft_ctx.h"

using namespace cdft;

namespace {
typedef std::tuple<int, int, int, int, int, int> TuneKey;  // nx, ny, nz, model, lj, precision
std::mutex g_mu;
std::map<TuneKey, std::array<std::vector<int>, 3>> g_plans;

TuneKey key_of(const cdft_ctx* c, int precision) { return TuneKey(c->p.nx, c->p.ny, c->p.nz, c->p.model, c->p.lj ? 1 : 0, precision); }

// Orderings of the power-of-two part into radix-8/4/2 stages with the fewest
// stages (and, for short lengths, one more), each with the odd prime factors
// placed first or last.
void compositions(int a, int parts_left, std::vector<int>& cur, std::vector<std::vector<int>>& out) {
  if (a == 0) {
    if (parts_left == 0) out.push_back(cur);
    return;
  }
  if (parts_left == 0) return;
  for (int e = 3; e >= 1; --e)
    if (e <= a) {
      cur.push_back(1 << e);
      compositions(a - e, parts_left - 1, cur, out);
      cur.pop_back();
    }
}
}  // namespace

std::vector<std::vector<int>> cdft_internal_radix_candidates(int n) {
  int a = 0, m = n;
  while (m % 2 == 0) { m /= 2; ++a; }
  std::vector<int> odd;
  for (int q = 3; m > 1; q += 2)
    while (m % q == 0) { odd.push_back(q); m /= q; }
  std::vector<std::vector<int>> pow2;
  if (a == 0) pow2.push_back({});
  const int smin = (a + 2) / 3;
  for (int st = smin; a > 0 && st <= smin + (a <= 5 ? 1 : 0); ++st) {
    std::vector<int> cur;
    compositions(a, st, cur, pow2);
  }
  std::set<std::vector<int>> seen;
  std::vector<std::vector<int>> out;
  auto add = [&](const std::vector<int>& r) {
    if (seen.insert(r).second) out.push_back(r);
  };
  add(default_radices(n));
  for (const auto& p : pow2) {
    std::vector<int> r = odd;
    r.insert(r.end(), p.begin(), p.end());
    add(r);
    r = p;
    r.insert(r.end(), odd.begin(), odd.end());
    add(r);
  }
  if (out.size() > 12) out.resize(12);
  return out;
}

// Plans remembered for the context's shape, model and precision (false if none).
bool cdft_internal_tuned_plans(const cdft_ctx* c, int precision, std::array<std::vector<int>, 3>* plans) {
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_plans.find(key_of(c, precision));
  if (it == g_plans.end()) return false;
  *plans = it->second;
  return true;
}

static float time_evals(cdft_ctx* c, int reps, cudaEvent_t e0, cudaEvent_t e1) {
  auto run = [&]() {
    if (c->precision == CDFT_FP64) c->e64->launch(c->rho, c->vext, c->dF, c->info.dV, c->mu, 1, c->stream, nullptr);
    else c->e32->launch(c->rho, c->vext, c->dF, c->info.dV, c->mu, 1, c->stream, nullptr);
  };
  run();  // warm
  cudaEventRecord(e0, c->stream);
  for (int i = 0; i < reps; ++i) run();
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  return ms / reps;
}

static void install(cdft_ctx* c, const std::shared_ptr<FFTTable> t[3]) {
  ++c->plan_gen;  // captured evaluation graphs hold the old plans
  c->tx = t[0];
  c->ty = t[1];
  c->tz = t[2];
  if (c->e64) c->e64->set_tables(t[0].get(), t[1].get(), t[2].get());
  if (c->e32) c->e32->set_tables(t[0].get(), t[1].get(), t[2].get());
}

extern "C" int cdft_autotune(cdft_ctx* c, int reps, int* radices_out, double* ms_out) {
  if (!c || reps <= 0) return CDFT_ERR_ARG;
  const int prec = c->precision;
  if ((prec == CDFT_FP64 && !c->e64) || (prec == CDFT_FP32 && !c->e32)) {
    int rc = cdft_set_precision(c, prec);
    if (rc) return rc;
  }
  const int n[3] = {c->p.nx, c->p.ny, c->p.nz};
  std::shared_ptr<FFTTable> cur[3] = {c->tx, c->ty, c->tz};
  std::vector<int> best_r[3];
  for (int a = 0; a < 3; ++a) {
    const FFTPlan& P = cur[a]->plan;
    best_r[a].assign(P.radix, P.radix + P.nst);
  }
  // each axis gets its own tables while tuning (a cubic grid shares one by default)
  std::string err;
  for (int a = 0; a < 3; ++a) {
    cur[a] = make_fft_table(n[a], &err, &best_r[a]);
    if (!cur[a]) return cdft_internal_fail(c, CDFT_ERR_ARG, err);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return cdft_internal_fail(c, CDFT_ERR_CUDA, "autotune events");
  }
  install(c, cur);
  float best = time_evals(c, reps, e0, e1);
  const float base = best;
  const int order[3] = {2, 0, 1};  // z (rows, Phi), x (convolutions), y (columns)
  for (int oi = 0; oi < 3; ++oi) {
    const int a = order[oi];
    for (const auto& r : cdft_internal_radix_candidates(n[a])) {
      if (r == best_r[a]) continue;
      std::shared_ptr<FFTTable> trial[3] = {cur[0], cur[1], cur[2]};
      trial[a] = make_fft_table(n[a], &err, &r);
      if (!trial[a]) continue;
      install(c, trial);
      const float ms = time_evals(c, reps, e0, e1);
      if (ms < best) {
        best = ms;
        best_r[a] = r;
        cur[a] = trial[a];
      }
    }
    install(c, cur);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return cdft_internal_fail(c, CDFT_ERR_CUDA, "autotune launch failed");
  {
    std::lock_guard<std::mutex> g(g_mu);
    g_plans[key_of(c, prec)] = {best_r[0], best_r[1], best_r[2]};
  }
  if (radices_out) {
    for (int a = 0; a < 3; ++a) {
      for (int i = 0; i < 8; ++i) radices_out[a * 8 + i] = i < (int)best_r[a].size() ? best_r[a][i] : 0;
    }
  }
  if (ms_out) {
    ms_out[0] = base;
    ms_out[1] = best;
  }
  return CDFT_OK;
}

extern "C" int cdft_get_radices(const cdft_ctx* c, int* radices_out) {
  if (!c || !radices_out) return CDFT_ERR_ARG;
  const FFTTable* t[3] = {c->tx.get(), c->ty.get(), c->tz.get()};
  for (int a = 0; a < 3; ++a)
    for (int i = 0; i < 8; ++i) radices_out[a * 8 + i] = i < t[a]->plan.nst ? t[a]->plan.radix[i] : 0;
  return CDFT_OK;
}

extern "C" int cdft_radix_candidates(int n, int* out, int max_plans, int* count) {
  if (n < 2 || !count) return CDFT_ERR_ARG;
  const auto cand = cdft_internal_radix_candidates(n);
  *count = (int)cand.size();
  if (out)
    for (int k = 0; k < std::min(max_plans, (int)cand.size()); ++k)
      for (int i = 0; i < 8; ++i) out[k * 8 + i] = i < (int)cand[k].size() ? cand[k][i] : 0;
  return CDFT_OK;
}

// ------------------------------------------- FP64 / FP32 pipe rate probes ---
// Sustained FMA rate of the current device in one precision: every thread runs
// kChains independent dependent-FMA chains (enough in flight to cover the pipe's
// latency), the grid fills every SM several times over. The result is what a pass
// bound by that pipe can reach at best, the denominator of its roofline.
namespace {
constexpr int kChains = 8, kIters = 2048;
template <class T>
__global__ void __launch_bounds__(256) k_fma_chains(T b, T c, T* __restrict__ sink) {
  T a[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) a[j] = (T)(threadIdx.x + j) * (T)1e-3;
  for (int i = 0; i < kIters; ++i)
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = fma(a[j], b, c);
  T s = 0;
#pragma unroll
  for (int j = 0; j < kChains; ++j) s += a[j];
  if (s == (T)12345.678) sink[0] = s;  // never true for these inputs: keeps the chains live
}

template <class T>
int fma_rate(double* tflops, void* stream) {
  if (!tflops) return CDFT_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return CDFT_ERR_CUDA;
  T* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(T)) != cudaSuccess) return CDFT_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // FP32 runs 64x faster than FP64 here: a longer grid keeps its launches well above the timer's resolution
  const unsigned grid = (unsigned)sms * (sizeof(T) == 8 ? 16 : 256);
  k_fma_chains<T><<<grid, 256, 0, s>>>((T)0.999999, (T)1e-7, sink);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0, s);
    k_fma_chains<T><<<grid, 256, 0, s>>>((T)0.999999, (T)1e-7, sink);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess) return CDFT_ERR_CUDA;
  const double flops = 2.0 * kChains * kIters * (double)grid * 256;
  *tflops = flops / (best * 1e-3) / 1e12;
  return CDFT_OK;
}
}  // namespace

int cdft_fp64_fma_rate(double* tflops, void* stream) { return fma_rate<double>(tflops, stream); }
int cdft_fp32_fma_rate(double* tflops, void* stream) { return fma_rate<float>(tflops, stream); }

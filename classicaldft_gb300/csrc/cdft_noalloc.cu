// Number of atoms of a device density without any allocation.
//
// Some callers cannot call cudaMalloc: an application that hands this library
// only device pointers carved from its own memory pool (a cudaMalloc would
// draw device memory outside the pool's budget, and can synchronise the whole
// device while the application's other streams are running). For them this
// file offers a variant of the compensated density sum (Density::getNumberAtoms,
// the reduction behind the fixed-mass constraint) whose scratch lives in a
// file-scope device array instead of context buffers.
//
// The scratch array (64 KiB: one Neumaier (sum, compensation) pair per block
// for at most kMaxBlocks blocks, plus the result) is held by every GPU that
// loads this library until the process exits. Each call writes every scratch
// slot it later reads, so nothing has to be cleared between calls; the array
// keeps the last call's contents. All calls share it: calls whose work
// overlaps on the GPU (different streams, or several host threads) race and
// must be serialised by the caller.
#include <cuda.h>
#include <cuda_runtime.h>
#include <mutex>
#include "../../include/cdft.h"
#include "cdft_kernels.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 32;  // points per thread, so one block covers 8192 points
constexpr long kMaxBlocks = 4096;
constexpr long kMaxPoints = kMaxBlocks * kThreads * kPerThread;  // 2^25 = 33,554,432

static __device__ __align__(256) double g_noalloc_scratch[2 * kMaxBlocks + 8];

__global__ void __launch_bounds__(kThreads) k_sum_blocks(const double* __restrict__ x, long n, double* __restrict__ part) {
  cdft::Acc acc;
  acc.init();
  const long base = (long)blockIdx.x * kThreads * kPerThread;
  for (int j = 0; j < kPerThread; ++j) {
    const long i = base + (long)j * kThreads + threadIdx.x;
    if (i < n) acc.add(x[i]);
  }
  cdft::block_reduce_store<1>(&acc, part, blockIdx.x);
}

__global__ void k_sum_finish(const double* __restrict__ part, long nblk, double scale, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    cdft::Acc a;
    a.init();
    for (long b = 0; b < nblk; ++b) a.merge(part[2 * b], part[2 * b + 1]);
    out[0] = (a.s + a.c) * scale;
  }
}

// Device address of g_noalloc_scratch, resolved with cudaGetSymbolAddress once per
// device (with that device current) on the first call made on it, and resolved
// again if the device's context has been replaced since (after cudaDeviceReset the
// module is loaded anew and the array may sit at another address). Contexts are
// told apart by the driver's never-reused context id.
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};
std::mutex g_scratch_mu;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// id of the calling thread's current context, 0 when there is none or it cannot be read
unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuCtxGetCurrent", &p, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPoint("cuCtxGetId", &p, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(p);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CDFT_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  const unsigned long long id = current_ctx_id();
  if (!g_scratch_ptr[dev] || id == 0 || id != g_scratch_ctx[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return CDFT_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
    g_scratch_ctx[dev] = current_ctx_id();  // the context is current now that the address has been resolved
  }
  *out = g_scratch_ptr[dev];
  return CDFT_OK;
}

}  // namespace

extern "C" int cdft_number_of_atoms_noalloc(const double* rho, long n, double dV, void* stream, double* out) {
  if (!rho || !out || n < 1) return CDFT_ERR_ARG;
  if (n > kMaxPoints) return CDFT_ERR_ARG;  // beyond the scratch array: 2^25 points at most
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long nblk = (n + (long)kThreads * kPerThread - 1) / ((long)kThreads * kPerThread);
  double* part = scratch;
  double* result = scratch + 2 * kMaxBlocks;
  k_sum_blocks<<<(unsigned)nblk, kThreads, 0, s>>>(rho, n, part);
  k_sum_finish<<<1, 32, 0, s>>>(part, nblk, dV, result);
  // a failed launch returns before the copy, so *out is never a previous call's result
  // (this reads, and clears, the runtime's last-error state, as cudaGetLastError does)
  if (cudaGetLastError() != cudaSuccess) return CDFT_ERR_CUDA;
  if (cudaMemcpyAsync(out, result, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return CDFT_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return CDFT_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? CDFT_OK : CDFT_ERR_CUDA;
}

// BF16 tensor-core GEMM for the neural-operator warm start (sm_103a, tcgen05):
//   Y[M x N] = act(X[M x K] . W[K x N] + bias[N] + add[M x N]),
// X and W in BF16, accumulation in FP32 in tensor memory, Y in FP32 (and,
// optionally, the pre-activation Z for the backward pass).
//
// One CTA (4 warps) walks 128-row tiles of X. W^T is staged once in shared
// memory; each X tile is staged by all threads in the no-swizzle K-major
// layout the MMA reads (8-row x 16-byte core matrices: K-adjacent ones 128 B
// apart, row-adjacent 8-row groups 256 B apart, one 128 x 16 sub-tile per
// K step). One elected thread issues K/16 MMAs of shape M128 x N x K16 into a
// TMEM accumulator and commits them to an mbarrier; every thread waits on it
// (bounded: a wait that runs out sets the status word and the CTA stops), then
// each warp reads its 32 accumulator lanes with tcgen05.ld and writes its rows.
// The TMEM columns are allocated once per CTA and freed before it exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include "../../include/cdft.h"
#include "cdft_tma.cuh"

namespace cdft {
namespace tc {

constexpr int kRows = 128;  // MMA M, one accumulator lane per row
constexpr unsigned kStatusTcTimeout = 16u;

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of sm_100-class tensor cores
  // base offset 0, absolute LBO mode off, layout type 0 = no swizzle
  return d;
}

// kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t instr_desc(int n) {
  return (1u << 4)                          // D format FP32
         | (1u << 7)                        // A format BF16
         | (1u << 10)                       // B format BF16
         | ((uint32_t)(n >> 3) << 17)       // N / 8
         | ((uint32_t)(kRows >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 32 columns of FP32 (bits) per warp: thread t gets lane (32 w + t), columns col..col+31.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// byte offset of element (row, k) in the canonical no-swizzle K-major layout of a tile with `rows` rows
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int rows) {
  const int kc = k >> 4, kk = k & 15;
  return (uint32_t)(kc * rows * 32 + (row >> 3) * 256 + (kk >> 3) * 128 + (row & 7) * 16 + (kk & 7) * 2);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }

// K multiple of 16 (<= 64), N multiple of 32 (<= 128), M any (rows past M are zero-filled, not written).
// Dynamic shared memory: the X tile, W^T, and a 32 x 33 FP32 staging block per warp through which the
// accumulator rows are turned into coalesced row-major stores; with N = 32 also the tile's rows of
// the residual input `add`, copied in with the X tile so that the epilogue does not wait on them.
template <int N> struct StageAdd { static constexpr bool value = N == 32; };
template <int N, int K>
__host__ __device__ constexpr size_t smem_bytes() {
  return (size_t)2 * kRows * K * 2 + (size_t)N * K * 2 + (size_t)4 * 32 * 33 * 4  // two X tiles (double buffer)
         + (StageAdd<N>::value ? (size_t)2 * kRows * N * 4 : 0);                   // two add tiles
}

// 16-byte asynchronous copy global -> shared; zero-fills when `valid` is false
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int N, int K>
__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16* __restrict__ X, const __nv_bfloat16* __restrict__ W,
                                                   const float* __restrict__ bias, const float* __restrict__ add, float* __restrict__ Y,
                                                   float* __restrict__ Z, long M, int act, unsigned* __restrict__ status) {
  static_assert(K % 16 == 0 && K <= 64 && N % 32 == 0 && N <= 128, "tile shape");
  constexpr int TCOLS = N <= 32 ? 32 : (N <= 64 ? 64 : 128);  // power of two >= 32
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // the two X tiles by address arithmetic (a pointer array indexed by the buffer would live in local memory)
  auto sxb = [&](int b) { return smem_raw + (size_t)b * kRows * K * 2; };
  unsigned char* sw = smem_raw + (size_t)2 * kRows * K * 2;
  float* ep = reinterpret_cast<float*>(sw + (size_t)N * K * 2);
  constexpr bool SA = StageAdd<N>::value;
  float* sadd0 = ep + 4 * 32 * 33;  // add tiles (SA only): [kRows][N], two buffers
  const bool stage_add = SA && add != nullptr && (reinterpret_cast<uintptr_t>(add) & 15u) == 0;  // 16-byte copies
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int stop;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* my = ep + warp * 32 * 33;
  // W^T (N rows of K) into the canonical layout, once
  for (int e = tid; e < N * K; e += blockDim.x) {
    const int n = e / K, k = e - n * K;
    *reinterpret_cast<__nv_bfloat16*>(sw + kmajor_off(n, k, N)) = W[(long)k * N + n];
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    stop = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)), "r"(TCOLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_base;
  const long ntile = (M + kRows - 1) / kRows;
  constexpr uint32_t idesc = instr_desc(N);
  unsigned phase = 0;
  // X tile t into buffer b: 16-byte chunks (8 BF16 along K), asynchronous, rows past M zero-filled;
  // with stage_add the tile's add rows too (4 floats per chunk)
  auto load_tile = [&](long t, int b) {
    unsigned char* buf = sxb(b);
    const long r0 = t * kRows;
    for (int e = tid; e < kRows * (K / 8); e += blockDim.x) {
      const int r = e / (K / 8), k8 = (e - r * (K / 8)) * 8;
      const bool valid = r0 + r < M;
      cp_async16(buf + kmajor_off(r, k8, kRows), X + (valid ? (r0 + r) * K + k8 : 0), valid);
    }
    if (stage_add) {
      float* sa = sadd0 + (size_t)b * kRows * N;
      for (int e = tid; e < kRows * (N / 4); e += blockDim.x) {
        const int r = e / (N / 4), c4 = (e - r * (N / 4)) * 4;
        const bool valid = r0 + r < M;
        cp_async16(sa + r * N + c4, add + (valid ? (r0 + r) * N + c4 : 0), valid);
      }
    }
    cp_async_commit();
  };
  if (blockIdx.x < ntile) load_tile(blockIdx.x, 0);
  int b = 0;
  for (long t = blockIdx.x; t < ntile; t += gridDim.x, b ^= 1) {
    const long row0 = t * kRows;
    unsigned char* sx = sxb(b);
    cp_async_wait_all();  // this tile's copies (the only group in flight)
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    // the next tile streams into the other buffer while this one is multiplied and stored
    if (t + gridDim.x < ntile) load_tile(t + gridDim.x, b ^ 1);
    if (tid == 0) {
      const uint32_t ax = smem_u32(sx), aw = smem_u32(sw);
#pragma unroll
      for (int kc = 0; kc < K / 16; ++kc)
        mma_bf16(tmem, smem_desc(ax + kc * kRows * 32, 128, 256), smem_desc(aw + kc * N * 32, 128, 256), idesc, kc > 0);
      mma_commit(&bar);
    }
    bool ok = mbar_wait(&bar, phase, status);
    phase ^= 1u;
    if (!ok) atomicOr(&stop, 1);
    fence_after();
    __syncthreads();
    if (stop) break;
    // epilogue: warp w owns accumulator lanes 32w..32w+31 (rows of the tile); each 32-column
    // block goes through the warp's staging block so that a store instruction writes one row
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 32) {
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) my[lane * 33 + j] = __uint_as_float(v[j]);
      __syncwarp();
      const int col = c0 + lane;
      const float bc = bias ? bias[col] : 0.f;
      const float* sa = sadd0 + (size_t)b * kRows * N;
      for (int r = 0; r < 32; ++r) {
        const long row = row0 + warp * 32 + r;
        if (row >= M) break;
        float z = my[r * 33 + lane] + bc;
        if (stage_add) z += sa[(warp * 32 + r) * N + col];
        else if (add) z += add[row * N + col];
        if (Z) Z[row * N + col] = z;
        Y[row * N + col] = act ? gelu(z) : z;
      }
      __syncwarp();
    }
    fence_before();
    __syncthreads();  // the tile buffer and the accumulator are reused by the next tile
    fence_after();
  }
  cp_async_wait_all();  // no copy may still target shared memory when the CTA exits
  if (stop && tid == 0) {
    atomicOr(status, kStatusTcTimeout);
    mbar_wait(&bar, phase ^ 1u, nullptr);  // bounded: the MMAs still in flight before their columns are freed
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS) : "memory");
}

}  // namespace tc
}  // namespace cdft

using namespace cdft::tc;

template <int N, int K>
static int launch_gemm(const void* X, const void* W, const float* bias, const float* add, float* Y, float* Z, long M, int act,
                       unsigned* status, cudaStream_t s) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long ntile = (M + kRows - 1) / kRows;
  constexpr size_t sm = smem_bytes<N, K>();
  static int per_sm = 0;  // resident CTAs per SM: the persistent grid is that many per SM
  if (!per_sm) {
    cudaFuncSetAttribute(k_gemm_bf16<N, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_bf16<N, K>, 128, sm);
    per_sm = std::max(1, std::min(per_sm, 4));
  }
  const unsigned grid = (unsigned)std::min<long>(ntile, (long)nsm * per_sm);
  k_gemm_bf16<N, K><<<grid, 128, sm, s>>>(reinterpret_cast<const __nv_bfloat16*>(X), reinterpret_cast<const __nv_bfloat16*>(W), bias, add,
                                          Y, Z, M, act, status);
  return cudaGetLastError() == cudaSuccess ? CDFT_OK : CDFT_ERR_CUDA;
}

// Y = act(X . W + bias + add); X: M x K BF16 row-major, W: K x N BF16 row-major,
// bias (N), add (M x N) and Z (pre-activation out) may be NULL; act 0 none, 1 GELU (erf).
// K in {16, 32, 48, 64}, N in {32, 64, 128}. All device pointers; X rows 16-byte aligned.
extern "C" int cdft_tc_gemm_bf16(const void* X, const void* W, const float* bias, const float* add, float* Y, float* Z, long M, int K,
                                 int N, int act, void* status_dev, void* stream) {
  if (!X || !W || !Y || M <= 0 || !status_dev) return CDFT_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(X) & 15u) != 0) return CDFT_ERR_ARG;
  unsigned* st = static_cast<unsigned*>(status_dev);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
#define CDFT_TC_CASE(NN, KK) \
  if (N == NN && K == KK) return launch_gemm<NN, KK>(X, W, bias, add, Y, Z, M, act, st, s);
  CDFT_TC_CASE(32, 16) CDFT_TC_CASE(32, 32) CDFT_TC_CASE(32, 48) CDFT_TC_CASE(32, 64)
  CDFT_TC_CASE(64, 16) CDFT_TC_CASE(64, 32) CDFT_TC_CASE(64, 64)
  CDFT_TC_CASE(128, 16) CDFT_TC_CASE(128, 32) CDFT_TC_CASE(128, 64)
#undef CDFT_TC_CASE
  return CDFT_ERR_ARG;
}

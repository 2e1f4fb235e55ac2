// Exhaustive / structured check of the integer-pipe FP64 <-> FP32 conversions
// (cdft_convert.cuh) against the hardware conversions:
//   float -> double: all 2^32 bit patterns;
//   double -> float: every exponent with fractions at and around the rounding
//   boundaries of the normal and the subnormal ranges, plus random patterns.
// NaN inputs only need a NaN output. Prints the mismatch counts; exit 0.
#include <cstdio>
#include <cuda_runtime.h>
#include "../../classicaldft_gb300/csrc/cdft_convert.cuh"

using cdft::cvt_f32;
using cdft::cvt_f64;

__device__ unsigned long long mix64(unsigned long long x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_f64_all(unsigned long long* bad, unsigned int* first) {
  const unsigned long long total = 1ull << 32;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const float f = __uint_as_float((unsigned int)i);
    const double a = cvt_f64(f), b = (double)f;
    const bool ok = (f != f) ? (a != a) : (__double_as_longlong(a) == __double_as_longlong(b));
    if (!ok && atomicAdd(bad, 1ull) == 0ull) *first = (unsigned int)i;
  }
}

__global__ void k_f32_structured(unsigned long long* bad, unsigned long long* first, long per_exp) {
  // one (exponent, sign) pair per blockIdx.y; per_exp patterns each
  const int ex = blockIdx.y >> 1;
  const unsigned long long sign = (unsigned long long)(blockIdx.y & 1) << 63;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < per_exp; i += (long)gridDim.x * blockDim.x) {
    const unsigned long long r = mix64((unsigned long long)i * 4096ull + (unsigned long long)blockIdx.y);
    unsigned long long frac = r & 0xFFFFFFFFFFFFFull;
    // force the bits below a rounding position to 0, half - 1, half or half + 1
    const int kind = (int)(i & 7);
    int s = 29;                          // normal results drop 29 bits
    if (ex <= 896) s = 926 - ex;         // subnormal results drop more
    if (kind >= 4 && s >= 1 && s <= 52) {
      const unsigned long long mask = (1ull << s) - 1, half = 1ull << (s - 1);
      unsigned long long low = kind == 4 ? 0ull : kind == 5 ? half - 1 : kind == 6 ? half : half + 1;
      frac = (frac & ~mask) | (low & mask);
    }
    const unsigned long long bits = sign | ((unsigned long long)ex << 52) | frac;
    const double x = __longlong_as_double((long long)bits);
    const float a = cvt_f32(x), b = __double2float_rn(x);
    const bool ok = (x != x) ? (a != a) : (__float_as_uint(a) == __float_as_uint(b));
    if (!ok && atomicAdd(bad, 1ull) == 0ull) *first = bits;
  }
}

int main() {
  unsigned long long* bad;
  unsigned int* first32;
  unsigned long long* first64;
  if (cudaMalloc(&bad, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMalloc(&first32, sizeof(unsigned int));
  cudaMalloc(&first64, sizeof(unsigned long long));
  cudaMemset(bad, 0, 2 * sizeof(unsigned long long));
  cudaMemset(first32, 0, sizeof(unsigned int));
  cudaMemset(first64, 0, sizeof(unsigned long long));
  k_f64_all<<<152 * 8, 256>>>(bad, first32);
  const long per_exp = 1L << 16;  // 2^16 patterns x 2048 exponents x 2 signs
  k_f32_structured<<<dim3(64, 4096), 256>>>(bad + 1, first64, per_exp);
  const cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    printf("cuda error %s\n", cudaGetErrorString(e));
    return 3;
  }
  unsigned long long hb[2], f64;
  unsigned int f32;
  cudaMemcpy(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
  cudaMemcpy(&f32, first32, sizeof(f32), cudaMemcpyDeviceToHost);
  cudaMemcpy(&f64, first64, sizeof(f64), cudaMemcpyDeviceToHost);
  printf("f32_to_f64_checked %llu mismatches %llu first 0x%08x\n", 1ull << 32, hb[0], f32);
  printf("f64_to_f32_checked %llu mismatches %llu first 0x%016llx\n", (unsigned long long)per_exp * 4096ull, hb[1], f64);
  return 0;
}

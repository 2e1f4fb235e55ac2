// FP64 <-> FP32 conversions on the integer pipes (sm_103a device code).
#pragma once

namespace cdft {

// FP64 <-> FP32 conversions on the integer pipes. GB300 runs F2F conversions
// through its small FP64 unit, which made them the bottleneck of the row passes
// that read the FP64 density and write the FP64 dF. Both restate IEEE 754
// round-to-nearest-even conversion in integer arithmetic for every input,
// normal or not, so that no hardware conversion can be executed speculatively
// on the common path: zeros, subnormal results, overflow to infinity,
// infinities and (quietened) NaNs included.
__device__ __forceinline__ float cvt_f32(double x) {
  const unsigned long long d = (unsigned long long)__double_as_longlong(x);
  const unsigned int sign = (unsigned int)(d >> 63) << 31;
  const int ex = (int)((d >> 52) & 0x7FF);
  const int e = ex - 1023 + 127;
  if (e > 0 && e < 255) {
    unsigned int u = sign | ((unsigned int)e << 23) | (unsigned int)((d >> 29) & 0x7FFFFFu);
    const unsigned long long rest = d & 0x1FFFFFFFull;  // the 29 bits dropped
    if (rest > 0x10000000ull || (rest == 0x10000000ull && (u & 1u))) u += 1u;  // a carry moves into the exponent correctly
    return __uint_as_float(u);
  }
  const unsigned long long frac = d & 0xFFFFFFFFFFFFFull;
  if (ex == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (frac ? (0x400000u | (unsigned int)(frac >> 29)) : 0u));
  if (e >= 255) return __uint_as_float(sign | 0x7F800000u);  // finite overflow rounds to infinity
  // |x| < 2^-126: a subnormal float q * 2^-149 with q = m * 2^(ex - 926), m the 53-bit significand
  const int shift = 926 - ex;  // >= 30
  if (ex == 0 || shift >= 54) return __uint_as_float(sign);  // below half the smallest subnormal
  const unsigned long long m = frac | (1ull << 52);
  unsigned long long q = m >> shift;
  const unsigned long long rem = m & ((1ull << shift) - 1), half = 1ull << (shift - 1);
  if (rem > half || (rem == half && (q & 1ull))) q += 1ull;  // q = 2^23 encodes the smallest normal
  return __uint_as_float(sign | (unsigned int)q);
}
__device__ __forceinline__ double cvt_f64(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e != 0u && e != 0xFFu)
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29)));
  if (e == 0xFFu)
    return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull | ((unsigned long long)m << 29) | (m ? (1ull << 51) : 0ull)));
  if (m == 0u) return __longlong_as_double((long long)sign);
  // subnormal float m * 2^-149 = 1.f * 2^(p - 149), p the position of m's leading bit
  const int p = 31 - __clz((int)m);
  return __longlong_as_double((long long)(sign | ((unsigned long long)(p + 874) << 52) |
                                          (((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFull)));
}

}  // namespace cdft

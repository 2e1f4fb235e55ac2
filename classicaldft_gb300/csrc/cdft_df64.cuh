// Double-float ("df64") arithmetic for the FP64 transforms on sm_103a.
//
// GB300 issues FP64 instructions at 1/64 of its FP32 rate, and the FP64 passes of an
// evaluation keep that pipe ~84% busy, most of it in FFT butterflies. A transform
// needs only normwise accuracy, so its stages run here on pairs of floats: a value
// is hi + lo with |lo| <= ulp(hi) / 2, 48 significant bits, the unit roundoff
// 2^-48 ~ 3.6e-15 (against FP64's 1.1e-16). The arithmetic is the classical
// error-free transformations: TwoSum (Knuth) and the FMA form of TwoProduct, the
// double-word addition whose error is bounded by u^2 (|a| + |b|) (normwise, which is
// what an FFT's error analysis needs) and the double-word product with error
// ~2 u^2 |ab| (Joldes, Muller, Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44, 2017: algorithms
// "DWPlusDW" in its sloppy form and "DWTimesDW"). Every operation is an explicit
// round-to-nearest intrinsic, so the compiler cannot contract or reassociate it.
//
// Values enter and leave a transform as doubles: dfs_split (hi the rounded float,
// lo the rounded remainder: one FP64 subtraction, the conversions on the integer
// pipe) and dfs_join (one FP64 addition). A complex df64 value is 16 bytes, the size
// of a double2, so the shared-memory tiles keep their layout.
#pragma once
#include <cuda_runtime.h>
#include "cdft_convert.cuh"
#include "cdft_types.h"

namespace cdft {

struct dfs {
  float h, l;
  __host__ __device__ dfs() {}
  __host__ __device__ constexpr dfs(float a, float b) : h(a), l(b) {}
  __host__ __device__ constexpr dfs(int z) : h((float)z), l(0.f) {}  // small integer constants, exact
  // a constant (folded at compile time for literals): hi the nearest float, lo the rest
  __host__ __device__ constexpr explicit dfs(double d) : h((float)d), l((float)(d - (double)(float)d)) {}
};
struct dfc {
  dfs x, y;
};
template <> struct Cx<dfs> { typedef dfc type; };

__device__ __forceinline__ dfs df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  const float e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
  return dfs(s, e);
}
__device__ __forceinline__ dfs df_fast_two_sum(float a, float b) {  // |a| >= |b| or a = 0
  const float s = __fadd_rn(a, b);
  return dfs(s, __fadd_rn(b, -__fadd_rn(s, -a)));
}
__device__ __forceinline__ dfs operator+(dfs a, dfs b) {
  const dfs s = df_two_sum(a.h, b.h);
  return df_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfs operator-(dfs a) { return dfs(-a.h, -a.l); }
__device__ __forceinline__ dfs operator-(dfs a, dfs b) { return a + (-b); }
__device__ __forceinline__ dfs operator*(dfs a, dfs b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ dfs& operator+=(dfs& a, dfs b) { return a = a + b; }
__device__ __forceinline__ dfs& operator-=(dfs& a, dfs b) { return a = a - b; }
__device__ __forceinline__ dfs& operator*=(dfs& a, dfs b) { return a = a * b; }

// a / 2, exact (both parts scaled by a power of two)
__device__ __forceinline__ dfs df_half(dfs a) { return dfs(__fmul_rn(0.5f, a.h), __fmul_rn(0.5f, a.l)); }

// double -> df64: hi = RN(d), lo = RN(d - hi); d - hi is exact in FP64
__device__ __forceinline__ dfs dfs_split(double d) {
  const float h = cvt_f32(d);
  return dfs(h, cvt_f32(d - cvt_f64(h)));
}
// df64 -> double: hi + lo, rounded once
__device__ __forceinline__ double dfs_join(dfs a) { return cvt_f64(a.h) + cvt_f64(a.l); }
__device__ __forceinline__ dfc dfc_split(double2 z) {
  dfc r;
  r.x = dfs_split(z.x);
  r.y = dfs_split(z.y);
  return r;
}
__device__ __forceinline__ double2 dfc_join(dfc z) { return make_double2(dfs_join(z.x), dfs_join(z.y)); }

}  // namespace cdft

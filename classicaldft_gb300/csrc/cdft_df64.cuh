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
#include "cdft_df_log_table.h"
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

// ---- inside a transform's butterfly: arithmetic without the closing renormalisation ----
// TwoSum of the high parts is exact whatever their sizes, so a butterfly may carry a pair
// (h, l) whose low part exceeds ulp(h) / 2 (after a cancellation), as long as l stays of
// the order of u times the magnitudes summed into it, which is what an FFT's normwise
// bound needs. The sums skip the closing FastTwoSum (8 FP32 operations instead of 11), a
// twiddle product forms each component as one two-term dot product (16 instead of 25),
// and the values a transform leaves are renormalised once (df_renorm), while its inner
// stages pass unnormalised pairs on. In a float32 emulation of the 128- and 256-point
// transforms (tests/cpp/df64_fft_emulation.cpp: random, near-constant and DC-dominated
// inputs) the normwise error stays within 3x of that of the renormalising operations above
// (worst 4.7e-14 against 1.6e-14); a transform's first stage is given normalised pairs
// (unnormalised weight products there raised the evaluation's Omega error tenfold).
__device__ __forceinline__ dfs dfl_add(dfs a, dfs b) {
  const dfs s = df_two_sum(a.h, b.h);
  return dfs(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfs dfl_mul(dfs a, dfs b) {  // the product's error term left unnormalised
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  return dfs(p, __fmaf_rn(a.l, b.h, e));
}
// a1 b1 + a2 b2: both exact products of the high parts summed by TwoSum, the cross terms
// and the products' errors gathered in one float
__device__ __forceinline__ dfs dfl_dot2(dfs a1, dfs b1, dfs a2, dfs b2) {
  const float p = __fmul_rn(a1.h, b1.h), q = __fmul_rn(a2.h, b2.h);
  const float e1 = __fmaf_rn(a1.h, b1.h, -p), e2 = __fmaf_rn(a2.h, b2.h, -q);
  const dfs s = df_two_sum(p, q);
  float c = __fmaf_rn(a1.h, b1.l, e1);
  c = __fmaf_rn(a1.l, b1.h, c);
  c = __fmaf_rn(a2.h, b2.l, c);
  c = __fmaf_rn(a2.l, b2.h, c);
  c = __fadd_rn(c, e2);
  return dfs(s.h, __fadd_rn(c, s.l));
}
__device__ __forceinline__ dfs df_renorm(dfs a) { return df_fast_two_sum(a.h, a.l); }

// a / 2, exact (both parts scaled by a power of two)
__device__ __forceinline__ dfs df_half(dfs a) { return dfs(__fmul_rn(0.5f, a.h), __fmul_rn(0.5f, a.l)); }

// double -> df64: hi = RN(d), lo = RN(d - hi); d - hi is exact in FP64
__device__ __forceinline__ dfs dfs_split(double d) {
  const float h = cvt_f32(d);
  return dfs(h, cvt_f32(d - cvt_f64(h)));
}
// df64 -> double: hi + lo, rounded once
__device__ __forceinline__ double dfs_join(dfs a) { return cvt_f64(a.h) + cvt_f64(a.l); }
__device__ __forceinline__ bool operator<(dfs a, dfs b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ dfs df_abs(dfs a) { return a.h < 0.f ? -a : a; }

// 1 / b: the FP32 reciprocal refined by two residual corrections in df64 (each residual
// 1 - b q is formed with exact products), relative error ~5e-15
__device__ __forceinline__ dfs df_rcp(dfs b) {
  const float y = __frcp_rn(b.h);
  dfs r = dfs(1) - b * dfs(y, 0.f);
  const float q2 = __fmul_rn(r.h, y);
  r = r - b * dfs(q2, 0.f);
  const float q3 = __fmul_rn(r.h, y);
  return df_fast_two_sum(y, q2) + dfs(q3, 0.f);
}
__device__ __forceinline__ dfs operator/(dfs a, dfs b) { return a * df_rcp(b); }

// ---- logarithms in df64, table-driven (P. T. P. Tang, "Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 16, 1990): 1 + x = 2^k F (1 + r)
// with F = 1 + j/128 (j = -32..64, so that F and 2^-k (1 + x) lie within 1/256 of each
// other), u = 2^-k (1 + x) - F formed exactly (Sterbenz), r = u / F, and
// log(1 + x) = k ln2 + log F + log1p(r), |r| <= 2^-8, where log1p(r) = r - r^2/2 + r^3/3
// + r^4 q(r) takes its first three terms in df64 and q (a cubic) in FP32. Near x = 0 the
// reduction is skipped (k = 0, F = 1), so the result keeps its relative accuracy there.
// Relative error ~1.3e-14 (against ~1e-16 in FP64; a float32 emulation of these operations,
// tests/cpp/df64_log_emulation.cpp), far inside the evaluation's 1e-12.
// The table (log F and 1/F as df64, from 50-digit decimal arithmetic: cdft_df_log_table.h)
// is read from shared memory: a kernel calls df_log_table_init once, which copies it there
// from global memory, and synchronises before the first logarithm.
constexpr int kDfLogLo = -32, kDfLogN = 97;
static __device__ const float4 kDfLogTable[kDfLogN] = {CDFT_DF_LOG_TABLE};
__device__ __forceinline__ float4* df_log_table() {
  __shared__ float4 t[kDfLogN];
  return t;
}
__device__ __forceinline__ void df_log_table_init(int tid, int nthreads) {
  float4* t = df_log_table();
  for (int i = tid; i < kDfLogN; i += nthreads) t[i] = __ldg(&kDfLogTable[i]);
}
__device__ __forceinline__ dfs df_ln2() { return dfs(0.6931471805599453094); }
__device__ __forceinline__ dfs df_third() { return dfs(0.3333333333333333333); }
__device__ __forceinline__ dfs df_log1p_reduced(dfs r) {  // |r| <= 2^-8
  const dfs r2 = r * r, r3 = r2 * r;
  const float rh = r.h;
  const float q = __fmaf_rn(rh, __fmaf_rn(rh, __fmaf_rn(rh, 0.142857142857f, -0.166666666667f), 0.2f), -0.25f);
  const float r4q = __fmul_rn(__fmul_rn(r2.h, r2.h), q);
  return (r + (r3 * df_third() + (-df_half(r2)))) + dfs(r4q, 0.f);
}
__device__ __forceinline__ dfs df_log1p(dfs x) {
  if (fabsf(x.h) < 0.00390625f) return df_log1p_reduced(x);
  const float y = __fadd_rn(1.0f, x.h);
  if (!(y >= 1.17549435e-38f && y <= 1.0e30f)) return dfs_split(log1p(dfs_join(x)));  // 1 + x <= 0, huge, NaN: FP64
  const int bits = __float_as_int(y);
  int k = ((bits >> 23) & 0xff) - 127;
  float m = __int_as_float((bits & 0x007fffff) | 0x3f800000);  // y = 2^k m, m in [1, 2)
  if (m >= 1.5f) {
    m = __fmul_rn(m, 0.5f);
    ++k;
  }
  int j = __float2int_rn(__fmul_rn(__fadd_rn(m, -1.0f), 128.0f));
  j = j < kDfLogLo ? kDfLogLo : (j > kDfLogLo + kDfLogN - 1 ? kDfLogLo + kDfLogN - 1 : j);
  const float F = __fmaf_rn((float)j, 0.0078125f, 1.0f);
  const float p = __int_as_float((127 - k) << 23);  // 2^-k (k in [-126, 100] here)
  const dfs u = dfs(__fadd_rn(p, -F), 0.f) + dfs(__fmul_rn(x.h, p), __fmul_rn(x.l, p));
  const float4 t = df_log_table()[j - kDfLogLo];
  const dfs lf = dfs(t.x, t.y) + dfs((float)k, 0.f) * df_ln2();
  return lf + df_log1p_reduced(u * dfs(t.z, t.w));
}
// log x for x > 0: x = 2^k m, m in [0.75, 1.5), log x = k ln2 + log1p(m - 1 + lo 2^-k)
__device__ __forceinline__ dfs df_log(dfs x) {
  if (!(x.h >= 1.17549435e-38f && x.h <= 1.0e30f)) return dfs_split(log(dfs_join(x)));  // zero, subnormal, huge, NaN: FP64
  const int bits = __float_as_int(x.h);
  int k = ((bits >> 23) & 0xff) - 127;
  float m = __int_as_float((bits & 0x007fffff) | 0x3f800000);
  if (m >= 1.5f) {
    m = __fmul_rn(m, 0.5f);
    ++k;
  }
  const float p = __int_as_float((127 - k) << 23);
  const dfs u = df_two_sum(__fadd_rn(m, -1.0f), __fmul_rn(x.l, p));
  return dfs((float)k, 0.f) * df_ln2() + df_log1p(u);
}

// df64 with the butterflies' sums and products (dfl_add, dfl_mul) as its operators, for the
// per-point functional of the Phi pass: its outputs feed the forward transforms and its value
// the Phi sum, both with normwise bounds. The logarithm, reciprocals and comparisons
// renormalise their arguments first (norm()).
struct dfl {
  float h, l;
  __device__ dfl() {}
  __device__ constexpr dfl(int z) : h((float)z), l(0.f) {}  // small integer constants, exact
  __device__ constexpr explicit dfl(double d) : h((float)d), l((float)(d - (double)(float)d)) {}
  __device__ explicit dfl(dfs a) : h(a.h), l(a.l) {}
  __device__ dfs norm() const { return df_fast_two_sum(h, l); }
  __device__ dfs raw() const { return dfs(h, l); }
};
__device__ __forceinline__ dfl mk_dfl(dfs a) { return dfl(a); }
__device__ __forceinline__ dfl operator+(dfl a, dfl b) { return mk_dfl(dfl_add(a.raw(), b.raw())); }
__device__ __forceinline__ dfl operator-(dfl a) { return mk_dfl(dfs(-a.h, -a.l)); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) { return mk_dfl(dfl_mul(a.raw(), b.raw())); }
__device__ __forceinline__ dfl operator/(dfl a, dfl b) { return a * mk_dfl(df_rcp(b.norm())); }
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { return a = a - b; }
__device__ __forceinline__ bool operator<(dfl a, dfl b) { return a.norm() < b.norm(); }

__device__ __forceinline__ dfc dfc_split(double2 z) {
  dfc r;
  r.x = dfs_split(z.x);
  r.y = dfs_split(z.y);
  return r;
}
__device__ __forceinline__ double2 dfc_join(dfc z) { return make_double2(dfs_join(z.x), dfs_join(z.y)); }

}  // namespace cdft

// Float32 emulation of the double-float logarithm and reciprocal of the FP64 evaluation
// (df_log1p, df_log, df_rcp in classicaldft_gb300/csrc/cdft_df64.cuh), operation for
// operation, with the same table (cdft_df_log_table.h), against long double. Prints the
// largest relative error of each over a spread of arguments.
// Build: g++ -O2 -ffp-contract=off -I classicaldft_gb300/csrc
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include "cdft_df_log_table.h"

typedef long double LD;
struct dw {
  float h, l;
};
static const float kTable[97][4] = {CDFT_DF_LOG_TABLE};

static dw two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
static dw fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
static dw add(dw a, dw b) {
  const dw s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, s.l + (a.l + b.l));
}
static dw neg(dw a) { return {-a.h, -a.l}; }
static dw mul(dw a, dw b) {
  const float p = a.h * b.h;
  float e = std::fmaf(a.h, b.h, -p);
  e = std::fmaf(a.h, b.l, e);
  e = std::fmaf(a.l, b.h, e);
  return fast_two_sum(p, e);
}
static dw constant(double d) {
  const float h = (float)d;
  return {h, (float)(d - (double)h)};
}
static dw split(LD v) {
  const float h = (float)v;
  return {h, (float)(v - (LD)h)};
}
static LD value(dw a) { return (LD)a.h + (LD)a.l; }
static int bits_of(float f) {
  int b;
  std::memcpy(&b, &f, 4);
  return b;
}
static float float_of(int b) {
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

static dw rcp(dw b) {
  const float y = 1.0f / b.h;
  dw r = add({1.0f, 0.0f}, neg(mul(b, {y, 0.0f})));
  const float q2 = r.h * y;
  r = add(r, neg(mul(b, {q2, 0.0f})));
  const float q3 = r.h * y;
  return add(fast_two_sum(y, q2), {q3, 0.0f});
}
static dw log1p_reduced(dw r) {
  const dw r2 = mul(r, r), r3 = mul(r2, r);
  const float rh = r.h;
  const float q = std::fmaf(rh, std::fmaf(rh, std::fmaf(rh, 0.142857142857f, -0.166666666667f), 0.2f), -0.25f);
  const float r4q = (r2.h * r2.h) * q;
  const dw half_r2 = {0.5f * r2.h, 0.5f * r2.l};
  return add(add(r, add(mul(r3, constant(0.3333333333333333333)), neg(half_r2))), {r4q, 0.0f});
}
static dw log1p_df(dw x) {  // the arguments here keep 1 + x in the normal float range
  if (std::fabs(x.h) < 0.00390625f) return log1p_reduced(x);
  const float y = 1.0f + x.h;
  const int bits = bits_of(y);
  int k = ((bits >> 23) & 0xff) - 127;
  float m = float_of((bits & 0x007fffff) | 0x3f800000);
  if (m >= 1.5f) {
    m = m * 0.5f;
    ++k;
  }
  int j = (int)std::nearbyint((m - 1.0f) * 128.0f);
  j = j < -32 ? -32 : (j > 64 ? 64 : j);
  const float F = std::fmaf((float)j, 0.0078125f, 1.0f);
  const float p = float_of((127 - k) << 23);
  const dw u = add({p - F, 0.0f}, {x.h * p, x.l * p});
  const float* t = kTable[j + 32];
  const dw lf = add({t[0], t[1]}, mul({(float)k, 0.0f}, constant(0.6931471805599453094)));
  return add(lf, log1p_reduced(mul(u, {t[2], t[3]})));
}
static dw log_df(dw x) {  // x a normal float range value
  const int bits = bits_of(x.h);
  int k = ((bits >> 23) & 0xff) - 127;
  float m = float_of((bits & 0x007fffff) | 0x3f800000);
  if (m >= 1.5f) {
    m = m * 0.5f;
    ++k;
  }
  const float p = float_of((127 - k) << 23);
  const dw u = two_sum(m - 1.0f, x.l * p);
  return add(mul({(float)k, 0.0f}, constant(0.6931471805599453094)), log1p_df(u));
}

int main() {
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> U(0, 1);
  double w_log1p = 0, w_log = 0, w_rcp = 0;
  for (int i = 0; i < 200000; ++i) {
    const int kind = i % 4;
    LD x;
    if (kind == 0) x = -0.999 + 1.899 * U(g);                 // eta-like arguments and beyond
    else if (kind == 1) x = -std::pow(10.0L, -12 + 11.99 * U(g));  // small negative (log(1 - eta) near 0)
    else if (kind == 2) x = std::pow(10.0L, -12 + 12.5 * U(g));    // small and moderate positive
    else x = -0.004 + 0.008 * U(g);                             // around the reduction's threshold
    const dw xd = split(x);
    const LD xe = value(xd);
    const LD ref = std::log1p(xe);
    if (ref != 0) w_log1p = std::max(w_log1p, (double)(std::fabs(value(log1p_df(xd)) - ref) / std::fabs(ref)));
    const LD z = std::pow(10.0L, -30 + 55 * U(g));  // densities and other positive values
    const dw zd = split(z);
    const LD ze = value(zd), lz = std::log(ze);
    if (std::fabs(lz) > 1e-6) w_log = std::max(w_log, (double)(std::fabs(value(log_df(zd)) - lz) / std::fabs(lz)));
    else w_log = std::max(w_log, (double)std::fabs(value(log_df(zd)) - lz));
    const LD b = (U(g) < 0.5 ? -1 : 1) * std::pow(10.0L, -20 + 40 * U(g));
    const dw bd = split(b);
    const LD be = value(bd);
    w_rcp = std::max(w_rcp, (double)(std::fabs(value(rcp(bd)) - 1 / be) * std::fabs(be)));
  }
  std::printf("%.4e %.4e %.4e\n", w_log1p, w_log, w_rcp);
  return 0;
}

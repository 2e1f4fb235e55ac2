// Float32 emulation of the double-float ("df64") transforms of the FP64 evaluation
// (classicaldft_gb300/csrc/cdft_df64.cuh, cdft_fft_df.cuh): the 128- and 256-point
// Stockham transforms with the device's radix order (4 4 8 and 4 4 4 4), computed
//   R: with the renormalising double-word operations (sum: TwoSum of the high parts, the low
//      parts added, FastTwoSum; product: FMA TwoProduct plus the cross terms, FastTwoSum),
//   L: as the device does it: sums without the closing FastTwoSum, each twiddle product's
//      component as one two-term dot product, and only the values that leave the transform
//      renormalised,
// against a long-double DFT of the same (exactly representable) input. Prints, per length,
// input kind and direction, the largest normwise error (|error| / max |output|) of each.
// Build: g++ -O2 -ffp-contract=off (every float operation rounded as written).
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

typedef long double LD;
struct dw {
  float h, l;
};
struct dwc {
  dw x, y;
};

static dw two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
static dw fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
static dw neg(dw a) { return {-a.h, -a.l}; }
// renormalising operations
static dw r_add(dw a, dw b) {
  const dw s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, s.l + (a.l + b.l));
}
static dw r_mul(dw a, dw b) {
  const float p = a.h * b.h;
  float e = std::fmaf(a.h, b.h, -p);
  e = std::fmaf(a.h, b.l, e);
  e = std::fmaf(a.l, b.h, e);
  return fast_two_sum(p, e);
}
// the device's lazy operations
static dw l_add(dw a, dw b) {
  const dw s = two_sum(a.h, b.h);
  return {s.h, s.l + (a.l + b.l)};
}
static dw l_mul(dw a, dw b) {
  const float p = a.h * b.h;
  float e = std::fmaf(a.h, b.h, -p);
  e = std::fmaf(a.h, b.l, e);
  return {p, std::fmaf(a.l, b.h, e)};
}
static dw l_dot2(dw a1, dw b1, dw a2, dw b2) {
  const float p = a1.h * b1.h, q = a2.h * b2.h;
  const float e1 = std::fmaf(a1.h, b1.h, -p), e2 = std::fmaf(a2.h, b2.h, -q);
  const dw s = two_sum(p, q);
  float c = std::fmaf(a1.h, b1.l, e1);
  c = std::fmaf(a1.l, b1.h, c);
  c = std::fmaf(a2.h, b2.l, c);
  c = std::fmaf(a2.l, b2.h, c);
  c = c + e2;
  return {s.h, c + s.l};
}
static dw split(LD v) {
  const float h = (float)v;
  return {h, (float)(v - (LD)h)};
}
static LD value(dw a) { return (LD)a.h + (LD)a.l; }

template <bool LAZY>
struct Ops {
  static dw add(dw a, dw b) { return LAZY ? l_add(a, b) : r_add(a, b); }
  static dw mul(dw a, dw b) { return LAZY ? l_mul(a, b) : r_mul(a, b); }
  static dwc cadd(dwc a, dwc b) { return {add(a.x, b.x), add(a.y, b.y)}; }
  static dwc csub(dwc a, dwc b) { return {add(a.x, neg(b.x)), add(a.y, neg(b.y))}; }
  static dwc mul_i(dwc a, int dir) { return dir < 0 ? dwc{a.y, neg(a.x)} : dwc{neg(a.y), a.x}; }
  static dwc twiddle(dwc a, dwc w, int dir) {  // a w (forward) or a conj(w) (backward)
    if (LAZY) {
      if (dir < 0) return {l_dot2(a.x, w.x, neg(a.y), w.y), l_dot2(a.x, w.y, a.y, w.x)};
      return {l_dot2(a.x, w.x, a.y, w.y), l_dot2(a.y, w.x, neg(a.x), w.y)};
    }
    if (dir < 0) return {r_add(r_mul(a.x, w.x), neg(r_mul(a.y, w.y))), r_add(r_mul(a.x, w.y), r_mul(a.y, w.x))};
    return {r_add(r_mul(a.x, w.x), r_mul(a.y, w.y)), r_add(r_mul(a.y, w.x), neg(r_mul(a.x, w.y)))};
  }
  static void dft4(dwc* a, int dir) {
    const dwc t0 = cadd(a[0], a[2]), t1 = csub(a[0], a[2]), t2 = cadd(a[1], a[3]), t3 = mul_i(csub(a[1], a[3]), dir);
    a[0] = cadd(t0, t2);
    a[2] = csub(t0, t2);
    a[1] = cadd(t1, t3);
    a[3] = csub(t1, t3);
  }
  static void dft8(dwc* a, int dir) {
    const dw r = split(0.70710678118654752440084436210484903928L);
    dwc e[4] = {a[0], a[2], a[4], a[6]}, o[4] = {a[1], a[3], a[5], a[7]};
    dft4(e, dir);
    dft4(o, dir);
    const dwc o1 = o[1], o3 = o[3];
    if (dir < 0) {
      o[1] = {mul(r, add(o1.x, o1.y)), mul(r, add(o1.y, neg(o1.x)))};
      o[3] = {mul(r, add(o3.y, neg(o3.x))), neg(mul(r, add(o3.x, o3.y)))};
    } else {
      o[1] = {mul(r, add(o1.x, neg(o1.y))), mul(r, add(o1.x, o1.y))};
      o[3] = {neg(mul(r, add(o3.x, o3.y))), mul(r, add(o3.x, neg(o3.y)))};
    }
    o[2] = mul_i(o[2], dir);
    for (int k = 0; k < 4; ++k) {
      a[k] = cadd(e[k], o[k]);
      a[k + 4] = csub(e[k], o[k]);
    }
  }
  // Stockham, decimation in frequency: y[k + s(p q + t)] = (sum_j x[k + s(q + m j)] w_p^jt) w_len^qt
  static std::vector<dwc> fft(std::vector<dwc> x, int dir) {
    const int n = (int)x.size();
    std::vector<int> radix;
    for (int m = n; m > 1;) {
      int a = 0;
      while ((1 << (a + 1)) <= m) ++a;
      const int f = a == 3 ? 8 : 4;
      radix.push_back(f);
      m /= f;
    }
    std::vector<dwc> y(n);
    int len = n;
    for (size_t st = 0; st < radix.size(); ++st) {
      const int p = radix[st], m = len / p, s = n / len;
      for (int q = 0; q < m; ++q)
        for (int k = 0; k < s; ++k) {
          dwc a[8];
          for (int j = 0; j < p; ++j) a[j] = x[k + s * (q + m * j)];
          if (p == 8) dft8(a, dir);
          else dft4(a, dir);
          for (int t = 0; t < p; ++t) {
            dwc v = a[t];
            if (m > 1 && t > 0) {
              const LD ang = -2.0L * 3.141592653589793238462643383279502884L * q * t / len;
              v = twiddle(v, dwc{split(std::cos(ang)), split(std::sin(ang))}, dir);
            }
            y[k + s * (p * q + t)] = v;
          }
        }
      std::swap(x, y);
      len = m;
    }
    if (LAZY)
      for (auto& v : x) v = {fast_two_sum(v.x.h, v.x.l), fast_two_sum(v.y.h, v.y.l)};
    return x;
  }
};

int main() {
  std::mt19937_64 g(1);
  std::uniform_real_distribution<double> U(-1, 1);
  for (int n : {128, 256})
    for (int kind = 0; kind < 3; ++kind)
      for (int dir : {-1, 1}) {
        double worst[2] = {0, 0};
        for (int trial = 0; trial < 60; ++trial) {
          std::vector<dwc> xd(n);
          std::vector<std::complex<LD>> xs(n);
          for (int i = 0; i < n; ++i) {
            LD re, im;
            if (kind == 0) {  // random
              re = U(g);
              im = U(g);
            } else if (kind == 1) {  // near-constant field: a large mean, small variations
              re = 0.5 + 1e-6 * U(g);
              im = 0.5 + 1e-6 * U(g);
            } else {  // a spectrum dominated by its first coefficient
              re = i == 0 ? 1e4 : 1e-3 * U(g);
              im = i == 0 ? -3e3 : 1e-3 * U(g);
            }
            xd[i] = {split(re), split(im)};
            xs[i] = {value(xd[i].x), value(xd[i].y)};
          }
          std::vector<std::complex<LD>> ref(n);
          LD norm = 0;
          for (int k = 0; k < n; ++k) {
            std::complex<LD> acc = 0;
            for (int j = 0; j < n; ++j) {
              const LD ang = dir * 2.0L * 3.141592653589793238462643383279502884L * (LD)((long)j * k % n) / n;
              acc += xs[j] * std::complex<LD>(std::cos(ang), std::sin(ang));
            }
            ref[k] = acc;
            norm = std::max(norm, std::abs(acc));
          }
          const std::vector<dwc> out[2] = {Ops<false>::fft(xd, dir), Ops<true>::fft(xd, dir)};
          for (int v = 0; v < 2; ++v)
            for (int k = 0; k < n; ++k) {
              const LD e = std::abs(std::complex<LD>(value(out[v][k].x), value(out[v][k].y)) - ref[k]);
              worst[v] = std::max(worst[v], (double)(e / norm));
            }
        }
        std::printf("%d %d %d %.4e %.4e\n", n, kind, dir, worst[0], worst[1]);
      }
  return 0;
}

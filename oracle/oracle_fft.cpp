// FP64 FFT for the oracle: mixed-radix Stockham (radices 4, 2, 3, 5 and a
// direct DFT for any other prime), unnormalised, sign -1 forward / +1 backward.
// 3D real transforms follow FFTW's r2c/c2r conventions, which the reference
// uses through DFT_FFT (include/DFT_LinAlg.h:163-211): the half spectrum keeps
// kz = 0..nz/2, and c2r ignores the imaginary parts of the kz = 0 and kz = nz/2
// planes. Two real rows are transformed as one complex row.
// TEST INFRASTRUCTURE ONLY (see oracle.h).
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>
#include "oracle.h"

typedef std::complex<double> cd;

namespace {

struct Plan1D {
  int n;
  std::vector<int> radix;
  std::vector<std::vector<cd>> tw_fwd;  // per stage: twiddles exp(-2 pi i q t / len)
  std::vector<std::vector<cd>> root_fwd;  // per stage: exp(-2 pi i t / p) for generic radices
};

cd expi(long num, long den, int sign) {
  // exp(sign * 2 pi i num/den) with the angle reduced to [0, 2pi)
  num %= den;
  if (num < 0) num += den;
  const long double a = 6.283185307179586476925286766559005768L * (long double)num / (long double)den;
  return cd((double)cosl(a), (double)(sign * sinl(a)));
}

std::shared_ptr<Plan1D> make_plan(int n) {
  auto P = std::make_shared<Plan1D>();
  P->n = n;
  int m = n;
  while (m > 1) {
    int r = 0;
    if (m % 4 == 0) r = 4;
    else if (m % 2 == 0) r = 2;
    else if (m % 3 == 0) r = 3;
    else if (m % 5 == 0) r = 5;
    else {
      for (int f = 7; f <= m; f += 2)
        if (m % f == 0) { r = f; break; }
    }
    P->radix.push_back(r);
    m /= r;
  }
  int len = n;
  for (int r : P->radix) {
    int sub = len / r;
    std::vector<cd> tw((size_t)sub * r);
    for (int q = 0; q < sub; ++q)
      for (int t = 0; t < r; ++t) tw[(size_t)q * r + t] = expi((long)q * t, len, -1);
    P->tw_fwd.push_back(tw);
    std::vector<cd> roots(r);
    for (int t = 0; t < r; ++t) roots[t] = expi(t, r, -1);
    P->root_fwd.push_back(roots);
    len = sub;
  }
  return P;
}

std::shared_ptr<Plan1D> get_plan(int n) {
  static std::mutex mu;
  static std::map<int, std::shared_ptr<Plan1D>> cache;
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(n);
  if (it != cache.end()) return it->second;
  auto p = make_plan(n);
  cache[n] = p;
  return p;
}

// Stockham decimation-in-frequency: at each stage of radix p on sub-length len
// (stride s), output y[q' + s*(p*q + t)] = (sum_j x[q' + s*(q + m*j)] w_p^{jt}) w_len^{qt}.
void fft1d(const Plan1D& P, cd* x, cd* work, int sign) {
  const int n = P.n;
  cd* a = x;
  cd* b = work;
  int len = n, s = 1;
  for (size_t st = 0; st < P.radix.size(); ++st) {
    const int p = P.radix[st];
    const int m = len / p;
    const std::vector<cd>& tw = P.tw_fwd[st];
    const std::vector<cd>& rt = P.root_fwd[st];
    cd in[64], out[64];
    for (int q = 0; q < m; ++q) {
      for (int k = 0; k < s; ++k) {
        for (int j = 0; j < p; ++j) in[j] = a[k + s * (q + m * j)];
        if (p == 2) {
          out[0] = in[0] + in[1];
          out[1] = in[0] - in[1];
        } else if (p == 4) {
          cd t0 = in[0] + in[2], t1 = in[0] - in[2], t2 = in[1] + in[3], t3 = in[1] - in[3];
          cd jt3 = (sign < 0) ? cd(t3.imag(), -t3.real()) : cd(-t3.imag(), t3.real());
          out[0] = t0 + t2;
          out[2] = t0 - t2;
          out[1] = t1 + jt3;
          out[3] = t1 - jt3;
        } else {
          for (int t = 0; t < p; ++t) {
            cd acc = 0;
            for (int j = 0; j < p; ++j) {
              cd w = rt[((long)j * t) % p];
              if (sign > 0) w = std::conj(w);
              acc += in[j] * w;
            }
            out[t] = acc;
          }
        }
        for (int t = 0; t < p; ++t) {
          cd w = tw[(size_t)q * p + t];
          if (sign > 0) w = std::conj(w);
          b[k + s * (p * q + t)] = out[t] * w;
        }
      }
    }
    std::swap(a, b);
    len = m;
    s *= p;
  }
  if (a != x) std::memcpy(x, a, sizeof(cd) * n);
}

// Complex FFT along one axis of a [n0][n1][n2c] complex array.
void fft_axis(cd* data, int n0, int n1, int n2c, int axis, int sign) {
  const int n = axis == 0 ? n0 : n1;
  auto P = get_plan(n);
  const long stride = axis == 0 ? (long)n1 * n2c : (long)n2c;
  const long lines = axis == 0 ? (long)n1 * n2c : (long)n0 * n2c;
#pragma omp parallel
  {
    std::vector<cd> buf(n), work(n);
#pragma omp for schedule(static)
    for (long L = 0; L < lines; ++L) {
      long base;
      if (axis == 0) base = L;
      else base = (L / n2c) * (long)n1 * n2c + (L % n2c);
      for (int i = 0; i < n; ++i) buf[i] = data[base + i * stride];
      fft1d(*P, buf.data(), work.data(), sign);
      for (int i = 0; i < n; ++i) data[base + i * stride] = buf[i];
    }
  }
}

}  // namespace

extern "C" void orc_r2c(int nx, int ny, int nz, const double* in, double* out_c) {
  const int nzc = nz / 2 + 1;
  cd* out = reinterpret_cast<cd*>(out_c);
  auto P = get_plan(nz);
  const long rows = (long)nx * ny;
#pragma omp parallel
  {
    std::vector<cd> buf(nz), work(nz);
#pragma omp for schedule(static)
    for (long r = 0; r < rows; r += 2) {
      const bool two = (r + 1 < rows);
      for (int k = 0; k < nz; ++k) buf[k] = cd(in[r * nz + k], two ? in[(r + 1) * nz + k] : 0.0);
      fft1d(*P, buf.data(), work.data(), -1);
      for (int k = 0; k < nzc; ++k) {
        cd X = buf[k], Y = std::conj(buf[(nz - k) % nz]);
        out[r * nzc + k] = 0.5 * (X + Y);
        if (two) out[(r + 1) * nzc + k] = cd(0, -0.5) * (X - Y);
      }
    }
  }
  fft_axis(out, nx, ny, nzc, 1, -1);
  fft_axis(out, nx, ny, nzc, 0, -1);
}

extern "C" void orc_c2r(int nx, int ny, int nz, const double* in_c, double* out) {
  const int nzc = nz / 2 + 1;
  std::vector<cd> w(reinterpret_cast<const cd*>(in_c), reinterpret_cast<const cd*>(in_c) + (size_t)nx * ny * nzc);
  fft_axis(w.data(), nx, ny, nzc, 0, +1);
  fft_axis(w.data(), nx, ny, nzc, 1, +1);
  auto P = get_plan(nz);
  const long rows = (long)nx * ny;
#pragma omp parallel
  {
    std::vector<cd> buf(nz), work(nz);
#pragma omp for schedule(static)
    for (long r = 0; r < rows; r += 2) {
      const bool two = (r + 1 < rows);
      // Hermitian-extend both rows; drop Im of kz = 0 and kz = nz/2 (even nz).
      auto row = [&](long rr, int k) -> cd {
        cd v;
        if (k < nzc) v = w[rr * nzc + k];
        else v = std::conj(w[rr * nzc + (nz - k)]);
        if (k == 0 || (nz % 2 == 0 && k == nz / 2)) v = cd(v.real(), 0.0);
        return v;
      };
      for (int k = 0; k < nz; ++k) {
        cd A = row(r, k);
        cd B = two ? row(r + 1, k) : cd(0, 0);
        buf[k] = A + cd(0, 1) * B;
      }
      fft1d(*P, buf.data(), work.data(), +1);
      for (int k = 0; k < nz; ++k) {
        out[r * nz + k] = buf[k].real();
        if (two) out[(r + 1) * nz + k] = buf[k].imag();
      }
    }
  }
}

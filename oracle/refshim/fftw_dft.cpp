// Restatement of the DFTs that FFTW3 computes for the reference's 3D r2c/c2r
// plans (FFTW manual, "What FFTW Really Computes"): forward
//   Y[k] = sum_n X[n] exp(-2 pi i k.n/N)    (r2c keeps kz = 0..Nz/2)
// backward
//   Y[n] = sum_k X[k] exp(+2 pi i k.n/N)    (c2r, Hermitian-extended along z;
//   the imaginary parts of the kz = 0 and kz = Nz/2 planes are ignored, as
//   FFTW's c2r does).
// Each axis is a radix-2 FFT (power-of-two lengths) or a direct O(n^2) DFT in
// long double with twiddles reduced mod n: slower than FFTW but at least as
// accurate. It is only used on the small grids of the golden-vector runs.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <vector>
#include "fftw3.h"

typedef std::complex<long double> cld;

struct refshim_fftw_plan_s {
  int n0, n1, n2;
  bool r2c;
  double* real;
  fftw_complex* cplx;
};

static std::vector<cld> twiddles(int n, int sign) {
  std::vector<cld> t(n);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int k = 0; k < n; ++k) {
    long double a = two_pi * (long double)k / (long double)n;
    t[k] = cld(cosl(a), sign * sinl(a));
  }
  return t;
}

// Iterative radix-2 decimation-in-time FFT of one gathered line (n a power of 2).
static void fft_pow2(std::vector<cld>& a, const std::vector<cld>& tw) {
  const int n = (int)a.size();
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int step = n / len;
    for (int i = 0; i < n; i += len)
      for (int k = 0; k < len / 2; ++k) {
        cld u = a[i + k], v = a[i + k + len / 2] * tw[k * step];
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
  }
}

// In-place DFT of lines of length n with element stride `stride`; line starts
// given by base offsets. Direct summation unless n is a power of two.
static void dft_lines(cld* data, int n, long stride, const std::vector<long>& bases, int sign) {
  std::vector<cld> tw = twiddles(n, sign);
  std::vector<cld> tmp(n);
  const bool pow2 = (n & (n - 1)) == 0;
  for (long b : bases) {
    if (pow2) {
      for (int j = 0; j < n; ++j) tmp[j] = data[b + (long)j * stride];
      fft_pow2(tmp, tw);
    } else {
      for (int k = 0; k < n; ++k) {
        cld s(0, 0);
        for (int j = 0; j < n; ++j) s += data[b + (long)j * stride] * tw[((long)j * k) % n];
        tmp[k] = s;
      }
    }
    for (int k = 0; k < n; ++k) data[b + (long)k * stride] = tmp[k];
  }
}

extern "C" {

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double* in, fftw_complex* out, unsigned) {
  return new refshim_fftw_plan_s{n0, n1, n2, true, in, out};
}
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex* in, double* out, unsigned) {
  return new refshim_fftw_plan_s{n0, n1, n2, false, out, in};
}
void fftw_destroy_plan(fftw_plan p) { delete p; }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int) {}

void fftw_execute(const fftw_plan p) {
  const int n0 = p->n0, n1 = p->n1, n2 = p->n2, nc = n2 / 2 + 1;
  if (p->r2c) {
    std::vector<cld> w((size_t)n0 * n1 * n2);
    for (size_t i = 0; i < w.size(); ++i) w[i] = cld(p->real[i], 0);
    std::vector<long> bases;
    for (long i = 0; i < (long)n0 * n1; ++i) bases.push_back(i * n2);
    dft_lines(w.data(), n2, 1, bases, -1);
    bases.clear();
    for (long i = 0; i < n0; ++i) for (long k = 0; k < n2; ++k) bases.push_back(i * n1 * n2 + k);
    dft_lines(w.data(), n1, n2, bases, -1);
    bases.clear();
    for (long j = 0; j < n1; ++j) for (long k = 0; k < n2; ++k) bases.push_back(j * n2 + k);
    dft_lines(w.data(), n0, (long)n1 * n2, bases, -1);
    for (long i = 0; i < (long)n0 * n1; ++i)
      for (int k = 0; k < nc; ++k) {
        p->cplx[i * nc + k][0] = (double)w[i * n2 + k].real();
        p->cplx[i * nc + k][1] = (double)w[i * n2 + k].imag();
      }
  } else {
    std::vector<cld> w((size_t)n0 * n1 * nc);
    for (size_t i = 0; i < w.size(); ++i) w[i] = cld(p->cplx[i][0], p->cplx[i][1]);
    std::vector<long> bases;
    for (long i = 0; i < n0; ++i) for (long k = 0; k < nc; ++k) bases.push_back(i * n1 * nc + k);
    dft_lines(w.data(), n1, nc, bases, +1);
    bases.clear();
    for (long j = 0; j < n1; ++j) for (long k = 0; k < nc; ++k) bases.push_back(j * nc + k);
    dft_lines(w.data(), n0, (long)n1 * nc, bases, +1);
    std::vector<cld> tw = twiddles(n2, +1);
    for (long i = 0; i < (long)n0 * n1; ++i) {
      const cld* X = &w[i * nc];
      for (int n = 0; n < n2; ++n) {
        long double s = X[0].real();
        int kmax = (n2 % 2 == 0) ? n2 / 2 - 1 : (n2 - 1) / 2;
        for (int k = 1; k <= kmax; ++k) s += 2.0L * (X[k] * tw[((long)k * n) % n2]).real();
        if (n2 % 2 == 0) s += ((n % 2) ? -1.0L : 1.0L) * X[n2 / 2].real();
        p->real[i * n2 + n] = (double)s;
      }
    }
  }
}

}  // extern "C"

// Storage for the reference's DFT_Vec / DFT_Vec_Complex (declared in its
// include/DFT_LinAlg.h). The reference ships this part as an optional adapter
// over Armadillo (additionalCode/DFT_Armadillo.cpp); Armadillo is not
// installed here, so this file restates the same element-wise semantics over
// std::vector: zero-initialised storage, BLAS-1 updates, max-abs / 2-norms,
// dot products and the complex Schur product with optional conjugation.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <vector>
using namespace std;
#include "DFT_LinAlg.h"

typedef std::vector<double> rvec;
typedef std::vector<std::complex<double>> cvec;
#define R(p) (*static_cast<rvec*>(p))
#define C(p) (*static_cast<cvec*>(p))

DFT_Vec::DFT_Vec(unsigned N) : data_(new rvec(N, 0.0)) {}
DFT_Vec::DFT_Vec(const DFT_Vec& v) : data_(new rvec(R(v.data_))) {}
DFT_Vec::DFT_Vec() : data_(new rvec(1, 0.0)) {}
DFT_Vec& DFT_Vec::operator=(const DFT_Vec& v) { R(data_) = R(v.data_); return *this; }
DFT_Vec::~DFT_Vec() { delete static_cast<rvec*>(data_); }

void DFT_Vec::set(unsigned pos, double val) { R(data_)[pos] = val; }
double DFT_Vec::get(unsigned pos) const { return R(data_)[pos]; }
void DFT_Vec::set(const DFT_Vec& v) { R(data_) = R(v.data_); }
void DFT_Vec::set(const DFT_Vec& v1, const DFT_Vec& v2, double scale) {
  const rvec &a = R(v1.data_), &b = R(v2.data_);
  rvec out(a.size());
  for (size_t i = 0; i < a.size(); ++i) out[i] = a[i] + b[i] * scale;
  R(data_) = out;
}
void DFT_Vec::set(double d) { std::fill(R(data_).begin(), R(data_).end(), d); }
void DFT_Vec::set(const double* x, unsigned n) { R(data_).assign(x, x + n); }
void DFT_Vec::set_random_normal() { throw std::runtime_error("refshim: set_random_normal unused"); }
void DFT_Vec::set_random() { throw std::runtime_error("refshim: set_random unused"); }
void DFT_Vec::resize(long N) { R(data_).resize(N, 0.0); }
void DFT_Vec::zeros(long N) { R(data_).assign(N, 0.0); }
void DFT_Vec::zeros() { std::fill(R(data_).begin(), R(data_).end(), 0.0); }
double DFT_Vec::inf_norm() const {
  double m = 0;
  for (double x : R(data_)) m = std::max(m, std::fabs(x));
  return m;
}
double DFT_Vec::euclidean_norm() const {
  double s = 0;
  for (double x : R(data_)) s += x * x;
  return std::sqrt(s);
}
void DFT_Vec::normalise() { MultBy(1.0 / euclidean_norm()); }
double DFT_Vec::min() const { return *std::min_element(R(data_).begin(), R(data_).end()); }
double DFT_Vec::max() const { return *std::max_element(R(data_).begin(), R(data_).end()); }
double* DFT_Vec::memptr() { return R(data_).data(); }
unsigned DFT_Vec::size() const { return R(data_).size(); }
double DFT_Vec::dotWith(const DFT_Vec& v) const {
  const rvec &a = R(data_), &b = R(v.data_);
  if (a.size() != b.size()) throw std::runtime_error("refshim: dot of vectors of different sizes");
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
double DFT_Vec::accu() const {
  double s = 0;
  for (double x : R(data_)) s += x;
  return s;
}
void DFT_Vec::MultBy(double val) { for (double& x : R(data_)) x *= val; }
void DFT_Vec::IncrementBy(const DFT_Vec& v) { rvec& a = R(data_); const rvec& b = R(v.data_); for (size_t i = 0; i < a.size(); ++i) a[i] += b[i]; }
void DFT_Vec::DecrementBy(const DFT_Vec& v) { rvec& a = R(data_); const rvec& b = R(v.data_); for (size_t i = 0; i < a.size(); ++i) a[i] -= b[i]; }
void DFT_Vec::add(double shift) { for (double& x : R(data_)) x += shift; }
void DFT_Vec::IncrementBy(unsigned pos, double val) { R(data_)[pos] += val; }
void DFT_Vec::IncrementBy_Scaled_Vector(const DFT_Vec& v, double scale) {
  rvec& a = R(data_); const rvec& b = R(v.data_);
  for (size_t i = 0; i < a.size(); ++i) a[i] += b[i] * scale;
}
void DFT_Vec::Schur(const DFT_Vec& v1, const DFT_Vec& v2) {
  const rvec &a = R(v1.data_), &b = R(v2.data_);
  rvec out(a.size());
  for (size_t i = 0; i < a.size(); ++i) out[i] = a[i] * b[i];
  R(data_) = out;
}
void DFT_Vec::save(ofstream& of) const { of << *this; }
void DFT_Vec::load(ifstream& in) { in >> *this; }

DFT_Vec_Complex::DFT_Vec_Complex(unsigned N) : data_(new cvec(N)) {}
DFT_Vec_Complex::DFT_Vec_Complex(const DFT_Vec_Complex& v) : data_(new cvec(C(v.data_))) {}
DFT_Vec_Complex::DFT_Vec_Complex() : data_(new cvec(1)) {}
DFT_Vec_Complex::~DFT_Vec_Complex() { delete static_cast<cvec*>(data_); }
void DFT_Vec_Complex::set(const DFT_Vec_Complex& v) { C(data_) = C(v.data_); }
void DFT_Vec_Complex::set(unsigned pos, complex<double> val) { C(data_)[pos] = val; }
complex<double> DFT_Vec_Complex::get(unsigned pos) const { return C(data_)[pos]; }
void DFT_Vec_Complex::MultBy(double val) { for (auto& x : C(data_)) x *= val; }
void DFT_Vec_Complex::Schur(const DFT_Vec_Complex& v1, const DFT_Vec_Complex& v2, bool conj_) {
  const cvec &a = C(v1.data_), &b = C(v2.data_);
  cvec out(a.size());
  for (size_t i = 0; i < a.size(); ++i) out[i] = a[i] * (conj_ ? std::conj(b[i]) : b[i]);
  C(data_) = out;
}
void DFT_Vec_Complex::incrementSchur(const DFT_Vec_Complex& v1, const DFT_Vec_Complex& v2, bool conj_) {
  cvec& o = C(data_);
  const cvec &a = C(v1.data_), &b = C(v2.data_);
  for (size_t i = 0; i < a.size(); ++i) o[i] += a[i] * (conj_ ? std::conj(b[i]) : b[i]);
}
void DFT_Vec_Complex::resize(long N) { C(data_).resize(N); }
void DFT_Vec_Complex::zeros(long N) { C(data_).assign(N, std::complex<double>(0, 0)); }
void DFT_Vec_Complex::zeros() { std::fill(C(data_).begin(), C(data_).end(), std::complex<double>(0, 0)); }
complex<double> DFT_Vec_Complex::max() const { throw std::runtime_error("refshim: complex max unused"); }
complex<double> DFT_Vec_Complex::min() const { throw std::runtime_error("refshim: complex min unused"); }
complex<double>* DFT_Vec_Complex::memptr() { return C(data_).data(); }
unsigned DFT_Vec_Complex::size() const { return C(data_).size(); }

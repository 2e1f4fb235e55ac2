// FP64 CPU restatement of classicalDFT's F+dF evaluation, FIRE2 and DDFT.
// TEST INFRASTRUCTURE ONLY (see oracle.h). Citations are paths in the
// reference project.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

typedef std::complex<double> cd;

namespace {

// ------------------------------------------------------------------ sums ---
// Neumaier compensated sum (include/Summation.h:15-56); partial sums from
// threads are combined by adding (sum, c) componentwise (:39-44).
struct Neumaier {
  double s = 0, c = 0;
  void add(double v) {
    double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) c += (s - t) + v;
    else c += (v - t) + s;
    s = t;
  }
  void merge(const Neumaier& o) { s += o.s; c += o.c; }
  double sum() const { return s + c; }
};

template <class F>
double par_sum(long n, F f) {
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  std::vector<Neumaier> part(nt);
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
#pragma omp for schedule(static)
    for (long i = 0; i < n; ++i) part[t].add(f(i));
  }
  Neumaier tot;
  for (auto& p : part) tot.merge(p);
  return tot.sum();
}

// ---------------------------------------------------------- FMT weights ---
// Analytic cell-averaged weights of a sphere (src/FMT_Species.cpp:112-308).
struct IInt { double v[5]; };
// The polynomial terms below keep the reference's left-to-right evaluation
// order so that the weights agree to the last bit.
IInt integrals_I(double X, double A) {  // getI, :112-123
  double a = std::asin(X / A), b = std::sqrt(std::fabs(A * A - X * X));
  IInt I;
  I.v[0] = 0.5 * X * b + 0.5 * A * A * a;
  I.v[1] = -(1.0 / 3) * (A * A - X * X) * b;
  I.v[2] = 0.125 * X * (2 * X * X - A * A) * b + 0.125 * A * A * A * A * a;
  I.v[3] = -(1.0 / 15) * (A * A - X * X) * (3 * X * X + 2 * A * A) * b;
  I.v[4] = (1.0 / 48) * (8 * X * X * X * X - 2 * A * A * X * X - 3 * A * A * A * A) * X * b + 0.0625 * A * A * A * A * A * A * a;
  return I;
}
const double kTinyDen = 1e-15;  // :125
inline double clamp1(double x) { return std::max(-1.0, std::min(1.0, x)); }
IInt integrals_J(double X, double V, double R) {  // getJ, :127-145
  double aV = std::asin(clamp1(V / std::max(kTinyDen, std::sqrt(R * R - X * X))));
  double aX = std::asin(clamp1(X / std::sqrt(R * R - V * V)));
  double aVX = std::asin(clamp1(X * V / std::max(kTinyDen, std::sqrt((R * R - V * V) * (R * R - X * X)))));
  double b = std::sqrt(std::fabs(R * R - V * V - X * X));
  IInt J;
  J.v[0] = X * aV + V * aX - R * aVX;
  J.v[1] = -0.5 * V * b + 0.5 * (X * X - R * R) * aV;
  J.v[2] = -(1.0 / 6) * V * (V * V - 3 * R * R) * aX + (1.0 / 3) * X * X * X * aV - (1.0 / 3) * R * R * R * aVX - (1.0 / 6) * V * X * b;
  J.v[3] = 0.25 * (X * X * X * X - R * R * R * R) * aV + (M_PI / 8) * R * R * R * R - (V / 12.0) * (5 * R * R + X * X - 2 * V * V) * b;
  J.v[4] = 0.025 * X * V * (3 * V * V - 2 * X * X - 7 * R * R) * b + 0.025 * V * (3 * V * V * V * V - 10 * V * V * R * R + 15 * R * R * R * R) * aX +
           0.2 * X * X * X * X * X * aV - 0.2 * R * R * R * R * R * aVX;
  return J;
}

struct GArgs {  // the shared pieces of G_eta/G_s/G_vx/G_txx/G_txy
  double R, X, Vy, Vz, Tx, Ty, Tz;
  IInt Iy, Iz, Jy, Jz;
};
GArgs g_args(double R, double X, double Vy, double Vz, double Tx, double Ty, double Tz) {
  GArgs g;
  R += 1e-15;  // the reference's guard against NaN, :152
  g.R = R; g.X = X; g.Vy = Vy; g.Vz = Vz; g.Tx = Tx; g.Ty = Ty; g.Tz = Tz;
  g.Iy = integrals_I(X, std::sqrt(R * R - Vy * Vy));
  g.Iz = integrals_I(X, std::sqrt(R * R - Vz * Vz));
  g.Jy = integrals_J(X, Vy, R);
  g.Jz = integrals_J(X, Vz, R);
  return g;
}

double G_eta(const GArgs& g) {  // :147-191
  const double R = g.R, X = g.X, Vy = g.Vy, Vz = g.Vz, Tx = g.Tx, Ty = g.Ty, Tz = g.Tz;
  const double* Iy = g.Iy.v; const double* Iz = g.Iz.v; const double* Jy = g.Jy.v; const double* Jz = g.Jz.v;
  double A = Ty * Tz * Vy * Vz + 0.25 * Vy * Vy * Vz * Vz + 0.125 * R * R * R * R - (1.0 / 6) * (Ty * Vy * Vy * Vy + Tz * Vz * Vz * Vz) -
             0.5 * Tz * Vz * Vy * Vy - 0.5 * Ty * Vy * Vz * Vz + 0.125 * Vy * Vy * Vy * Vy + 0.125 * Vz * Vz * Vz * Vz +
             0.5 * R * R * (Ty * Vy + Tz * Vz - 0.5 * Vy * Vy - 0.5 * Vz * Vz + 0.5 * M_PI * Ty * Tz);
  double B = 0.5 * Ty * Vy + 0.5 * Tz * Vz - 0.25 * Vy * Vy - 0.25 * Vz * Vz + (M_PI / 4) * Ty * Tz + 0.25 * R * R;
  double C = 0.5 * Ty * Vy + (1.0 / 3) * (R * R - Vy * Vy);
  double D = 0.5 * Tz * Vz + (1.0 / 3) * (R * R - Vz * Vz);
  double v = Tx * A * X - 0.5 * A * X * X - (1.0 / 3) * B * Tx * X * X * X + 0.25 * X * X * X * X * B + 0.025 * Tx * X * X * X * X * X -
             (1.0 / 48) * X * X * X * X * X * X;
  v -= 0.5 * Ty * Tz * (Tx * R * R * Jy[0] - R * R * Jy[1] - Tx * Jy[2] + Jy[3]);
  v -= 0.5 * Ty * Tz * (Tx * R * R * Jz[0] - R * R * Jz[1] - Tx * Jz[2] + Jz[3]);
  v -= (Tx * Tz * C * Iy[0] - Tz * C * Iy[1] - (1.0 / 3) * Tx * Tz * Iy[2] + (1.0 / 3) * Tz * Iy[3]);
  v -= (Tx * Ty * D * Iz[0] - Ty * D * Iz[1] - (1.0 / 3) * Tx * Ty * Iz[2] + (1.0 / 3) * Ty * Iz[3]);
  return v;
}
double G_s(const GArgs& g) {  // :193-218
  const double R = g.R, X = g.X, Vy = g.Vy, Vz = g.Vz, Tx = g.Tx, Ty = g.Ty, Tz = g.Tz;
  double A = Ty * Vy + Tz * Vz - 0.5 * Vy * Vy - 0.5 * Vz * Vz + 0.5 * R * R + (M_PI / 2) * Ty * Tz;
  double v = 0.125 * R * X * X * X * X - (1.0 / 6) * R * Tx * X * X * X - 0.5 * R * A * X * X + R * A * Tx * X;
  v -= R * Tz * (Tx * g.Iy.v[0] - g.Iy.v[1]);
  v -= R * Ty * (Tx * g.Iz.v[0] - g.Iz.v[1]);
  v -= R * Ty * Tz * (Tx * g.Jy.v[0] - g.Jy.v[1]);
  v -= R * Ty * Tz * (Tx * g.Jz.v[0] - g.Jz.v[1]);
  return v;
}
// G_vx and G_txx share one shape with the I/J orders shifted by one (:220-270).
double G_moment(const GArgs& g, int order) {
  const double R = g.R, X = g.X, Vy = g.Vy, Vz = g.Vz, Tx = g.Tx, Ty = g.Ty, Tz = g.Tz;
  double A = Ty * Vy + Tz * Vz - 0.5 * Vy * Vy - 0.5 * Vz * Vz + 0.5 * R * R + (M_PI / 2) * Ty * Tz;
  double v;
  if (order == 1)
    v = 0.1 * R * X * X * X * X * X - 0.125 * R * Tx * X * X * X * X - (1.0 / 3) * R * A * X * X * X + 0.5 * R * A * Tx * X * X;
  else
    v = (1.0 / 12) * R * X * X * X * X * X * X - 0.1 * R * Tx * X * X * X * X * X - 0.25 * R * A * X * X * X * X +
        (1.0 / 3) * R * A * Tx * X * X * X;
  const int a = order, b = order + 1;
  v -= R * Tz * (Tx * g.Iy.v[a] - g.Iy.v[b]);
  v -= R * Ty * (Tx * g.Iz.v[a] - g.Iz.v[b]);
  v -= R * Ty * Tz * (Tx * g.Jy.v[a] - g.Jy.v[b]);
  v -= R * Ty * Tz * (Tx * g.Jz.v[a] - g.Jz.v[b]);
  return v;
}
double G_txy(const GArgs& g) {  // :272-299
  const double R = g.R, X = g.X, Vy = g.Vy, Vz = g.Vz, Tx = g.Tx, Ty = g.Ty, Tz = g.Tz;
  const double* Iy = g.Iy.v; const double* Iz = g.Iz.v; const double* Jy = g.Jy.v; const double* Jz = g.Jz.v;
  double A = (1.0 / 6) * (3 * Ty * R * R + 2 * Vy * Vy * Vy - 3 * Ty * Vy * Vy - 3 * Ty * Vz * Vz + 6 * Ty * Tz * Vz + 1.5 * M_PI * R * R * Tz);
  double B = 0.25 * M_PI * Tz + 0.5 * Ty;
  double C = -(1.0 / 6) * (2 * R * R - 2 * Vz * Vz + 3 * Tz * Vz);
  double v = -0.5 * R * A * Tx * X * X + (1.0 / 3) * R * A * X * X * X + 0.25 * R * B * Tx * X * X * X * X - 0.2 * R * B * X * X * X * X * X;
  v += 0.5 * R * Tz * (Tx * R * R * Jy[1] - R * R * Jy[2] - Tx * Jy[3] + Jy[4]);
  v += 0.5 * R * Tz * (Tx * R * R * Jz[1] - R * R * Jz[2] - Tx * Jz[3] + Jz[4]);
  v += 0.5 * R * Tz * (2 * Ty - Vy) * (Tx * Iy[1] - Iy[2]);
  v += R * (-Tx * C * Iz[1] + C * Iz[2] - (1.0 / 3) * Tx * Iz[3] + (1.0 / 3) * Iz[4]);
  return v;
}

enum GKind { K_ETA, K_S, K_V, K_TXX, K_TXY };
double G_of(GKind k, const GArgs& g) {
  switch (k) {
    case K_ETA: return G_eta(g);
    case K_S: return G_s(g);
    case K_V: return G_moment(g, 1);
    case K_TXX: return G_moment(g, 2);
    default: return G_txy(g);
  }
}
// The difference the reference takes for every corner: G at the corner minus G
// at the point where the sphere crosses the line through it (:449-466).
double corner_term(GKind k, double R, double a, double b, double c, double ta, double tb, double tc) {
  return G_of(k, g_args(R, a, b, c, ta, tb, tc)) - G_of(k, g_args(R, std::sqrt(R * R - b * b - c * c), b, c, ta, tb, tc));
}

inline long wrap(long i, long n) { i %= n; if (i < 0) i += n; return i; }

// FMT_Species::generateWeights (src/FMT_Species.cpp:310-496): w[a][pos] for
// a = eta, s, v0, v1, v2, T00, T01, T02, T11, T12, T22.
void generate_fmt_weights(int nx, int ny, int nz, double dx, double dy, double dz, double hsd, std::vector<double>* w) {
  const double dV = dx * dy * dz;
  const double R = hsd / 2;
  if (hsd < std::min(std::min(dx, dy), dz)) throw std::runtime_error("hsd is less than the lattice spacing");
  const int Sx_max = 2 + int(R / dx), Sy_max = 2 + int(R / dy), Sz_max = 2 + int(R / dz);
  const int I[2] = {-1, 1};
  for (int a = 0; a < 11; ++a) w[a].assign((size_t)nx * ny * nz, 0.0);
  const double tiny = std::nextafter(0.0, 1.0);
  for (int Sx = 0; Sx <= Sx_max; Sx++)
    for (int Sy = 0; Sy <= Sy_max; Sy++)
      for (int Sz = 0; Sz <= Sz_max; Sz++) {
        auto lo = [](int S) { return S - (S == 0 ? 0 : 1); };
        double R2_min = dx * dx * lo(Sx) * lo(Sx) + dy * dy * lo(Sy) * lo(Sy) + dz * dz * lo(Sz) * lo(Sz);
        double R2_max = dx * dx * (Sx + 1) * (Sx + 1) + dy * dy * (Sy + 1) * (Sy + 1) + dz * dz * (Sz + 1) * (Sz + 1);
        double w_eta = 0, w_s = 0, w_v[3] = {0, 0, 0}, w_T[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (R * R > R2_max) {
          w_eta = dV;
        } else if (R * R > R2_min) {
          for (int ax : I) {
            int ix = ax;
            double Tx = dx * (Sx + ix);
            int px = (Tx < 0 ? -1 : 1);
            if (Tx < 0) { ix = 1; Tx = dx; }
            for (int ay : I) {
              int iy = ay;
              double Ty = dy * (Sy + iy);
              int py = (Ty < 0 ? -1 : 1);
              if (Ty < 0) { iy = 1; Ty = dy; }
              for (int az : I) {
                int iz = az;
                double Tz = dz * (Sz + iz);
                int pz = (Tz < 0 ? -1 : 1);
                if (Tz < 0) { iz = 1; Tz = dz; }
                const int vx[2] = {0, ix}, vy[2] = {0, iy}, vz[2] = {0, iz};
                for (int jx = 0; jx < 2; jx++)
                  for (int jy = 0; jy < 2; jy++)
                    for (int jz = 0; jz < 2; jz++) {
                      double Vx = Tx - dx * vx[jx], Vy = Ty - dy * vy[jy], Vz = Tz - dz * vz[jz];
                      int sgn = ((jx + jy + jz) % 2) ? -1 : 1;
                      if ((R * R - (Vx * Vx + Vy * Vy + Vz * Vz)) < tiny) continue;
                      const double f = (1 / dV) * sgn;
                      w_eta += f * corner_term(K_ETA, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      w_s += f * corner_term(K_S, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      w_v[0] += (1 / dV) * px * (1.0 / R) * sgn * corner_term(K_V, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      w_v[1] += (1 / dV) * py * (1.0 / R) * sgn * corner_term(K_V, R, Vy, Vx, Vz, Ty, Tx, Tz);
                      w_v[2] += (1 / dV) * pz * (1.0 / R) * sgn * corner_term(K_V, R, Vz, Vy, Vx, Tz, Ty, Tx);
                      w_T[0][0] += (1 / dV) * (1.0 / (R * R)) * sgn * corner_term(K_TXX, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      w_T[1][1] += (1 / dV) * (1.0 / (R * R)) * sgn * corner_term(K_TXX, R, Vy, Vx, Vz, Ty, Tx, Tz);
                      w_T[2][2] += (1 / dV) * (1.0 / (R * R)) * sgn * corner_term(K_TXX, R, Vz, Vy, Vx, Tz, Ty, Tx);
                      w_T[0][1] += (1 / dV) * px * py * (1.0 / (R * R)) * sgn * corner_term(K_TXY, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      w_T[0][2] += (1 / dV) * px * pz * (1.0 / (R * R)) * sgn * corner_term(K_TXY, R, Vx, Vz, Vy, Tx, Tz, Ty);
                      w_T[1][2] += (1 / dV) * py * pz * (1.0 / (R * R)) * sgn * corner_term(K_TXY, R, Vy, Vz, Vx, Ty, Tz, Tx);
                    }
              }
            }
          }
        }
        // Octant fill with the parity of vector and tensor components (:471-492).
        for (int ox = 0; ox < (Sx == 0 ? 1 : 2); ox++)
          for (int oy = 0; oy < (Sy == 0 ? 1 : 2); oy++)
            for (int oz = 0; oz < (Sz == 0 ? 1 : 2); oz++) {
              const int sx = 1 - 2 * ox, sy = 1 - 2 * oy, sz = 1 - 2 * oz;
              long pos = wrap(sz * Sz, nz) + (long)nz * (wrap(sy * Sy, ny) + (long)ny * wrap(sx * Sx, nx));
              const int sg[3] = {sx, sy, sz};
              w[0][pos] += w_eta;
              w[1][pos] += w_s;
              int slot = 5;
              for (int iv = 0; iv < 3; iv++) w[2 + iv][pos] += sg[iv] * w_v[iv];
              for (int iv = 0; iv < 3; iv++)
                for (int it = iv; it < 3; it++) w[slot++][pos] += sg[iv] * sg[it] * w_T[iv][it];
            }
      }
}

// ------------------------------------------------------ LJ + QF kernel ---
// Cut-and-shifted LJ with the Barker-Henderson split (include/Potential1.h:136-189, :56-70).
struct LJPot {
  double sigma, eps, rc, shift, r0;
  LJPot(double s, double e, double c) : sigma(s), eps(e), rc(c) {
    shift = (rc < 0 ? 0.0 : vr(rc));
    r0 = std::pow(0.5 * std::sqrt(1 + shift) + 0.5, -1.0 / 6.0);
  }
  double vr(double r) const { double y = sigma / r, y3 = y * y * y, y6 = y3 * y3; return 4 * eps * (y6 * y6 - y6); }
  double vr2(double r2) const { double y2 = sigma * sigma / r2, y6 = y2 * y2 * y2; return 4 * eps * (y6 * y6 - y6); }
  double V(double r) const { return vr(r) - shift; }
  double Watt2(double r2) const {  // BH branch of Potential1::Watt2
    if (r2 < rc * rc) return (r2 < r0 * r0 ? 0.0 : vr2(r2) - shift);
    return 0.0;
  }
};

double gl10(const LJPot& lj, double kT, double a, double b) {
  static const double xs[5] = {0.1488743389816312, 0.4333953941292472, 0.6794095682990244, 0.8650633666889845, 0.9739065285171717};
  static const double ws[5] = {0.2955242247147529, 0.2692667193099963, 0.2190863625159820, 0.1494513491505806, 0.0666713443086881};
  double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0;
  for (int i = 0; i < 5; ++i)
    for (int sg = -1; sg <= 1; sg += 2) s += ws[i] * (1.0 - std::exp(-lj.V(c + sg * h * xs[i]) / kT));
  return s * h;
}
double adapt(const LJPot& lj, double kT, double a, double b, double whole, int depth) {
  double m = 0.5 * (a + b), l = gl10(lj, kT, a, m), r = gl10(lj, kT, m, b);
  if (depth > 40 || std::fabs(l + r - whole) < 1e-15) return l + r;
  return adapt(lj, kT, a, m, l, depth + 1) + adapt(lj, kT, m, b, r, depth + 1);
}
// Potential1::getHSD (include/Potential1.h:73-83): int_0^{r0} (1 - exp(-V0/kT)) dr.
double bh_diameter(const LJPot& lj, double kT) {
  double lo = 1e-3;  // the integrand equals 1 to machine precision below this
  return lo + adapt(lj, kT, lo, lj.r0, gl10(lj, kT, lo, lj.r0), 0);
}

// Interaction_Base::generateWeightsXYZSym + Interaction_Interpolation::generateWeight
// with the QF points {-1/2,0,1/2} and weights 1/3 (src/Interaction.cpp:178-307,
// 522-534; include/Interaction.h:416-431), then /kT (:32-52).
void generate_qf_kernel(int nx, int ny, int nz, double dx, const LJPot& lj, double kT, std::vector<double>& w_att, double& a_vdw) {
  const double dy = dx, dz = dx;
  const int Nlim = 1 + int(lj.rc / dx);
  const long Nmax = (((long)(Nlim + 1) * (Nlim + 2) * (Nlim + 3)) / 6) + (((long)(Nlim + 1) * (Nlim + 2)) / 2) + Nlim + 1;
  std::vector<double> w2(Nmax + 1, 0.0);
  const double pt[3] = {-0.5, 0.0, 0.5};
  const double vv = 1.0 / 3;
  const double gfac = dx * dx * dy * dy * dz * dz;
  for (int Sx = 0; Sx <= Nlim + 1; ++Sx)
    for (int Sy = 0; Sy <= Sx; ++Sy)
      for (int Sz = 0; Sz <= Sy; ++Sz) {
        long p = ((long)Sx * (Sx + 1) * (Sx + 2)) / 6 + ((long)Sy * (Sy + 1)) / 2 + Sz;
        if (p > Nmax) continue;
        double sum = 0.0;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
              double r2 = (Sx + pt[i]) * (Sx + pt[i]) * dx * dx + (Sy + pt[j]) * (Sy + pt[j]) * dy * dy + (Sz + pt[k]) * (Sz + pt[k]) * dz * dz;
              sum += vv * vv * vv * lj.Watt2(r2);
            }
        w2[p] = gfac * sum;
      }
  w_att.assign((size_t)nx * ny * nz, 0.0);
  a_vdw = 0.0;
  for (int ix = -Nlim - 1; ix <= Nlim + 1; ix++)
    for (int iy = -Nlim - 1; iy <= Nlim + 1; iy++)
      for (int iz = -Nlim - 1; iz <= Nlim + 1; iz++) {
        int a = std::abs(ix), b = std::abs(iy), c = std::abs(iz);
        if (b > a) std::swap(a, b);
        if (c > a) std::swap(a, c);
        if (c > b) std::swap(b, c);
        long p = ((long)a * (a + 1) * (a + 2)) / 6 + ((long)b * (b + 1)) / 2 + c;
        double w = w2[p];
        long pos = wrap(iz, nz) + (long)nz * (wrap(iy, ny) + (long)ny * wrap(ix, nx));
        w_att[pos] += w / (dx * dy * dz);
        a_vdw += w;
      }
  a_vdw /= (dx * dy * dz);
  for (double& x : w_att) x *= 1.0 / kT;
  a_vdw /= kT;
}

// ------------------------------------------------------------ FMT models ---
// Fundamental measures in the reference's 19-slot order (include/Fundamental_Measures.h:112-134).
struct FM {
  double eta, s0, s1, s2, v1[3], v2[3], T[3][3];
  double v1_v2, v2_v2, vTv, T2, T3, vT[3], Tv[3], TT[3][3];
  void derived() {  // :76-106
    for (int i = 0; i < 3; i++) {
      vT[i] = v2[0] * T[0][i] + v2[1] * T[1][i] + v2[2] * T[2][i];
      Tv[i] = T[i][0] * v2[0] + T[i][1] * v2[1] + T[i][2] * v2[2];
    }
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) TT[i][j] = T[i][0] * T[0][j] + T[i][1] * T[1][j] + T[i][2] * T[2][j];
    v1_v2 = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
    v2_v2 = v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2];
    vTv = v2[0] * vT[0] + v2[1] * vT[1] + v2[2] * vT[2];
    T2 = TT[0][0] + TT[1][1] + TT[2][2];
    T3 = 0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) T3 += TT[i][j] * T[j][i];
  }
  void from19(const double* f) {
    eta = f[0]; s0 = f[1]; s1 = f[2]; s2 = f[3];
    for (int i = 0; i < 3; i++) { v1[i] = f[4 + i]; v2[i] = f[7 + i]; }
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) T[i][j] = f[10 + 3 * i + j];
    derived();
  }
  void uniform(double rho, double d) {  // fillUniform, :20-31
    eta = M_PI * rho * d * d * d / 6; s0 = M_PI * rho; s1 = s0 * d; s2 = s1 * d;
    for (int i = 0; i < 3; i++) { v1[i] = v2[i] = 0; for (int j = 0; j < 3; j++) T[i][j] = (i == j ? s2 / 3 : 0.0); }
    derived();
  }
  void to19(double* f) const {
    f[0] = eta; f[1] = s0; f[2] = s1; f[3] = s2;
    for (int i = 0; i < 3; i++) { f[4 + i] = v1[i]; f[7 + i] = v2[i]; }
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) f[10 + 3 * i + j] = T[i][j];
  }
};

struct Model {
  int kind;  // orc_model
  double A = 1, B = 0;
  bool tensor() const { return kind >= ORC_ESFMT; }
  // f1, f2, f3 and first derivatives (include/FMT.h:139-643)
  void f(double e, double& f1, double& f2, double& f3, double& f1p, double& f2p, double& f3p) const {
    f1 = std::log(1.0 - e);
    f1p = -1.0 / (1.0 - e);
    if (kind == ORC_WHITEBEAR_II) {  // :576-622
      if (e < 1e-12) { f2 = 1 + e * (1 + e * ((10.0 / 9) + (7.0 / 6) * e)); f2p = 1 + e * ((20.0 / 9) + 3.5 * e); }
      else {
        f2 = (1.0 / 3.0) + (4.0 / 3.0) * (1.0 / (1.0 - e)) + (2.0 / (3.0 * e)) * std::log(1 - e);
        f2p = (2 * (3 * e - 1) / (3 * e * (1 - e) * (1 - e))) - (2.0 / (3.0 * e * e)) * std::log(1 - e);
      }
      if (e < 1e-12) { f3 = 1.5 + (7.0 / 3) * e + 3.25 * e * e + 4.2 * e * e * e; f3p = (7.0 / 3) + 7.5 * e + 12.6 * e * e; }
      else {
        f3 = -((1.0 - 3 * e + e * e) / (e * (1 - e) * (1 - e))) - (1.0 / (e * e)) * std::log(1 - e);
        f3p = ((2 - 5 * e + 6 * e * e - e * e * e) / (e * e * (1 - e) * (1 - e) * (1 - e))) + (2.0 / (e * e * e)) * std::log(1 - e);
      }
      return;
    }
    double g = 1.0 / (1.0 - e);
    f2 = g;
    f2p = g * g;
    if (kind == ORC_RSLT) {  // :276-294
      if (e < 1e-12) { f3 = 1.5 + (8.0 / 3) * e + 3.75 * e * e + 4.8 * e * e * e; f3p = (8.0 / 3) + 7.5 * e + 14.4 * e * e; }
      else {
        f3 = (1.0 / (e * (1 - e) * (1 - e))) + (std::log(1 - e) / (e * e));
        f3p = -(1.0 / (e * e)) * (1.0 / ((1.0 - e) * (1.0 - e) * (1.0 - e))) * (e * e - 5 * e + 2) - (2.0 / (e * e * e)) * std::log(1 - e);
      }
    } else if (kind == ORC_WHITEBEAR_I) {  // :541-557
      if (e < 1e-12) { f3 = 1.5 + (8.0 / 3) * e + 3.75 * e * e + 4.8 * e * e * e; f3p = (8.0 / 3) + 7.5 * e + 14.4 * e * e; }
      else {
        f3 = (1.0 / (e * (1 - e) * (1 - e))) + (std::log(1 - e) / (e * e));
        f3p = ((-2 + 5 * e - e * e) / (e * e * (1 - e) * (1 - e) * (1 - e))) - (2 / (e * e * e)) * std::log(1 - e);
      }
    } else {  // Rosenfeld, esFMT: f3 = 1/(1-e)^2 (:194-204)
      f3 = g * g;
      f3p = 2 * g * g * g;
    }
  }
  double Phi3(const FM& m) const {
    if (kind == ORC_ROSENFELD) return (1.0 / (24 * M_PI)) * (m.s2 * m.s2 * m.s2 - 3 * m.s2 * m.v2_v2);
    if (kind == ORC_RSLT) {
      if (m.s2 < 1e-20) return 0.0;
      double psi = m.v2_v2 / (m.s2 * m.s2);
      return (1.0 / (36 * M_PI)) * m.s2 * m.s2 * m.s2 * (1 - psi) * (1 - psi) * (1 - psi);
    }
    double a = esA(), b = esB();
    return (a / (24 * M_PI)) * (m.s2 * m.s2 * m.s2 - 3 * m.s2 * m.v2_v2 + 3 * m.vTv - m.T3) +
           (b / (24 * M_PI)) * (m.s2 * m.s2 * m.s2 - 3 * m.s2 * m.T2 + 2 * m.T3);
  }
  double esA() const { return kind == ORC_ESFMT ? A : 1.0; }
  double esB() const { return kind == ORC_ESFMT ? B : -1.0; }
  double dPhi3_dS2(const FM& m) const {
    if (kind == ORC_ROSENFELD) return (1.0 / (24 * M_PI)) * (3 * m.s2 * m.s2 - 3 * m.v2_v2);
    if (kind == ORC_RSLT) {
      if (m.s2 < 1e-20) return 0.0;
      double psi = m.v2_v2 / (m.s2 * m.s2);
      return (1.0 / (12 * M_PI)) * m.s2 * m.s2 * (1 + psi) * (1 - psi) * (1 - psi);
    }
    return (esA() / (24 * M_PI)) * (3 * m.s2 * m.s2 - 3 * m.v2_v2) + (esB() / (24 * M_PI)) * (3 * m.s2 * m.s2 - 3 * m.T2);
  }
  double dPhi3_dV2(int k, const FM& m) const {
    if (kind == ORC_ROSENFELD) return (1.0 / (24 * M_PI)) * (-6 * m.s2 * m.v2[k]);
    if (kind == ORC_RSLT) {
      if (m.s2 < 1e-20) return 0.0;
      double psi = m.v2_v2 / (m.s2 * m.s2);
      return -(1.0 / (6 * M_PI)) * m.s2 * m.v2[k] * (1 - psi) * (1 - psi);
    }
    return (esA() / (24 * M_PI)) * (-6 * m.s2 * m.v2[k] + 3 * m.vT[k] + 3 * m.Tv[k]);
  }
  double dPhi3_dT(int j, int k, const FM& m) const {  // esFMT, include/FMT.h:441-450
    if (!tensor()) return 0.0;
    return (esA() / (8 * M_PI)) * (m.v2[j] * m.v2[k] - m.TT[k][j]) + (esB() / (4 * M_PI)) * (-m.s2 * m.T[k][j] + m.TT[k][j]);
  }
  // Second derivatives of f1, f2, f3 (include/FMT.h: Rosenfeld :163-199, RSLT :284-289,
  // WhiteBearI :530-556, WhiteBearII :604-632).
  void fpp(double e, double& f1pp, double& f2pp, double& f3pp) const {
    f1pp = -1.0 / (1.0 - 2 * e + e * e);
    const double g = 1.0 / (1.0 - e);
    f2pp = 2 * g * g * g;
    f3pp = 6 * g * g * g * g;
    const double L = std::log(1 - e);
    if (kind == ORC_RSLT) {
      if (e < 1e-12) f3pp = 7.5 + 28.8 * e;
      else f3pp = -(1.0 / (e * e * e)) * (1.0 / ((1.0 - e) * (1.0 - e) * (1.0 - e) * (1 - e))) * (5 * e * e * e - 26 * e * e + 21 * e - 6) +
                  (6.0 / (e * e * e * e)) * L;
    } else if (kind == ORC_WHITEBEAR_I) {
      if (e < 1e-12) f3pp = 7.5 + 28.8 * e;
      else f3pp = ((6 - 21 * e + 26 * e * e - 5 * e * e * e) / (e * e * e * (1 - e) * (1 - e) * (1 - e) * (1 - e))) + (6 * L) / (e * e * e * e);
    } else if (kind == ORC_WHITEBEAR_II) {
      if (e < 1e-12) f2pp = (20.0 / 9) + 7 * e;
      else f2pp = (2 * (7 * e * e - 5 * e + 2) / (3 * e * e * (1 - e) * (1 - e) * (1 - e))) + (4.0 / (3.0 * e * e * e)) * L;
      if (e < 1e-12) f3pp = 7.5 + 25.2 * e;
      else f3pp = (-(6 - 21 * e + 26 * e * e - 19 * e * e * e + 2 * e * e * e * e) / (e * e * e * (1 - e) * (1 - e) * (1 - e) * (1 - e))) -
                  (6.0 / (e * e * e * e)) * L;
    }
  }
  // Second derivatives of Phi3 (Rosenfeld include/FMT.h:218-231, RSLT :313-345, esFMT :417-480).
  double d2_S2S2(const FM& m) const {
    if (kind == ORC_ROSENFELD) return (1.0 / (24 * M_PI)) * (6 * m.s2);
    if (kind == ORC_RSLT) {
      if (m.s2 < 1e-20) return 0.0;
      const double psi = m.v2_v2 / (m.s2 * m.s2);
      return (1.0 / (6 * M_PI)) * m.s2 * (1 - psi) * (1 + psi + 2 * psi * psi);
    }
    return (esA() / (24 * M_PI)) * (6 * m.s2) + (esB() / (24 * M_PI)) * (6 * m.s2);
  }
  double d2_V2S2(int i, const FM& m) const {
    if (kind == ORC_RSLT) {
      if (m.s2 < 1e-20) return 0.0;
      const double psi = m.v2_v2 / (m.s2 * m.s2);
      return (1.0 / (36 * M_PI)) * (-6 * m.v2[i]) * (1 - psi) * (1 + 3 * psi);
    }
    return (esA() / (24 * M_PI)) * (-6 * m.v2[i]);  // Rosenfeld: A = 1
  }
  double d2_V2V2(int i, int j, const FM& m) const {
    if (kind == ORC_ROSENFELD) return i == j ? (1.0 / (24 * M_PI)) * (-6 * m.s2) : 0.0;
    if (kind == ORC_RSLT) {
      if (m.s2 < 1e-20) return 0.0;
      const double psi = m.v2_v2 / (m.s2 * m.s2);
      if (i == j) return (1.0 / (36 * M_PI)) * (-6 * m.s2) * (1 - psi) * (1 - psi - 4 * m.v2[i] * m.v2[i] / (m.s2 * m.s2));
      return (1.0 / (36 * M_PI)) * (24 / m.s2) * m.v2[i] * m.v2[j] * (1 - psi);
    }
    return (esA() / (24 * M_PI)) * (3 * m.T[i][j] + 3 * m.T[j][i] - 6 * (i == j ? m.s2 : 0.0));
  }
  double d2_S2T(int j, int k, const FM& m) const { return tensor() ? (esB() / (4 * M_PI)) * (-m.T[k][j]) : 0.0; }
  double d2_V2T(int i, int j, int k, const FM& m) const {
    if (!tensor()) return 0.0;
    double val = 0;
    if (i == j) val += esA() * m.v2[k];
    if (i == k) val += esA() * m.v2[j];
    return val / (8 * M_PI);
  }
  double d2_TT(int j, int k, int l, int mm, const FM& m) const {
    if (!tensor()) return 0.0;
    const double A = esA(), B = esB();
    double val = 0;
    if (l == k) val += -A * m.T[mm][j] + 2 * B * m.T[mm][j];
    if (mm == j) val += -A * m.T[k][l] + 2 * B * m.T[k][l];
    if (l == k && mm == j) val += -2 * B * m.s2;
    return val / (8 * M_PI);
  }
  // FMT::calculate_d2Phi_dot_V (src/FMT.cpp:181-280): r = (d2Phi/dn dn) . v, 19 slots.
  void d2phi_dot(const FM& n, const FM& v, FM& r) const {
    double f1, f2, f3, f1p, f2p, f3p, f1pp, f2pp, f3pp;
    f(n.eta, f1, f2, f3, f1p, f2p, f3p);
    fpp(n.eta, f1pp, f2pp, f3pp);
    const double s0 = n.s0, s1 = n.s1, s2 = n.s2;
    std::memset(&r, 0, sizeof(FM));
    const double ip = 1 / M_PI, i2p = 1 / (2 * M_PI);
    r.eta += (-ip * s0 * f1pp + i2p * (s1 * s2 - n.v1_v2) * f2pp + Phi3(n) * f3pp) * v.eta;
    r.eta += -ip * f1p * v.s0;
    r.s0 += -ip * f1p * v.eta;
    r.eta += i2p * s2 * f2p * v.s1;
    r.s1 += i2p * s2 * f2p * v.eta;
    const double es2 = i2p * s1 * f2p + dPhi3_dS2(n) * f3p;
    r.eta += es2 * v.s2;
    r.s2 += es2 * v.eta;
    for (int i = 0; i < 3; i++) {
      r.eta += -i2p * n.v2[i] * f2p * v.v1[i];
      r.v1[i] += -i2p * n.v2[i] * f2p * v.eta;
    }
    for (int i = 0; i < 3; i++) {
      const double ev2 = -i2p * n.v1[i] * f2p + dPhi3_dV2(i, n) * f3p;
      r.eta += ev2 * v.v2[i];
      r.v2[i] += ev2 * v.eta;
    }
    r.s1 += i2p * f2 * v.s2;
    r.s2 += i2p * f2 * v.s1;
    r.s2 += d2_S2S2(n) * f3 * v.s2;
    for (int i = 0; i < 3; i++) {
      r.s2 += d2_V2S2(i, n) * f3 * v.v2[i];
      r.v2[i] += d2_V2S2(i, n) * f3 * v.s2;
      r.v1[i] += -i2p * f2 * v.v2[i];
      r.v2[i] += -i2p * f2 * v.v1[i];
      for (int j = 0; j < 3; j++) {
        r.v2[i] += d2_V2V2(i, j, n) * f3 * v.v2[j];
        r.eta += dPhi3_dT(i, j, n) * f3p * v.T[i][j];
        r.T[i][j] += dPhi3_dT(i, j, n) * f3p * v.eta;
        r.s2 += d2_S2T(i, j, n) * f3 * v.T[i][j];
        r.T[i][j] += d2_S2T(i, j, n) * f3 * v.s2;
        for (int k = 0; k < 3; k++) {
          r.v2[i] += d2_V2T(i, j, k, n) * f3 * v.T[j][k];
          r.T[j][k] += d2_V2T(i, j, k, n) * f3 * v.v2[i];
          for (int l = 0; l < 3; l++) r.T[i][j] += d2_TT(i, j, k, l, n) * f3 * v.T[k][l];
        }
      }
    }
  }
  // FMT::calculate_Phi and calculate_dPhi_wrt_fundamental_measures (src/FMT.cpp:114-176)
  double phi(const FM& m, FM* d) const {
    double f1, f2, f3, f1p, f2p, f3p;
    f(m.eta, f1, f2, f3, f1p, f2p, f3p);
    double p3 = Phi3(m);
    double phi = 0;
    phi -= (1 / M_PI) * m.s0 * f1;
    phi += (1 / (2 * M_PI)) * (m.s1 * m.s2 - m.v1_v2) * f2;
    phi += p3 * f3;
    if (d) {
      std::memset(d, 0, sizeof(FM));
      d->eta -= (1 / M_PI) * m.s0 * f1p;
      d->eta += (1 / (2 * M_PI)) * (m.s1 * m.s2 - m.v1_v2) * f2p;
      d->eta += p3 * f3p;
      d->s0 += -(1 / M_PI) * f1;
      d->s1 += (1 / (2 * M_PI)) * m.s2 * f2;
      d->s2 += (1 / (2 * M_PI)) * m.s1 * f2;
      d->s2 += dPhi3_dS2(m) * f3;
      for (int k = 0; k < 3; k++) {
        d->v1[k] += (1 / (2 * M_PI)) * (-m.v2[k]) * f2;
        d->v2[k] += (1 / (2 * M_PI)) * (-m.v1[k]) * f2;
        d->v2[k] += dPhi3_dV2(k, m) * f3;
      }
      if (tensor())
        for (int k = 0; k < 3; k++)
          for (int j = 0; j < 3; j++) d->T[j][k] = dPhi3_dT(j, k, m) * f3;
    }
    return phi;
  }
};

// ---------------------------------------------------------------- context ---
struct Ctx {
  orc_params p;
  long N, Nc;
  int nzc;
  double dV, vol;
  Model model;
  double hsd = 0;
  std::vector<cd> wk[11];  // r2c(w_a)/N
  std::vector<double> wreal[11];
  bool lj = false;
  LJPot* pot = nullptr;
  std::vector<double> watt;  // real, already / kT
  std::vector<cd> wattk;     // r2c(w_att)
  double a_vdw = 0;
  double mu = 0;
  double fixed_mass = -1;
  std::vector<double> vext;  // zero external field (Density::vWall_)
};

void r2c(const Ctx& c, const double* in, std::vector<cd>& out) {
  out.resize(c.Nc);
  orc_r2c(c.p.nx, c.p.ny, c.p.nz, in, reinterpret_cast<double*>(out.data()));
}
void c2r(const Ctx& c, const std::vector<cd>& in, double* out) {
  orc_c2r(c.p.nx, c.p.ny, c.p.nz, reinterpret_cast<const double*>(in.data()), out);
}

// FMT bulk Muex / Fex for one species (src/FMT.cpp:616-709).
double bulk_muex(const Ctx& c, double rho) {
  FM fm;
  fm.uniform(rho, c.hsd);
  FM d;
  c.model.phi(fm, &d);
  double dv[19], wv[19];
  d.to19(dv);
  FM wts;
  wts.uniform(1.0, c.hsd);
  wts.to19(wv);
  double mu = 0;
  for (int i = 0; i < 19; i++) mu += dv[i] * wv[i];
  return mu;
}
double bulk_fex(const Ctx& c, double rho) {
  FM fm;
  fm.uniform(rho, c.hsd);
  return c.model.phi(fm, nullptr);
}

// The F+dF evaluation: DFT::calculateFreeEnergyAndDerivatives (src/DFT.cpp:360-425).
int eval(Ctx& c, double* rho, double* dF, double* terms) {
  const long N = c.N;
  const double dV = c.dV;
  // Species::beginForceCalculation (src/Species.cpp:64-71): fixed-mass rescale.
  if (c.fixed_mass > 0) {
    Neumaier sn;
    for (long i = 0; i < N; ++i) sn.add(rho[i]);
    double Nat = sn.sum() * dV;
    double s = c.fixed_mass / Nat;
    for (long i = 0; i < N; ++i) rho[i] *= s;
    c.mu = 0.0;
  }
  // Ideal gas (:381-395)
  double F_id = par_sum(N, [&](long i) { double d0 = rho[i]; return (d0 * std::log(d0) - d0) * dV; });
#pragma omp parallel for schedule(static)
  for (long i = 0; i < N; ++i) dF[i] = std::log(rho[i]) * dV;

  std::vector<cd> rhok;
  r2c(c, rho, rhok);
  double F_hs = 0;
  int status = 0;
  if (c.model.kind != ORC_NONE) {
    // FMT::calculateFreeEnergy (src/FMT.cpp:310-352): weighted densities by convolution.
    const int M = c.model.tensor() ? 11 : 5;
    std::vector<std::vector<double>> n(M, std::vector<double>(N));
    std::vector<cd> tmp(c.Nc);
    for (int a = 0; a < M; ++a) {
      for (long k = 0; k < c.Nc; ++k) tmp[k] = rhok[k] * c.wk[a][k];
      c2r(c, tmp, n[a].data());
    }
    // per point Phi and dPhi (FMT::dPHI, :283-305; FMT_Species::set_fundamental_measure_derivatives, include/Species.h:310-329)
    std::vector<std::vector<double>> dphi(M, std::vector<double>(N));
    const double h = c.hsd;
    int bad = 0;
    F_hs = par_sum(N, [&](long i) {
      FM fm;
      double S = n[1][i];
      fm.eta = n[0][i]; fm.s0 = S / (h * h); fm.s1 = S / h; fm.s2 = S;
      for (int j = 0; j < 3; j++) { fm.v1[j] = n[2 + j][i] / h; fm.v2[j] = n[2 + j][i]; }
      static const int TI[3][3] = {{5, 6, 7}, {6, 8, 9}, {7, 9, 10}};
      for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++) fm.T[j][k] = (M == 11) ? n[TI[j][k]][i] : 0.0;
      fm.derived();
      FM d;
      double phi = c.model.phi(fm, &d);
      if (fm.eta > 0.5 && 1 - fm.eta < 0.0) {
#pragma omp atomic write
        bad = 1;
      }
      dphi[0][i] = d.eta;
      dphi[1][i] = (d.s0 / (h * h)) + (d.s1 / h) + d.s2;
      for (int j = 0; j < 3; j++) {
        dphi[2 + j][i] = -(d.v2[j] + d.v1[j] / h);
        if (M == 11)
          for (int k = j; k < 3; k++) dphi[TI[j][k]][i] = (j == k ? 1 : 2) * d.T[j][k];
      }
      return phi;
    });
    if (bad) status = 1;
    // dF_hs = c2r(sum_a r2c(dPhi_a) . w_a) * dV (src/FMT.cpp:363-427; include/FMT_Weighted_Density.h:50-54)
    std::vector<cd> acc(c.Nc, cd(0, 0)), t;
    for (int a = 0; a < M; ++a) {
      r2c(c, dphi[a].data(), t);
      for (long k = 0; k < c.Nc; ++k) acc[k] += t[k] * c.wk[a][k];
    }
    std::vector<double> out(N);
    c2r(c, acc, out.data());
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) dF[i] += out[i] * dV;
    F_hs *= dV;
  }
  // Mean field, self pair (src/Interaction.cpp:76-96)
  double F_mf = 0;
  if (c.lj) {
    std::vector<cd> t(c.Nc);
    for (long k = 0; k < c.Nc; ++k) t[k] = rhok[k] * c.wattk[k];
    std::vector<double> v(N);
    c2r(c, t, v.data());
    for (long i = 0; i < N; ++i) v[i] *= dV / N;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) dF[i] += v[i];
    Neumaier E;  // Density::get_dot_with is a serial compensated sum (src/Density.cpp:144-150)
    for (long i = 0; i < N; ++i) E.add(rho[i] * v[i]);
    F_mf = 0.5 * E.sum();
  }
  // External field + chemical potential (src/Species.cpp:51-61), zero wall field.
  Neumaier Nat;
  for (long i = 0; i < N; ++i) Nat.add(rho[i]);
  double F_ext = 0.0 * dV - Nat.sum() * dV * c.mu;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < N; ++i) { dF[i] += 0.0 * dV; dF[i] += -c.mu * dV; }
  // Species::endForceCalculation, fixed mass (src/Species.cpp:97-109): serial sum in the reference.
  if (c.fixed_mass > 0) {
    double m = 0;
    for (long i = 0; i < N; ++i) m += dF[i] * rho[i];
    c.mu = m / c.fixed_mass;
    for (long i = 0; i < N; ++i) dF[i] = dF[i] - c.mu * dV;
  }
  Neumaier F;
  F.add(F_id);
  F.add(F_hs);
  F.add(F_mf);
  F.add(F_ext);
  if (terms) {
    terms[0] = F.sum(); terms[1] = F_id; terms[2] = F_hs; terms[3] = F_mf; terms[4] = F_ext; terms[5] = c.mu;
  }
  return status;
}

// DFT::matrix_dot_v_intern (src/DFT.cpp:435-488) with the full Hessian: the
// ideal-gas term dV v/rho, FMT::add_second_derivative (src/FMT.cpp:437-567) and
// Interaction_Base::add_second_derivative (src/Interaction.cpp:119-147), at the
// density rho (the state of the last evaluation in the reference).
void hessian_dot_v(const Ctx& c, const double* rho, const double* v, double* out) {
  const long N = c.N;
  const double dV = c.dV;
  for (long i = 0; i < N; ++i) out[i] = dV * v[i] / rho[i];
  std::vector<cd> rhok, vk;
  r2c(c, rho, rhok);
  r2c(c, v, vk);
  if (c.model.kind != ORC_NONE) {
    const double h = c.hsd;
    static const int TI[3][3] = {{5, 6, 7}, {6, 8, 9}, {7, 9, 10}};
    // weighted densities of rho and convolutions of v with every weight
    std::vector<std::vector<double>> n(11, std::vector<double>(N)), cv(11, std::vector<double>(N));
    std::vector<cd> tmp(c.Nc);
    for (int a = 0; a < 11; ++a) {
      for (long k = 0; k < c.Nc; ++k) tmp[k] = rhok[k] * c.wk[a][k];
      c2r(c, tmp, n[a].data());
      for (long k = 0; k < c.Nc; ++k) tmp[k] = vk[k] * c.wk[a][k];
      c2r(c, tmp, cv[a].data());
    }
    // Lambda_a(K) = sum_b d2Phi/dn_a dn_b Psi_b(K), 19 slots
    std::vector<std::vector<double>> lam(19, std::vector<double>(N));
    const bool T = c.model.tensor();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) {
      FM fm, ps, r;
      std::memset(&fm, 0, sizeof(FM));
      std::memset(&ps, 0, sizeof(FM));
      const double S = n[1][i];
      fm.eta = n[0][i]; fm.s0 = S / (h * h); fm.s1 = S / h; fm.s2 = S;
      ps.eta = cv[0][i]; ps.s0 = cv[1][i] / (h * h); ps.s1 = cv[1][i] / h; ps.s2 = cv[1][i];
      for (int j = 0; j < 3; j++) {
        fm.v1[j] = n[2 + j][i] / h; fm.v2[j] = n[2 + j][i];
        ps.v1[j] = cv[2 + j][i] / h; ps.v2[j] = cv[2 + j][i];
        for (int k = 0; k < 3; k++) {
          fm.T[j][k] = T ? n[TI[j][k]][i] : 0.0;
          ps.T[j][k] = cv[TI[j][k]][i];
        }
      }
      fm.derived();
      c.model.d2phi_dot(fm, ps, r);
      double r19[19];
      r.to19(r19);
      for (int a = 0; a < 19; ++a) lam[a][i] = r19[a];
    }
    // sum_a conv(Lambda_a, w_a) with conjugated weights, scaled as the reference does
    std::vector<cd> acc(c.Nc, cd(0, 0)), t;
    auto add_conv = [&](int slot, int w, double scale) {
      r2c(c, lam[slot].data(), t);
      for (long k = 0; k < c.Nc; ++k) acc[k] += scale * t[k] * std::conj(c.wk[w][k]);
    };
    add_conv(0, 0, 1.0);
    add_conv(1, 1, 1.0 / (h * h));
    add_conv(2, 1, 1.0 / h);
    add_conv(3, 1, 1.0);
    for (int j = 0; j < 3; j++) {
      add_conv(4 + j, 2 + j, 1.0 / h);
      add_conv(7 + j, 2 + j, 1.0);
    }
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) add_conv(10 + 3 * j + k, TI[j][k], 1.0);
    std::vector<double> o(N);
    c2r(c, acc, o.data());
    for (long i = 0; i < N; ++i) out[i] += o[i] * dV;
  }
  if (c.lj) {
    std::vector<cd> t(c.Nc);
    for (long k = 0; k < c.Nc; ++k) t[k] = vk[k] * c.wattk[k];
    std::vector<double> o(N);
    c2r(c, t, o.data());
    for (long i = 0; i < N; ++i) out[i] += o[i] * (dV / N);
  }
}

// Alias maps for FMT_Species (src/FMT_Species.cpp:29-93); SMALL_VALUE = 1e-18 (include/Density.h:24).
struct Alias {
  double dmin, c;
  Alias(double hsd, double dV) {
    dmin = 1e-18;
    double etamin = dmin * (4 * M_PI * hsd * hsd * hsd / 3);
    c = (1.0 - etamin) / dV;
  }
  double rho(double y) const { return dmin + c * y * y / (1 + y * y); }
  double y(double rho) const { double z = (rho - dmin) / c; return std::sqrt(std::fabs(z / (1 - z))); }
  double drho_dy(double y) const { return 2 * c * y / ((1 + y * y) * (1 + y * y)); }
};

}  // namespace

struct orc_ctx : Ctx {};

extern "C" {

double orc_bh_diameter(double rc, double kT) {
  LJPot lj(1.0, 1.0, rc);
  return bh_diameter(lj, kT);
}

orc_ctx* orc_create(const orc_params* p) {
  orc_ctx* c = new orc_ctx();
  c->p = *p;
  c->N = (long)p->nx * p->ny * p->nz;
  c->nzc = p->nz / 2 + 1;
  c->Nc = (long)p->nx * p->ny * c->nzc;
  c->dV = p->dx * p->dx * p->dx;
  c->vol = c->N * c->dV;
  c->model.kind = p->model;
  c->model.A = p->es_A;
  c->model.B = p->es_B;
  c->mu = p->mu;
  c->fixed_mass = p->fixed_mass;
  if (p->fixed_mass > 0) c->mu = 0.0;  // Species::setFixedMass (include/Species.h:25)
  c->lj = p->lj != 0;
  if (c->lj) c->pot = new LJPot(p->lj_sigma, p->lj_eps, p->lj_rc);
  c->hsd = p->hsd > 0 ? p->hsd : (c->pot ? bh_diameter(*c->pot, p->kT) : 1.0);
  if (c->model.kind != ORC_NONE) {
    generate_fmt_weights(p->nx, p->ny, p->nz, p->dx, p->dx, p->dx, c->hsd, c->wreal);
    for (int a = 0; a < 11; ++a) {  // FMT_Weighted_Density::transformWeights (include/FMT_Weighted_Density.h:35-39)
      r2c(*c, c->wreal[a].data(), c->wk[a]);
      for (auto& z : c->wk[a]) z *= 1.0 / c->N;
    }
  }
  if (c->lj) {
    generate_qf_kernel(p->nx, p->ny, p->nz, p->dx, *c->pot, p->kT, c->watt, c->a_vdw);
    r2c(*c, c->watt.data(), c->wattk);
  }
  return c;
}
void orc_destroy(orc_ctx* c) { delete c->pot; delete c; }
double orc_hsd(const orc_ctx* c) { return c->hsd; }
double orc_a_vdw(const orc_ctx* c) { return c->a_vdw; }
void orc_set_mu(orc_ctx* c, double mu) { c->mu = mu; c->fixed_mass = -1; }
double orc_get_mu(const orc_ctx* c) { return c->mu; }
void orc_weights(const orc_ctx* c, double* out) {
  for (int a = 0; a < 11; ++a) std::memcpy(out + a * c->N, c->wreal[a].data(), sizeof(double) * c->N);
}
void orc_w_att(const orc_ctx* c, double* out) {
  if (c->lj) std::memcpy(out, c->watt.data(), sizeof(double) * c->N);
}
int orc_eval(orc_ctx* c, double* rho, double* dF, double* terms) { return eval(*c, rho, dF, terms); }

void orc_hessian_dot_v(const orc_ctx* c, const double* rho, const double* v, double* out) { hessian_dot_v(*c, rho, v, out); }

// DDFT::matrix_dot_v_intern (src/DDFT.cpp:353-361): g . (H v), with DDFT::g_dot_x
// (:320-351, forward differences): gx = sum_axes D [(rho+ + rho0)(x+ - x0) - (rho0 + rho-)(x0 - x-)], D = 1/(2 dx^2).
void orc_ddft_matrix_dot_v(const orc_ctx* c, const double* rho, const double* v, double* out) {
  const int nx = c->p.nx, ny = c->p.ny, nz = c->p.nz;
  const long N = c->N;
  std::vector<double> hv(N);
  hessian_dot_v(*c, rho, v, hv.data());
  const double D = 1.0 / (2 * c->p.dx * c->p.dx);
  auto idx = [&](int i, int j, int k) { return (long)((k + nz) % nz) + (long)nz * (((j + ny) % ny) + (long)ny * ((i + nx) % nx)); };
  const int off[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        const long p = idx(i, j, k);
        const double x0 = hv[p], d0 = rho[p];
        double g = 0;
        for (int a = 0; a < 3; a++) {
          const long pp = idx(i + off[a][0], j + off[a][1], k + off[a][2]);
          const long pm = idx(i - off[a][0], j - off[a][1], k - off[a][2]);
          g += D * ((rho[pp] + d0) * (hv[pp] - x0) - (d0 + rho[pm]) * (x0 - hv[pm]));
        }
        out[p] = g;
      }
}

// DFT::mu_times_beta (src/DFT.cpp:58-71), Interaction_Base::Mu (src/Interaction.cpp:61-72)
double orc_mu_times_beta(const orc_ctx* c, double rho) {
  Neumaier mu;
  mu.add(std::log(rho));
  if (c->model.kind != ORC_NONE) mu.add(bulk_muex(*c, rho));
  if (c->lj) mu.add(0.5 * c->a_vdw * rho + 0.5 * c->a_vdw * rho);
  return mu.sum();
}
// DFT::fhelmholtz_times_beta_over_volume (src/DFT.cpp:90-115)
double orc_fhelmholtz_times_beta_over_volume(const orc_ctx* c, double rho) {
  double F = rho * std::log(rho) - rho;
  if (c->model.kind != ORC_NONE) F += bulk_fex(*c, rho);
  if (c->lj) F += 0.5 * c->a_vdw * rho * rho;
  return F;
}
double orc_omega_times_beta_over_volume(const orc_ctx* c, double rho) {
  return orc_fhelmholtz_times_beta_over_volume(c, rho) - rho * orc_mu_times_beta(c, rho);
}
double orc_phi(int model, double A, double B, const double* fm19, double* dphi19) {
  Model m;
  m.kind = model; m.A = A; m.B = B;
  FM fm;
  fm.from19(fm19);
  FM d;
  double phi = m.phi(fm, &d);
  if (dphi19) d.to19(dphi19);
  return phi;
}

void orc_fill_noise(double* rho, long n, double rho0, double amp, uint64_t seed) {
  uint64_t s = seed;
  for (long i = 0; i < n; ++i) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    rho[i] = rho0 * (1.0 + amp * (2.0 * u - 1.0));
  }
}

// fireMinimizer2 (src/Minimizer.cpp:18-327; include/Minimizer.h:13-182).
int orc_fire(orc_ctx* c, double* rho, int nsteps, double dt0, double dt_max0, double force_limit,
             double* rec_F, double* rec_dt, double* rec_alpha, double* rec_vv, double* rec_fmax, double* rec_resid) {
  const long N = c->N;
  const double dV = c->dV;
  Alias al(c->hsd, dV);
  std::vector<double> x(N), v(N, 0.0), dF(N), xr(N), vr(N), dFr(N);
  // Minimizer::Minimizer: x = alias(rho) (:18-28)
  for (long i = 0; i < N; ++i) x[i] = al.y(rho[i]);
  double terms[6];
  double resid_true = 0;
  // getDF_DX (:90-115): density from alias, eval, convert dF to alias derivative
  auto getDF_DX = [&](double& F) -> int {
    for (long i = 0; i < N; ++i) rho[i] = al.rho(x[i]);
    int st = eval(*c, rho, dF.data(), terms);
    if (st) return st;
    F = terms[0];
    double m = 0;
    for (long i = 0; i < N; ++i) m = std::max(m, std::fabs(dF[i]));
    resid_true = m / dV;
    for (long i = 0; i < N; ++i) dF[i] *= al.drho_dy(x[i]);
    return 0;
  };
  double dt = dt0, dt_max = dt_max0;
  const int N_delay = 5;
  const double alpha_start = 0.1, f_dec = 0.5, f_inc = 1.1, f_alf = 0.99, dt_min = 0.0;
  const int N_P_negative_max = 20;
  double alpha = alpha_start;
  int Npos = 0, Nneg = 0, backtracks = 0;
  unsigned it = 0;
  double vv = 1.0, dt_best = 1e-3, fmax = -1.0;  // dt_best_ = the constructor's dt_ (:130-140)
  double F = 0;
  if (getDF_DX(F)) return -2;
  double fold = F;  // `static double fold = F_` on the first step (:164)
  int steps = 0;
  for (int s = 0; s < nsteps; ++s) {
    // fireMinimizer2::step (:160-271)
    it++;
    double vdotf = 0;
    for (long i = 0; i < N; ++i) vdotf += v[i] * dF[i];
    Neumaier P;
    P.add(-vdotf);
    fold = F;
    xr = x; vr = v; dFr = dF;
    if (P.sum() > 0) {
      Npos++;
      Nneg = 0;
      if (Npos > N_delay) { dt = std::min(dt * f_inc, dt_max); alpha = alpha * f_alf; }
    } else {
      Npos = 0;
      Nneg++;
      if (Nneg > N_P_negative_max) return -1;
      if (!(it < (unsigned)N_delay)) {  // initial_delay_ = true
        if (dt * f_dec >= dt_min) dt *= f_dec;
        alpha = alpha_start;
      }
      for (long i = 0; i < N; ++i) { x[i] += v[i] * (-0.5 * dt); v[i] *= 0.1; }
      backtracks++;
    }
    // SemiImplicitEuler (:273-327)
    double vnorm = 0, fnorm = 0;
    for (long i = 0; i < N; ++i) v[i] += dF[i] * (-dt);
    {
      double sv = 0, sf = 0;
      for (long i = 0; i < N; ++i) { sv += v[i] * v[i]; sf += dF[i] * dF[i]; }
      double nv = std::sqrt(sv), nf = std::sqrt(sf);  // euclidean_norm, then squared (:283-289)
      vnorm = nv * nv;
      fnorm = nf * nf;
    }
    for (long i = 0; i < N; ++i) {
      v[i] *= (1 - alpha);
      v[i] += dF[i] * (-alpha * std::sqrt(vnorm / fnorm));
      x[i] += v[i] * dt;
    }
    double Fnew;
    if (getDF_DX(Fnew) == 0) {
      F = Fnew;
      double m = 0;
      for (long i = 0; i < N; ++i) m = std::max(m, std::fabs(dF[i]));
      fmax = m / dV;
      vv = vv * 0.9 + 0.1 * (std::fabs(F - fold) / dt);
      dt_best = std::max(dt, dt_best);
    } else {  // Eta_Too_Large_Exception (:233-245)
      x = xr;
      v = vr;
      for (long i = 0; i < N; ++i) v[i] *= 0.5;
      dF = dFr;
      dt /= 2;
      fmax = 1000;
      backtracks++;
    }
    if (backtracks >= 10) { dt_max = std::min(dt_best, 0.9 * dt_max); dt_best = 0; backtracks = 0; }
    if (rec_F) rec_F[s] = F;
    if (rec_dt) rec_dt[s] = dt;
    if (rec_alpha) rec_alpha[s] = alpha;
    if (rec_vv) rec_vv[s] = vv;
    if (rec_fmax) rec_fmax[s] = fmax;
    if (rec_resid) rec_resid[s] = resid_true;
    steps = s + 1;
    // Minimizer::resume stop test on |vv/V| (:55-63; include/Minimizer.h:105)
    if (std::fabs(vv / c->vol) < force_limit) break;
  }
  // rho keeps the density of the last evaluation, as the reference's Density does
  // (rescaled under fixed mass; the rejected density after a final backtrack).
  return steps;
}

// DDFT integrating-factor step (src/DDFT.cpp:42-351), single species, periodic.
int orc_ddft(orc_ctx* c, double* rho, int nsteps, double dt_init, double dt_max,
             double* rec_F, double* rec_t, double* rec_dt, double* rec_mass, double* rec_rhs) {
  const int nx = c->p.nx, ny = c->p.ny, nz = c->p.nz, nzc = c->nzc;
  const long N = c->N;
  const double dx = c->p.dx, dV = c->dV;
  std::vector<double> Lx(nx), Ly(ny), Lz(nzc);
  const double D2 = 1.0 / (dx * dx);
  for (int i = 0; i < nx; i++) Lx[i] = 2 * D2 * (std::cos((2 * M_PI * i) / nx) - 1);
  for (int i = 0; i < ny; i++) Ly[i] = 2 * D2 * (std::cos((2 * M_PI * i) / ny) - 1);
  for (int i = 0; i < nzc; i++) Lz[i] = 2 * D2 * (std::cos((2 * M_PI * i) / nz) - 1);
  std::vector<double> fx(nx), fy(ny), fz(nzc);
  double dt = dt_init;
  bool have_factors = false;
  auto change_timestep = [&](double ndt) {  // :194-215, including its early return
    if (std::fabs(dt - ndt) < 1e-10) return;
    dt = ndt;
    have_factors = true;
    for (int i = 0; i < nx; i++) fx[i] = std::exp(Lx[i] * dt);
    for (int i = 0; i < ny; i++) fy[i] = std::exp(Ly[i] * dt);
    for (int i = 0; i < nzc; i++) fz[i] = std::exp(Lz[i] * dt);
  };
  std::vector<double> dF(N), terms(6);
  auto idx = [&](int i, int j, int k) { return (long)((k + nz) % nz) + (long)nz * (((j + ny) % ny) + (long)ny * ((i + nx) % nx)); };
  // calculate_excess_RHS (:212-235): g_dot_x(dF)/dV - Laplacian_h(rho), then r2c
  auto excess_rhs = [&](const double* d, std::vector<cd>& out) -> double {
    std::vector<double> R(N);
    const double D = 1.0 / (2 * dx * dx);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
      for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz; k++) {
          long p = idx(i, j, k);
          double x0 = dF[p], d0 = d[p];
          double g = 0;
          const int off[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
          for (int a = 0; a < 3; a++) {
            long pp = idx(i + off[a][0], j + off[a][1], k + off[a][2]);
            long pm = idx(i - off[a][0], j - off[a][1], k - off[a][2]);
            g += D * ((d[pp] + d0) * (dF[pp] - x0) - (d0 + d[pm]) * (x0 - dF[pm]));
          }
          R[p] = g;
        }
    double rmax = 0;
    for (long p = 0; p < N; ++p) { R[p] *= 1.0 / dV; rmax = std::max(rmax, std::fabs(R[p])); }
    rmax /= dV;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
      for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz; k++) {
          long p = idx(i, j, k);
          double d0 = d[p];
          R[p] += -D2 * (d[idx(i + 1, j, k)] + d[idx(i - 1, j, k)] - 2 * d0) - D2 * (d[idx(i, j + 1, k)] + d[idx(i, j - 1, k)] - 2 * d0) -
                  D2 * (d[idx(i, j, k + 1)] + d[idx(i, j, k - 1)] - 2 * d0);
        }
    r2c(*c, R.data(), out);
    return rmax;
  };
  // The DDFT constructor evaluates once (:52); its first step sets the factors (:119).
  if (eval(*c, rho, dF.data(), terms.data())) return -2;
  double time = 0;
  int successes = 0;
  std::vector<double> d0(N), d1(N);
  std::vector<cd> R0, R1, rk;
  for (int s = 0; s < nsteps; ++s) {
    if (!have_factors) { double tmp = dt; dt = 0; change_timestep(tmp); }
    if (eval(*c, rho, dF.data(), terms.data())) return -2;
    d0.assign(rho, rho + N);
    d1 = d0;
    bool decreased = false, restart;
    double rhs_max = excess_rhs(d0.data(), R0);
    do {
      double deviation = 1;
      restart = false;
      for (int i = 0; i < 100 && deviation > 1e-4 && !restart; i++) {
        if (eval(*c, d1.data(), dF.data(), terms.data())) return -2;
        excess_rhs(d1.data(), R1);
        // apply_diffusion_propogator (:239-292), with the density set back to d0
        r2c(*c, d0.data(), rk);
        std::vector<cd> work(c->Nc);
        long pos = 0;
        for (int ix = 0; ix < nx; ix++)
          for (int iy = 0; iy < ny; iy++)
            for (int iz = 0; iz < nzc; iz++, pos++) {
              double Lam = Lx[ix] + Ly[iy] + Lz[iz];
              double e = fx[ix] * fy[iy] * fz[iz];
              double U0 = e;
              double U1 = (pos == 0 ? dt : (e - 1) / Lam);
              double U2 = (pos == 0 ? dt / 2 : (e - 1 - dt * Lam) / (Lam * Lam * dt));
              work[pos] = U0 * rk[pos] + U1 * R0[pos] + U2 * (R1[pos] - R0[pos]);
            }
        std::vector<double> nd(N);
        c2r(*c, work, nd.data());
        double old = deviation, maxdev = 0, mn = 1e300;
        for (long p = 0; p < N; ++p) {
          nd[p] *= 1.0 / N;
          maxdev = std::max(maxdev, std::fabs(d1[p] - nd[p]));
        }
        d1 = nd;
        deviation = maxdev;
        for (long p = 0; p < N; ++p) mn = std::min(mn, d1[p]);
        if (mn < 0 || (i > 0 && old < deviation)) restart = true;
      }
      if (restart || deviation > 1e-4) { change_timestep(dt / 10); d1 = d0; decreased = true; restart = true; }
    } while (restart);
    time += dt;
    if (decreased) successes = 0;
    else successes++;
    if (successes >= 5 && dt < dt_max) { change_timestep(std::min(2 * dt, dt_max)); successes = 0; }
    std::memcpy(rho, d1.data(), sizeof(double) * N);
    if (eval(*c, rho, dF.data(), terms.data())) return -2;
    if (rec_F) rec_F[s] = terms[0];
    if (rec_t) rec_t[s] = time;
    if (rec_dt) rec_dt[s] = dt;
    if (rec_mass) { Neumaier m; for (long p = 0; p < N; ++p) m.add(rho[p]); rec_mass[s] = m.sum() * dV; }
    if (rec_rhs) rec_rhs[s] = rhs_max;
  }
  return nsteps;
}

// Log_Det::calculate_log_det (src/Log_Det.cpp:84-166) with the coefficients of
// Log_Det::get_coefficients (:34-57): a Chebyshev expansion of log on the spectrum
// [lam_min, lam_max] scaled by 1/(lam_min + lam_max), traced by Hutchinson with +-1
// vectors from std::mt19937(seed) and uniform_int_distribution<>(0, 1), drawn in
// point order, sample after sample. dynamic = 1 uses -(g . H), the DDFT matrix the
// reference negates (is_dynamic). has_zero adds lam_mid * sum(v) / N to every entry.
double orc_log_det(const orc_ctx* c, const double* rho, int dynamic, int order, double lam_max, double lam_min, long seed, int num_samples,
                   int has_zero, double* variance) {
  const long N = c->N;
  const double scale = 1.0 / (lam_min + lam_max), a = lam_min * scale, b = lam_max * scale, lam_mid = 0.5 * (lam_max + lam_min);
  std::vector<double> cf(order + 1, 0.0);
  for (int k = 0; k <= order; ++k) {
    const double xk = std::cos(M_PI * (k + 0.5) / (order + 1));
    double Tm2 = 0, Tm1 = 0, T = 1;
    for (int j = 0; j <= order; ++j) {
      T = j == 0 ? 1.0 : j == 1 ? xk : 2 * xk * Tm1 - Tm2;
      cf[j] += std::log(0.5 * (b - a) * xk + 0.5 * (b + a)) * T;
      Tm2 = Tm1;
      Tm1 = T;
    }
  }
  for (int j = 0; j <= order; ++j) cf[j] *= (j == 0 ? 1.0 : 2.0) / (order + 1);
  std::vector<double> v(N), w0(N), w1(N), w2(N), u(N), r(N);
  auto op = [&](const std::vector<double>& x, std::vector<double>& y) {
    if (dynamic) {
      orc_ddft_matrix_dot_v(c, rho, x.data(), y.data());
      for (double& t : y) t = -t;
    } else {
      hessian_dot_v(*c, rho, x.data(), y.data());
    }
    if (has_zero) {
      double s = 0;
      for (double t : x) s += t;
      for (double& t : y) t += lam_mid * s / N;
    }
  };
  std::mt19937 rng((unsigned long)seed);
  std::uniform_int_distribution<> distrib(0, 1);
  double log_det = 0, var_log_det = 0;
  for (int i = 1; i <= num_samples; ++i) {
    for (long p = 0; p < N; ++p) v[p] = distrib(rng) > 0 ? 1 : -1;
    op(v, r);
    for (long p = 0; p < N; ++p) {
      w0[p] = v[p];
      w1[p] = r[p] * scale * (2.0 / (b - a)) - (b + a) / (b - a) * v[p];
      u[p] = cf[0] * w0[p] + cf[1] * w1[p];
    }
    for (int k = 2; k <= order; ++k) {
      op(w1, r);
      for (long p = 0; p < N; ++p) {
        w2[p] = r[p] * scale * (4.0 / (b - a)) - 2 * (b + a) / (b - a) * w1[p] - w0[p];
        u[p] += cf[k] * w2[p];
      }
      w0.swap(w1);
      w1.swap(w2);
    }
    double vu = 0;
    for (long p = 0; p < N; ++p) vu += v[p] * u[p];
    log_det += vu;
    var_log_det += vu * vu;
    const double av = log_det / i, av2 = var_log_det / i;
    if (variance) *variance = std::sqrt(std::fabs(av2 - av * av));
  }
  log_det /= num_samples;
  if (has_zero) log_det -= std::log(lam_mid);
  return log_det - N * std::log(scale);
}

}  // extern "C"

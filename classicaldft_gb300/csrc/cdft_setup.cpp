// Host-side set-up maths of the GB300 engine (run once per context, FP64):
// the Barker-Henderson diameter of the cut-and-shifted LJ, the analytic
// cell-averaged FMT weights of a sphere, the quadratic-force (QF) mean-field
// kernel, and the bulk thermodynamics used for chemical potentials.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>
#include "cdft_internal.h"

namespace cdft {

// ----------------------------------------------------------------- LJ ---
// Potential1 / LJ with setBH() (include/Potential1.h:23-189): V(r) = 4 eps
// ((s/r)^12 - (s/r)^6) - V(rc); r0 = (sqrt(1 + shift)/2 + 1/2)^(-1/6) is the
// zero of the shifted potential for s = eps = 1 as the reference writes it.
namespace {
struct ShiftedLJ {
  double sigma, eps, rc, shift, r0;
  ShiftedLJ(double s, double e, double c) : sigma(s), eps(e), rc(c) {
    shift = rc < 0 ? 0.0 : raw(rc);
    r0 = std::pow(0.5 * std::sqrt(1 + shift) + 0.5, -1.0 / 6.0);
  }
  double raw(double r) const { double y = sigma / r, y3 = y * y * y, y6 = y3 * y3; return 4 * eps * (y6 * y6 - y6); }
  double raw2(double r2) const { double y2 = sigma * sigma / r2, y6 = y2 * y2 * y2; return 4 * eps * (y6 * y6 - y6); }
  double V(double r) const { return raw(r) - shift; }
  // attractive tail of the BH split (Potential1::Watt2)
  double tail2(double r2) const { return (r2 < rc * rc) ? (r2 < r0 * r0 ? 0.0 : raw2(r2) - shift) : 0.0; }
};

// 10-point Gauss-Legendre nodes and weights on [-1, 1] (symmetric half).
const double kGLx[5] = {0.1488743389816312, 0.4333953941292472, 0.6794095682990244, 0.8650633666889845, 0.9739065285171717};
const double kGLw[5] = {0.2955242247147529, 0.2692667193099963, 0.2190863625159820, 0.1494513491505806, 0.0666713443086881};

template <class F>
double gauss10(F f, double a, double b) {
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  double s = 0;
  for (int i = 0; i < 5; ++i) {
    s += kGLw[i] * f(c - h * kGLx[i]);
    s += kGLw[i] * f(c + h * kGLx[i]);
  }
  return s * h;
}
template <class F>
double adaptive(F f, double a, double b, double whole, int depth) {
  const double m = 0.5 * (a + b);
  const double l = gauss10(f, a, m), r = gauss10(f, m, b);
  if (depth > 40 || std::fabs(l + r - whole) < 1e-15) return l + r;
  return adaptive(f, a, m, l, depth + 1) + adaptive(f, m, b, r, depth + 1);
}
}  // namespace

// Potential1::getHSD (include/Potential1.h:73-83): hsd = int_0^{r0} (1 - exp(-V/kT)) dr,
// integrated to 1e-15 (the integrand is 1 to machine precision below r = 1e-3).
double bh_diameter_lj(double sigma, double eps, double rc, double kT) {
  ShiftedLJ lj(sigma, eps, rc);
  auto f = [&](double r) { return 1.0 - std::exp(-lj.V(r) / kT); };
  const double lo = 1e-3;
  return lo + adaptive(f, lo, lj.r0, gauss10(f, lo, lj.r0), 0);
}

// ------------------------------------------------------------ QF kernel ---
// Interaction_Interpolation_QF weights (src/Interaction.cpp:178-307, 522-534;
// include/Interaction.h:416-431): for every lattice vector S within
// (1 + int(rc/dx)) + 1 cells, w(S) = dx^6 sum_ijk (1/3)^3 Watt(|S + p_ijk| dx)
// with p in {-1/2, 0, 1/2}^3, tabulated once per sorted (|Sx| >= |Sy| >= |Sz|)
// triple, folded periodically, divided by dV and kT.
void qf_kernel_real(int nx, int ny, int nz, double dx, double sigma, double eps, double rc, double kT, std::vector<double>& w_att,
                    double& a_vdw) {
  ShiftedLJ lj(sigma, eps, rc);
  const int lim = 1 + int(rc / dx);
  auto tri = [](long a, long b, long c) { return a * (a + 1) * (a + 2) / 6 + b * (b + 1) / 2 + c; };
  const long nmax = tri(lim + 1, lim + 1, lim + 1);
  std::vector<double> table(nmax + 1, 0.0);
  const double pts[3] = {-0.5, 0.0, 0.5};
  const double third = 1.0 / 3;
  const double dx2 = dx * dx, pref = dx2 * dx2 * dx2;
  for (int a = 0; a <= lim + 1; ++a)
    for (int b = 0; b <= a; ++b)
      for (int c = 0; c <= b; ++c) {
        double sum = 0.0;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
              const double r2 = (a + pts[i]) * (a + pts[i]) * dx * dx + (b + pts[j]) * (b + pts[j]) * dx * dx + (c + pts[k]) * (c + pts[k]) * dx * dx;
              sum += third * third * third * lj.tail2(r2);
            }
        table[tri(a, b, c)] = pref * sum;
      }
  w_att.assign((size_t)nx * ny * nz, 0.0);
  a_vdw = 0.0;
  const double dV = dx * dx * dx;
  for (int ix = -lim - 1; ix <= lim + 1; ix++)
    for (int iy = -lim - 1; iy <= lim + 1; iy++)
      for (int iz = -lim - 1; iz <= lim + 1; iz++) {
        int s[3] = {std::abs(ix), std::abs(iy), std::abs(iz)};
        if (s[1] > s[0]) std::swap(s[0], s[1]);
        if (s[2] > s[0]) std::swap(s[0], s[2]);
        if (s[2] > s[1]) std::swap(s[1], s[2]);
        const double w = table[tri(s[0], s[1], s[2])];
        const long i = ((ix % nx) + nx) % nx, j = ((iy % ny) + ny) % ny, k = ((iz % nz) + nz) % nz;
        w_att[k + (long)nz * (j + (long)ny * i)] += w / dV;
        a_vdw += w;
      }
  a_vdw /= dV;
  for (double& x : w_att) x *= 1.0 / kT;
  a_vdw /= kT;
}

// ---------------------------------------------------------- FMT weights ---
// Exact cell averages of the FMT weight functions of a sphere of radius
// R = hsd/2 (FMT_Species::generateWeights, src/FMT_Species.cpp:310-496): for
// each lattice offset S >= 0 the weights are sums over the corners of the
// adjoining cells of analytic antiderivatives G(R; X, Vy, Vz, Tx, Ty, Tz)
// (:112-308), then copied to the 2-8 mirror images with the parity of the
// vector (odd) and tensor components.
namespace {
struct Moments { double v[5]; };

// int_0^X x^n sqrt(A^2 - x^2) type moments (getI)
Moments moments_I(double X, double A) {
  const double a = std::asin(X / A), b = std::sqrt(std::fabs(A * A - X * X));
  Moments m;
  m.v[0] = 0.5 * X * b + 0.5 * A * A * a;
  m.v[1] = -(1.0 / 3) * (A * A - X * X) * b;
  m.v[2] = 0.125 * X * (2 * X * X - A * A) * b + 0.125 * A * A * A * A * a;
  m.v[3] = -(1.0 / 15) * (A * A - X * X) * (3 * X * X + 2 * A * A) * b;
  m.v[4] = (1.0 / 48) * (8 * X * X * X * X - 2 * A * A * X * X - 3 * A * A * A * A) * X * b + 0.0625 * A * A * A * A * A * A * a;
  return m;
}
inline double unit_clamp(double x) { return std::max(-1.0, std::min(1.0, x)); }
// arcsine moments over the spherical cap (getJ)
Moments moments_J(double X, double V, double R) {
  const double floor_den = 1e-15;
  const double aV = std::asin(unit_clamp(V / std::max(floor_den, std::sqrt(R * R - X * X))));
  const double aX = std::asin(unit_clamp(X / std::sqrt(R * R - V * V)));
  const double aVX = std::asin(unit_clamp(X * V / std::max(floor_den, std::sqrt((R * R - V * V) * (R * R - X * X)))));
  const double b = std::sqrt(std::fabs(R * R - V * V - X * X));
  Moments m;
  m.v[0] = X * aV + V * aX - R * aVX;
  m.v[1] = -0.5 * V * b + 0.5 * (X * X - R * R) * aV;
  m.v[2] = -(1.0 / 6) * V * (V * V - 3 * R * R) * aX + (1.0 / 3) * X * X * X * aV - (1.0 / 3) * R * R * R * aVX - (1.0 / 6) * V * X * b;
  m.v[3] = 0.25 * (X * X * X * X - R * R * R * R) * aV + (M_PI / 8) * R * R * R * R - (V / 12.0) * (5 * R * R + X * X - 2 * V * V) * b;
  m.v[4] = 0.025 * X * V * (3 * V * V - 2 * X * X - 7 * R * R) * b + 0.025 * V * (3 * V * V * V * V - 10 * V * V * R * R + 15 * R * R * R * R) * aX +
           0.2 * X * X * X * X * X * aV - 0.2 * R * R * R * R * R * aVX;
  return m;
}

enum Antiderivative { G_ETA, G_S, G_V, G_TXX, G_TXY };

double antiderivative(Antiderivative kind, double R, double X, double Vy, double Vz, double Tx, double Ty, double Tz) {
  R += 1e-15;  // as the reference, keeps the square roots below real
  const Moments Iy = moments_I(X, std::sqrt(R * R - Vy * Vy)), Iz = moments_I(X, std::sqrt(R * R - Vz * Vz));
  const Moments Jy = moments_J(X, Vy, R), Jz = moments_J(X, Vz, R);
  switch (kind) {
    case G_ETA: {
      const double A = Ty * Tz * Vy * Vz + 0.25 * Vy * Vy * Vz * Vz + 0.125 * R * R * R * R - (1.0 / 6) * (Ty * Vy * Vy * Vy + Tz * Vz * Vz * Vz) -
                       0.5 * Tz * Vz * Vy * Vy - 0.5 * Ty * Vy * Vz * Vz + 0.125 * Vy * Vy * Vy * Vy + 0.125 * Vz * Vz * Vz * Vz +
                       0.5 * R * R * (Ty * Vy + Tz * Vz - 0.5 * Vy * Vy - 0.5 * Vz * Vz + 0.5 * M_PI * Ty * Tz);
      const double B = 0.5 * Ty * Vy + 0.5 * Tz * Vz - 0.25 * Vy * Vy - 0.25 * Vz * Vz + (M_PI / 4) * Ty * Tz + 0.25 * R * R;
      const double C = 0.5 * Ty * Vy + (1.0 / 3) * (R * R - Vy * Vy);
      const double D = 0.5 * Tz * Vz + (1.0 / 3) * (R * R - Vz * Vz);
      double g = Tx * A * X - 0.5 * A * X * X - (1.0 / 3) * B * Tx * X * X * X + 0.25 * X * X * X * X * B + 0.025 * Tx * X * X * X * X * X -
                 (1.0 / 48) * X * X * X * X * X * X;
      g -= 0.5 * Ty * Tz * (Tx * R * R * Jy.v[0] - R * R * Jy.v[1] - Tx * Jy.v[2] + Jy.v[3]);
      g -= 0.5 * Ty * Tz * (Tx * R * R * Jz.v[0] - R * R * Jz.v[1] - Tx * Jz.v[2] + Jz.v[3]);
      g -= (Tx * Tz * C * Iy.v[0] - Tz * C * Iy.v[1] - (1.0 / 3) * Tx * Tz * Iy.v[2] + (1.0 / 3) * Tz * Iy.v[3]);
      g -= (Tx * Ty * D * Iz.v[0] - Ty * D * Iz.v[1] - (1.0 / 3) * Tx * Ty * Iz.v[2] + (1.0 / 3) * Ty * Iz.v[3]);
      return g;
    }
    case G_TXY: {
      const double A = (1.0 / 6) * (3 * Ty * R * R + 2 * Vy * Vy * Vy - 3 * Ty * Vy * Vy - 3 * Ty * Vz * Vz + 6 * Ty * Tz * Vz + 1.5 * M_PI * R * R * Tz);
      const double B = 0.25 * M_PI * Tz + 0.5 * Ty;
      const double C = -(1.0 / 6) * (2 * R * R - 2 * Vz * Vz + 3 * Tz * Vz);
      double g = -0.5 * R * A * Tx * X * X + (1.0 / 3) * R * A * X * X * X + 0.25 * R * B * Tx * X * X * X * X - 0.2 * R * B * X * X * X * X * X;
      g += 0.5 * R * Tz * (Tx * R * R * Jy.v[1] - R * R * Jy.v[2] - Tx * Jy.v[3] + Jy.v[4]);
      g += 0.5 * R * Tz * (Tx * R * R * Jz.v[1] - R * R * Jz.v[2] - Tx * Jz.v[3] + Jz.v[4]);
      g += 0.5 * R * Tz * (2 * Ty - Vy) * (Tx * Iy.v[1] - Iy.v[2]);
      g += R * (-Tx * C * Iz.v[1] + C * Iz.v[2] - (1.0 / 3) * Tx * Iz.v[3] + (1.0 / 3) * Iz.v[4]);
      return g;
    }
    default: {
      // surface (order 0), vector (order 1) and diagonal tensor (order 2) share one form
      const int o = (kind == G_S) ? 0 : (kind == G_V ? 1 : 2);
      const double A = Ty * Vy + Tz * Vz - 0.5 * Vy * Vy - 0.5 * Vz * Vz + 0.5 * R * R + (M_PI / 2) * Ty * Tz;
      double g;
      if (o == 0) g = 0.125 * R * X * X * X * X - (1.0 / 6) * R * Tx * X * X * X - 0.5 * R * A * X * X + R * A * Tx * X;
      else if (o == 1) g = 0.1 * R * X * X * X * X * X - 0.125 * R * Tx * X * X * X * X - (1.0 / 3) * R * A * X * X * X + 0.5 * R * A * Tx * X * X;
      else
        g = (1.0 / 12) * R * X * X * X * X * X * X - 0.1 * R * Tx * X * X * X * X * X - 0.25 * R * A * X * X * X * X + (1.0 / 3) * R * A * Tx * X * X * X;
      g -= R * Tz * (Tx * Iy.v[o] - Iy.v[o + 1]);
      g -= R * Ty * (Tx * Iz.v[o] - Iz.v[o + 1]);
      g -= R * Ty * Tz * (Tx * Jy.v[o] - Jy.v[o + 1]);
      g -= R * Ty * Tz * (Tx * Jz.v[o] - Jz.v[o + 1]);
      return g;
    }
  }
}

// G at a corner minus G where the sphere cuts the line through the corner.
inline double corner(Antiderivative k, double R, double a, double b, double c, double ta, double tb, double tc) {
  return antiderivative(k, R, a, b, c, ta, tb, tc) - antiderivative(k, R, std::sqrt(R * R - b * b - c * c), b, c, ta, tb, tc);
}
}  // namespace

void fmt_weights_real(int nx, int ny, int nz, double dx, double hsd, std::vector<double> w[11]) {
  const double dV = dx * dx * dx;
  const double R = 0.5 * hsd;
  if (hsd < dx) throw std::runtime_error("hsd is less than the lattice spacing");
  const int smax = 2 + int(R / dx);
  for (int a = 0; a < 11; ++a) w[a].assign((size_t)nx * ny * nz, 0.0);
  const double dmin = std::nextafter(0.0, 1.0);
  auto lo = [](int S) { return S == 0 ? 0 : S - 1; };
  for (int Sx = 0; Sx <= smax; Sx++)
    for (int Sy = 0; Sy <= smax; Sy++)
      for (int Sz = 0; Sz <= smax; Sz++) {
        const double near2 = dx * dx * lo(Sx) * lo(Sx) + dx * dx * lo(Sy) * lo(Sy) + dx * dx * lo(Sz) * lo(Sz);
        const double far2 = dx * dx * (Sx + 1) * (Sx + 1) + dx * dx * (Sy + 1) * (Sy + 1) + dx * dx * (Sz + 1) * (Sz + 1);
        double we = 0, ws = 0, wv[3] = {0, 0, 0}, wt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (R * R > far2) {
          we = dV;  // cell entirely inside the sphere
        } else if (R * R > near2) {
          const int S[3] = {Sx, Sy, Sz};
          for (int cx = 0; cx < 2; ++cx)
            for (int cy = 0; cy < 2; ++cy)
              for (int cz = 0; cz < 2; ++cz) {
                // the adjoining cell on side (-1 or +1) of each axis; cells
                // across the origin are reflected with a parity factor
                const int side[3] = {2 * cx - 1, 2 * cy - 1, 2 * cz - 1};
                int step[3], par[3];
                double Tc[3];
                for (int ax = 0; ax < 3; ++ax) {
                  step[ax] = side[ax];
                  Tc[ax] = dx * (S[ax] + step[ax]);
                  par[ax] = Tc[ax] < 0 ? -1 : 1;
                  if (Tc[ax] < 0) { step[ax] = 1; Tc[ax] = dx; }
                }
                for (int jx = 0; jx < 2; jx++)
                  for (int jy = 0; jy < 2; jy++)
                    for (int jz = 0; jz < 2; jz++) {
                      const double Vx = Tc[0] - dx * (jx ? step[0] : 0), Vy = Tc[1] - dx * (jy ? step[1] : 0),
                                   Vz = Tc[2] - dx * (jz ? step[2] : 0);
                      const int sgn = ((jx + jy + jz) & 1) ? -1 : 1;
                      if ((R * R - (Vx * Vx + Vy * Vy + Vz * Vz)) < dmin) continue;
                      const double Tx = Tc[0], Ty = Tc[1], Tz = Tc[2];
                      we += (1 / dV) * sgn * corner(G_ETA, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      ws += (1 / dV) * sgn * corner(G_S, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      wv[0] += (1 / dV) * par[0] * (1.0 / R) * sgn * corner(G_V, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      wv[1] += (1 / dV) * par[1] * (1.0 / R) * sgn * corner(G_V, R, Vy, Vx, Vz, Ty, Tx, Tz);
                      wv[2] += (1 / dV) * par[2] * (1.0 / R) * sgn * corner(G_V, R, Vz, Vy, Vx, Tz, Ty, Tx);
                      wt[0][0] += (1 / dV) * (1.0 / (R * R)) * sgn * corner(G_TXX, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      wt[1][1] += (1 / dV) * (1.0 / (R * R)) * sgn * corner(G_TXX, R, Vy, Vx, Vz, Ty, Tx, Tz);
                      wt[2][2] += (1 / dV) * (1.0 / (R * R)) * sgn * corner(G_TXX, R, Vz, Vy, Vx, Tz, Ty, Tx);
                      wt[0][1] += (1 / dV) * par[0] * par[1] * (1.0 / (R * R)) * sgn * corner(G_TXY, R, Vx, Vy, Vz, Tx, Ty, Tz);
                      wt[0][2] += (1 / dV) * par[0] * par[2] * (1.0 / (R * R)) * sgn * corner(G_TXY, R, Vx, Vz, Vy, Tx, Tz, Ty);
                      wt[1][2] += (1 / dV) * par[1] * par[2] * (1.0 / (R * R)) * sgn * corner(G_TXY, R, Vy, Vz, Vx, Ty, Tz, Tx);
                    }
              }
        }
        for (int mx = 0; mx < (Sx ? 2 : 1); mx++)
          for (int my = 0; my < (Sy ? 2 : 1); my++)
            for (int mz = 0; mz < (Sz ? 2 : 1); mz++) {
              const int sg[3] = {1 - 2 * mx, 1 - 2 * my, 1 - 2 * mz};
              const long i = ((sg[0] * Sx) % nx + nx) % nx, j = ((sg[1] * Sy) % ny + ny) % ny, k = ((sg[2] * Sz) % nz + nz) % nz;
              const long pos = k + (long)nz * (j + (long)ny * i);
              w[0][pos] += we;
              w[1][pos] += ws;
              for (int v = 0; v < 3; v++) w[2 + v][pos] += sg[v] * wv[v];
              int slot = 5;
              for (int v = 0; v < 3; v++)
                for (int t = v; t < 3; t++) w[slot++][pos] += sg[v] * sg[t] * wt[v][t];
            }
      }
}

// ------------------------------------------------- bulk thermodynamics ---
// A value and its derivative along one direction, for exact forward-mode
// differentiation of the host functional (the AO bulk chemical potential needs
// the second derivative of Phi along the uniform measures).
struct Dual {
  double v = 0, d = 0;
  Dual() = default;
  Dual(double x) : v(x) {}
  Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) { return Dual(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
inline Dual operator+(double a, Dual b) { return Dual(a) + b; }
inline Dual operator-(double a, Dual b) { return Dual(a) - b; }
inline Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
inline Dual operator/(double a, Dual b) { return Dual(a) / b; }
inline Dual operator+(Dual a, double b) { return a + Dual(b); }
inline Dual operator-(Dual a, double b) { return a - Dual(b); }
inline Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
inline Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
inline Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
inline Dual& operator-=(Dual& a, Dual b) { return a = a - b; }
inline bool operator<(Dual a, double b) { return a.v < b; }
inline Dual log(Dual a) { return Dual(std::log(a.v), a.d / a.v); }

// FMT on the 19 fundamental measures (FMT::calculate_Phi / calculate_dPhi, src/FMT.cpp:114-176).
template <class R>
R fmt_phi_t(int model, double A, double B, const R f[19], R d[19]) {
  using std::log;
  const R eta = f[0], s0 = f[1], s1 = f[2], s2 = f[3];
  const R* v1 = f + 4;
  const R* v2 = f + 7;
  R T[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) T[i][j] = f[10 + 3 * i + j];
  R vT[3], TT[3][3];
  for (int i = 0; i < 3; i++) vT[i] = v2[0] * T[0][i] + v2[1] * T[1][i] + v2[2] * T[2][i];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) TT[i][j] = T[i][0] * T[0][j] + T[i][1] * T[1][j] + T[i][2] * T[2][j];
  const R v1_v2 = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
  const R v2_v2 = v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2];
  const R vTv = v2[0] * vT[0] + v2[1] * vT[1] + v2[2] * vT[2];
  const R T2 = TT[0][0] + TT[1][1] + TT[2][2];
  R T3 = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) T3 += TT[i][j] * T[j][i];
  // f-functions
  const R L = log(1.0 - eta);
  R f1 = L, f1p = -1.0 / (1.0 - eta), f2, f2p, f3, f3p;
  const R g = 1.0 / (1.0 - eta);
  if (model == MODEL_WHITEBEAR_II) {
    if (eta < 1e-12) {
      f2 = 1 + eta * (1 + eta * ((10.0 / 9) + (7.0 / 6) * eta));
      f2p = 1 + eta * ((20.0 / 9) + 3.5 * eta);
      f3 = 1.5 + (7.0 / 3) * eta + 3.25 * eta * eta + 4.2 * eta * eta * eta;
      f3p = (7.0 / 3) + 7.5 * eta + 12.6 * eta * eta;
    } else {
      f2 = (1.0 / 3.0) + (4.0 / 3.0) * (1.0 / (1.0 - eta)) + (2.0 / (3.0 * eta)) * L;
      f2p = (2 * (3 * eta - 1) / (3 * eta * (1 - eta) * (1 - eta))) - (2.0 / (3.0 * eta * eta)) * L;
      f3 = -((1.0 - 3 * eta + eta * eta) / (eta * (1 - eta) * (1 - eta))) - (1.0 / (eta * eta)) * L;
      f3p = ((2 - 5 * eta + 6 * eta * eta - eta * eta * eta) / (eta * eta * (1 - eta) * (1 - eta) * (1 - eta))) + (2.0 / (eta * eta * eta)) * L;
    }
  } else {
    f2 = g;
    f2p = g * g;
    if (model == MODEL_RSLT || model == MODEL_WHITEBEAR_I) {
      if (eta < 1e-12) {
        f3 = 1.5 + (8.0 / 3) * eta + 3.75 * eta * eta + 4.8 * eta * eta * eta;
        f3p = (8.0 / 3) + 7.5 * eta + 14.4 * eta * eta;
      } else {
        f3 = (1.0 / (eta * (1 - eta) * (1 - eta))) + (L / (eta * eta));
        f3p = model == MODEL_RSLT
                  ? -(1.0 / (eta * eta)) * (1.0 / ((1.0 - eta) * (1.0 - eta) * (1.0 - eta))) * (eta * eta - 5 * eta + 2) - (2.0 / (eta * eta * eta)) * L
                  : ((-2 + 5 * eta - eta * eta) / (eta * eta * (1 - eta) * (1 - eta) * (1 - eta))) - (2 / (eta * eta * eta)) * L;
      }
    } else {
      f3 = g * g;
      f3p = 2 * g * g * g;
    }
  }
  R P3, dS2, dV2[3], dT[3][3];
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++) dT[j][k] = 0.0;
  const bool tensor = model >= MODEL_ESFMT;
  if (tensor) {
    const double a = model == MODEL_ESFMT ? A : 1.0, b = model == MODEL_ESFMT ? B : -1.0;
    P3 = (a / (24 * M_PI)) * (s2 * s2 * s2 - 3 * s2 * v2_v2 + 3 * vTv - T3) + (b / (24 * M_PI)) * (s2 * s2 * s2 - 3 * s2 * T2 + 2 * T3);
    dS2 = (a / (24 * M_PI)) * (3 * s2 * s2 - 3 * v2_v2) + (b / (24 * M_PI)) * (3 * s2 * s2 - 3 * T2);
    for (int k = 0; k < 3; k++) dV2[k] = (a / (24 * M_PI)) * (-6 * s2 * v2[k] + 3 * vT[k] + 3 * vT[k]);
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) dT[j][k] = (a / (8 * M_PI)) * (v2[j] * v2[k] - TT[k][j]) + (b / (4 * M_PI)) * (-s2 * T[k][j] + TT[k][j]);
  } else if (model == MODEL_RSLT) {
    if (s2 < 1e-20) {
      P3 = dS2 = dV2[0] = dV2[1] = dV2[2] = 0.0;
    } else {
      const R psi = v2_v2 / (s2 * s2);
      P3 = (1.0 / (36 * M_PI)) * s2 * s2 * s2 * (1 - psi) * (1 - psi) * (1 - psi);
      dS2 = (1.0 / (12 * M_PI)) * s2 * s2 * (1 + psi) * (1 - psi) * (1 - psi);
      for (int k = 0; k < 3; k++) dV2[k] = -(1.0 / (6 * M_PI)) * s2 * v2[k] * (1 - psi) * (1 - psi);
    }
  } else {
    P3 = (1.0 / (24 * M_PI)) * (s2 * s2 * s2 - 3 * s2 * v2_v2);
    dS2 = (1.0 / (24 * M_PI)) * (3 * s2 * s2 - 3 * v2_v2);
    for (int k = 0; k < 3; k++) dV2[k] = (1.0 / (24 * M_PI)) * (-6 * s2 * v2[k]);
  }
  R phi = 0.0;
  phi -= (1 / M_PI) * s0 * f1;
  phi += (1 / (2 * M_PI)) * (s1 * s2 - v1_v2) * f2;
  phi += P3 * f3;
  if (d) {
    for (int i = 0; i < 19; i++) d[i] = 0.0;
    d[0] -= (1 / M_PI) * s0 * f1p;
    d[0] += (1 / (2 * M_PI)) * (s1 * s2 - v1_v2) * f2p;
    d[0] += P3 * f3p;
    d[1] += -(1 / M_PI) * f1;
    d[2] += (1 / (2 * M_PI)) * s2 * f2;
    d[3] += (1 / (2 * M_PI)) * s1 * f2;
    d[3] += dS2 * f3;
    for (int k = 0; k < 3; k++) {
      d[4 + k] += (1 / (2 * M_PI)) * (-v2[k]) * f2;
      d[7 + k] += (1 / (2 * M_PI)) * (-v1[k]) * f2;
      d[7 + k] += dV2[k] * f3;
    }
    if (tensor)
      for (int k = 0; k < 3; k++)
        for (int j = 0; j < 3; j++) d[10 + 3 * j + k] = dT[j][k] * f3;
  }
  return phi;
}


// The same in FP64, and along a direction (Dual: value and derivative, exact
// forward-mode differentiation) for the AO bulk terms below.
double fmt_phi_host(int model, double A, double B, const double f[19], double d[19]) { return fmt_phi_t<double>(model, A, B, f, d); }

static void uniform_measures(double rho, double d, double f[19]) {  // FundamentalMeasures::fillUniform
  std::memset(f, 0, 19 * sizeof(double));
  f[0] = M_PI * rho * d * d * d / 6;
  f[1] = M_PI * rho;
  f[2] = f[1] * d;
  f[3] = f[2] * d;
  f[10] = f[14] = f[18] = f[3] / 3;
}

// FMT::BulkMuex / BulkFex for one species (src/FMT.cpp:616-709)
double bulk_muex(int model, double A, double B, double hsd, double rho) {
  double f[19], d[19], w[19];
  uniform_measures(rho, hsd, f);
  fmt_phi_host(model, A, B, f, d);
  uniform_measures(1.0, hsd, w);
  double mu = 0;
  for (int i = 0; i < 19; i++) mu += d[i] * w[i];
  return mu;
}
double bulk_fex(int model, double A, double B, double hsd, double rho) {
  double f[19];
  uniform_measures(rho, hsd, f);
  return fmt_phi_host(model, A, B, f, nullptr);
}

// The AO terms of FMT::BulkMuex / BulkFex (src/FMT.cpp:640-700) for colloids of
// diameter hsd and polymers of diameter hsdp at reservoir density rhop:
//   arg(rho) = sum_i dPhi_i(n(rho)) wp_i,  wp = the uniform measures of unit density
//   and diameter hsdp;  f_AO = rhop (1 - exp(-arg));
//   mu_AO = rhop exp(-arg) sum_i (d2Phi(n) . w)_i wp_i = rhop exp(-arg) d arg / d rho,
// since the uniform measures n(rho) = rho w are linear in rho: the second derivative
// along w is the rho-derivative of arg, taken here exactly by forward differentiation.
static Dual ao_arg(int model, double A, double B, double hsd, double hsdp, double rho) {
  double fu[19], wp[19];
  uniform_measures(rho, hsd, fu);
  double w1[19];
  uniform_measures(1.0, hsd, w1);
  Dual f[19], d[19];
  for (int i = 0; i < 19; i++) f[i] = Dual(fu[i], w1[i]);
  fmt_phi_t<Dual>(model, A, B, f, d);
  uniform_measures(1.0, hsdp, wp);
  Dual arg = 0.0;
  for (int i = 0; i < 19; i++) arg += d[i] * wp[i];
  return arg;
}
double bulk_muex_ao(int model, double A, double B, double hsd, double hsdp, double rhop, double rho) {
  const Dual a = ao_arg(model, A, B, hsd, hsdp, rho);
  return rhop * a.d * std::exp(-a.v);
}
double bulk_fex_ao(int model, double A, double B, double hsd, double hsdp, double rhop, double rho) {
  const Dual a = ao_arg(model, A, B, hsd, hsdp, rho);
  return rhop - rhop * std::exp(-a.v);
}

}  // namespace cdft

// Golden-vector driver for the reference (jimlutsko/classicalDFT), compiled
// from the reference's own sources by oracle/Makefile (target `ref`) into
// oracle/_ref/ref_driver. It drives the reference through its public C++ API
// (Density, FMT_Species, FMT models, LJ, Interaction_Interpolation_QF, DFT,
// fireMinimizer2, DDFT) and writes named float64 arrays to a binary file that
// tests/golden/make_golden.py packs into fixtures.
//
// Usage: ref_driver <case> <out.bin>
// Every case takes its inputs from the seeded splitmix64 stream below, which
// tests/golden/make_golden.py and the oracle reproduce exactly.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
using namespace std;

#include "DFT.h"
#include "FMT.h"
#include "Interaction.h"
#include "Log_Det.h"
#include "Minimizer.h"
#include "Potential1.h"

// ---------------------------------------------------------------- output ---
static std::vector<std::pair<std::string, std::vector<double>>> g_out;
static void put(const std::string& name, const std::vector<double>& v) { g_out.push_back({name, v}); }
static void put1(const std::string& name, double x) { put(name, std::vector<double>(1, x)); }
static void write_out(const char* path) {
  FILE* f = std::fopen(path, "wb");
  if (!f) throw std::runtime_error("cannot open output");
  for (auto& kv : g_out) {
    uint32_t nl = (uint32_t)kv.first.size();
    uint64_t n = kv.second.size();
    std::fwrite(&nl, 4, 1, f);
    std::fwrite(kv.first.data(), 1, nl, f);
    std::fwrite(&n, 8, 1, f);
    std::fwrite(kv.second.data(), 8, n, f);
  }
  std::fclose(f);
}

// ------------------------------------------------------------- inputs -----
// splitmix64; uniform(s) = (next >> 11) * 2^-53 in [0, 1).
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// rho_i = rho0 * (1 + amp * (2u - 1)), row-major fill.
static void fill_noise(Density& d, double rho0, double amp, uint64_t seed) {
  SplitMix64 g(seed);
  for (long p = 0; p < d.Ntot(); ++p) d.set((unsigned)p, rho0 * (1.0 + amp * (2.0 * g.uniform() - 1.0)));
}

// rho(r) = rho_v + (rho_l - rho_v) * 0.5 * (1 - tanh((r - R)/w)), r from the box
// centre with x = getX(i) = dx (i - Nx/2).
static void fill_droplet(Density& d, double rho_v, double rho_l, double R, double w) {
  for (int i = 0; i < d.Nx(); ++i)
    for (int j = 0; j < d.Ny(); ++j)
      for (int k = 0; k < d.Nz(); ++k) {
        double x = d.getX(i), y = d.getY(j), z = d.getZ(k);
        double r = std::sqrt(x * x + y * y + z * z);
        d.set(i, j, k, rho_v + (rho_l - rho_v) * 0.5 * (1.0 - std::tanh((r - R) / w)));
      }
}

static std::vector<double> vec_of(const DFT_Vec& v) {
  std::vector<double> o(v.size());
  for (unsigned i = 0; i < v.size(); ++i) o[i] = v.get(i);
  return o;
}
static std::vector<double> density_of(const Density& d) { return vec_of(d.get_density_real()); }

// Barker-Henderson diameter: hsd = int_0^{r0} (1 - exp(-V(r)/kT)) dr for the
// cut-and-shifted LJ (the integral Potential1::getHSD evaluates with GSL qags),
// here by adaptive 10-point Gauss-Legendre to 1e-15.
static double lj_V(double r, double rc) {
  auto v = [](double x) { double y6 = std::pow(1.0 / x, 6); return 4.0 * (y6 * y6 - y6); };
  return v(r) - v(rc);
}
static double gl10(double a, double b, double rc, double kT) {
  static const double xs[5] = {0.1488743389816312, 0.4333953941292472, 0.6794095682990244, 0.8650633666889845, 0.9739065285171717};
  static const double ws[5] = {0.2955242247147529, 0.2692667193099963, 0.2190863625159820, 0.1494513491505806, 0.0666713443086881};
  double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0;
  for (int i = 0; i < 5; ++i)
    for (int sg = -1; sg <= 1; sg += 2) {
      double r = c + sg * h * xs[i];
      s += ws[i] * (1.0 - std::exp(-lj_V(r, rc) / kT));
    }
  return s * h;
}
static double adapt(double a, double b, double whole, double rc, double kT, int depth) {
  double m = 0.5 * (a + b);
  double l = gl10(a, m, rc, kT), r = gl10(m, b, rc, kT);
  if (depth > 40 || std::fabs(l + r - whole) < 1e-15) return l + r;
  return adapt(a, m, l, rc, kT, depth + 1) + adapt(m, b, r, rc, kT, depth + 1);
}
static double bh_diameter(double rc, double kT) {
  double shift = 4.0 * (std::pow(rc, -12) - std::pow(rc, -6));
  double r0 = std::pow(0.5 * std::sqrt(1.0 + shift) + 0.5, -1.0 / 6.0);
  double lo = 1e-3;  // integrand is 1 to machine precision below this
  return lo + adapt(lo, r0, gl10(lo, r0, rc, kT), rc, kT, 0);
}

static FMT* make_fmt(const std::string& name) {
  if (name == "WhiteBearI") return new WhiteBearI();
  if (name == "WhiteBearII") return new WhiteBearII();
  if (name == "RSLT") return new RSLT();
  if (name == "Rosenfeld") return new Rosenfeld();
  if (name == "esFMT") return new esFMT(1.0, 0.0);
  if (name == "esFMT_A1_Bm1") return new esFMT(1.0, -1.0);
  throw std::runtime_error("unknown model " + name);
}

// Sampled positions for large arrays: every `stride`-th point plus a hashed set.
static std::vector<double> sample_positions(long N, int count, uint64_t seed) {
  SplitMix64 g(seed);
  std::vector<double> p;
  for (int i = 0; i < count; ++i) p.push_back((double)(g.next() % (uint64_t)N));
  return p;
}
static std::vector<double> take(const std::vector<double>& a, const std::vector<double>& pos) {
  std::vector<double> o;
  for (double p : pos) o.push_back(a[(long)p]);
  return o;
}

struct Sums { double s1, s2, amax; };
static Sums sums(const std::vector<double>& a) {
  long double s1 = 0, s2 = 0; double m = 0;
  for (double x : a) { s1 += x; s2 += (long double)x * x; m = std::max(m, std::fabs(x)); }
  return {(double)s1, (double)s2, m};
}
static void put_field(const std::string& name, const std::vector<double>& a, bool full, const std::vector<double>& pos) {
  if (full) put(name, a);
  else put(name + ".sample", take(a, pos));
  Sums s = sums(a);
  put(name + ".sum", {s.s1});
  put(name + ".sumsq", {s.s2});
  put(name + ".absmax", {s.amax});
}

// --------------------------------------------------------------- cases -----

// FMT weights (real space) for a sphere of diameter hsd on an n^3 lattice.
static void case_weights(const std::string& tag, double dx, int n, double hsd) {
  double L[3] = {dx * n, dx * n, dx * n};
  Density d(dx, L);
  FMT_Species s(d, hsd, 0.0, 0);
  put1(tag + ".hsd", hsd);
  put1(tag + ".dx", dx);
  put1(tag + ".n", n);
  for (int a = 0; a < 11; ++a) {
    std::vector<double> w(d.Ntot());
    for (long p = 0; p < d.Ntot(); ++p) w[p] = s.getWeight(a, p);
    put(tag + ".w" + std::to_string(a), w);
  }
}

// Pointwise Phi and dPhi/dn for every model on seeded fundamental measures.
static void case_phi() {
  const char* models[] = {"Rosenfeld", "RSLT", "esFMT", "esFMT_A1_Bm1", "WhiteBearI", "WhiteBearII"};
  SplitMix64 g(777);
  const int npts = 64;
  std::vector<double> in;
  for (int p = 0; p < npts; ++p) {
    // A self-consistent single-species set: eta, s, v (|v| < s), T (symmetric).
    double hsd = 0.8 + 0.4 * g.uniform();
    double eta = (p < 4) ? (p == 0 ? 1e-14 : p == 1 ? 1e-13 : p == 2 ? 0.3 : 0.62) : 0.6 * g.uniform();
    double s2 = 6.0 * eta / hsd * (0.7 + 0.6 * g.uniform());
    double v[3], T[3][3];
    for (int i = 0; i < 3; ++i) v[i] = s2 * 0.5 * (2.0 * g.uniform() - 1.0) / std::sqrt(3.0);
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) T[i][j] = T[j][i] = (i == j ? s2 / 3.0 : 0.0) + 0.2 * s2 * (2.0 * g.uniform() - 1.0);
    double f[19] = {eta, s2 / (hsd * hsd), s2 / hsd, s2, v[0] / hsd, v[1] / hsd, v[2] / hsd, v[0], v[1], v[2],
                    T[0][0], T[0][1], T[0][2], T[1][0], T[1][1], T[1][2], T[2][0], T[2][1], T[2][2]};
    in.insert(in.end(), f, f + 19);
  }
  put("phi.inputs", in);
  for (const char* m : models) {
    FMT* fmt = make_fmt(m);
    std::vector<double> phi, dphi;
    for (int p = 0; p < npts; ++p) {
      FundamentalMeasures fm(&in[19 * p]);
      phi.push_back(fmt->calculate_Phi(fm));
      FundamentalMeasures d;
      fmt->calculate_dPhi_wrt_fundamental_measures(fm, d);
      std::vector<double> dv = d.get_as_vector();
      dphi.insert(dphi.end(), dv.begin(), dv.end());
    }
    put(std::string("phi.") + m + ".phi", phi);
    put(std::string("phi.") + m + ".dphi", dphi);
    delete fmt;
  }
}

// Density::write_VTK_File (src/Density.cpp:197-225, the reference's VisIt writer
// src/visit_writer.cpp) on two small seeded densities: 4x3x5 (the last line of values
// partly filled) and 3x3x3 (27 values: every line full). The files go next to the
// output file as <out>.a.vtk and <out>.b.vtk; the densities go into the output.
static void case_files(const std::string& out) {
  SplitMix64 g(4242);
  struct Box { const char* tag; double dx; double L[3]; };
  const Box boxes[2] = {{"a", 0.25, {1.0, 0.75, 1.25}}, {"b", 0.5, {1.5, 1.5, 1.5}}};
  for (const Box& b : boxes) {
    double L[3] = {b.L[0], b.L[1], b.L[2]};
    Density d(b.dx, L);
    std::vector<double> rho;
    for (long i = 0; i < d.Nx(); ++i)
      for (long j = 0; j < d.Ny(); ++j)
        for (long k = 0; k < d.Nz(); ++k) {
          const double v = 0.05 + 0.8 * g.uniform();
          d.set((int)i, (int)j, (int)k, v);
        }
    for (long p = 0; p < d.Ntot(); ++p) rho.push_back(d.get_density_real().get(p));
    put(std::string("files.") + b.tag + ".rho", rho);
    put(std::string("files.") + b.tag + ".shape", {(double)d.Nx(), (double)d.Ny(), (double)d.Nz()});
    d.write_VTK_File(out + "." + b.tag + ".vtk");
  }
}

// Bulk thermodynamics of one species (hard spheres, and LJ mean field).
static void case_bulk() {
  const char* models[] = {"Rosenfeld", "RSLT", "esFMT", "WhiteBearI", "WhiteBearII"};
  std::vector<double> rhos = {0.01, 0.1, 0.3, 0.5, 0.7, 0.9};
  double L[3] = {3.2, 3.2, 3.2};
  for (const char* m : models) {
    Density d(0.2, L);
    FMT_Species s(d, 1.0, 0.0, 0);
    FMT* fmt = make_fmt(m);
    DFT dft(&s);
    dft.addHardCoreContribution(fmt);
    std::vector<double> mu, om, fh;
    for (double r : rhos) { mu.push_back(dft.mu_times_beta(r)); om.push_back(dft.omega_times_beta_over_volume(r)); fh.push_back(dft.fhelmholtz_times_beta_over_volume(r)); }
    put(std::string("bulk.") + m + ".mu", mu);
    put(std::string("bulk.") + m + ".omega", om);
    put(std::string("bulk.") + m + ".fhelm", fh);
    delete fmt;
  }
  put("bulk.rho", rhos);
}

// One F+dF evaluation.
struct System {
  Density* d = nullptr;
  FMT_Species* s = nullptr;
  FMT* fmt = nullptr;
  LJ* lj = nullptr;
  Interaction_Interpolation_QF* inter = nullptr;
  DFT* dft = nullptr;
  double hsd = 1.0;
};
static System make_system(double dx, int n, const std::string& model, bool lj, double kT) {
  System S;
  double L[3] = {dx * n, dx * n, dx * n};
  S.d = new Density(dx, L);
  if (lj) S.hsd = bh_diameter(3.0, kT);
  S.s = new FMT_Species(*S.d, S.hsd, 0.0, 0);  // seq 0: one species per system
  S.fmt = make_fmt(model);
  S.dft = new DFT(S.s);
  S.dft->addHardCoreContribution(S.fmt);
  if (lj) {
    S.lj = new LJ(1.0, 1.0, 3.0);
    S.lj->setBH();
    S.inter = new Interaction_Interpolation_QF(S.s, S.s, S.lj, kT);
    S.dft->addInteraction(S.inter);
  }
  return S;
}

// The dense matrix of a Dynamical_Matrix (include/Dynamical_Matrix.h): column j =
// matrix_dot_v1 of the j-th unit vector (src/Dynamical_Matrix.cpp), stored column-major.
static std::vector<double> dense_matrix(const Dynamical_Matrix& m, long N) {
  std::vector<double> H((size_t)N * N);
  DFT_Vec e(N), r(N);
  for (long j = 0; j < N; ++j) {
    e.zeros(N);
    e.set(j, 1.0);
    m.matrix_dot_v1(e, r, nullptr);
    for (long i = 0; i < N; ++i) H[(size_t)j * N + i] = r.get(i);
  }
  return H;
}
// Largest eigenvalue of a + b H (H dense, symmetric, column-major) by power iteration
// from a seeded start; used only to bracket spectra for Log_Det.
static double power_extreme(const std::vector<double>& H, long N, double a, double b, int iters) {
  std::vector<double> x(N), y(N);
  SplitMix64 g(99);
  for (long i = 0; i < N; ++i) x[i] = 2.0 * g.uniform() - 1.0;
  double lam = 0;
  for (int it = 0; it < iters; ++it) {
    double nx = 0;
    for (long i = 0; i < N; ++i) nx += x[i] * x[i];
    nx = std::sqrt(nx);
    for (long i = 0; i < N; ++i) x[i] /= nx;
    for (long i = 0; i < N; ++i) y[i] = a * x[i];
    for (long j = 0; j < N; ++j)
      for (long i = 0; i < N; ++i) y[i] += b * H[(size_t)j * N + i] * x[j];
    lam = 0;
    for (long i = 0; i < N; ++i) lam += x[i] * y[i];
    x.swap(y);
  }
  return lam;
}

static void record_eval(const std::string& tag, System& S, bool full_fields, const std::vector<double>& pos) {
  double F = S.dft->calculateFreeEnergyAndDerivatives(false);
  put1(tag + ".Omega", F);
  put1(tag + ".F_id", S.dft->get_f_id());
  put1(tag + ".F_hs", S.dft->get_f_hs());
  put1(tag + ".F_mf", S.dft->get_f_mf());
  put1(tag + ".F_ext", S.dft->get_f_ext());
  put1(tag + ".mu", S.s->getChemPotential());
  put_field(tag + ".dF", vec_of(S.dft->getDF(0)), full_fields, pos);
  put_field(tag + ".rho", density_of(S.d[0]), full_fields, pos);
}

// FIRE2 probe: records per-step scalars through the draw_after() hook.
class FireProbe : public fireMinimizer2 {
 public:
  explicit FireProbe(DFT* dft) : fireMinimizer2(dft) {}
  std::vector<double> F, dt, alpha, vv, fmax, rms, resid;
  virtual void draw_after() {
    F.push_back(F_); dt.push_back(dt_); alpha.push_back(alpha_); vv.push_back(vv_); fmax.push_back(fmax_);
    rms.push_back(rms_force_);
    resid.push_back(dft_->getDF(0).inf_norm());
  }
  double getDt() const { return dt_; }
};

class DDFTProbe : public DDFT {
 public:
  DDFTProbe(DFT* dft) : DDFT(dft, false) {}
  std::vector<double> F, t, dt, mass, rhs;
  virtual void draw_after() {
    F.push_back(F_); t.push_back(time_); dt.push_back(dt_); rhs.push_back(RHS_max_);
    mass.push_back(dft_->getNumberAtoms(0));
  }
};

int main(int argc, char** argv) {
  if (argc != 3) { std::fprintf(stderr, "usage: %s <case> <out.bin>\n", argv[0]); return 2; }
  std::string c = argv[1];
  std::cout.setstate(std::ios_base::failbit);  // silence the reference's progress prints
  try {
    if (c == "weights") {
      case_weights("w_d1_dx0.2_n16", 0.2, 16, 1.0);
      case_weights("w_d0.9786_dx0.1_n16", 0.1, 16, 0.9786);
      case_weights("w_d1.3_dx0.25_n12", 0.25, 12, 1.3);
    } else if (c == "phi") {
      case_phi();
    } else if (c == "bulk") {
      case_bulk();
      put1("bulk.lj_hsd_kT0.8", bh_diameter(3.0, 0.8));
      put1("bulk.lj_hsd_kT1.0", bh_diameter(3.0, 1.0));
    } else if (c == "eval_models16") {
      const char* models[] = {"Rosenfeld", "RSLT", "esFMT", "WhiteBearI", "WhiteBearII"};
      for (const char* m : models) {
        System S = make_system(0.2, 16, m, false, 1.0);
        fill_noise(*S.d, 0.6, 0.2, 11);
        S.s->setChemPotential(S.dft->mu_times_beta(0.6));
        record_eval(std::string("m16.") + m, S, true, {});
      }
    } else if (c == "hessian") {
      // DFT::matrix_dot_v1 (src/Dynamical_Matrix.cpp; DFT::matrix_dot_v_intern,
      // src/DFT.cpp:435-488): the full Hessian (ideal gas + FMT + mean field)
      // times a seeded vector, at the state of the preceding F+dF evaluation.
      const char* models[] = {"Rosenfeld", "RSLT", "esFMT", "esFMT_A1_Bm1", "WhiteBearI", "WhiteBearII"};
      for (const char* m : models) {
        System S = make_system(0.2, 16, m, false, 1.0);
        fill_noise(*S.d, 0.6, 0.2, 11);
        S.s->setChemPotential(S.dft->mu_times_beta(0.6));
        S.dft->calculateFreeEnergyAndDerivatives(false);
        const long N = S.d->Ntot();
        DFT_Vec v(N), r(N);
        SplitMix64 g(77);
        for (long i = 0; i < N; ++i) v.set(i, 0.3 * (2.0 * g.uniform() - 1.0));
        S.dft->matrix_dot_v1(v, r, nullptr);
        put(std::string("h16.") + m + ".Hv", vec_of(r));
      }
      System S = make_system(0.1, 16, "WhiteBearI", true, 0.8);
      fill_noise(*S.d, 0.3, 0.1, 5);
      S.s->setChemPotential(S.dft->mu_times_beta(0.3));
      S.dft->calculateFreeEnergyAndDerivatives(false);
      const long N = S.d->Ntot();
      DFT_Vec v(N), r(N);
      SplitMix64 g(77);
      for (long i = 0; i < N; ++i) v.set(i, 0.3 * (2.0 * g.uniform() - 1.0));
      S.dft->matrix_dot_v1(v, r, nullptr);
      put("hlj16.Hv", vec_of(r));
      put1("hlj16.hsd", S.hsd);
      // DDFT::matrix_dot_v_intern (src/DDFT.cpp:353-361): g . (H v), the DDFT dynamical matrix
      DDFT ddft(S.dft, false);
      DFT_Vec gr(N);
      ddft.matrix_dot_v1(v, gr, nullptr);
      put("hlj16.GHv", vec_of(gr));
    } else if (c == "eval_hs32") {
      System S = make_system(0.2, 32, "WhiteBearI", false, 1.0);
      fill_noise(*S.d, 0.7, 0.05, 20240601);
      S.s->setChemPotential(S.dft->mu_times_beta(0.7));
      std::vector<double> pos = sample_positions(S.d->Ntot(), 2048, 99);
      put("hs32.pos", pos);
      record_eval("hs32", S, false, pos);
    } else if (c == "fire_hs32") {
      System S = make_system(0.2, 32, "WhiteBearI", false, 1.0);
      fill_noise(*S.d, 0.7, 0.05, 20240601);
      S.s->setChemPotential(S.dft->mu_times_beta(0.7));
      FireProbe fire(S.dft);
      fire.setForceTerminationCriterion(0.0);
      fire.run(200);
      put("fire32.F", fire.F); put("fire32.dt", fire.dt); put("fire32.alpha", fire.alpha);
      put("fire32.vv", fire.vv); put("fire32.fmax", fire.fmax); put("fire32.rms", fire.rms); put("fire32.resid_alias", fire.resid);
      std::vector<double> pos = sample_positions(S.d->Ntot(), 2048, 99);
      put("fire32.pos", pos);
      put_field("fire32.rho_final", density_of(*S.d), false, pos);
    } else if (c == "eval_lj") {
      // LJ fluid, WhiteBearI + QF mean field, kT = 0.8, 24^3 at dx = 0.2 (the
      // rc = 3 kernel is folded by the periodic box) and 16^3 at dx = 0.1.
      System S = make_system(0.2, 24, "WhiteBearI", true, 0.8);
      fill_droplet(*S.d, 0.01, 0.75, 1.6, 0.5);
      S.s->setChemPotential(S.dft->mu_times_beta(0.01));
      put1("lj24.hsd", S.hsd);
      put1("lj24.a_vdw", S.inter->getVDWParameter());
      std::vector<double> watt(S.d->Ntot());
      for (long p = 0; p < S.d->Ntot(); ++p) watt[p] = S.inter->getW(p);
      put("lj24.w_att", watt);
      record_eval("lj24", S, true, {});
      System T = make_system(0.1, 16, "WhiteBearI", true, 0.8);
      fill_noise(*T.d, 0.3, 0.1, 5);
      T.s->setChemPotential(T.dft->mu_times_beta(0.3));
      record_eval("lj16", T, true, {});
      // fixed mass variant (the droplet ensemble)
      System U = make_system(0.2, 24, "WhiteBearI", true, 0.8);
      fill_droplet(*U.d, 0.01, 0.75, 1.6, 0.5);
      double mass = U.d->getNumberAtoms();
      U.s->setFixedMass(mass * 1.01);
      put1("lj24fm.fixed_mass", mass * 1.01);
      record_eval("lj24fm", U, true, {});
    } else if (c == "fire_lj24") {
      System S = make_system(0.2, 24, "WhiteBearI", true, 0.8);
      fill_droplet(*S.d, 0.01, 0.75, 1.6, 0.5);
      double mass = S.d->getNumberAtoms();
      S.s->setFixedMass(mass);
      FireProbe fire(S.dft);
      fire.setForceTerminationCriterion(0.0);
      fire.run(60);
      put("firelj.F", fire.F); put("firelj.dt", fire.dt); put("firelj.alpha", fire.alpha);
      put("firelj.vv", fire.vv); put("firelj.fmax", fire.fmax); put("firelj.resid_alias", fire.resid);
      put("firelj.rho_final", density_of(*S.d));
    } else if (c == "ddft_lj16") {
      System S = make_system(0.1, 16, "WhiteBearI", true, 0.8);
      fill_noise(*S.d, 0.3, 0.1, 5);
      DDFTProbe ddft(S.dft);
      ddft.setTimeStep(1e-4);
      ddft.set_max_time_step(1e-4);
      ddft.setForceTerminationCriterion(0.0);
      ddft.run(10);
      put("ddft16.F", ddft.F); put("ddft16.t", ddft.t); put("ddft16.dt", ddft.dt);
      put("ddft16.mass", ddft.mass); put("ddft16.rhs", ddft.rhs);
      put("ddft16.rho_final", density_of(*S.d));
    } else if (c == "coex") {
      // bulk coexistence of the LJ fluid (WhiteBearI + QF at dx = 0.1): DFT::findCoex
      std::vector<double> kts = {0.7, 0.8, 0.9}, xv, xl, mu, xs1, xs2;
      for (double kT : kts) {
        System S = make_system(0.1, 16, "WhiteBearI", true, kT);
        double a, b, s1, s2;
        S.dft->findSpinodal(1.0, 1e-3, s1, s2, 1e-8);
        S.dft->findCoex(1.0, 1e-3, a, b, 1e-8);
        xv.push_back(a); xl.push_back(b); mu.push_back(S.dft->mu_times_beta(a)); xs1.push_back(s1); xs2.push_back(s2);
        put1("coex.hsd_kT" + std::to_string(kT).substr(0, 3), S.hsd);
        put1("coex.avdw_kT" + std::to_string(kT).substr(0, 3), S.inter->getVDWParameter());
      }
      put("coex.kT", kts); put("coex.x_vap", xv); put("coex.x_liq", xl); put("coex.mu", mu);
      put("coex.spinodal1", xs1); put("coex.spinodal2", xs2);
    } else if (c == "ddft_adapt16") {
      // default adaptive time step (dt grows x2 after 5 successes up to dtMax)
      System S = make_system(0.1, 16, "WhiteBearI", true, 0.8);
      fill_noise(*S.d, 0.3, 0.1, 5);
      DDFTProbe ddft(S.dft);
      ddft.setTimeStep(1e-5);
      ddft.set_max_time_step(4e-5);
      ddft.setForceTerminationCriterion(0.0);
      ddft.run(14);
      put("ddfta.F", ddft.F); put("ddfta.t", ddft.t); put("ddfta.dt", ddft.dt);
      put("ddfta.mass", ddft.mass); put("ddfta.rhs", ddft.rhs);
      put("ddfta.rho_final", density_of(*S.d));
    } else if (c == "ao") {
      // FMT_AO_Species (src/FMT_Species.cpp:645-738, src/FMT.cpp:340-421): hard-sphere colloids
      // (d = 1) with ideal polymers of radius Rp = 0.35 at reservoir density 0.4 (the
      // Asakura-Oosawa model), one F+dF evaluation each for a model without and with the
      // tensor measures, and the bulk mu / omega with the AO terms (src/FMT.cpp:616-709).
      const char* models[] = {"Rosenfeld", "WhiteBearI"};
      for (const char* m : models) {
        double L[3] = {3.2, 3.2, 3.2};
        Density* d = new Density(0.2, L);
        FMT_AO_Species* s = new FMT_AO_Species(*d, 1.0, 0.35, 0.4, 0.0, 0);
        FMT* fmt = make_fmt(m);
        DFT* dft = new DFT(s);
        dft->addHardCoreContribution(fmt);
        fill_noise(*d, 0.4, 0.2, 13);
        s->setChemPotential(dft->mu_times_beta(0.4));
        double F = dft->calculateFreeEnergyAndDerivatives(false);
        const std::string tag = std::string("ao16.") + m;
        put1(tag + ".Omega", F);
        put1(tag + ".F_id", dft->get_f_id());
        put1(tag + ".F_hs", dft->get_f_hs());
        put1(tag + ".F_ext", dft->get_f_ext());
        put1(tag + ".mu", s->getChemPotential());
        put(tag + ".dF", vec_of(dft->getDF(0)));
        put(tag + ".rho", density_of(*d));
        std::vector<double> mu, om;
        for (double r : {0.05, 0.2, 0.4, 0.6}) { mu.push_back(dft->mu_times_beta(r)); om.push_back(dft->omega_times_beta_over_volume(r)); }
        put(tag + ".bulk_mu", mu);
        put(tag + ".bulk_omega", om);
        // Dynamical_Matrix::matrix_dot_v1 of the AO system at this density: the reference's
        // FMT::add_second_derivative (src/FMT.cpp:437-567) takes the AO species through the
        // plain FMT_Species branch, so this is the hard-sphere FMT Hessian plus the ideal gas
        {
          const long N = d->Ntot();
          DFT_Vec v(N), r(N);
          SplitMix64 g(77);
          for (long i = 0; i < N; ++i) v.set(i, 0.3 * (2.0 * g.uniform() - 1.0));
          dft->matrix_dot_v1(v, r, nullptr);
          put(tag + ".Hv", vec_of(r));
        }
      }
    } else if (c == "files") {
      case_files(argv[2]);
    } else if (c == "boundary") {
      // Species::setFixedBackground / setHomogeneousBoundary (src/Species.cpp:74-95): the
      // boundary planes i = 0, j = 0, k = 0 in the evaluation, the Hessian
      // (src/DFT.cpp:441-487, Dynamical_Matrix::matrix_dot_v1), FIRE2 and Log_Det.
      const long N = 16 * 16 * 16;
      {
        System S = make_system(0.2, 16, "WhiteBearI", false, 1.0);
        fill_noise(*S.d, 0.6, 0.2, 11);
        S.s->setChemPotential(S.dft->mu_times_beta(0.6));
        S.s->setFixedBackground(true);
        record_eval("bfix", S, true, {});
        DFT_Vec v(N), r(N);
        SplitMix64 g(77);
        for (long i = 0; i < N; ++i) v.set(i, 0.3 * (2.0 * g.uniform() - 1.0));
        S.dft->matrix_dot_v1(v, r, nullptr);
        put("bfix.Hv", vec_of(r));
        Log_Det ld(*S.dft, 10, 0.16, 0.008, false);
        double var = 0;
        const double val = ld.calculate_log_det(1234, 2, false, var);
        put("bfix.logdet", {val, var});
        FireProbe fire(S.dft);
        fire.setForceTerminationCriterion(0.0);
        fire.run(30);
        put("bfix.fire.F", fire.F);
        put("bfix.fire.rho", density_of(*S.d));
      }
      {
        System S = make_system(0.2, 16, "WhiteBearI", false, 1.0);
        fill_noise(*S.d, 0.6, 0.2, 11);
        S.s->setChemPotential(S.dft->mu_times_beta(0.6));
        S.s->setHomogeneousBoundary(true);
        record_eval("bhom", S, true, {});
      }
      {
        System S = make_system(0.2, 16, "WhiteBearI", false, 1.0);
        fill_noise(*S.d, 0.6, 0.2, 11);
        const double mass = S.d->getNumberAtoms();
        S.s->setFixedMass(0.98 * mass);
        S.s->setHomogeneousBoundary(true);
        put1("bhomfm.fixed_mass", 0.98 * mass);
        record_eval("bhomfm", S, true, {});
      }
      // DDFT with each boundary mode (src/DDFT.cpp:280-281, 333-338): the LJ system of ddft_lj16
      for (int mode = 0; mode < 2; ++mode) {
        System S = make_system(0.1, 16, "WhiteBearI", true, 0.8);
        fill_noise(*S.d, 0.3, 0.1, 5);
        if (mode == 0) S.s->setFixedBackground(true);
        else S.s->setHomogeneousBoundary(true);
        DDFTProbe ddft(S.dft);
        ddft.setTimeStep(1e-4);
        ddft.set_max_time_step(1e-4);
        ddft.setForceTerminationCriterion(0.0);
        ddft.run(10);
        const std::string tag = mode == 0 ? "bddft_fix" : "bddft_hom";
        put(tag + ".F", ddft.F); put(tag + ".mass", ddft.mass); put(tag + ".dt", ddft.dt);
        put(tag + ".rho_final", density_of(*S.d));
      }
    } else if (c == "spectral") {
      // Pins of the spectral drivers (Eigenvalues, Arnoldi, Log_Det consume matrix_dot_v1):
      // the dense Hessian of a hard-sphere state and of an LJ state (tests/golden/make_golden.py
      // takes their eigenvalues with LAPACK and keeps those), and Log_Det::calculate_log_det
      // (src/Log_Det.cpp:84-166) of the hard-sphere DFT matrix and of its DDFT matrix.
      System S = make_system(0.2, 16, "WhiteBearI", false, 1.0);
      fill_noise(*S.d, 0.6, 0.2, 11);
      S.s->setChemPotential(S.dft->mu_times_beta(0.6));
      S.dft->calculateFreeEnergyAndDerivatives(false);
      const long N = S.d->Ntot();
      std::vector<double> H = dense_matrix(*S.dft, N);
      put("sp16.H", H);
      const double lmax = power_extreme(H, N, 0.0, 1.0, 400);
      const double lmin = lmax - power_extreme(H, N, lmax, -1.0, 4000);
      const double lam_max = 1.02 * lmax, lam_min = 0.9 * lmin;
      put("sp16.logdet.bounds", {lam_min, lam_max});
      for (int order : {10, 40}) {
        Log_Det ld(*S.dft, order, lam_max, lam_min, false);
        double var = 0;
        const double val = ld.calculate_log_det(1234, 3, false, var);
        put(std::string("sp16.logdet.o") + std::to_string(order), {val, var});
      }
      {
        Log_Det ld(*S.dft, 20, lam_max, lam_min, false);
        double var = 0;
        const double val = ld.calculate_log_det(77, 2, true, var);
        put("sp16.logdet.zero", {val, var});
      }
      DDFT ddft(S.dft, false);
      // the dominant eigenvalue of -g.H (the matrix Log_Det uses for a dynamic matrix) by
      // power iteration through the reference's own product
      double gmax = 0;
      {
        DFT_Vec x(N), y(N);
        SplitMix64 g(5);
        for (long i = 0; i < N; ++i) x.set(i, 2.0 * g.uniform() - 1.0);
        for (int it = 0; it < 300; ++it) {
          x.MultBy(1.0 / x.euclidean_norm());
          ddft.matrix_dot_v1(x, y, nullptr);
          y.MultBy(-1.0);
          gmax = x.dotWith(y);
          x.set(y);
        }
      }
      const double g_max = 1.05 * gmax, g_min = 1e-3 * gmax;
      put("sp16.logdet.ddft.bounds", {g_min, g_max});
      Log_Det lg(ddft, 16, g_max, g_min, false);
      double var = 0;
      const double val = lg.calculate_log_det(4321, 2, true, var);
      put("sp16.logdet.ddft", {val, var});
      // the dense DDFT dynamical matrix g.H (every column a DDFT::matrix_dot_v1), whose
      // spectrum pins the eigen drivers on it (make_golden.py keeps its eigenvalues)
      put("sp16.G", dense_matrix(ddft, N));
      System T = make_system(0.1, 16, "WhiteBearI", true, 0.8);
      fill_noise(*T.d, 0.3, 0.1, 5);
      T.s->setChemPotential(T.dft->mu_times_beta(0.3));
      T.dft->calculateFreeEnergyAndDerivatives(false);
      put("splj16.H", dense_matrix(*T.dft, N));
      put1("splj16.hsd", T.hsd);
    } else {
      std::fprintf(stderr, "unknown case %s\n", c.c_str());
      return 2;
    }
  } catch (std::exception& e) {
    std::fprintf(stderr, "reference threw: %s\n", e.what());
    return 1;
  }
  write_out(argv[2]);
  return 0;
}

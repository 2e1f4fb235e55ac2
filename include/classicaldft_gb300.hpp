// classicaldft_gb300.hpp — the reference's C++ class API over the GB300 C ABI.
//
// Header-only. Code written against jimlutsko/classicalDFT's DFT / Species /
// FMT / Interaction / Minimizer classes for the free-energy-and-derivative
// path compiles against this header with the same class names and method
// signatures, and runs on the GPU through include/cdft.h
// (link with classicaldft_gb300/libcdft.so and the CUDA runtime).
//
// Covered: Lattice/Density (include/Lattice.h, include/Density.h), FMT models
// Rosenfeld / RSLT / esFMT / WhiteBearI / WhiteBearII (include/FMT.h),
// FMT_Species (include/Species.h), LJ with setBH (include/Potential1.h),
// Interaction_Interpolation_QF (include/Interaction.h), DFT (include/DFT.h),
// fireMinimizer2 and DDFT (include/Minimizer.h), Log_Det (include/Log_Det.h),
// Eigenvalues (include/Eigenvalues.h), Arnoldi (include/Arnoldi.h),
// Eta_Too_Large_Exception.
#ifndef CLASSICALDFT_GB300_HPP
#define CLASSICALDFT_GB300_HPP

#include <algorithm>
#include <cmath>
#include <cstring>
#include <istream>
#include <ostream>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "cdft.h"

namespace classicaldft_gb300 {

class Eta_Too_Large_Exception : public std::runtime_error {
 public:
  Eta_Too_Large_Exception() : std::runtime_error("Eta too large in FMT::dPHI") {}
};

inline void check(int code, const cdft_ctx* ctx) {
  if (code == CDFT_OK) return;
  if (code == CDFT_ERR_ETA) throw Eta_Too_Large_Exception();
  throw std::runtime_error(std::string("classicaldft_gb300: ") + (ctx ? cdft_last_error(ctx) : "error") + " (code " +
                           std::to_string(code) + ")");
}

// include/Lattice.h:57-134
class Lattice {
 public:
  Lattice(double dx, const double L[]) : dx_(dx) {
    for (int a = 0; a < 3; ++a) {
      n_[a] = long((L[a] + 1e-8 * dx) / dx);
      if (std::fabs(L[a] - n_[a] * dx) > 1e-5 * dx) throw std::runtime_error("Box length incommensurate with lattice");
    }
  }
  long Nx() const { return n_[0]; }
  long Ny() const { return n_[1]; }
  long Nz() const { return n_[2]; }
  long Ntot() const { return n_[0] * n_[1] * n_[2]; }
  long Nout() const { return n_[0] * n_[1] * (n_[2] / 2 + 1); }
  double getDX() const { return dx_; }
  double dV() const { return dx_ * dx_ * dx_; }
  double getVolume() const { return Ntot() * dV(); }
  double getX(int i) const { return dx_ * (i - double(n_[0]) / 2); }
  double getY(int i) const { return dx_ * (i - double(n_[1]) / 2); }
  double getZ(int i) const { return dx_ * (i - double(n_[2]) / 2); }
  long pos(int i, int j, int k) const { return k + n_[2] * (j + n_[1] * i); }

 protected:
  double dx_;
  long n_[3];
};

// include/DFT_LinAlg.h:14-98: the reference's real vector, with the behaviour of its
// Armadillo adapter (additionalCode/DFT_Armadillo.cpp), in host memory. getDF returns one.
class DFT_Vec {
 public:
  DFT_Vec() : d_(1, 0.0) {}
  explicit DFT_Vec(unsigned N) : d_(N, 0.0) {}
  void set(unsigned pos, double val) { d_[pos] = val; }
  double get(unsigned pos) const { return d_[pos]; }
  void set(const DFT_Vec& x) { d_ = x.d_; }
  void set(const DFT_Vec& v1, const DFT_Vec& v2, double scale) {  // v1 + v2 * scale
    d_.resize(v1.size());
    for (size_t i = 0; i < d_.size(); ++i) d_[i] = v1.d_[i] + v2.d_[i] * scale;
  }
  void set(const double* x, unsigned n) { d_.assign(x, x + n); }
  void set(double v) { std::fill(d_.begin(), d_.end(), v); }
  void set_random_normal() {
    std::mt19937_64 g(std::random_device{}());
    std::normal_distribution<double> nd(0.0, 1.0);
    for (double& x : d_) x = nd(g);
  }
  void set_random() {  // uniform in (-1, 1)
    std::mt19937_64 g(std::random_device{}());
    std::uniform_real_distribution<double> u(0.0, 1.0);
    for (double& x : d_) x = 2 * u(g) - 1;
  }
  void resize(long N) { d_.resize(N, 0.0); }
  void zeros(long N) { d_.assign(N, 0.0); }
  void zeros() { std::fill(d_.begin(), d_.end(), 0.0); }
  double inf_norm() const {
    double m = 0;
    for (double x : d_) m = std::max(m, std::fabs(x));
    return m;
  }
  double euclidean_norm() const { return std::sqrt(dotWith(*this)); }
  void normalise() { MultBy(1.0 / euclidean_norm()); }
  double min() const { return *std::min_element(d_.begin(), d_.end()); }
  double max() const { return *std::max_element(d_.begin(), d_.end()); }
  double* memptr() { return d_.data(); }
  const void* get_raw_data() const { return d_.data(); }
  unsigned size() const { return (unsigned)d_.size(); }
  double dotWith(const DFT_Vec& v) const {
    double s = 0;
    for (size_t i = 0; i < d_.size(); ++i) s += v.d_[i] * d_[i];
    return s;
  }
  double accu() const {
    double s = 0;
    for (double x : d_) s += x;
    return s;
  }
  void MultBy(double val) { for (double& x : d_) x *= val; }
  void IncrementBy(const DFT_Vec& v) { for (size_t i = 0; i < d_.size(); ++i) d_[i] += v.d_[i]; }
  void DecrementBy(const DFT_Vec& v) { for (size_t i = 0; i < d_.size(); ++i) d_[i] -= v.d_[i]; }
  void add(double shift) { for (double& x : d_) x += shift; }
  void IncrementBy(unsigned pos, double val) { d_[pos] += val; }
  void IncrementBy_Scaled_Vector(const DFT_Vec& v, double scale) { for (size_t i = 0; i < d_.size(); ++i) d_[i] += v.d_[i] * scale; }
  void Schur(const DFT_Vec& v1, const DFT_Vec& v2) {
    d_.resize(v1.size());
    for (size_t i = 0; i < d_.size(); ++i) d_[i] = v1.d_[i] * v2.d_[i];
  }
  // the reference's stream format: unsigned N, then N doubles
  friend std::ostream& operator<<(std::ostream& of, const DFT_Vec& v) {
    const unsigned N = v.size();
    of.write((const char*)&N, sizeof(unsigned));
    of.write((const char*)v.d_.data(), N * sizeof(double));
    return of;
  }
  friend std::istream& operator>>(std::istream& in, DFT_Vec& v) {
    unsigned N = 0;
    in.read((char*)&N, sizeof(unsigned));
    v.resize(N);
    in.read((char*)v.d_.data(), N * sizeof(double));
    return in;
  }

 private:
  std::vector<double> d_;
};

// include/Density.h:35-118 (the host copy of the field; the GPU holds the working copy)
class Density : public Lattice {
 public:
  Density(double dx, const double L[]) : Lattice(dx, L), rho_(Ntot(), 0.0) {}
  void set(long pos, double v) { rho_[pos] = v; }
  void set(int i, int j, int k, double v) { rho_[pos(i, j, k)] = v; }
  void set(const std::vector<double>& x) { rho_ = x; }
  double get(long pos) const { return rho_[pos]; }
  double getNumberAtoms() const {
    double s = 0, c = 0;
    for (double x : rho_) {
      double t = s + x;
      c += (std::fabs(s) >= std::fabs(x)) ? (s - t) + x : (x - t) + s;
      s = t;
    }
    return (s + c) * dV();
  }
  const double* data() const { return rho_.data(); }
  double* data() { return rho_.data(); }
  // src/Density.cpp:197-244: Armadillo binary snapshot, and the VisIt-writer VTK file
  void writeDensity(const std::string& filename) const {
    if (cdft_density_write(filename.c_str(), rho_.data(), (long)rho_.size()) != CDFT_OK)
      throw std::runtime_error("could not write " + filename);
  }
  void readDensity(const char* filename) {
    if (cdft_density_read(filename, rho_.data(), (long)rho_.size()) != CDFT_OK)
      throw std::runtime_error(std::string("Could not open input file ") + filename + " ... aborting ... ");
  }
  void write_VTK_File(const std::string& filename) const {
    if (cdft_density_write_vtk(filename.c_str(), rho_.data(), (int)Nx(), (int)Ny(), (int)Nz()) != CDFT_OK)
      throw std::runtime_error("could not write " + filename);
  }

 private:
  std::vector<double> rho_;
};

// include/FMT.h:139-643
class FMT {
 public:
  virtual ~FMT() {}
  virtual int model() const = 0;
  virtual double A() const { return 1.0; }
  virtual double B() const { return 0.0; }
  bool needsTensor() const { return model() >= CDFT_ESFMT; }
};
class Rosenfeld : public FMT { public: int model() const override { return CDFT_ROSENFELD; } };
class RSLT : public FMT { public: int model() const override { return CDFT_RSLT; } };
class esFMT : public FMT {
 public:
  esFMT(double A = 1, double B = 0) : A_(A), B_(B) {}
  int model() const override { return CDFT_ESFMT; }
  double A() const override { return A_; }
  double B() const override { return B_; }
 private:
  double A_, B_;
};
class WhiteBearI : public FMT { public: int model() const override { return CDFT_WHITEBEAR_I; } };
class WhiteBearII : public FMT { public: int model() const override { return CDFT_WHITEBEAR_II; } };

// include/Potential1.h:136-189 (Barker-Henderson split only)
class LJ {
 public:
  LJ(double sigma, double eps, double rcut) : sigma_(sigma), eps_(eps), rcut_(rcut) {}
  void setBH() { bh_ = true; }
  double getHSD(double kT) const {
    if (!bh_) throw std::runtime_error("only the Barker-Henderson split is on the GPU path");
    double d = 0;
    check(cdft_bh_diameter(sigma_, eps_, rcut_, kT, &d), nullptr);
    return d;
  }
  double sigma() const { return sigma_; }
  double eps() const { return eps_; }
  double getRcut() const { return rcut_; }
  bool isBH() const { return bh_; }
 private:
  double sigma_, eps_, rcut_;
  bool bh_ = false;
};

// include/Species.h:13-380
class FMT_Species {
 public:
  FMT_Species(Density& density, double hsd, double mu = 0, int seq = -1) : density_(density), hsd_(hsd), mu_(mu) {
    (void)seq;
  }
  virtual ~FMT_Species() {}
  // the polymer radius and reservoir density of an FMT_AO_Species (0 for a plain FMT_Species)
  virtual double aoRp() const { return 0.0; }
  virtual double getReservoirDensity() const { return 0.0; }
  void setChemPotential(double m) { mu_ = m; fixedMass_ = -1; }
  double getChemPotential() const { return mu_; }
  void setFixedMass(double m) { fixedMass_ = m; if (m > 0.0) mu_ = 0.0; }
  bool is_mass_fixed() const { return fixedMass_ > 0; }
  // include/Species.h:24-29 (src/Species.cpp:74-95)
  void setFixedBackground(bool fixed) { fixedBackground_ = fixed; }
  void setHomogeneousBoundary(bool homo) { homogeneousBoundary_ = homo; }
  bool is_background_fixed() const { return fixedBackground_; }
  bool is_fixed_boundary() const { return fixedBackground_; }
  bool is_boundary_homogeneous() const { return homogeneousBoundary_; }
  double getHSD() const { return hsd_; }
  Density& getDensity() { return density_; }
  const Density& getLattice() const { return density_; }
  DFT_Vec& getDF() { return dF_; }
  const DFT_Vec& getDF() const { return dF_; }
  double get_convergence_monitor() const { return dF_.inf_norm() / density_.dV(); }
  double fixedMass() const { return fixedMass_; }
  void setMuInternal(double m) { mu_ = m; }

 private:
  Density& density_;
  double hsd_, mu_;
  double fixedMass_ = -1;
  bool fixedBackground_ = false, homogeneousBoundary_ = false;
  DFT_Vec dF_;
};

// include/Species.h:380-461, src/FMT_Species.cpp:645-738: hard-sphere colloids with ideal
// polymers of radius Rp at the given reservoir density (the Asakura-Oosawa model)
class FMT_AO_Species : public FMT_Species {
 public:
  FMT_AO_Species(Density& density, double hsd, double Rp, double reservoir_density, double mu = 0, int seq = -1)
      : FMT_Species(density, hsd, mu, seq), Rp_(Rp), reservoir_(reservoir_density) {}
  double aoRp() const override { return Rp_; }
  double getReservoirDensity() const override { return reservoir_; }
  double getHSDP() const { return 2 * Rp_; }
 private:
  double Rp_, reservoir_;
};

// include/Interaction.h:416-441 (self interaction of one species)
class Interaction_Interpolation_QF {
 public:
  Interaction_Interpolation_QF(FMT_Species* s1, FMT_Species* s2, LJ* v, double kT) : s_(s1), v_(v), kT_(kT) {
    if (s1 != s2) throw std::runtime_error("only the self interaction of one species is on the GPU path");
  }
  FMT_Species* species() const { return s_; }
  LJ* potential() const { return v_; }
  double kT() const { return kT_; }
 private:
  FMT_Species* s_;
  LJ* v_;
  double kT_;
};

// include/DFT.h:44-190
class DFT {
 public:
  explicit DFT(FMT_Species* s = nullptr, int precision = CDFT_FP64) : s_(s), precision_(precision) {}
  ~DFT() { if (ctx_) cdft_destroy(ctx_); }
  DFT(const DFT&) = delete;
  DFT& operator=(const DFT&) = delete;

  void addSpecies(FMT_Species* s) { s_ = s; reset(); }
  void addHardCoreContribution(FMT* fmt) { fmt_ = fmt; reset(); }
  void addInteraction(Interaction_Interpolation_QF* i) { inter_ = i; reset(); }

  double calculateFreeEnergyAndDerivatives(bool onlyFex) {
    push();
    double t[8];
    DFT_Vec& dF = s_->getDF();
    dF.resize(s_->getDensity().Ntot());
    int rc = cdft_eval(context(), onlyFex ? 1 : 0, t, dF.memptr(), 0);
    check(rc, ctx_);
    pull(t);
    return t[0];
  }
  double mu_times_beta(double rho) { double o[3]; check(cdft_bulk(context(), rho, o), ctx_); return o[0]; }
  double omega_times_beta_over_volume(double rho) { double o[3]; check(cdft_bulk(context(), rho, o), ctx_); return o[1]; }
  double fhelmholtz_times_beta_over_volume(double rho) { double o[3]; check(cdft_bulk(context(), rho, o), ctx_); return o[2]; }
  double get_f_id() const { return F_[0]; }
  double get_f_hs() const { return F_[1]; }
  double get_f_mf() const { return F_[2]; }
  double get_f_ext() const { return F_[3]; }
  DFT_Vec& getDF(int) { return s_->getDF(); }
  FMT_Species* getSpecies(int) const { return s_; }
  double get_convergence_monitor() const { return s_->get_convergence_monitor(); }

  // Dynamical_Matrix::matrix_dot_v1 (src/Dynamical_Matrix.cpp): the full Hessian of Omega
  // (DFT::matrix_dot_v_intern, src/DFT.cpp:435-488) times v, at the current density.
  void matrix_dot_v1(const DFT_Vec& v, DFT_Vec& result, void* param = nullptr) {
    (void)param;
    push();
    result.resize(v.size());
    check(cdft_hessian_dot_v(context(), (const double*)v.get_raw_data(), result.memptr(), 0), ctx_);
  }
  void matrix_dot_v1(const std::vector<double>& v, std::vector<double>& result) {
    push();
    result.resize(v.size());
    check(cdft_hessian_dot_v(context(), v.data(), result.data(), 0), ctx_);
  }
  // DFT::findCoex (src/DFT_Coex.cpp:159-196): coexisting vapour and liquid densities.
  void findCoex(double xmax, double dx, double& x1, double& x2, double tol = 1e-8) {
    double o[5];
    check(cdft_find_coex(context(), xmax, dx, tol, o), ctx_);
    x1 = o[0];
    x2 = o[1];
  }

  // GPU handle for the minimizers
  cdft_ctx* context() {
    if (!ctx_) {
      cdft_params p;
      std::memset(&p, 0, sizeof(p));
      const Density& d = s_->getDensity();
      p.nx = (int)d.Nx(); p.ny = (int)d.Ny(); p.nz = (int)d.Nz(); p.dx = d.getDX();
      p.model = fmt_ ? fmt_->model() : CDFT_MODEL_NONE;
      p.es_A = fmt_ ? fmt_->A() : 1; p.es_B = fmt_ ? fmt_->B() : 0;
      p.hsd = s_->getHSD();
      if (inter_) {
        p.lj = 1; p.lj_sigma = inter_->potential()->sigma(); p.lj_eps = inter_->potential()->eps();
        p.lj_rc = inter_->potential()->getRcut(); p.kT = inter_->kT();
      }
      p.mu = s_->getChemPotential();
      p.fixed_mass = s_->fixedMass();
      p.precision = precision_;
      p.ao_rp = s_->aoRp();
      p.ao_reservoir = s_->getReservoirDensity();
      check(cdft_create(&p, &ctx_), nullptr);
    }
    return ctx_;
  }
  void push() {
    cdft_ctx* c = context();
    check(cdft_set_density(c, s_->getDensity().data(), 0), c);
    check(cdft_set_boundary(c, s_->is_background_fixed() ? 1 : 0, s_->is_boundary_homogeneous() ? 1 : 0), c);
    if (s_->is_mass_fixed()) check(cdft_set_fixed_mass(c, s_->fixedMass()), c);
    else check(cdft_set_chem_potential(c, s_->getChemPotential()), c);
  }
  void pull_density() { check(cdft_get_density(ctx_, s_->getDensity().data(), 0), ctx_); }

 private:
  void reset() { if (ctx_) { cdft_destroy(ctx_); ctx_ = nullptr; } }
  void pull(const double* t) {
    F_[0] = t[1]; F_[1] = t[2]; F_[2] = t[3]; F_[3] = t[4];
    s_->setMuInternal(t[5]);
    // a fixed mass rescales the density, as the reference's Density does; otherwise the
    // evaluation leaves it as pushed and nothing comes back
    if (s_->is_mass_fixed()) pull_density();
  }
  FMT_Species* s_;
  FMT* fmt_ = nullptr;
  Interaction_Interpolation_QF* inter_ = nullptr;
  int precision_;
  cdft_ctx* ctx_ = nullptr;
  double F_[4] = {0, 0, 0, 0};
};

// include/Minimizer.h:80-182
class fireMinimizer2 {
 public:
  explicit fireMinimizer2(DFT* dft) : dft_(dft) { cdft_fire_default_params(&p_); }
  void setTimeStep(double dt) { p_.dt = dt; }
  void setTimeStepMax(double dt) { p_.dt_max = dt; }
  void setAlphaStart(double a) { p_.alpha_start = a; }
  void setAlphaFac(double a) { p_.f_alf = a; }
  void setForceTerminationCriterion(double v) { p_.force_limit = v; }
  double step() {
    start();
    check(cdft_fire_step(dft_->context(), 1, &r_), dft_->context());
    snapshot_after(1);
    return r_.F;
  }
  // Minimizer::run (src/Minimizer.cpp:36-87), steps on the GPU; with snapshots on, the run
  // is cut where the reference's step() writes one, and the density comes back there
  void run(long maxSteps = -1) {
    start();
    if (!snapshots_) {
      check(cdft_fire_run(dft_->context(), maxSteps, &r_), dft_->context());
      dft_->pull_density();
      return;
    }
    long done = 0;
    for (;;) {
      long chunk = (10 - counter() % 10) % 10 + 1;  // steps up to and including the next writing one
      if (maxSteps >= 0) chunk = std::min(chunk, maxSteps - done);
      if (chunk <= 0) break;
      cdft_fire_report r;
      check(cdft_fire_run(dft_->context(), chunk, &r), dft_->context());
      r_ = r;
      done += r.steps;
      snapshot_after(r.steps);
      if (r.steps < chunk || r.stop != 0) break;
    }
    dft_->pull_density();
  }
  void resume(long maxSteps = -1) { run(maxSteps); }
  // fireMinimizer2::step writes snapshot_s0.dat (Density::writeDensity) at every tenth call
  // counted over the process (src/Minimizer.cpp:258-268); off: no files, no density reads
  void setSnapshots(bool on) { snapshots_ = on; }
  // the minimizer's state (Boost serialisation in the reference, include/Minimizer.h:145-180)
  // to a file and back; a loaded minimizer continues the saved run
  void save_state(const std::string& path) {
    start();
    check(cdft_fire_save(dft_->context(), path.c_str()), dft_->context());
  }
  void load_state(const std::string& path) {
    dft_->push();
    check(cdft_fire_load(dft_->context(), path.c_str()), dft_->context());
    started_ = true;
    dft_->pull_density();
  }
  double getF() const { return r_.F; }
  double get_convergence_monitor() const { return std::fabs(r_.vv / dft_->getSpecies(0)->getDensity().getVolume()); }
  const cdft_fire_report& report() const { return r_; }

 private:
  void start() {
    if (!started_) {
      dft_->push();
      check(cdft_fire_init(dft_->context(), &p_), dft_->context());
      started_ = true;
    }
  }
  static long& counter() {  // the reference's static step counter, shared by every minimizer
    static long ic = 0;
    return ic;
  }
  // after n more step() calls: write snapshot_s0.dat for each that lands on a multiple of 10
  void snapshot_after(long n) {
    if (n <= 0) return;
    const long first = counter(), last = counter() + n - 1;
    counter() += n;
    if (!snapshots_) return;
    if ((last / 10) * 10 < first) return;  // no multiple of 10 in [first, last]
    dft_->pull_density();
    dft_->getSpecies(0)->getDensity().writeDensity("snapshot_s0.dat");
  }
  DFT* dft_;
  cdft_fire_params p_;
  cdft_fire_report r_{};
  bool started_ = false;
  bool snapshots_ = true;
};

// include/Minimizer.h:189-266 (periodic boundaries)
class DDFT {
 public:
  DDFT(DFT* dft, bool showGraphics = false) : dft_(dft) {
    (void)showGraphics;
    const double dx = dft->getSpecies(0)->getDensity().getDX();
    dt_ = 1e-4 * dx * dx;
  }
  void setTimeStep(double dt) { dt_ = dt; }
  void set_max_time_step(double t) { dt_max_ = t; }
  void set_tolerence_fixed_point(double e) { tol_ = e; }
  double step() {
    start();
    check(cdft_ddft_step(dft_->context(), 1, &r_), dft_->context());
    dft_->pull_density();
    return r_.F;
  }
  void run(long maxSteps) {
    start();
    check(cdft_ddft_step(dft_->context(), (int)maxSteps, &r_), dft_->context());
    dft_->pull_density();
  }
  double get_time() const { return r_.time; }
  double getTimeStep() const { return r_.dt > 0 ? r_.dt : dt_; }
  double get_convergence_monitor() const { return r_.rhs_max; }
  DFT* dft() const { return dft_; }  // the system whose dynamical matrix g.H the spectral drivers take

 private:
  void start() {
    if (!started_) {
      dft_->push();
      check(cdft_ddft_init(dft_->context(), dt_, dt_max_, tol_), dft_->context());
      started_ = true;
    }
  }
  DFT* dft_;
  double dt_, dt_max_ = 1.0, tol_ = 1e-4;
  cdft_ddft_report r_{};
  bool started_ = false;
};

// include/Log_Det.h:21-51 (src/Log_Det.cpp): on the DFT's Hessian or the DDFT matrix.
class Log_Det {
 public:
  Log_Det(DFT& dft, int order, double lam_max, double lam_min, bool verbose = false)
      : dft_(&dft), matrix_(CDFT_MATRIX_HESSIAN), order_(order), lam_max_(lam_max), lam_min_(lam_min) { (void)verbose; }
  Log_Det(DFT& dft, const DDFT&, int order, double lam_max, double lam_min, bool verbose = false)
      : dft_(&dft), matrix_(CDFT_MATRIX_DDFT), order_(order), lam_max_(lam_max), lam_min_(lam_min) { (void)verbose; }
  double calculate_log_det(long seed, int num_samples, bool has_zero_eigenvalue, double& variance) {
    dft_->push();
    double v = 0;
    check(cdft_log_det(dft_->context(), matrix_, order_, lam_max_, lam_min_, seed, num_samples, has_zero_eigenvalue ? 1 : 0, &v, &variance),
          dft_->context());
    return v;
  }

 private:
  DFT* dft_;
  int matrix_, order_;
  double lam_max_, lam_min_;
};

// include/Eigenvalues.h:16-57 (src/Eigenvalues.cpp) on the DFT's Hessian.
class Eigenvalues {
 public:
  explicit Eigenvalues(DFT& dft, bool verbose = false) : dft_(&dft) { (void)verbose; }
  void set_scale(double d) { scale_ = d; }
  void set_tolerence(double d) { tol_ = d; }
  void set_change_sign(bool b) { change_sign_ = b; }
  void set_vshift(const std::vector<double>& v) { vshift_ = v; }
  void set_eigen_vec_(const std::vector<double>& v) { eigen_vec_ = v; }
  double get_scale() const { return scale_; }
  double get_tolerence() const { return tol_; }
  bool get_change_sign() const { return change_sign_; }
  double get_eigenvalue() const { return eigen_val_; }
  int get_num_eval() const { return (int)rep_.matvecs; }
  int get_return_code() const { return rep_.converged; }
  const std::vector<double>& get_eigen_vec() const { return eigen_vec_; }
  void calculate_eigenvector(long max_matvecs = 1000000) {
    dft_->push();
    cdft_ctx* c = dft_->context();
    std::vector<double> out(dft_->getSpecies(0)->getDensity().Ntot());
    const double* guess = eigen_vec_.size() == out.size() ? eigen_vec_.data() : nullptr;
    check(cdft_eigenvalue(c, scale_, tol_, change_sign_ ? 1 : 0, vshift_.size() == out.size() ? vshift_.data() : nullptr, guess, max_matvecs,
                          &eigen_val_, out.data(), 0, &rep_),
          c);
    eigen_vec_.swap(out);
  }
  void clear() { eigen_vec_.clear(); }

 private:
  DFT* dft_;
  double scale_ = 1e6, tol_ = 1e-6, eigen_val_ = 0;
  bool change_sign_ = false;
  std::vector<double> vshift_, eigen_vec_;
  cdft_eigen_report rep_{};
};

// include/Arnoldi.h:19-84 (src/Arnoldi.cpp) on the DFT's Hessian.
class Arnoldi {
 public:
  // Arnoldi(const Dynamical_Matrix&): the DFT's Hessian, or a DDFT's dynamical matrix g.H
  explicit Arnoldi(DFT& dft, bool verbose = false) : dft_(&dft), matrix_(CDFT_MATRIX_HESSIAN) { (void)verbose; }
  explicit Arnoldi(DDFT& ddft, bool verbose = false) : dft_(ddft.dft()), matrix_(CDFT_MATRIX_DDFT) { (void)verbose; }
  void set_initial_guess(const std::vector<double>& v) { guess_ = v; }
  void determine_largest_eigenpairs(double shift, int k, int p, bool compute_all_k_largest = true, long maxSteps = 1000000,
                                    double tol = 1e-8) {
    dft_->push();
    cdft_ctx* c = dft_->context();
    const long N = dft_->getSpecies(0)->getDensity().Ntot();
    vals_.assign(k, 0.0);
    vecs_.assign((size_t)k * N, 0.0);
    executed_ = true;
    const int rc = cdft_arnoldi_largest_matrix(c, matrix_, shift, k, p, compute_all_k_largest ? 1 : 0, maxSteps, tol,
                                               guess_.size() == (size_t)N ? guess_.data() : nullptr, vals_.data(), vecs_.data(), 0, &rep_);
    success_ = rc == CDFT_OK;
    check(rc, c);
  }
  bool is_success() const {
    if (!executed_) throw std::runtime_error("Arnoldi: Solver has yet not been executed");
    return success_;
  }
  double get_eigenvalue(int i) const {
    if (!executed_) throw std::runtime_error("Arnoldi: Solver has yet not been executed");
    if (i < 0 || i >= (int)vals_.size()) throw std::runtime_error("Arnoldi: Requesting eigenvalue that has not been computed (index larger than k)");
    return vals_[i];
  }
  std::vector<double> get_eigenvector(int i) const {
    if (!executed_) throw std::runtime_error("Arnoldi: Solver has yet not been executed");
    if (i < 0 || i >= (int)vals_.size()) throw std::runtime_error("Arnoldi: Requesting eigenvector that has not been computed (index larger than k)");
    const size_t N = vecs_.size() / vals_.size();
    return std::vector<double>(vecs_.begin() + (long)(i * N), vecs_.begin() + (long)((i + 1) * N));
  }

 private:
  DFT* dft_;
  int matrix_;
  std::vector<double> guess_, vals_, vecs_;
  cdft_eigen_report rep_{};
  bool executed_ = false, success_ = false;
};

}  // namespace classicaldft_gb300

#endif

// Internal host-side declarations of the GB300 evaluation engine.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>
#include <cuda.h>
#include "cdft_types.h"

namespace cdft {

struct Dims;

// Twiddle tables for one transform length, in both precisions, on the device.
struct FFTTable {
  FFTPlan plan;
  void* d64 = nullptr;  // double2[]
  void* d32 = nullptr;  // float2[]
  ~FFTTable();
};
// Twiddle tables of the mixed-radix plan `radices` (default_radices(n) when
// null; stages in order of execution, product n). nullptr if n has a prime
// factor above 31 or the radices do not multiply to n.
std::shared_ptr<FFTTable> make_fft_table(int n, std::string* err, const std::vector<int>* radices = nullptr);
std::vector<int> default_radices(int n);

// Host-side setup maths (cdft_setup.cpp).
double bh_diameter_lj(double sigma, double eps, double rc, double kT);
void fmt_weights_real(int nx, int ny, int nz, double dx, double hsd, std::vector<double> w[11]);
void qf_kernel_real(int nx, int ny, int nz, double dx, double sigma, double eps, double rc, double kT, std::vector<double>& w_att,
                    double& a_vdw);
double fmt_phi_host(int model, double A, double B, const double fm19[19], double dphi19[19]);
double bulk_muex(int model, double A, double B, double hsd, double rho);
double bulk_fex(int model, double A, double B, double hsd, double rho);
// the AO (polymer) terms of the same, src/FMT.cpp:640-700
double bulk_muex_ao(int model, double A, double B, double hsd, double hsdp, double rhop, double rho);
double bulk_fex_ao(int model, double A, double B, double hsd, double hsdp, double rhop, double rho);

struct EvalTerms {
  double F_id, F_hs, F_mf, F_ext, Omega;
  double sum_rho, sum_vext_rho, sum_dF_rho;
  unsigned status;
};

// Device buffers and launch sequence of one F+dF evaluation in precision T.
template <class T>
class Evaluator {
 public:
  typedef typename Cx<T>::type C;
  Evaluator() {}
  ~Evaluator();
  // w_fmt: 11 real-space weights (host, FP64) or null; w_att: real-space MF kernel or null.
  int init(int nx, int ny, int nz, int model, double hsd, double esA, double esB, const std::vector<double>* w_fmt,
           const std::vector<double>* w_att, FFTTable* tx, FFTTable* ty, FFTTable* tz, cudaStream_t s, std::string* err,
           const double* dev_w = nullptr, const double* dev_watt = nullptr);
  // dev_w / dev_watt (optional): the compact FP64 weight spectra of an FP64 evaluator of the
  // same system (M x Nc and Nc values); when given they are rounded to T on the device in
  // place of w_fmt / w_att (the same values the host path gives: both round one FP64 product).
  const T* weight_spectra() const { return w_; }
  const T* att_spectrum() const { return watt_; }
  // rho (device FP64) -> dF (device FP64), scalar terms (host). Synchronous at the end.
  int eval(const double* rho, const double* vext, double* dF, double dV, double mu, int ideal, EvalTerms* out, cudaStream_t s);
  // Launches the pass sequence without host synchronisation; partial sums land in dev_terms.
  // ev (optional, 10 events) are recorded before pass 0 and after each of the 9 passes.
  // RT: storage type of rho and dF (double, or T for an all-T pipeline).
  // nrm (optional, 2 * final_blocks() doubles): the final row pass also stores
  // per block (sum dF^2, max |dF|) there, the partials k_dF_norms would make.
  // dF_mirror (optional, N values, device-visible, e.g. pinned host memory): the final row
  // pass stores dF there too, so that a caller's host copy needs no separate transfer.
  template <class RT>
  int launch(const RT* rho, const double* vext, RT* dF, double dV, double mu, int ideal, cudaStream_t s, cudaEvent_t* ev = nullptr,
             double* nrm = nullptr, RT* dF_mirror = nullptr);
  int launch(const double* rho, const double* vext, double* dF, double dV, double mu, int ideal, cudaStream_t s,
             cudaEvent_t* ev = nullptr, double* nrm = nullptr, double* dF_mirror = nullptr) {
    return launch<double>(rho, vext, dF, dV, mu, ideal, s, ev, nrm, dF_mirror);
  }
  long final_blocks() const { return grid_blocks_rows(); }
  bool has_mf() const { return mf_; }
  // Hessian-vector products (DFT::matrix_dot_v_intern with the full Hessian):
  // hess_prepare stores the M weighted densities of the state rho0 in real
  // space (allocated on first use); hess_apply then maps v -> H v at that
  // state, rho0 giving the ideal-gas term v/rho0. Asynchronous on s.
  int hess_prepare(const double* rho0, cudaStream_t s);
  bool hess_ready() const { return M_ == 0 || NA_ != nullptr; }
  template <class RT>
  int hess_apply(const RT* v, const double* rho0, RT* out, double dV, cudaStream_t s);
  // Algorithmic bytes each of the 9 passes must move (reads + writes once).
  void pass_bytes(double* bytes) const;
  // FMT_AO_Species (src/FMT_Species.cpp:645-738, src/FMT.cpp:340-421), after init: ideal
  // polymers of diameter hsdp at reservoir density `reservoir`. w_ao: the polymer weights in
  // real space (host), or dev_wao: an FP64 evaluator's compact polymer spectra to round.
  // Every later evaluation adds the AO free energy to F_hs and its force to dF.
  int enable_ao(double hsdp, double reservoir, const std::vector<double>* w_ao, const double* dev_wao, cudaStream_t s,
                std::string* err);
  bool has_ao() const { return ao_; }
  const T* ao_spectra() const { return wao_; }
  bool setup_tma(std::string* err);
  int finish(double dV, double mu, EvalTerms* out, cudaStream_t s);
  // the host side of finish: raw device sums h[8] and status -> terms
  int terms_from(const double* h, unsigned st, double dV, double mu, EvalTerms* out) const;
  // Transforms used by DDFT and tests: real FP64 (device) -> spectrum (device C), and back (x scale).
  void r2c(const double* in, C* out, cudaStream_t s);
  void c2r(const C* in, double* out, T scale, cudaStream_t s);
  C* spectrum_buffer() const { return A_; }
  const T* weights() const { return w_; }
  const T* w_att() const { return watt_; }
  int M() const { return M_; }
  // swap the transform plans (same lengths, another radix ordering)
  void set_tables(FFTTable* tx, FFTTable* ty, FFTTable* tz) {
    tx_ = tx; ty_ = ty; tz_ = tz;
    fixed_plans();
    if (tma_) setup_phi_tma();
  }
  long spectrum_len() const { return Nc_; }  // complex values per spectrum (padded rows)
  int pitch() const { return pz_; }
  bool uses_tma() const { return tma_; }
  double* dev_terms() const { return terms_; }
  unsigned* dev_status() const { return status_; }
  long grid_blocks_rows() const;

 private:
  int nx_ = 0, ny_ = 0, nz_ = 0, nzc_ = 0, pz_ = 0;
  long N_ = 0, Nc_ = 0, rows_ = 0;
  int model_ = -1, M_ = 0;
  double hsd_ = 1, esA_ = 1, esB_ = 0;
  bool mf_ = false;
  FFTTable *tx_ = nullptr, *ty_ = nullptr, *tz_ = nullptr;
  C* A_ = nullptr;    // forward-transformed density (after z, y)
  C* Cf_ = nullptr;   // M weighted-density / derivative spectra
  C* E_ = nullptr;    // back-convolution
  T* w_ = nullptr;    // M compact weight spectra (w~_a / N, the non-zero component)
  T* watt_ = nullptr; // compact mean-field kernel spectrum (w~_att / N)
  double* part_ = nullptr;  // block partial sums
  long part_len_ = 0;
  double* terms_ = nullptr;  // reduced sums: [0] sum Phi, [1] Parseval MF, [2] F_id, [3] sum rho, [4] sum V rho, [5] sum dF rho
  unsigned* status_ = nullptr;
  long phi_blocks_last_ = 0;  // blocks of the last Phi launch (its partial sums)
  T* NA_ = nullptr;  // Hessian: M weighted densities of the state, real space (M x N)
  // AO: polymer weight spectra (M x Nc), the real fields of the AO passes (M x N), their spectra
  // (M x Nc), Psi's spectrum and real field, and the block partials of sum exp(-Psi)
  void ao_block(cudaStream_t s);
  bool ao_ = false;
  double ao_hp_ = 0, ao_res_ = 0;
  T* wao_ = nullptr;
  T* XA_ = nullptr;
  C* S_ = nullptr;
  C* psi_ = nullptr;
  T* psir_ = nullptr;
  double* part_ao_ = nullptr;
  int gao_ = 0, grid_tao_ = 0;
  // row pairs per block of the z-row passes: 8 in FP64 (1024 blocks at 128^3, fewer idle SMs in
  // the last wave than 512 blocks of 16 pairs: r2c + final 0.126 -> 0.108 ms), 16 in FP32
  int rb_rows_ = sizeof(T) == 8 ? 8 : 16, rb_phi_ = 4, tc_ = 16;
  size_t smem_rows_ = 0, smem_phi_ = 0, smem_colx_ = 0, smem_coly_ = 0, smem_xconv_ = 0, smem_xback_ = 0;
  // tensor-copy path (cdft_kernels_tma.cuh)
  bool tma_ = false;
  CUtensorMap mapA_, mapCf_, mapE_, mapW_, mapWatt_, mapYA_, mapYC_, mapYE_;
  // FP64: the weight spectra again as df64 (hi, lo float pairs, 8 bytes like a double) for
  // the x passes on double-float spectra, which then split no weight per tile
  void* wdf_ = nullptr;
  void* wattdf_ = nullptr;
  CUtensorMap mapWdf_, mapWattdf_;
  size_t smem_ty_ = 0, smem_tconv_ = 0, smem_tback_ = 0;
  int grid_ty1_[2] = {0, 0}, grid_tyM_[2] = {0, 0};  // y-pass persistent grids, by df64 spectra or not
  bool tma_phi_ = false;
  // the tensor-copy kernels' compile-time plans (length 128, default radix order) apply to x / y / z
  int fx_ = 0, fy_ = 0, fz_ = 0;  // compile-time plan length per axis (128, 256) or 0
  void fixed_plans();
  // FP64 spectra kept in double-float between passes: every pass of an evaluation and of a
  // Hessian product on the tensor-copy path with compile-time plans on all three axes (not
  // with the AO passes, whose spectra go through the runtime-plan kernels). Each complex
  // value is then a dfc (two float pairs, 16 bytes like a double2) in A_, Cf_ and E_, and no
  // pass splits or joins at its edges.
  bool df_candidate() const;
  bool df_spectra() const { return df_candidate() && tma_phi_; }
  // the plan length of the Phi pass's instance: in FP64 its compile-time instance reads and
  // writes double-float spectra, so it runs only when every pass does
  int phi_nf() const;
  bool setup_phi_tma();
  CUtensorMap mapR_;
  size_t smem_tphi_ = 0;
  int grid_tphi_ = 0, grid_thess_ = 0;
};

}  // namespace cdft

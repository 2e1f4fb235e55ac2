// FP64 CPU oracle for the free-energy-and-derivative path of classicalDFT.
//
// TEST INFRASTRUCTURE ONLY. This is a CPU restatement of the reference's
// arithmetic (each routine cites the reference file:line it follows). Only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and
// only as a checker. The product (classicaldft_gb300) never links or calls it.
//
// Pinning: tests/golden/ holds outputs of the reference's own sources,
// compiled here by `make ref` against stand-ins for FFTW/GSL/Boost/Armadillo
// (oracle/refshim); tests/test_oracle_golden.py checks this oracle against them.
#pragma once
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum orc_model { ORC_NONE = -1, ORC_ROSENFELD = 0, ORC_RSLT = 1, ORC_ESFMT = 2, ORC_WHITEBEAR_I = 3, ORC_WHITEBEAR_II = 4 };

typedef struct {
  int nx, ny, nz;
  double dx;
  int model;          /* orc_model */
  double es_A, es_B;  /* esFMT coefficients (model ORC_ESFMT) */
  double hsd;         /* hard-sphere diameter; <= 0: Barker-Henderson diameter of the LJ at kT */
  int lj;             /* 1: add the QF mean-field interaction of a cut-and-shifted LJ with BH split */
  double lj_sigma, lj_eps, lj_rc, kT;
  double mu;          /* chemical potential (beta mu) */
  double fixed_mass;  /* > 0: fixed-mass ensemble */
} orc_params;

typedef struct orc_ctx orc_ctx;

orc_ctx* orc_create(const orc_params* p);
void orc_destroy(orc_ctx* c);
double orc_hsd(const orc_ctx* c);
double orc_a_vdw(const orc_ctx* c);
void orc_set_mu(orc_ctx* c, double mu);
double orc_get_mu(const orc_ctx* c);
/* real-space FMT weights, 11 arrays of N (eta, s, v0..2, T00,T01,T02,T11,T12,T22) */
void orc_weights(const orc_ctx* c, double* out);
/* real-space mean-field kernel w_att (already / kT), N values */
void orc_w_att(const orc_ctx* c, double* out);
/* one F+dF evaluation: rho (N) is read (and rescaled in place under fixed
   mass), dF (N) written with the x dV convention, terms[6] = Omega, F_id,
   F_hs, F_mf, F_ext, mu. Returns 0, or 1 if eta > 1 somewhere (F not valid). */
int orc_eval(orc_ctx* c, double* rho, double* dF, double* terms);
/* bulk thermodynamics */
double orc_mu_times_beta(const orc_ctx* c, double rho);
double orc_omega_times_beta_over_volume(const orc_ctx* c, double rho);
double orc_fhelmholtz_times_beta_over_volume(const orc_ctx* c, double rho);
/* pointwise Phi and the 19 derivatives for one set of 19 measures */
double orc_phi(int model, double A, double B, const double* fm19, double* dphi19);
/* Barker-Henderson diameter of the cut-and-shifted LJ(sigma=eps=1) */
double orc_bh_diameter(double rc, double kT);

/* FIRE2 (fireMinimizer2) for nsteps from rho; rho overwritten with the final
   density. Per-step records (each nsteps long, may be NULL): F, dt, alpha, vv,
   fmax, resid_true (max|dF|/dV before alias conversion). Returns the number
   of steps taken, or -1 (uphill limit). */
int orc_fire(orc_ctx* c, double* rho, int nsteps, double dt0, double dt_max, double force_limit,
             double* rec_F, double* rec_dt, double* rec_alpha, double* rec_vv, double* rec_fmax, double* rec_resid);
/* DDFT integrating-factor steps. rho overwritten. Records per step: F, time, dt, mass, RHS max. */
int orc_ddft(orc_ctx* c, double* rho, int nsteps, double dt, double dt_max,
             double* rec_F, double* rec_t, double* rec_dt, double* rec_mass, double* rec_rhs);

/* DFT::matrix_dot_v_intern with the full Hessian (src/DFT.cpp:435-488): out =
   (d2Omega/drho drho) . v in the reference's scaling, at the density rho. */
void orc_hessian_dot_v(const orc_ctx* c, const double* rho, const double* v, double* out);
/* DDFT::matrix_dot_v_intern (src/DDFT.cpp:353-361): g_dot_x of the full Hessian times v. */
void orc_ddft_matrix_dot_v(const orc_ctx* c, const double* rho, const double* v, double* out);

/* Log_Det::calculate_log_det (src/Log_Det.cpp:84-166) of the Hessian (dynamic = 0) or
   of -(DDFT matrix) (dynamic = 1) at the density rho; variance (may be NULL) as the
   reference reports it. */
double orc_log_det(const orc_ctx* c, const double* rho, int dynamic, int order, double lam_max, double lam_min, long seed, int num_samples,
                   int has_zero, double* variance);

/* FFT helpers exposed for tests: unnormalised r2c / c2r of an nx*ny*nz grid
   (complex stored interleaved, nx*ny*(nz/2+1) values). */
void orc_r2c(int nx, int ny, int nz, const double* in, double* out_c);
void orc_c2r(int nx, int ny, int nz, const double* in_c, double* out);

/* splitmix64 noise fill, rho_i = rho0 * (1 + amp * (2u - 1)) */
void orc_fill_noise(double* rho, long n, double rho0, double amp, uint64_t seed);

#ifdef __cplusplus
}
#endif

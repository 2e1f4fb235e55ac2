/*
 * classicaldft_gb300 — C ABI of the GB300 (sm_103a) engine for classicalDFT's
 * free-energy-and-derivative path and the FIRE2 / DDFT loops that drive it.
 *
 * One context = one single-species system (a Density on a periodic Lattice,
 * one FMT_Species, an FMT model, optionally one LJ mean-field interaction,
 * a chemical potential or a fixed mass) resident on one GPU. Every entry point
 * returns CDFT_OK (0) or an error code; cdft_last_error() gives the message.
 * Arrays are FP64 in the reference's row-major layout pos = k + Nz*(j + Ny*i)
 * (include/Lattice.h:120-126). dF follows the reference's convention: it holds
 * dOmega/drho_i * dV (include/Species.h:57, src/DFT.cpp:377-425).
 * Host pointers are plain host memory; `on_device` = 1 means a CUDA device
 * pointer on the context's device. A context is not thread-safe; use one per
 * host thread. All work is ordered on the context's stream (cdft_set_stream).
 */
#ifndef CLASSICALDFT_GB300_CDFT_H
#define CLASSICALDFT_GB300_CDFT_H
#ifdef __cplusplus
extern "C" {
#endif

/* Return codes */
#define CDFT_OK 0
#define CDFT_ERR_ETA 1       /* eta > 1 at some site: Eta_Too_Large_Exception (include/FMT.h:649-663, src/FMT.cpp:289) */
#define CDFT_ERR_NONFINITE 2 /* a non-finite free-energy density */
#define CDFT_ERR_TIMEOUT 3   /* a device-side wait or iteration cap ran out */
#define CDFT_ERR_ARG 4       /* bad argument (incommensurate lattice, hsd < dx, unsupported grid length, ...) */
#define CDFT_ERR_CUDA 5      /* CUDA runtime error */
#define CDFT_ERR_UPHILL 6    /* fireMinimizer2: "Cannot stop going uphill" (src/Minimizer.cpp:207) */
#define CDFT_ERR_STATE 7     /* call out of order (e.g. cdft_fire_step before cdft_fire_init) */

/* FMT models (include/FMT.h:139-643) */
#define CDFT_MODEL_NONE (-1) /* ideal gas only (no FMT object) */
#define CDFT_ROSENFELD 0
#define CDFT_RSLT 1
#define CDFT_ESFMT 2 /* esFMT(A, B) */
#define CDFT_WHITEBEAR_I 3
#define CDFT_WHITEBEAR_II 4

/* Arithmetic of the bulk FFT / pointwise passes. Reductions are FP64 always.
 * CDFT_FP64 is the reference's precision: its transforms along 128- and 256-point axes
 * run in double-float (float pairs, 48 significant bits) on the FP32 pipe, and when all
 * three axes have those lengths so do the per-point terms and the spectra between passes;
 * at 128^3 Omega stays within ~1e-14 relative and dF within ~2e-16 absolute of an
 * all-FP64 evaluation (the parity bars are 1e-12 and 1e-10 dV). Transforms along other
 * axis lengths run in FP64. CDFT_FP32 runs the transforms and the pointwise terms in
 * FP32 (Omega ~2.5e-7 relative, dF ~5e-7 of max|dF| from FP64). */
#define CDFT_FP64 0
#define CDFT_FP32 1

typedef struct cdft_ctx cdft_ctx;

typedef struct cdft_params {
  int nx, ny, nz;  /* lattice points: Lattice(dx, L) with N = L/dx (include/Lattice.h:57-85) */
  double dx;       /* lattice spacing (dx = dy = dz) */
  int model;       /* CDFT_* model, or CDFT_MODEL_NONE */
  double es_A, es_B; /* esFMT coefficients (CDFT_ESFMT only) */
  double hsd;      /* FMT_Species hard-sphere diameter; <= 0 with lj: Barker-Henderson diameter at kT */
  int lj;          /* 1: LJ(sigma, eps, rc) with setBH() and Interaction_Interpolation_QF(s, s, &lj, kT) */
  double lj_sigma, lj_eps, lj_rc, kT;
  double mu;         /* Species::setChemPotential (beta mu) */
  double fixed_mass; /* > 0: Species::setFixedMass */
  int precision;     /* CDFT_FP64 or CDFT_FP32 */
  double ao_rp;        /* > 0: FMT_AO_Species (src/FMT_Species.cpp:645-738): ideal polymers of radius ao_rp */
  double ao_reservoir; /*   at reservoir density ao_reservoir (the Asakura-Oosawa model); needs an FMT model */
} cdft_params;

typedef struct cdft_info {
  double hsd, a_vdw, dV, volume;
  long N, Nc;
  int nx, ny, nz;
} cdft_info;

/* Context life cycle. cdft_create builds the weights (FMT_Species::generateWeights,
 * src/FMT_Species.cpp:310-496; Interaction_Base::initialize, src/Interaction.cpp:32-52)
 * and allocates every device buffer of the path; later calls allocate nothing
 * except the first cdft_fire_init / cdft_ddft_init (that loop's state), the first
 * Hessian product (its two vectors and the weighted densities) and the spectral
 * drivers (their Krylov bases and probe buffers, for the duration of the call). */
int cdft_create(const cdft_params* p, cdft_ctx** out);
int cdft_destroy(cdft_ctx* ctx);
const char* cdft_last_error(const cdft_ctx* ctx);
int cdft_set_stream(cdft_ctx* ctx, void* cuda_stream);
int cdft_get_info(const cdft_ctx* ctx, cdft_info* out);
int cdft_set_precision(cdft_ctx* ctx, int precision);

/* Density::set / Species::set_density (include/Density.h:51-54, include/Species.h:45) */
int cdft_set_density(cdft_ctx* ctx, const double* rho, int on_device);
int cdft_get_density(const cdft_ctx* ctx, double* rho, int on_device);
/* Density::vWall_ external field (include/Density.h:116); NULL clears it */
int cdft_set_external_field(cdft_ctx* ctx, const double* v, int on_device);
/* Species::setChemPotential / setFixedMass / getChemPotential (include/Species.h:24-31) */
int cdft_set_chem_potential(cdft_ctx* ctx, double mu);
int cdft_set_fixed_mass(cdft_ctx* ctx, double mass);
int cdft_get_chem_potential(const cdft_ctx* ctx, double* mu);

/* Species::setFixedBackground / setHomogeneousBoundary (include/Species.h:24-25). The
 * boundary is the planes i = 0, j = 0 and k = 0 (Lattice::is_boundary_point,
 * include/Lattice.h:184-196). fixed_background = 1: after each evaluation dF = 0 there
 * (Species::endForceCalculation, src/Species.cpp:78-82), so the minimizers leave those
 * densities where they are; Hessian products take and give zero boundary entries
 * (Dynamical_Matrix::matrix_dot_v1, src/DFT.cpp:441-487, src/DDFT.cpp:330-338); Log_Det
 * zeroes its probes there and counts only the other points (src/Log_Det.cpp:91, 111);
 * Eigenvalues and Arnoldi start from a vector that is zero there; the DDFT step's g . dF
 * is zero there and the boundary densities stay as they are (src/DDFT.cpp:280-281).
 * homogeneous = 1: dF on the boundary is replaced by its mean over the boundary
 * (src/Species.cpp:84-95). A fixed background with a fixed mass makes the next
 * evaluation fail with CDFT_ERR_ARG (the reference throws). Every FIRE2 call (host-stepped,
 * device-resident, batched) and the DDFT step take both modes; Newton-Krylov takes the
 * fixed background (its corrections live on the interior points) but not the homogeneous
 * boundary (cdft_newton_refine returns CDFT_ERR_ARG; cdft_fire_run_device and
 * cdft_fire_run_batch take the FIRE2 policy, mixed = 1, instead of 2 or 3). */
int cdft_set_boundary(cdft_ctx* ctx, int fixed_background, int homogeneous);

/* DFT::calculateFreeEnergyAndDerivatives(onlyFex) (include/DFT.h:77, src/DFT.cpp:360-425);
 * only_fex = 1 leaves out the ideal-gas term, as the reference does.
 * terms (may be NULL) receives 8 values: Omega, F_id, F_hs, F_mf, F_ext (the
 * reference's get_f_* of include/DFT.h:121-124), mu after the call, the
 * convergence monitor max|dF|/dV (Species::get_convergence_monitor,
 * include/Species.h:55) and the number of atoms. dF (may be NULL) receives N
 * values (on_device = 1: a device pointer); a page-locked host dF (cudaHostAlloc,
 * cudaHostRegister) is written by the evaluation's last pass itself, with no copy
 * after it (the first call with a new such buffer re-captures the evaluation).
 * Under fixed mass the context's density is rescaled first, as
 * Species::beginForceCalculation does (src/Species.cpp:64-71).
 * Returns CDFT_ERR_ETA where the reference throws Eta_Too_Large_Exception. */
int cdft_eval(cdft_ctx* ctx, int only_fex, double* terms, double* dF, int on_device);

/* DFT::matrix_dot_v1 with the full Hessian (src/Dynamical_Matrix.cpp;
 * DFT::matrix_dot_v_intern, src/DFT.cpp:435-488): out = H v with H the second
 * derivative of Omega in the reference's scaling (ideal gas dV v/rho,
 * FMT::add_second_derivative src/FMT.cpp:437-567, the mean-field convolution
 * src/Interaction.cpp:119-147), taken at the context's current density (the
 * reference uses the fundamental measures of the last evaluation: call
 * cdft_eval first for the same state). v and out hold N values. For an
 * FMT_AO_Species system this is the reference's product too: its
 * add_second_derivative takes the AO species through the hard-sphere branch, so the
 * AO free energy has no term in it (Newton-Krylov, which needs the Jacobian of the
 * AO force, is therefore not offered for the AO model). */
int cdft_hessian_dot_v(cdft_ctx* ctx, const double* v, double* out, int on_device);
/* DDFT::matrix_dot_v_intern (src/DDFT.cpp:353-361): the DDFT dynamical matrix
 * times v, g . (H v), with DDFT::g_dot_x's forward-difference mobility operator
 * (src/DDFT.cpp:320-351), at the context's current density. */
int cdft_ddft_matrix_dot_v(cdft_ctx* ctx, const double* v, double* out, int on_device);

/* Spectral drivers on those matrices (the reference's consumers of Dynamical_Matrix,
 * include/Dynamical_Matrix.h), at the context's current density. Every vector stays
 * on the device; each product is one Hessian pass in the context's precision. */
#define CDFT_MATRIX_HESSIAN 0 /* DFT: the Hessian of Omega (Dynamical_Matrix::is_dynamic() false) */
#define CDFT_MATRIX_DDFT 1    /* DDFT: g . H (is_dynamic() true; Log_Det expands -g . H) */

/* Log_Det(matrix, order, lam_max, lam_min).calculate_log_det(seed, num_samples,
 * has_zero_eigenvalue, variance) (include/Log_Det.h:21-51, src/Log_Det.cpp:22-166): the
 * stochastic Chebyshev estimate of log det of the matrix whose spectrum lies in
 * [lam_min, lam_max], with the reference's +-1 probe vectors for the same seed
 * (std::mt19937(seed), uniform_int_distribution<>(0, 1), point order; seed <= 0 draws
 * one from std::random_device). variance (may be NULL) receives the reference's spread
 * sqrt|<(v.u)^2> - <v.u>^2|. Periodic lattices: every point is active. */
int cdft_log_det(cdft_ctx* ctx, int matrix, int order, double lam_max, double lam_min, long seed, int num_samples,
                 int has_zero_eigenvalue, double* log_det, double* variance);

typedef struct cdft_eigen_report {
  long matvecs;    /* Hessian products used */
  int restarts;    /* restarts of the Krylov basis */
  int converged;   /* 1 when the stopping rule was met */
  double residual; /* |H y - lambda y| of the (first) returned pair, in the matrix's own units */
} cdft_eigen_report;

/* Eigenvalues(dft).calculate_eigenvector (include/Eigenvalues.h:16-57,
 * src/Eigenvalues.cpp:44-99) with set_scale(scale), set_tolerence(tol),
 * set_change_sign(change_sign), set_vshift(vshift) (NULL: none): the smallest eigenvalue
 * of s (H + vshift vshift^T / 2), s = scale (change_sign = 0) or -scale (1), returned as
 * the reference's get_eigenvalue() does (divided by scale, sign restored; so change_sign
 * gives the largest eigenvalue of H + vshift vshift^T / 2), with its unit eigenvector
 * (eigvec, N values, may be NULL). Stops when |residual| <= tol |lambda| (the reference
 * stops nlopt's L-BFGS at a relative change tol of the Rayleigh quotient), or after
 * about max_matvecs products (checked at restarts; rep->converged = 0 then). guess (N
 * values, may be NULL) is the start vector, as set_eigen_vec_. Hessian only. */
int cdft_eigenvalue(cdft_ctx* ctx, double scale, double tol, int change_sign, const double* vshift, const double* guess,
                    long max_matvecs, double* eigval, double* eigvec, int on_device, cdft_eigen_report* rep);

/* Arnoldi(dft).determine_largest_eigenpairs(shift, k, p, compute_all_k_largest,
 * maxSteps, tol) (include/Arnoldi.h:19-84, src/Arnoldi.cpp:72-283): the k eigenpairs of
 * H + shift of largest magnitude, in that order, from a (k + p)-vector Krylov basis;
 * eigvals (k values) are reported without the shift and eigvecs (k * N values, may be
 * NULL) are unit vectors. A pair has converged when its Ritz estimate is at most
 * tol |lambda| or it is degenerate (within tol) with the largest discarded Ritz value;
 * all_k = 0 asks only for the first. Returns CDFT_ERR_TIMEOUT after max_steps restarts
 * without convergence (the reference throws; the outputs then hold the last estimates).
 * The reference stores the first Ritz value under every index (src/Arnoldi.cpp:210);
 * here eigvals[i] is the i-th pair's own value. Hessian only. */
int cdft_arnoldi_largest(cdft_ctx* ctx, double shift, int k, int p, int all_k, long max_steps, double tol, const double* guess,
                         double* eigvals, double* eigvecs, int on_device, cdft_eigen_report* rep);
/* The same driver on either matrix of the path (Arnoldi takes any Dynamical_Matrix,
 * include/Arnoldi.h:21; DDFT is one, include/Minimizer.h:189): CDFT_MATRIX_HESSIAN is
 * cdft_arnoldi_largest; CDFT_MATRIX_DDFT gives the k eigenpairs of the DDFT matrix g.H
 * (cdft_ddft_matrix_dot_v) of largest |lambda + shift|, eigvals without the shift, each
 * eigenvector of unit norm (g.H is not symmetric: they are not orthogonal). Its spectrum
 * is real (g = -C^T C, so g.H shares its non-zero eigenvalues with -C H C^T), plus, on a
 * periodic lattice, the zero eigenvalue of the conserved mass (eigenvector H^-1 1, by
 * conjugate gradients). rep->matvecs counts Hessian products. The homogeneous boundary is
 * rejected (CDFT_ERR_ARG) for the DDFT matrix. */
int cdft_arnoldi_largest_matrix(cdft_ctx* ctx, int matrix, double shift, int k, int p, int all_k, long max_steps, double tol,
                                const double* guess, double* eigvals, double* eigvecs, int on_device, cdft_eigen_report* rep);

/* Times each pass of one evaluation in the current precision with CUDA events
 * on the context's stream (no reference counterpart; used by the benchmark's
 * roofline). reps evaluations are timed; ms receives the mean time per pass
 * (CDFT_NPASS values, in the order of the pass list in
 * classicaldft_gb300/csrc/cdft_kernels.cuh) and bytes the algorithmic bytes each
 * pass must move. Returns the number of passes through *npass. */
#define CDFT_NPASS 9
int cdft_time_passes(cdft_ctx* ctx, int reps, double* ms, double* bytes, int* npass);

/* Bulk thermodynamics of the uniform fluid: out = {DFT::mu_times_beta,
 * omega_times_beta_over_volume, fhelmholtz_times_beta_over_volume} (src/DFT.cpp:58-115). */
int cdft_bulk(const cdft_ctx* ctx, double rho, double* out3);

/* Bulk liquid-vapour coexistence of the context's functional:
 * DFT::findSpinodal + DFT::findCoex (src/DFT_Coex.cpp:53-196). Searches densities
 * up to xmax with step dx and tolerance tol; out = {x_vap, x_liq, mu_coex
 * (= mu_times_beta(x_vap)), spinodal x1, spinodal x2}. CDFT_ERR_ARG when no
 * coexistence is bracketed (e.g. above the critical temperature). */
int cdft_find_coex(const cdft_ctx* ctx, double xmax, double dx, double tol, double* out5);

/* Potential1::getHSD(kT) of LJ(sigma, eps, rc) with setBH() (include/Potential1.h:73-83):
 * the Barker-Henderson diameter int_0^{r0} (1 - exp(-V(r)/kT)) dr, integrated to 1e-15. */
int cdft_bh_diameter(double sigma, double eps, double rc, double kT, double* out);

/* Density files, host only (no context or GPU needed); rho is the row-major
 * pos = k + Nz*(j + Ny*i) density of n = Nx*Ny*Nz values.
 * Density::writeDensity (src/Density.cpp:227-231): Armadillo's arma_binary
 * column vector ("ARMA_MAT_BIN_FN008\n", "<n> 1\n", n native doubles).
 * Density::readDensity (src/Density.cpp:233-244): reads that format; CDFT_ERR_ARG
 * when the file cannot be opened (the reference throws) or does not hold n values.
 * Density::write_VTK_File (src/Density.cpp:197-225): the legacy-VTK ASCII file of the
 * reference's VisIt writer (".vtk" appended when missing). */
int cdft_density_write(const char* path, const double* rho, long n);
int cdft_density_read(const char* path, double* rho, long n);
int cdft_density_write_vtk(const char* path, const double* rho, int nx, int ny, int nz);

/* FMT_Species::generateWeights on the host (src/FMT_Species.cpp:310-496), no
 * context or GPU needed: the 11 real-space weight arrays (11*nx*ny*nz values) of a
 * sphere of diameter hsd on an nx*ny*nz lattice of spacing dx. */
int cdft_fmt_weights(int nx, int ny, int nz, double dx, double hsd, double* w11);

/* Real-space weights for inspection: w11 (11*N: eta, s, v0..2, T00, T01, T02,
 * T11, T12, T22 as FMT_Species holds them) and w_att (N, already / kT); either may be NULL. */
int cdft_get_weights(const cdft_ctx* ctx, double* w11, double* w_att);

/* fireMinimizer2 (include/Minimizer.h:80-182, src/Minimizer.cpp:117-327). */
typedef struct cdft_fire_params {
  double dt, dt_max, dt_min;        /* setTimeStep / setTimeStepMax; defaults 1e-3, 1e-2, 0 */
  double alpha_start, f_alf;        /* setAlphaStart / setAlphaFac; defaults 0.1, 0.99 */
  double f_dec, f_inc;              /* 0.5, 1.1 */
  double force_limit;               /* Minimizer::setForceTerminationCriterion on |vv/V|; default 0.1 */
  int n_delay, n_p_negative_max;    /* 5, 20 */
  int initial_delay;                /* 1 */
} cdft_fire_params;

typedef struct cdft_fire_report {
  long steps;        /* steps taken by this call */
  long total_steps;  /* since cdft_fire_init */
  long calls;        /* F+dF evaluations since cdft_fire_init */
  double F;          /* Omega at the current state (fireMinimizer2::F_) */
  double dt, dt_max, alpha;
  double vv;         /* the energy-rate monitor vv_; Minimizer stops when |vv/V| < force_limit */
  double fmax;       /* max |dF/dx|/dV in alias coordinates (fmax_) */
  double resid;      /* max |dOmega/drho| = max|dF|/dV before alias conversion, last accepted evaluation */
  int backtracks;    /* eta > 1 backtracks seen by this call */
  int stop;          /* 0 max steps, 1 force limit, 2 residual target */
  long steps_fp32;   /* steps of this call taken in the FP32 bulk phase (cdft_fire_run_device, mixed) */
  long newton, cg_iters; /* Newton-Krylov refinement of cdft_fire_run_device (mixed = 2): corrections, CG iterations */
} cdft_fire_report;

/* fireMinimizer2 serialisation (include/Minimizer.h:145-180, Boost archives there): the
 * whole FIRE2 state (density, alias coordinates x, velocities v, parameters, dt, alpha,
 * counters) to a file of raw native doubles behind a small header, and back. After
 * cdft_fire_load (no cdft_fire_init needed; the file must come from the same lattice) the
 * next steps continue the saved run, the state's dF recomputed by one evaluation.
 * CDFT_ERR_ARG when the file cannot be opened or does not fit the context. */
int cdft_fire_save(cdft_ctx* ctx, const char* path);
int cdft_fire_load(cdft_ctx* ctx, const char* path);

int cdft_fire_default_params(cdft_fire_params* p);
/* fireMinimizer2::fireMinimizer2: x = alias(rho), one evaluation, v = 0. */
int cdft_fire_init(cdft_ctx* ctx, const cdft_fire_params* p);
/* nsteps calls of fireMinimizer2::step(). */
int cdft_fire_step(cdft_ctx* ctx, int nsteps, cdft_fire_report* rep);
/* Minimizer::run / resume loop: steps until |vv/V| < force_limit or max_steps (> 0). */
int cdft_fire_run(cdft_ctx* ctx, long max_steps, cdft_fire_report* rep);
/* The same FIRE2 steps, stopping when max|dOmega/drho| <= resid_tol (the
 * residual the reference's Species::get_convergence_monitor reports) or max_steps. */
int cdft_fire_run_to_residual(cdft_ctx* ctx, double resid_tol, long max_steps, cdft_fire_report* rep);

/* The same FIRE2 steps, run device-resident: the step's scalar logic runs in
 * one-thread control kernels and one whole step (vector passes, evaluation,
 * Species constraints, alias conversion) is captured once as a CUDA graph, so
 * no host round trip sits inside a step; the host reads the state every 16
 * steps. Stops when max|dOmega/drho| <= resid_tol (taken from an FP64
 * evaluation), on the uphill limit, or after max_steps (> 0).
 * mixed = 0: FP64 throughout. mixed = 1: an FP32 bulk phase (vectors and
 * evaluations in FP32) until its residual drops below switch_tol or goes 96
 * steps without a 2% improvement (its noise floor), then one FP64 evaluation
 * at the same state and FP64 refinement. mixed = 2: the same FP32 bulk phase,
 * then Newton-Krylov refinement (cdft_newton_refine: FP32 Hessian products,
 * FP64 residuals), falling back to FP64 FIRE2 steps if it stalls. mixed = 3:
 * Newton-Krylov from the current state (up to 40 corrections; if that stalls,
 * again from the same start with FP64 residuals throughout, then with CG to
 * 1e-3 throughout, up to 80 corrections each), falling back to the mixed = 2
 * path if all stall. */
int cdft_fire_run_device(cdft_ctx* ctx, double resid_tol, double switch_tol, long max_steps, int mixed, cdft_fire_report* rep);

/* cdft_fire_run_device on n independent contexts at once (state points of a
 * parameter sweep, grids of different sizes). No counterpart in the reference,
 * which solves one system per process. Each context's steps run on its own
 * stream; one host thread queues a context's next 16 steps as soon as its
 * previous ones have finished, so systems too small to fill the GPU overlap.
 * mixed is cdft_fire_run_device's (0 to 3; with 2 a context's Newton-Krylov
 * refinement runs on its own stream while the others' steps continue; with 3
 * the contexts are spread over host threads, 8 unless the environment variable
 * CDFT_BATCH_THREADS sets 1 to 64, each driving its contexts' Newton iterations on
 * their own streams).
 * Every context must have had cdft_fire_init and must appear once. reps[i] and
 * rcs[i] (either array may be NULL) receive each context's report and status;
 * the return value is the first non-zero status, or CDFT_OK. */
int cdft_fire_run_batch(cdft_ctx* const* ctx, int n, double resid_tol, double switch_tol, long max_steps, int mixed,
                        cdft_fire_report* reps, int* rcs);

/* FFT-plan autotuner (no counterpart in the reference, which uses FFTW's
 * planner). Times `reps` evaluations in the context's current precision for
 * each candidate radix ordering of the z, then x, then y transforms, keeps
 * the fastest, and remembers it for the grid, model and precision: later
 * cdft_create calls with the same shape use the tuned plans. Overwrites the
 * last evaluation's outputs (dF); the density and FIRE/DDFT state are kept.
 * radices_out (3 x 8 ints, zero-padded, may be NULL) receives the x, y, z
 * orderings; ms_out (2 doubles, may be NULL) the default and tuned ms per eval. */
int cdft_autotune(cdft_ctx* ctx, int reps, int* radices_out, double* ms_out);
/* The context's current x, y, z radix orderings (3 x 8 ints, zero-padded). */
int cdft_get_radices(const cdft_ctx* ctx, int* radices_out);
/* The orderings the autotuner tries for a transform length n (host only, no
 * GPU): count receives the number of plans; out (max_plans x 8 ints) the first ones. */
int cdft_radix_candidates(int n, int* out, int max_plans, int* count);
/* Measurement aid, no reference counterpart: the current device's sustained FP64
 * FMA rate in TFLOP/s (independent FMA chains on every SM, best of five timed
 * launches on `stream`), the ceiling of an FP64-bound pass. Allocates 8 bytes. */
int cdft_fp64_fma_rate(double* tflops, void* stream);
/* The same for FP32 FMAs: the ceiling of a pass bound by the FP32 pipe (the FP64
 * passes' double-float arithmetic runs there). Allocates 4 bytes. */
int cdft_fp32_fma_rate(double* tflops, void* stream);

/* Newton-Krylov refinement of a minimum (no counterpart in the reference):
 * Newton corrections H d = -dF solved by preconditioned conjugate gradients
 * (at most max_cg iterations, to a relative residual cg_rtol) with FP32
 * Hessian-vector products, each step accepted only when the FP64 residual
 * max|dOmega/drho| decreases (halving the step up to 6 times). Fixed mass is
 * kept exactly (corrections sum to zero). Stops at resid_tol or after
 * max_newton corrections. The FIRE2 state, if any, is re-derived from the
 * refined density. */
typedef struct cdft_newton_report {
  long newton;    /* Newton corrections taken */
  long cg_iters;  /* conjugate-gradient iterations (FP32 Hessian products) */
  long evals;     /* FP64 evaluations */
  double F;       /* Omega at the final state */
  double resid;   /* max|dOmega/drho| there (FP64) */
  int stop;       /* 2 residual reached, 3 no decrease along a correction, 0 max_newton */
} cdft_newton_report;
int cdft_newton_refine(cdft_ctx* ctx, double resid_tol, int max_newton, int max_cg, double cg_rtol, cdft_newton_report* rep);
/* The same with every parameter explicit. eta_max > 0 makes the CG tolerance
 * of a correction max(cg_rtol, min(eta_max, resid)) (loose while the residual is
 * large); 0 keeps cg_rtol. Residuals above fp32_above come from FP32
 * evaluations (0: FP64 throughout). cdft_newton_refine uses eta_max = 0.1,
 * fp32_above = 1e-4, host_cg = 0. */
typedef struct cdft_newton_params {
  int max_newton, max_cg;
  double cg_rtol, eta_max, fp32_above;
  int host_cg; /* 1: drive the CG iterations from the host instead of the device graph */
} cdft_newton_params;
int cdft_newton_refine_ex(cdft_ctx* ctx, double resid_tol, const cdft_newton_params* p, cdft_newton_report* rep);

/* BF16 tensor-core GEMM (tcgen05, FP32 accumulation in tensor memory) for the
 * neural-operator warm start; no counterpart in the reference.
 * Y = act(X . W + bias + add) with X (M x K) and W (K x N) BF16 row-major,
 * bias (N), add (M x N), Y and the optional pre-activation Z (M x N) FP32; all
 * device pointers, X 16-byte aligned; bias, add and Z may be NULL; act 0 none,
 * 1 GELU. K in {16, 32, 48, 64}, N in {32, 64, 128}. A device wait that runs
 * out sets bits in *status_dev (a device unsigned); asynchronous on stream. */
int cdft_tc_gemm_bf16(const void* X, const void* W, const float* bias, const float* add, float* Y, float* Z, long M, int K, int N,
                      int act, void* status_dev, void* stream);

/* DDFT integrating-factor dynamics, single species, periodic (include/Minimizer.h:189-266, src/DDFT.cpp:42-351). */
typedef struct cdft_ddft_report {
  long steps;
  double F;        /* Omega after the last step */
  double time;     /* DDFT::get_time */
  double dt;       /* current time step */
  double mass;     /* sum rho dV (compensated FP64) */
  double rhs_max;  /* DDFT::get_convergence_monitor (RHS_max_) */
  int restarts;    /* time-step reductions in this call */
} cdft_ddft_report;

/* DDFT::DDFT then setTimeStep(dt), set_max_time_step(dt_max), set_tolerence_fixed_point(tol). */
int cdft_ddft_init(cdft_ctx* ctx, double dt, double dt_max, double tol_fixed_point);
/* nsteps calls of DDFT::step(). In CDFT_FP32 mode every propagated density is
 * shifted uniformly (in FP64) back to the mass sum(rho) dV the run started
 * with, which the FP32 transforms keep only to ~1e-7 per step; CDFT_FP64 mode is
 * the reference's arithmetic unchanged. */
int cdft_ddft_step(cdft_ctx* ctx, int nsteps, cdft_ddft_report* rep);
/* CDFT_FP32 mode only: on != 0 (the default) keeps the mass restore described
 * above; 0 leaves each propagated density as the FP32 transforms return it, so
 * the run shows the propagator's own FP32 mass drift. No reference counterpart
 * (the reference has no FP32 mode). */
int cdft_ddft_set_mass_restore(cdft_ctx* ctx, int on);
/* CDFT_FP32 mode: the largest relative deviation |sum rho - sum rho_0| / sum rho_0
 * of a propagated density from the run's starting mass, measured before any
 * restore, over every propagation since cdft_ddft_init (0 in CDFT_FP64 mode). */
int cdft_ddft_mass_deviation(cdft_ctx* ctx, double* max_rel);

/* Number of atoms, sum(rho) * dV with FP64 compensated summation, of a density
 * that is already on the device (rho: n doubles, a device pointer), written to
 * *out (host). Allocates nothing: for callers that cannot call cudaMalloc, such
 * as an application that hands this library only device memory from its own
 * pool (a cudaMalloc would draw memory outside that pool's budget and can
 * synchronise the whole device under the application's other streams). No
 * counterpart in the reference. Its scratch is a 64 KiB file-scope device array
 * that every GPU loading this library holds until exit; n above 2^25
 * (33,554,432) points is rejected with CDFT_ERR_ARG. The first call on a device
 * resolves the array's address there with cudaGetSymbolAddress; it is resolved
 * again if the device's context has been replaced (cudaDeviceReset). Calls share the array: calls that overlap
 * on the GPU race and must be serialised by the caller. The work runs on
 * `stream` (NULL: the legacy default stream), which is synchronised before
 * returning; the call reads and clears the runtime's last-error state. */
int cdft_number_of_atoms_noalloc(const double* rho, long n, double dV, void* stream, double* out);

#ifdef __cplusplus
}
#endif
#endif

"""classicaldft_gb300: GB300-native free-energy-and-derivative engine for
classical DFT (FMT hard spheres + mean-field attraction), with FIRE2 and
integrating-factor DDFT drivers, behind the C ABI in include/cdft.h.

Two layers:
  * `Context` — a thin ctypes binding of the C ABI (one system on one GPU);
  * reference-shaped classes (`Density`, `FMT_Species`, `WhiteBearI`, `RSLT`,
    `esFMT`, `Rosenfeld`, `WhiteBearII`, `LJ`, `Interaction_Interpolation_QF`,
    `DFT`, `fireMinimizer2`, `DDFT`) with the reference's method names
    (include/DFT.h, include/Species.h, include/FMT.h, include/Interaction.h,
    include/Minimizer.h), so code written against the reference ports over.

The compute path is the CUDA library libcdft.so built in-tree by
classicaldft_gb300/build.py; importing the compute API raises if it is absent.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcdft.so")

OK, ERR_ETA, ERR_NONFINITE, ERR_TIMEOUT, ERR_ARG, ERR_CUDA, ERR_UPHILL, ERR_STATE = range(8)
MODEL_NONE, ROSENFELD, RSLT_MODEL, ESFMT, WHITEBEAR_I, WHITEBEAR_II = -1, 0, 1, 2, 3, 4
FP64, FP32 = 0, 1
MATRIX_HESSIAN, MATRIX_DDFT = 0, 1

C_FUNCTIONS = [
    "cdft_create", "cdft_destroy", "cdft_last_error", "cdft_set_stream", "cdft_get_info", "cdft_set_precision",
    "cdft_set_density", "cdft_get_density", "cdft_set_external_field", "cdft_set_chem_potential",
    "cdft_set_fixed_mass", "cdft_get_chem_potential", "cdft_eval", "cdft_bulk", "cdft_bh_diameter",
    "cdft_get_weights", "cdft_fire_default_params", "cdft_fire_init", "cdft_fire_step", "cdft_fire_run",
    "cdft_fire_run_to_residual", "cdft_ddft_init", "cdft_ddft_step", "cdft_time_passes", "cdft_fmt_weights", "cdft_number_of_atoms_noalloc", "cdft_fire_run_device", "cdft_find_coex",
    "cdft_fire_run_batch", "cdft_autotune", "cdft_get_radices", "cdft_radix_candidates", "cdft_hessian_dot_v",
    "cdft_newton_refine", "cdft_tc_gemm_bf16", "cdft_newton_refine_ex", "cdft_ddft_matrix_dot_v",
    "cdft_density_write", "cdft_density_read", "cdft_density_write_vtk", "cdft_log_det", "cdft_eigenvalue",
    "cdft_arnoldi_largest", "cdft_set_boundary", "cdft_ddft_set_mass_restore", "cdft_ddft_mass_deviation",
    "cdft_fp64_fma_rate", "cdft_fp32_fma_rate", "cdft_arnoldi_largest_matrix", "cdft_fire_save", "cdft_fire_load",
]
PASS_NAMES = ("rows_r2c", "cols_y_fwd(rho)", "xconv", "cols_y_inv(n_a)", "phi_rows", "cols_y_fwd(dPhi_a)", "xbackconv",
              "cols_y_inv(E)", "final_rows")


class CDFTError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cdft error %d: %s" % (code, msg))
        self.code = code


class Eta_Too_Large_Exception(CDFTError):
    """eta > 1 somewhere on the lattice (the reference's Eta_Too_Large_Exception)."""


class Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("dx", ctypes.c_double),
                ("model", ctypes.c_int), ("es_A", ctypes.c_double), ("es_B", ctypes.c_double),
                ("hsd", ctypes.c_double), ("lj", ctypes.c_int), ("lj_sigma", ctypes.c_double),
                ("lj_eps", ctypes.c_double), ("lj_rc", ctypes.c_double), ("kT", ctypes.c_double),
                ("mu", ctypes.c_double), ("fixed_mass", ctypes.c_double), ("precision", ctypes.c_int),
                ("ao_rp", ctypes.c_double), ("ao_reservoir", ctypes.c_double)]


class Info(ctypes.Structure):
    _fields_ = [("hsd", ctypes.c_double), ("a_vdw", ctypes.c_double), ("dV", ctypes.c_double),
                ("volume", ctypes.c_double), ("N", ctypes.c_long), ("Nc", ctypes.c_long),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int)]


class FireParams(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("dt_max", ctypes.c_double), ("dt_min", ctypes.c_double),
                ("alpha_start", ctypes.c_double), ("f_alf", ctypes.c_double), ("f_dec", ctypes.c_double),
                ("f_inc", ctypes.c_double), ("force_limit", ctypes.c_double), ("n_delay", ctypes.c_int),
                ("n_p_negative_max", ctypes.c_int), ("initial_delay", ctypes.c_int)]


class FireReport(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_long), ("total_steps", ctypes.c_long), ("calls", ctypes.c_long),
                ("F", ctypes.c_double), ("dt", ctypes.c_double), ("dt_max", ctypes.c_double),
                ("alpha", ctypes.c_double), ("vv", ctypes.c_double), ("fmax", ctypes.c_double),
                ("resid", ctypes.c_double), ("backtracks", ctypes.c_int), ("stop", ctypes.c_int),
                ("steps_fp32", ctypes.c_long), ("newton", ctypes.c_long), ("cg_iters", ctypes.c_long)]


class NewtonParams(ctypes.Structure):
    _fields_ = [("max_newton", ctypes.c_int), ("max_cg", ctypes.c_int), ("cg_rtol", ctypes.c_double),
                ("eta_max", ctypes.c_double), ("fp32_above", ctypes.c_double), ("host_cg", ctypes.c_int)]


class NewtonReport(ctypes.Structure):
    _fields_ = [("newton", ctypes.c_long), ("cg_iters", ctypes.c_long), ("evals", ctypes.c_long),
                ("F", ctypes.c_double), ("resid", ctypes.c_double), ("stop", ctypes.c_int)]


class DdftReport(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_long), ("F", ctypes.c_double), ("time", ctypes.c_double),
                ("dt", ctypes.c_double), ("mass", ctypes.c_double), ("rhs_max", ctypes.c_double),
                ("restarts", ctypes.c_int)]


class EigenReport(ctypes.Structure):
    _fields_ = [("matvecs", ctypes.c_long), ("restarts", ctypes.c_int), ("converged", ctypes.c_int),
                ("residual", ctypes.c_double)]


_lib = None


def lib():
    """Loads libcdft.so; raises if the CUDA library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("classicaldft_gb300: %s is missing; run classicaldft_gb300/build.py "
                              "(there is no CPU fallback)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P, d, i, vp = ctypes.POINTER, ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        dp = P(d)
        sig = {
            "cdft_create": ([P(Params), P(vp)], i), "cdft_destroy": ([vp], i), "cdft_last_error": ([vp], ctypes.c_char_p),
            "cdft_set_stream": ([vp, vp], i), "cdft_get_info": ([vp, P(Info)], i), "cdft_set_precision": ([vp, i], i),
            "cdft_set_density": ([vp, vp, i], i), "cdft_get_density": ([vp, vp, i], i),
            "cdft_set_external_field": ([vp, vp, i], i), "cdft_set_chem_potential": ([vp, d], i),
            "cdft_set_fixed_mass": ([vp, d], i), "cdft_get_chem_potential": ([vp, dp], i),
            "cdft_eval": ([vp, i, dp, vp, i], i), "cdft_bulk": ([vp, d, dp], i),
            "cdft_bh_diameter": ([d, d, d, d, dp], i), "cdft_get_weights": ([vp, dp, dp], i),
            "cdft_fire_default_params": ([P(FireParams)], i), "cdft_fire_init": ([vp, P(FireParams)], i),
            "cdft_fire_step": ([vp, i, P(FireReport)], i), "cdft_fire_run": ([vp, ctypes.c_long, P(FireReport)], i),
            "cdft_fire_run_to_residual": ([vp, d, ctypes.c_long, P(FireReport)], i),
            "cdft_ddft_init": ([vp, d, d, d], i), "cdft_ddft_step": ([vp, i, P(DdftReport)], i),
            "cdft_ddft_set_mass_restore": ([vp, i], i), "cdft_ddft_mass_deviation": ([vp, dp], i),
            "cdft_fp64_fma_rate": ([dp, vp], i),
            "cdft_fp32_fma_rate": ([dp, vp], i),
            "cdft_fire_save": ([vp, ctypes.c_char_p], i), "cdft_fire_load": ([vp, ctypes.c_char_p], i),
            "cdft_time_passes": ([vp, i, dp, dp, P(i)], i),
            "cdft_fmt_weights": ([i, i, i, d, d, dp], i),
            "cdft_number_of_atoms_noalloc": ([vp, ctypes.c_long, d, vp, dp], i),
            "cdft_fire_run_device": ([vp, d, d, ctypes.c_long, i, P(FireReport)], i),
            "cdft_find_coex": ([vp, d, d, d, dp], i),
            "cdft_fire_run_batch": ([P(vp), i, d, d, ctypes.c_long, i, P(FireReport), P(i)], i),
            "cdft_autotune": ([vp, i, P(i), dp], i),
            "cdft_hessian_dot_v": ([vp, vp, vp, i], i),
            "cdft_ddft_matrix_dot_v": ([vp, vp, vp, i], i),
            "cdft_newton_refine": ([vp, d, i, i, d, P(NewtonReport)], i),
            "cdft_tc_gemm_bf16": ([vp, vp, vp, vp, vp, vp, ctypes.c_long, i, i, i, vp, vp], i),
            "cdft_newton_refine_ex": ([vp, d, P(NewtonParams), P(NewtonReport)], i),
            "cdft_get_radices": ([vp, P(i)], i),
            "cdft_radix_candidates": ([i, P(i), i, P(i)], i),
            "cdft_density_write": ([ctypes.c_char_p, dp, ctypes.c_long], i),
            "cdft_density_read": ([ctypes.c_char_p, dp, ctypes.c_long], i),
            "cdft_density_write_vtk": ([ctypes.c_char_p, dp, i, i, i], i),
            "cdft_set_boundary": ([vp, i, i], i),
            "cdft_log_det": ([vp, i, i, d, d, ctypes.c_long, i, i, dp, dp], i),
            "cdft_eigenvalue": ([vp, d, d, i, vp, vp, ctypes.c_long, dp, vp, i, P(EigenReport)], i),
            "cdft_arnoldi_largest": ([vp, d, i, i, i, ctypes.c_long, d, vp, dp, vp, i, P(EigenReport)], i),
            "cdft_arnoldi_largest_matrix": ([vp, i, d, i, i, i, ctypes.c_long, d, vp, dp, vp, i, P(EigenReport)], i),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def bh_diameter(sigma, eps, rc, kT):
    out = ctypes.c_double()
    rc_ = lib().cdft_bh_diameter(sigma, eps, rc, kT, ctypes.byref(out))
    if rc_:
        raise CDFTError(rc_, "bad arguments")
    return out.value


def fmt_weights(shape, dx, hsd):
    """FMT_Species::generateWeights on the host: the 11 real-space weight arrays."""
    w = np.zeros((11,) + tuple(shape))
    rc_ = lib().cdft_fmt_weights(shape[0], shape[1], shape[2], dx, hsd, _dptr(w))
    if rc_:
        raise CDFTError(rc_, "bad arguments (hsd < dx?)")
    return w


def write_density(path, rho):
    """Density::writeDensity: the density as an Armadillo arma_binary column vector."""
    a = np.ascontiguousarray(rho, dtype=np.float64)
    code = lib().cdft_density_write(os.fsencode(path), _dptr(a), a.size)
    if code:
        raise CDFTError(code, "could not write %s" % path)


def read_density(path, shape):
    """Density::readDensity: a density written by write_density (or the reference), as an array of `shape`."""
    a = np.empty(tuple(shape))
    code = lib().cdft_density_read(os.fsencode(path), _dptr(a), a.size)
    if code:
        raise CDFTError(code, "could not read %d values from %s" % (a.size, path))
    return a


def write_vtk(path, rho):
    """Density::write_VTK_File: the reference's legacy-VTK ASCII file of a (nx, ny, nz) density."""
    a = np.ascontiguousarray(rho, dtype=np.float64)
    if a.ndim != 3:
        raise ValueError("rho must be a 3D array")
    code = lib().cdft_density_write_vtk(os.fsencode(path), _dptr(a), *a.shape)
    if code:
        raise CDFTError(code, "could not write %s" % path)


TERM_NAMES = ("Omega", "F_id", "F_hs", "F_mf", "F_ext", "mu", "resid", "N")


class Context:
    """One system resident on the current CUDA device (the C ABI's cdft_ctx)."""

    def __init__(self, shape, dx, model=WHITEBEAR_I, hsd=1.0, lj=False, kT=1.0, rc=3.0, sigma=1.0, eps=1.0,
                 mu=0.0, fixed_mass=-1.0, precision=FP64, es_A=1.0, es_B=0.0, ao_rp=0.0, ao_reservoir=0.0):
        """ao_rp > 0: the species is an FMT_AO_Species, colloids with ideal polymers of radius
        ao_rp at reservoir density ao_reservoir (src/FMT_Species.cpp:645-738)."""
        if isinstance(shape, int):
            shape = (shape, shape, shape)
        self.shape = tuple(int(s) for s in shape)
        p = Params(self.shape[0], self.shape[1], self.shape[2], dx, model, es_A, es_B,
                   hsd if hsd is not None else -1.0, int(bool(lj)), sigma, eps, rc, kT, mu, fixed_mass, precision,
                   ao_rp, ao_reservoir)
        h = ctypes.c_void_p()
        code = lib().cdft_create(ctypes.byref(p), ctypes.byref(h))
        if code:
            raise CDFTError(code, "cdft_create failed")
        self._h = h
        info = Info()
        lib().cdft_get_info(self._h, ctypes.byref(info))
        self.info = info
        self.N = int(info.N)

    def close(self):
        if getattr(self, "_h", None):
            lib().cdft_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, code):
        if code == OK:
            return
        msg = lib().cdft_last_error(self._h).decode()
        if code == ERR_ETA:
            raise Eta_Too_Large_Exception(code, msg)
        raise CDFTError(code, msg)

    @property
    def hsd(self):
        return self.info.hsd

    def set_precision(self, precision):
        self._check(lib().cdft_set_precision(self._h, precision))

    def set_stream(self, stream_ptr):
        self._check(lib().cdft_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def set_density(self, rho):
        """rho: numpy array (host) or an object with data_ptr() (a CUDA tensor, float64, contiguous)."""
        if hasattr(rho, "data_ptr"):  # a torch tensor: device, or (pinned) host memory
            on_dev = 1 if getattr(rho, "is_cuda", True) else 0
            self._check(lib().cdft_set_density(self._h, ctypes.c_void_p(rho.data_ptr()), on_dev))
        else:
            a = np.ascontiguousarray(rho, dtype=np.float64)
            assert a.size == self.N
            self._check(lib().cdft_set_density(self._h, a.ctypes.data_as(ctypes.c_void_p), 0))

    def get_density(self):
        a = np.empty(self.shape)
        self._check(lib().cdft_get_density(self._h, a.ctypes.data_as(ctypes.c_void_p), 0))
        return a

    def set_external_field(self, v):
        if v is None:
            self._check(lib().cdft_set_external_field(self._h, None, 0))
        else:
            a = np.ascontiguousarray(v, dtype=np.float64)
            self._check(lib().cdft_set_external_field(self._h, a.ctypes.data_as(ctypes.c_void_p), 0))

    def set_chem_potential(self, mu):
        self._check(lib().cdft_set_chem_potential(self._h, mu))

    def set_fixed_mass(self, m):
        self._check(lib().cdft_set_fixed_mass(self._h, m))

    def set_boundary(self, fixed_background=False, homogeneous=False):
        """Species::setFixedBackground / setHomogeneousBoundary: dF on the planes i, j, k = 0
        set to zero, or to its mean over those planes, after each evaluation."""
        self._check(lib().cdft_set_boundary(self._h, int(fixed_background), int(homogeneous)))

    def chem_potential(self):
        v = ctypes.c_double()
        self._check(lib().cdft_get_chem_potential(self._h, ctypes.byref(v)))
        return v.value

    def eval(self, want_dF=True, only_fex=False, dF_out=None):
        """One F+dF evaluation. Returns (terms dict, dF numpy array or None).
        dF_out may be a torch float64 tensor of N elements: a CUDA tensor receives dF on the
        device, a (pinned) CPU tensor on the host."""
        t = np.zeros(8)
        if dF_out is not None:  # a torch tensor: device, or (pinned) host memory
            on_dev = 1 if getattr(dF_out, "is_cuda", True) else 0
            code = lib().cdft_eval(self._h, int(only_fex), _dptr(t), ctypes.c_void_p(dF_out.data_ptr()), on_dev)
            dF = None
        elif want_dF:
            dF = np.empty(self.shape)
            code = lib().cdft_eval(self._h, int(only_fex), _dptr(t), dF.ctypes.data_as(ctypes.c_void_p), 0)
        else:
            dF = None
            code = lib().cdft_eval(self._h, int(only_fex), _dptr(t), None, 0)
        self._check(code)
        return dict(zip(TERM_NAMES, t)), dF

    def bulk(self, rho):
        out = np.zeros(3)
        self._check(lib().cdft_bulk(self._h, rho, _dptr(out)))
        return {"mu": out[0], "omega": out[1], "fhelmholtz": out[2]}

    def find_coex(self, xmax=1.0, dx=1e-3, tol=1e-8):
        """DFT::findCoex: {x_vap, x_liq, mu, spinodal1, spinodal2}."""
        out = np.zeros(5)
        self._check(lib().cdft_find_coex(self._h, xmax, dx, tol, _dptr(out)))
        return dict(zip(("x_vap", "x_liq", "mu", "spinodal1", "spinodal2"), out))

    def weights(self):
        w = np.zeros((11,) + self.shape)
        a = np.zeros(self.shape)
        self._check(lib().cdft_get_weights(self._h, _dptr(w), _dptr(a)))
        return w, a

    def time_passes(self, reps=10):
        """Mean CUDA-event time (ms) and algorithmic bytes of each evaluation pass."""
        ms, by = np.zeros(9), np.zeros(9)
        n = ctypes.c_int()
        self._check(lib().cdft_time_passes(self._h, reps, _dptr(ms), _dptr(by), ctypes.byref(n)))
        return [{"pass": PASS_NAMES[k], "ms": ms[k], "bytes": by[k]} for k in range(n.value)]

    # FIRE2
    def fire_init(self, **kw):
        p = FireParams()
        lib().cdft_fire_default_params(ctypes.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        self._check(lib().cdft_fire_init(self._h, ctypes.byref(p)))

    def _rep(self, r):
        return {k: getattr(r, k) for k, _ in r._fields_}

    def fire_step(self, n=1):
        r = FireReport()
        self._check(lib().cdft_fire_step(self._h, n, ctypes.byref(r)))
        return self._rep(r)

    def fire_run(self, max_steps=-1):
        r = FireReport()
        self._check(lib().cdft_fire_run(self._h, max_steps, ctypes.byref(r)))
        return self._rep(r)

    def fire_run_to_residual(self, tol, max_steps=100000):
        r = FireReport()
        self._check(lib().cdft_fire_run_to_residual(self._h, tol, max_steps, ctypes.byref(r)))
        return self._rep(r)

    def fire_save(self, path):
        """The FIRE2 state (density, alias coordinates, velocities, step parameters and
        counters) to a file (fireMinimizer2's serialisation)."""
        self._check(lib().cdft_fire_save(self._h, os.fsencode(path)))

    def fire_load(self, path):
        """Resumes a FIRE2 run saved by fire_save on a context of the same lattice."""
        self._check(lib().cdft_fire_load(self._h, os.fsencode(path)))

    def fire_run_device(self, tol, max_steps=-1, mixed=False, switch_tol=1e-6):
        """Graph-captured FIRE2 to max|dOmega/drho| <= tol (FP64 test); mixed: FP32 bulk phase first
        (True or 1: then FP64 FIRE2; 2: then Newton-Krylov refinement)."""
        r = FireReport()
        self._check(lib().cdft_fire_run_device(self._h, tol, switch_tol, max_steps, int(mixed), ctypes.byref(r)))
        return self._rep(r)

    def newton_refine(self, tol, max_newton=12, max_cg=200, cg_rtol=1e-3, eta_max=0.1, fp32_above=1e-4, host_cg=False):
        """Newton-Krylov refinement with FP32 Hessian products, FP32 then FP64 residuals (cdft_newton_refine_ex)."""
        p = NewtonParams(max_newton, max_cg, cg_rtol, eta_max, fp32_above, int(host_cg))
        r = NewtonReport()
        self._check(lib().cdft_newton_refine_ex(self._h, tol, ctypes.byref(p), ctypes.byref(r)))
        return self._rep(r)

    def hessian_dot_v(self, v, out=None):
        """Full Hessian of Omega times v at the current density (DFT::matrix_dot_v1).
        v: numpy array (host) or CUDA float64 tensor (device; out must then be one too)."""
        if hasattr(v, "data_ptr"):
            self._check(lib().cdft_hessian_dot_v(self._h, ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(out.data_ptr()), 1))
            return out
        a = np.ascontiguousarray(v, dtype=np.float64).reshape(self.shape)
        o = np.empty(self.shape)
        self._check(lib().cdft_hessian_dot_v(self._h, a.ctypes.data_as(ctypes.c_void_p), o.ctypes.data_as(ctypes.c_void_p), 0))
        return o

    def ddft_matrix_dot_v(self, v):
        """DDFT dynamical matrix times v, g . (H v), at the current density (DDFT::matrix_dot_v1)."""
        a = np.ascontiguousarray(v, dtype=np.float64).reshape(self.shape)
        o = np.empty(self.shape)
        self._check(lib().cdft_ddft_matrix_dot_v(self._h, a.ctypes.data_as(ctypes.c_void_p), o.ctypes.data_as(ctypes.c_void_p), 0))
        return o

    # spectral drivers (Log_Det, Eigenvalues, Arnoldi on the Hessian)
    def log_det(self, order, lam_max, lam_min, seed, num_samples, has_zero_eigenvalue=False, matrix=MATRIX_HESSIAN):
        """Log_Det(matrix, order, lam_max, lam_min).calculate_log_det(seed, num_samples,
        has_zero_eigenvalue) at the current density; returns (log_det, variance)."""
        val, var = ctypes.c_double(), ctypes.c_double()
        self._check(lib().cdft_log_det(self._h, matrix, order, lam_max, lam_min, seed, num_samples, int(has_zero_eigenvalue),
                                       ctypes.byref(val), ctypes.byref(var)))
        return val.value, var.value

    @staticmethod
    def _eigen_rep(r):
        return {"matvecs": r.matvecs, "restarts": r.restarts, "converged": bool(r.converged), "residual": r.residual}

    def _host_vec(self, v):
        if v is None:
            return None, None
        a = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        if a.size != int(np.prod(self.shape)):
            raise ValueError("expected %d values" % int(np.prod(self.shape)))
        return a, a.ctypes.data_as(ctypes.c_void_p)

    def eigenvalue(self, scale=1e6, tol=1e-6, change_sign=False, vshift=None, guess=None, max_matvecs=20000):
        """Eigenvalues(dft).calculate_eigenvector with set_scale / set_tolerence /
        set_change_sign / set_vshift: the smallest eigenvalue of the Hessian plus
        vshift vshift^T / 2 (the largest with change_sign); returns (eigenvalue, unit
        eigenvector, report)."""
        vs, vsp = self._host_vec(vshift)
        gs, gsp = self._host_vec(guess)
        val = ctypes.c_double()
        vec = np.empty(self.shape)
        r = EigenReport()
        self._check(lib().cdft_eigenvalue(self._h, scale, tol, int(change_sign), vsp, gsp, max_matvecs, ctypes.byref(val),
                                          vec.ctypes.data_as(ctypes.c_void_p), 0, ctypes.byref(r)))
        return val.value, vec, self._eigen_rep(r)

    def arnoldi(self, shift, k, p, all_k=True, max_steps=1000, tol=1e-8, guess=None, matrix=MATRIX_HESSIAN):
        """Arnoldi(matrix).determine_largest_eigenpairs(shift, k, p, all_k, max_steps, tol):
        the k eigenpairs of M + shift of largest magnitude, M the Hessian (MATRIX_HESSIAN,
        Arnoldi(dft)) or the DDFT dynamical matrix g.H (MATRIX_DDFT, Arnoldi(ddft));
        returns (eigenvalues without the shift, unit eigenvectors (k, *shape), report)."""
        gs, gsp = self._host_vec(guess)
        vals = np.empty(k)
        vecs = np.empty((k,) + tuple(self.shape))
        r = EigenReport()
        self._check(lib().cdft_arnoldi_largest_matrix(self._h, matrix, shift, k, p, int(all_k), max_steps, tol, gsp, _dptr(vals),
                                                      vecs.ctypes.data_as(ctypes.c_void_p), 0, ctypes.byref(r)))
        return vals, vecs, self._eigen_rep(r)

    # FFT plans
    def autotune(self, reps=5):
        """Tunes the radix ordering of each axis; returns ({x, y, z orderings}, default ms, tuned ms)."""
        r = (ctypes.c_int * 24)()
        ms = np.zeros(2)
        self._check(lib().cdft_autotune(self._h, reps, r, _dptr(ms)))
        return _radices(r), float(ms[0]), float(ms[1])

    def radices(self):
        r = (ctypes.c_int * 24)()
        self._check(lib().cdft_get_radices(self._h, r))
        return _radices(r)

    # DDFT
    def ddft_init(self, dt, dt_max, tol=1e-4):
        self._check(lib().cdft_ddft_init(self._h, dt, dt_max, tol))

    def ddft_step(self, n=1):
        r = DdftReport()
        self._check(lib().cdft_ddft_step(self._h, n, ctypes.byref(r)))
        return self._rep(r)

    def ddft_set_mass_restore(self, on):
        """FP32 mode: keep (True, the default) or drop the uniform FP64 shift back to the
        starting mass after each propagation."""
        self._check(lib().cdft_ddft_set_mass_restore(self._h, int(bool(on))))

    def ddft_mass_deviation(self):
        """FP32 mode: the largest relative mass deviation of a propagated density from the
        run's start, before any restore, since ddft_init."""
        v = ctypes.c_double()
        self._check(lib().cdft_ddft_mass_deviation(self._h, ctypes.byref(v)))
        return v.value


def _radices(r):
    return {ax: [v for v in r[8 * a:8 * a + 8] if v] for a, ax in enumerate("xyz")}


def radix_candidates(n):
    """Radix orderings the autotuner tries for transform length n (host only)."""
    cnt = ctypes.c_int()
    code = lib().cdft_radix_candidates(n, None, 0, ctypes.byref(cnt))
    if code:
        raise CDFTError(code, "bad length")
    out = (ctypes.c_int * (8 * cnt.value))()
    lib().cdft_radix_candidates(n, out, cnt.value, ctypes.byref(cnt))
    return [[v for v in out[8 * k:8 * k + 8] if v] for k in range(cnt.value)]


def fire_run_batch(contexts, tol, max_steps=-1, mixed=True, switch_tol=2e-6):
    """Device FIRE2 on many contexts at once (cdft_fire_run_batch); mixed as in
    Context.fire_run_device (0 FP64, 1 FP32 then FP64 FIRE2, 2 FP32 then Newton-Krylov).

    Returns (reports, statuses): one report dict and one status code per context."""
    n = len(contexts)
    hs = (ctypes.c_void_p * n)(*[c._h for c in contexts])
    reps = (FireReport * n)()
    rcs = (ctypes.c_int * n)()
    rc = lib().cdft_fire_run_batch(hs, n, tol, switch_tol, max_steps, int(mixed), reps, rcs)
    out = [contexts[k]._rep(reps[k]) for k in range(n)]
    status = [int(rcs[k]) for k in range(n)]
    for k in range(n):
        if status[k]:
            out[k]["error"] = lib().cdft_last_error(contexts[k]._h).decode()
    if rc and not any(status):
        raise CDFTError(rc, "cdft_fire_run_batch")
    return out, status


# ------------------------------------------------- reference-shaped API ---
class Lattice:
    """Lattice(dx, L) (include/Lattice.h:57-85): N_i = int((L_i + 1e-8 dx)/dx); throws if incommensurate."""

    def __init__(self, dx, L):
        self.dx = float(dx)
        n = [int((float(l) + 1e-8 * dx) / dx) for l in L]
        for l, m in zip(L, n):
            if abs(l - m * dx) > 1e-5 * dx:
                raise RuntimeError("Box length incommensurate with lattice")
        self._n = tuple(n)

    def Nx(self): return self._n[0]
    def Ny(self): return self._n[1]
    def Nz(self): return self._n[2]
    def Ntot(self): return self._n[0] * self._n[1] * self._n[2]
    def dV(self): return self.dx ** 3
    def getVolume(self): return self.Ntot() * self.dV()
    def getX(self, i): return self.dx * (i - self._n[0] / 2.0)
    def getY(self, j): return self.dx * (j - self._n[1] / 2.0)
    def getZ(self, k): return self.dx * (k - self._n[2] / 2.0)
    def pos(self, i, j, k): return k + self._n[2] * (j + self._n[1] * i)

    @property
    def shape(self):
        return self._n


class Density(Lattice):
    """Density(dx, L): the density field (include/Density.h:35-118), held on the host until a DFT runs."""

    def __init__(self, dx, L):
        super().__init__(dx, L)
        self.values = np.zeros(self.shape)
        self.vWall = None

    def set(self, *args):
        if len(args) == 1:
            a = np.asarray(args[0], dtype=np.float64)
            self.values[...] = a.reshape(self.shape) if a.ndim else a
        elif len(args) == 2:
            self.values.reshape(-1)[args[0]] = args[1]
        else:
            i, j, k, v = args
            self.values[i, j, k] = v

    def get(self, *args):
        if len(args) == 1:
            return self.values.reshape(-1)[args[0]]
        i, j, k = (a % n for a, n in zip(args, self.shape))
        return self.values[i, j, k]

    def getNumberAtoms(self):
        return math.fsum(self.values.ravel()) * self.dV()


class FMT:
    model = MODEL_NONE
    A, B = 1.0, 0.0

    def needsTensor(self):
        return self.model >= ESFMT

    def get_name(self):
        return type(self).__name__


class Rosenfeld(FMT):
    model = ROSENFELD


class RSLT(FMT):
    model = RSLT_MODEL


class esFMT(FMT):
    model = ESFMT

    def __init__(self, A=1.0, B=0.0):
        self.A, self.B = float(A), float(B)


class WhiteBearI(FMT):
    model = WHITEBEAR_I


class WhiteBearII(FMT):
    model = WHITEBEAR_II


class LJ:
    """Cut-and-shifted Lennard-Jones (include/Potential1.h:136-189)."""

    def __init__(self, sigma, eps, rcut):
        self.sigma, self.eps, self.rcut = float(sigma), float(eps), float(rcut)
        self.bh = False

    def setBH(self):
        self.bh = True

    def getHSD(self, kT):
        if not self.bh:
            raise NotImplementedError("only the Barker-Henderson split (setBH) is on the GPU path")
        return bh_diameter(self.sigma, self.eps, self.rcut, kT)


class FMT_Species:
    """FMT_Species(density, hsd, mu) (include/Species.h:120-380)."""

    def __init__(self, density, hsd, mu=0.0, seq=-1):
        self.density = density
        self.hsd = float(hsd)
        self.mu = float(mu)
        self.fixedMass = -1.0
        self.dF = None

    def setChemPotential(self, mu):
        self.mu, self.fixedMass = float(mu), -1.0

    def getChemPotential(self):
        return self.mu

    def setFixedMass(self, m):
        self.fixedMass = float(m)
        if m > 0:
            self.mu = 0.0

    def getHSD(self):
        return self.hsd

    def getDF(self):
        return self.dF

    def get_convergence_monitor(self):
        return float(np.abs(self.dF).max()) / self.density.dV()


class Interaction_Interpolation_QF:
    """Mean-field interaction with the quadratic-force weights (include/Interaction.h:416-441)."""

    def __init__(self, s1, s2, potential, kT):
        if s1 is not s2:
            raise NotImplementedError("only the self interaction of one species is on the GPU path")
        if not potential.bh:
            raise NotImplementedError("only the Barker-Henderson split (setBH) is on the GPU path")
        self.species, self.potential, self.kT = s1, potential, float(kT)


class DFT:
    """DFT(species) aggregator (include/DFT.h:44-190) running on the GPU."""

    def __init__(self, species=None, precision=FP64):
        self.species = species
        self.fmt = None
        self.interaction = None
        self.precision = precision
        self._ctx = None
        self.F_id = self.F_hs = self.F_mf = self.F_ext = 0.0

    def addSpecies(self, s):
        self.species = s

    def addHardCoreContribution(self, fmt):
        self.fmt = fmt
        self._ctx = None

    def addInteraction(self, inter):
        self.interaction = inter
        self._ctx = None

    def context(self):
        if self._ctx is None:
            s, d = self.species, self.species.density
            lj = self.interaction is not None
            pot = self.interaction.potential if lj else None
            self._ctx = Context(d.shape, d.dx, model=self.fmt.model if self.fmt else MODEL_NONE, hsd=s.hsd,
                                lj=lj, kT=self.interaction.kT if lj else 1.0, rc=pot.rcut if lj else 3.0,
                                sigma=pot.sigma if lj else 1.0, eps=pot.eps if lj else 1.0, mu=s.mu,
                                fixed_mass=s.fixedMass, precision=self.precision,
                                es_A=self.fmt.A if self.fmt else 1.0, es_B=self.fmt.B if self.fmt else 0.0)
        return self._ctx

    def _push(self):
        c, s = self.context(), self.species
        c.set_density(s.density.values)
        if s.fixedMass > 0:
            c.set_fixed_mass(s.fixedMass)
        else:
            c.set_chem_potential(s.mu)

    def _pull(self, terms):
        s = self.species
        s.density.values[...] = self._ctx.get_density()
        s.mu = terms["mu"]
        self.F_id, self.F_hs, self.F_mf, self.F_ext = terms["F_id"], terms["F_hs"], terms["F_mf"], terms["F_ext"]

    def calculateFreeEnergyAndDerivatives(self, onlyFex=False):
        self._push()
        terms, dF = self._ctx.eval(only_fex=onlyFex)
        self.species.dF = dF
        self._pull(terms)
        return terms["Omega"]

    def getDF(self, i=0):
        return self.species.dF

    def get_f_id(self): return self.F_id
    def get_f_hs(self): return self.F_hs
    def get_f_mf(self): return self.F_mf
    def get_f_ext(self): return self.F_ext

    def mu_times_beta(self, rho):
        return self.context().bulk(rho)["mu"]

    def omega_times_beta_over_volume(self, rho):
        return self.context().bulk(rho)["omega"]

    def fhelmholtz_times_beta_over_volume(self, rho):
        return self.context().bulk(rho)["fhelmholtz"]

    def getNumberAtoms(self, i=0):
        return self.species.density.getNumberAtoms()


class fireMinimizer2:
    """FIRE2 minimizer (include/Minimizer.h:80-182) with the reference's setters."""

    def __init__(self, dft):
        self.dft = dft
        p = FireParams()
        lib().cdft_fire_default_params(ctypes.byref(p))
        self.p = p
        self._started = False
        self.report = None

    def setTimeStep(self, dt): self.p.dt = dt
    def setTimeStepMax(self, dt): self.p.dt_max = dt
    def setAlphaStart(self, a): self.p.alpha_start = a
    def setAlphaFac(self, a): self.p.f_alf = a
    def setForceTerminationCriterion(self, v): self.p.force_limit = v

    def _start(self):
        if not self._started:
            self.dft._push()
            self.dft._ctx._check(lib().cdft_fire_init(self.dft._ctx._h, ctypes.byref(self.p)))
            self._started = True

    def step(self):
        self._start()
        self.report = self.dft._ctx.fire_step(1)
        return self.report["F"]

    def run(self, maxSteps=-1):
        self._start()
        self.report = self.dft._ctx.fire_run(maxSteps)
        self._sync()

    def resume(self, maxSteps=-1):
        self.run(maxSteps)

    def _sync(self):
        c = self.dft._ctx
        self.dft.species.density.values[...] = c.get_density()

    def getF(self):
        return self.report["F"] if self.report else None

    def get_convergence_monitor(self):
        return abs(self.report["vv"] / self.dft.species.density.getVolume())


class DDFT:
    """Integrating-factor DDFT (include/Minimizer.h:189-266), periodic boundaries."""

    def __init__(self, dft, showGraphics=False):
        self.dft = dft
        self.dt = 1e-4 * dft.species.density.dx ** 2
        self.dt_max = 1.0
        self.tol = 1e-4
        self._started = False
        self.report = None

    def setTimeStep(self, dt): self.dt = dt
    def set_max_time_step(self, dt): self.dt_max = dt
    def set_tolerence_fixed_point(self, e): self.tol = e

    def _start(self):
        if not self._started:
            self.dft._push()
            self.dft._ctx.ddft_init(self.dt, self.dt_max, self.tol)
            self._started = True

    def step(self):
        self._start()
        self.report = self.dft._ctx.ddft_step(1)
        self.dft.species.density.values[...] = self.dft._ctx.get_density()
        return self.report["F"]

    def run(self, maxSteps):
        self._start()
        self.report = self.dft._ctx.ddft_step(maxSteps)
        self.dft.species.density.values[...] = self.dft._ctx.get_density()

    def get_time(self):
        return self.report["time"] if self.report else 0.0

"""ctypes loader for the FP64 CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; the product never imports it.
"""
import ctypes
import os
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MODELS = {"none": -1, "Rosenfeld": 0, "RSLT": 1, "esFMT": 2, "WhiteBearI": 3, "WhiteBearII": 4}


class Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("dx", ctypes.c_double),
                ("model", ctypes.c_int), ("es_A", ctypes.c_double), ("es_B", ctypes.c_double),
                ("hsd", ctypes.c_double), ("lj", ctypes.c_int), ("lj_sigma", ctypes.c_double),
                ("lj_eps", ctypes.c_double), ("lj_rc", ctypes.c_double), ("kT", ctypes.c_double),
                ("mu", ctypes.c_double), ("fixed_mass", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            import subprocess
            subprocess.check_call(["make", "-C", HERE, "oracle"], stdout=subprocess.DEVNULL)
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        d = ctypes.c_double
        dp = P(d)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [P(Params)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        for f in ("orc_hsd", "orc_a_vdw", "orc_get_mu"):
            getattr(L, f).restype = d
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.orc_set_mu.argtypes = [ctypes.c_void_p, d]
        L.orc_weights.argtypes = [ctypes.c_void_p, dp]
        L.orc_w_att.argtypes = [ctypes.c_void_p, dp]
        L.orc_eval.restype = ctypes.c_int
        L.orc_eval.argtypes = [ctypes.c_void_p, dp, dp, dp]
        for f in ("orc_mu_times_beta", "orc_omega_times_beta_over_volume", "orc_fhelmholtz_times_beta_over_volume"):
            getattr(L, f).restype = d
            getattr(L, f).argtypes = [ctypes.c_void_p, d]
        L.orc_phi.restype = d
        L.orc_phi.argtypes = [ctypes.c_int, d, d, dp, dp]
        L.orc_bh_diameter.restype = d
        L.orc_bh_diameter.argtypes = [d, d]
        L.orc_fire.restype = ctypes.c_int
        L.orc_fire.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, d, d, d, dp, dp, dp, dp, dp, dp]
        L.orc_ddft.restype = ctypes.c_int
        L.orc_ddft.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, d, d, dp, dp, dp, dp, dp]
        L.orc_r2c.argtypes = [ctypes.c_int] * 3 + [dp, dp]
        L.orc_c2r.argtypes = [ctypes.c_int] * 3 + [dp, dp]
        L.orc_fill_noise.argtypes = [dp, ctypes.c_long, d, d, ctypes.c_uint64]
        L.orc_hessian_dot_v.argtypes = [ctypes.c_void_p, dp, dp, dp]
        L.orc_ddft_matrix_dot_v.argtypes = [ctypes.c_void_p, dp, dp, dp]
        L.orc_log_det.restype = d
        L.orc_log_det.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_int, d, d, ctypes.c_long, ctypes.c_int, ctypes.c_int, dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fill_noise(shape, rho0, amp, seed):
    a = np.empty(shape, dtype=np.float64)
    lib().orc_fill_noise(_p(a), a.size, rho0, amp, seed)
    return a


def bh_diameter(rc, kT):
    return lib().orc_bh_diameter(rc, kT)


def phi(model, fm19, A=1.0, B=0.0):
    fm19 = np.ascontiguousarray(fm19, dtype=np.float64)
    d = np.zeros(19)
    v = lib().orc_phi(MODELS[model], A, B, _p(fm19), _p(d))
    return v, d


def r2c(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    nx, ny, nz = a.shape
    out = np.empty((nx, ny, nz // 2 + 1), dtype=np.complex128)
    lib().orc_r2c(nx, ny, nz, _p(a), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def c2r(c, nz):
    c = np.ascontiguousarray(c, dtype=np.complex128)
    nx, ny, _ = c.shape
    out = np.empty((nx, ny, nz))
    lib().orc_c2r(nx, ny, nz, c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _p(out))
    return out


class Oracle:
    """One system: grid, FMT model, optional LJ mean field, mu / fixed mass."""

    def __init__(self, n, dx, model="WhiteBearI", hsd=1.0, lj=False, kT=1.0, rc=3.0, mu=0.0,
                 fixed_mass=-1.0, es_A=1.0, es_B=0.0):
        if isinstance(n, int):
            n = (n, n, n)
        self.shape = tuple(n)
        p = Params(n[0], n[1], n[2], dx, MODELS[model], es_A, es_B, hsd if hsd else -1.0, int(lj), 1.0, 1.0,
                   rc, kT, mu, fixed_mass)
        self._c = lib().orc_create(ctypes.byref(p))
        self.N = int(np.prod(n))
        self.dx = dx

    def __del__(self):
        if getattr(self, "_c", None):
            lib().orc_destroy(self._c)
            self._c = None

    @property
    def hsd(self):
        return lib().orc_hsd(self._c)

    @property
    def a_vdw(self):
        return lib().orc_a_vdw(self._c)

    @property
    def mu(self):
        return lib().orc_get_mu(self._c)

    def set_mu(self, mu):
        lib().orc_set_mu(self._c, mu)

    def weights(self):
        w = np.zeros((11,) + self.shape)
        lib().orc_weights(self._c, _p(w))
        return w

    def w_att(self):
        w = np.zeros(self.shape)
        lib().orc_w_att(self._c, _p(w))
        return w

    def eval(self, rho):
        """Returns (status, terms dict, dF, rho_after) for one F+dF evaluation."""
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.shape).copy()
        dF = np.zeros(self.shape)
        t = np.zeros(6)
        st = lib().orc_eval(self._c, _p(r), _p(dF), _p(t))
        terms = dict(zip(["Omega", "F_id", "F_hs", "F_mf", "F_ext", "mu"], t))
        return st, terms, dF, r

    def hessian_dot_v(self, rho, v):
        """Full Hessian (ideal + FMT + mean field) times v at density rho (DFT::matrix_dot_v1)."""
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.shape)
        vv = np.ascontiguousarray(v, dtype=np.float64).reshape(self.shape)
        out = np.zeros(self.shape)
        lib().orc_hessian_dot_v(self._c, _p(r), _p(vv), _p(out))
        return out

    def ddft_matrix_dot_v(self, rho, v):
        """DDFT dynamical matrix times v: g_dot_x(H v) (DDFT::matrix_dot_v_intern)."""
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.shape)
        vv = np.ascontiguousarray(v, dtype=np.float64).reshape(self.shape)
        out = np.zeros(self.shape)
        lib().orc_ddft_matrix_dot_v(self._c, _p(r), _p(vv), _p(out))
        return out

    def log_det(self, rho, order, lam_max, lam_min, seed, num_samples, has_zero=False, dynamic=False):
        """Log_Det::calculate_log_det of the Hessian (or of the negated DDFT matrix with
        dynamic=True) at density rho; returns (log_det, variance)."""
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.shape)
        var = np.zeros(1)
        val = lib().orc_log_det(self._c, _p(r), int(dynamic), order, lam_max, lam_min, seed, num_samples, int(has_zero), _p(var))
        return val, var[0]

    def mu_times_beta(self, rho):
        return lib().orc_mu_times_beta(self._c, rho)

    def omega_times_beta_over_volume(self, rho):
        return lib().orc_omega_times_beta_over_volume(self._c, rho)

    def fhelmholtz_times_beta_over_volume(self, rho):
        return lib().orc_fhelmholtz_times_beta_over_volume(self._c, rho)

    def fire(self, rho, nsteps, dt=1e-3, dt_max=1e-2, force_limit=0.0):
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.shape).copy()
        rec = {k: np.zeros(nsteps) for k in ("F", "dt", "alpha", "vv", "fmax", "resid")}
        n = lib().orc_fire(self._c, _p(r), nsteps, dt, dt_max, force_limit, *[_p(rec[k]) for k in
                                                                           ("F", "dt", "alpha", "vv", "fmax", "resid")])
        return n, {k: v[:max(n, 0)] for k, v in rec.items()}, r

    def ddft(self, rho, nsteps, dt, dt_max):
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.shape).copy()
        rec = {k: np.zeros(nsteps) for k in ("F", "t", "dt", "mass", "rhs")}
        n = lib().orc_ddft(self._c, _p(r), nsteps, dt, dt_max, *[_p(rec[k]) for k in ("F", "t", "dt", "mass", "rhs")])
        return n, rec, r

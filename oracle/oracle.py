"""ctypes wrapper of the CPU oracle (``liblassie_oracle.so``).

TEST INFRASTRUCTURE: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` use this module, as the checker.  The product
(``lassie_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liblassie_oracle.so")
_lib = None
_lock = threading.Lock()

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class _Model(C.Structure):
    _fields_ = [("n_species", C.c_int), ("n_reactions", C.c_int),
                ("rxn_ptr", C.POINTER(C.c_int)), ("rxn_species", C.POINTER(C.c_int)),
                ("rxn_stoich", C.POINTER(C.c_int)), ("sp_ptr", C.POINTER(C.c_int)),
                ("sp_rxn", C.POINTER(C.c_int)), ("sp_coef", C.POINTER(C.c_int)),
                ("nnz_a", C.c_int), ("nnz_h", C.c_int)]


class Opts(C.Structure):
    _fields_ = [("rkf_step", C.c_double), ("be_step", C.c_double),
                ("newton_tol", C.c_double), ("stiffness_tol", C.c_double),
                ("newton_iter", C.c_int64), ("max_steps", C.c_int64),
                ("use_pow", C.c_int32), ("pad", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("outer_iters", C.c_int64), ("rkf_accepts", C.c_int64),
                ("rkf_retries", C.c_int64), ("be_steps", C.c_int64),
                ("newton_iters", C.c_int64), ("lu_factorisations", C.c_int64),
                ("lu_failures", C.c_int64), ("nan_reverts", C.c_int64),
                ("t_final", C.c_double), ("dt_be_final", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class BdfOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("first_step", C.c_double),
                ("max_step", C.c_double), ("max_order", C.c_int32), ("pad", C.c_int32),
                ("max_steps", C.c_int64)]


class BdfStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("rejected", C.c_int64), ("newton_failures", C.c_int64),
                ("newton_iters", C.c_int64), ("jac_evals", C.c_int64),
                ("lu_factorisations", C.c_int64), ("rhs_evals", C.c_int64),
                ("order_final", C.c_int32), ("pad", C.c_int32), ("h_final", C.c_double),
                ("t_final", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                build()
            L = C.CDLL(_LIB_PATH)
            L.lo_model_build.argtypes = [C.c_int, C.c_int, _i32p, _i32p, C.POINTER(_Model)]
            L.lo_model_build.restype = C.c_int
            L.lo_model_free.argtypes = [C.POINTER(_Model)]
            L.lo_rhs.argtypes = [C.POINTER(_Model), _f64p, _f64p, _f64p]
            L.lo_jacobian.argtypes = [C.POINTER(_Model), _f64p, _f64p, _f64p]
            L.lo_lu_factor.argtypes = [C.c_int, _f64p, _i32p]
            L.lo_lu_factor.restype = C.c_int
            L.lo_lu_solve.argtypes = [C.c_int, _f64p, _i32p, _f64p]
            L.lo_set_solve_perturbation.argtypes = [C.c_double, C.c_uint64]
            L.lo_set_solve_perturbation_normwise.argtypes = [C.c_double, C.c_uint64]
            L.lo_set_lu_variant.argtypes = [C.c_int]
            L.lo_set_trace.argtypes = [C.c_void_p, C.c_int64]
            L.lo_trace_len.restype = C.c_int64
            L.lo_set_root_perturbation.argtypes = [C.c_double, C.c_uint64]
            L.lo_qroot_rn.argtypes = [C.c_double]
            L.lo_qroot_rn.restype = C.c_double
            L.lo_solve_compat.argtypes = [C.POINTER(_Model), _f64p, _f64p, C.c_void_p,
                                          C.c_void_p, _f64p, C.c_int, C.c_void_p, C.c_int,
                                          C.POINTER(Opts), _f64p, C.POINTER(Stats)]
            L.lo_solve_compat.restype = C.c_int
            L.lo_solve_compat_f32.argtypes = L.lo_solve_compat.argtypes
            L.lo_solve_compat_f32.restype = C.c_int
            L.lo_solve_compat_rec.argtypes = [C.POINTER(_Model), _f64p, _f64p, C.c_void_p,
                                              C.c_void_p, _f64p, C.c_int, C.c_void_p, C.c_int,
                                              C.POINTER(Opts), _f64p, C.POINTER(Stats), C.c_int,
                                              _i32p, _f64p, C.POINTER(C.c_int), _i32p]
            L.lo_solve_compat_rec.restype = C.c_int
            L.lo_solve_batch.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, _i32p, C.POINTER(Opts), C.c_void_p,
                                         C.c_void_p, _i32p, C.c_int]
            L.lo_solve_batch.restype = C.c_int
            L.lo_jacobian_exact.argtypes = [C.POINTER(_Model), _f64p, _f64p, _f64p]
            L.lo_block_sum512.argtypes = [_f64p, C.c_int]
            L.lo_block_sum512.restype = C.c_double
            L.lo_bdf_opts_default.argtypes = [C.POINTER(BdfOpts)]
            L.lo_solve_bdf.argtypes = [C.POINTER(_Model), _f64p, _f64p, C.c_void_p, C.c_void_p,
                                       _f64p, C.c_int, C.c_void_p, C.c_int,
                                       C.POINTER(BdfOpts), _f64p, C.POINTER(BdfStats)]
            L.lo_solve_bdf.restype = C.c_int
            _lib = L
    return _lib


class OracleModel:
    """A compiled network in the oracle's CSR form."""

    def __init__(self, left: np.ndarray, right: np.ndarray):
        left = np.ascontiguousarray(left, dtype=np.int32)
        right = np.ascontiguousarray(right, dtype=np.int32)
        R, N = left.shape
        self._m = _Model()
        rc = lib().lo_model_build(R, N, left, right, C.byref(self._m))
        if rc != 0:
            raise ValueError(f"lo_model_build failed: {rc}")
        self.n_species, self.n_reactions = N, R

    def __del__(self):
        if _lib is not None and getattr(self, "_m", None) is not None:
            _lib.lo_model_free(C.byref(self._m))
            self._m = None

    def rhs(self, k, x) -> np.ndarray:
        dx = np.zeros(self.n_species)
        lib().lo_rhs(C.byref(self._m), np.ascontiguousarray(k, np.float64),
                     np.ascontiguousarray(x, np.float64), dx)
        return dx

    def jacobian_exact(self, k, x) -> np.ndarray:
        J = np.zeros((self.n_species, self.n_species))
        lib().lo_jacobian_exact(C.byref(self._m), np.ascontiguousarray(k, np.float64),
                                np.ascontiguousarray(x, np.float64), J)
        return J

    def jacobian(self, k, x) -> np.ndarray:
        J = np.zeros((self.n_species, self.n_species))
        lib().lo_jacobian(C.byref(self._m), np.ascontiguousarray(k, np.float64),
                          np.ascontiguousarray(x, np.float64), J)
        return J


# the step-size factor (atol/R)^(1/4): sqrt(sqrt()), the C library's pow(),
# or correctly rounded
ROOTS = {"sqrt": 0, "libm": 1, "rn": 2}


def make_opts(model=None, max_steps: int = 0, root: str = "sqrt") -> Opts:
    """Options of a solve; ``root`` picks how the step-size factor
    (atol/R)^(1/4) is computed (``ROOTS``): "rn" correctly rounded, which
    is what the reference's pow() call returns on the golden cases."""
    if root not in ROOTS:
        raise ValueError("root must be one of " + ", ".join(ROOTS))
    o = Opts()
    o.use_pow = ROOTS[root]
    o.rkf_step = getattr(model, "rkf_step", 1e-3)
    o.be_step = getattr(model, "be_step", 0.01)
    o.newton_tol = getattr(model, "newton_tol", 1e-6)
    o.stiffness_tol = getattr(model, "stiffness_tol", 1e-6)
    o.newton_iter = int(getattr(model, "newton_iter", 10000))
    o.max_steps = int(max_steps)
    return o


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def solve(model, max_steps: int = 0, om: Optional[OracleModel] = None, root: str = "sqrt",
          precision: str = "double"):
    """Integrate a ``lassie_gb300.model.Model`` with the oracle (``root`` as
    in ``make_opts``; ``precision`` "float": the reference's -p float loop).
    Returns (trajectory [nt, ncs], stats dict, status)."""
    om = om or OracleModel(model.left, model.right)
    N = model.n_species
    k = np.ascontiguousarray(model.k, np.float64)
    x0 = np.ascontiguousarray(model.x0[:N], np.float64)
    t = np.ascontiguousarray(model.t, np.float64)
    cs = model.sampled().astype(np.int32)
    feed = None if model.feed is None else np.ascontiguousarray(model.feed[:N], np.float64)
    atol = None if model.atol is None else np.ascontiguousarray(model.atol[:N], np.float64)
    out = np.zeros((t.shape[0], cs.shape[0]))
    st = Stats()
    o = make_opts(model, max_steps, root)
    fn = lib().lo_solve_compat_f32 if precision == "float" else lib().lo_solve_compat
    rc = fn(C.byref(om._m), k, x0, _ptr(feed), _ptr(atol), t,
                               t.shape[0], _ptr(cs), cs.shape[0], C.byref(o), out,
                               C.byref(st))
    return out, st.as_dict(), rc


def bdf_opts(rtol: float = 1e-6, atol: float = 1e-9, first_step: float = 0.0,
             max_step: float = 0.0, max_order: int = 5, max_steps: int = 0) -> BdfOpts:
    o = BdfOpts()
    lib().lo_bdf_opts_default(C.byref(o))
    o.rtol, o.atol, o.first_step, o.max_step = rtol, atol, first_step, max_step
    o.max_order, o.max_steps = max_order, max_steps
    return o


def solve_bdf(model, om: Optional[OracleModel] = None, **kw):
    """The standard controller (variable-order BDF, rtol/atol) on a
    ``Model``; ``kw`` as ``bdf_opts``.  The model's atol vector, when set,
    replaces the scalar atol.  Returns (trajectory [nt, ncs], stats, status)."""
    om = om or OracleModel(model.left, model.right)
    N = model.n_species
    k = np.ascontiguousarray(model.k, np.float64)
    x0 = np.ascontiguousarray(model.x0[:N], np.float64)
    t = np.ascontiguousarray(model.t, np.float64)
    cs = model.sampled().astype(np.int32)
    feed = None if model.feed is None else np.ascontiguousarray(model.feed[:N], np.float64)
    atol = None if model.atol is None else np.ascontiguousarray(model.atol[:N], np.float64)
    out = np.zeros((t.shape[0], cs.shape[0]))
    st = BdfStats()
    o = bdf_opts(**kw)
    rc = lib().lo_solve_bdf(C.byref(om._m), k, x0, _ptr(feed), _ptr(atol), t, t.shape[0],
                            _ptr(cs), cs.shape[0], C.byref(o), out, C.byref(st))
    return out, st.as_dict(), rc


def solve_recorded(model, cap: int = 1_000_000):
    """Integrate and return (trajectory, stats, status, kinds, dts, samp):
    the step sequence of the integration, for sensitivity checks."""
    om = OracleModel(model.left, model.right)
    N = model.n_species
    k = np.ascontiguousarray(model.k, np.float64)
    x0 = np.ascontiguousarray(model.x0[:N], np.float64)
    t = np.ascontiguousarray(model.t, np.float64)
    cs = model.sampled().astype(np.int32)
    feed = None if model.feed is None else np.ascontiguousarray(model.feed[:N], np.float64)
    out = np.zeros((t.shape[0], cs.shape[0]))
    st = Stats()
    o = make_opts(model)
    kind = np.zeros(cap, np.int32)
    dts = np.zeros(cap)
    ns = C.c_int(0)
    samp = np.zeros(max(1, t.shape[0]), np.int32)
    rc = lib().lo_solve_compat_rec(C.byref(om._m), k, x0, _ptr(feed), None, t, t.shape[0],
                                   _ptr(cs), cs.shape[0], C.byref(o), out, C.byref(st), cap,
                                   kind, dts, C.byref(ns), samp)
    n = ns.value
    return out, st.as_dict(), rc, kind[:n].copy(), dts[:n].copy(), samp[: t.shape[0]].copy()


def solve_batch(models: Sequence, threads: int = 0, max_steps: int = 0, root: str = "sqrt"):
    """Solve independent instances (all species sampled, no feed, default
    atol) on ``threads`` host threads.  Returns (list of trajectories, list
    of stats dicts, statuses)."""
    n = len(models)
    threads = threads or os.cpu_count() or 1
    oms = [OracleModel(m.left, m.right) for m in models]
    keep = []
    mp = (C.c_void_p * n)(*[C.cast(C.byref(om._m), C.c_void_p) for om in oms])
    ks, xs, ts, outs = [], [], [], []
    for m in models:
        ks.append(np.ascontiguousarray(m.k, np.float64))
        xs.append(np.ascontiguousarray(m.x0[: m.n_species], np.float64))
        ts.append(np.ascontiguousarray(m.t, np.float64))
        outs.append(np.zeros((m.t.shape[0], m.n_species)))
    keep += [ks, xs, ts, outs]
    arr = lambda lst: (C.c_void_p * n)(*[a.ctypes.data for a in lst])  # noqa: E731
    nt = np.array([m.t.shape[0] for m in models], np.int32)
    stats = (Stats * n)()
    status = np.zeros(n, np.int32)
    o = make_opts(models[0] if n else None, max_steps, root)
    lib().lo_solve_batch(n, mp, arr(ks), arr(xs), arr(ts), nt, C.byref(o), arr(outs),
                         C.cast(stats, C.c_void_p), status, threads)
    return outs, [s.as_dict() for s in stats], status


def lu_factor(a: np.ndarray):
    a = np.ascontiguousarray(a, np.float64).copy()
    piv = np.zeros(a.shape[0], np.int32)
    rc = lib().lo_lu_factor(a.shape[0], a, piv)
    return a, piv, rc


def lu_solve(lu: np.ndarray, piv: np.ndarray, b: np.ndarray) -> np.ndarray:
    b = np.ascontiguousarray(b, np.float64).copy()
    lib().lo_lu_solve(lu.shape[0], np.ascontiguousarray(lu), piv, b)
    return b


class solve_perturbation:
    """Context manager: inside it, every oracle Newton correction is scaled
    componentwise by (1 +- rel) with seeded signs -- a linear solver that
    differs from the oracle's in the last bits.  Single-threaded use only."""

    def __init__(self, rel: float, seed: int = 1):
        self.rel, self.seed = float(rel), int(seed)

    def __enter__(self):
        lib().lo_set_solve_perturbation(self.rel, self.seed)
        return self

    def __exit__(self, *exc):
        lib().lo_set_solve_perturbation(0.0, 0)
        return False


class normwise_perturbation:
    """Context manager: inside it, every oracle Newton correction component
    moves by +- rel * max|dx| with seeded signs -- a linear solver accurate
    to rel normwise, as the mixed form's refinement is.  Single-threaded
    use only."""

    def __init__(self, rel: float, seed: int = 1):
        self.rel, self.seed = float(rel), int(seed)

    def __enter__(self):
        lib().lo_set_solve_perturbation_normwise(self.rel, self.seed)
        return self

    def __exit__(self, *exc):
        lib().lo_set_solve_perturbation(0.0, 0)
        return False


class root_perturbation:
    """Context manager: inside it, every RKF45 quarter root (atol/R)^(1/4)
    is scaled by (1 +- rel) with seeded signs -- a pow() that is off by an
    ulp.  Single-threaded use only."""

    def __init__(self, rel: float, seed: int = 1):
        self.rel, self.seed = float(rel), int(seed)

    def __enter__(self):
        lib().lo_set_root_perturbation(self.rel, self.seed)
        return self

    def __exit__(self, *exc):
        lib().lo_set_root_perturbation(0.0, 0)
        return False


class lu_variant:
    """Context manager: inside it the oracle's LU rounds in another valid
    order (1: triangular solves without fma, 2: Schur update without fma,
    3: both) -- another FP64 getrf/getrs that differs in the last bits only.
    Single-threaded use only."""

    def __init__(self, variant: int):
        self.variant = int(variant)

    def __enter__(self):
        lib().lo_set_lu_variant(self.variant)
        return self

    def __exit__(self, *exc):
        lib().lo_set_lu_variant(0)
        return False

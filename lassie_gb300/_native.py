"""ctypes binding of ``liblassie_gb300.so`` (the C ABI in
``include/lassie_gb300.h``).  Loading fails loudly when the library is
missing: there is no CPU fallback."""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_native", "liblassie_gb300.so")

OK = 0
ERR_ARGS = -20
ERR_MAX_STEPS = -21
ERR_ALLOC = -22
ERR_TOO_LARGE = -23
ERR_DEADLINE = -24
ERR_NO_DEVICE = -25
ERR_RECORD_FULL = -26
ERR_STEP_TOO_SMALL = -27
ERR_CUDA = -13
PREC_FP64 = 0
PREC_MIXED = 1
PREC_FLOAT = 2
CTRL_COMPAT = 0
CTRL_BDF = 1
ROOT_POW = 0
ROOT_SQRT = 1

# every function the header declares (checked by the CPU test suite)
EXPORTS = (
    "lassie_opts_default", "lassie_status_string", "lassie_last_error", "lassie_device_ok",
    "lassie_model_create_dense", "lassie_model_create_csr", "lassie_model_destroy",
    "lassie_model_info", "lassie_solve", "lassie_solve_batch", "lassie_batch_create",
    "lassie_batch_run", "lassie_batch_sync", "lassie_batch_read", "lassie_batch_launches",
    "lassie_batch_order_by_cost",
    "lassie_batch_bytes", "lassie_batch_destroy", "lassie_rhs_device", "lassie_rhs", "lassie_newton_matrix",
    "lassie_newton_matrix_device", "lassie_jacobian_nnz", "lassie_jacobian_pattern",
    "lassie_lu_solve", "lassie_adjoint_batch", "lassie_solve_noalloc", "lassie_batch_tile_rows", "lassie_tc_selftest", "lassie_tc_selftest_bf16",
)


class Opts(C.Structure):
    _fields_ = [("rkf_step", C.c_double), ("be_step", C.c_double),
                ("newton_tol", C.c_double), ("stiffness_tol", C.c_double),
                ("newton_iter", C.c_int64), ("max_steps", C.c_int64),
                ("deadline_s", C.c_double), ("precision", C.c_int32),
                ("refine_max", C.c_int32), ("quarter_root", C.c_int32), ("lu_reuse", C.c_int32),
                ("tensor_cores", C.c_int32), ("controller", C.c_int32),
                ("rtol", C.c_double), ("atol", C.c_double), ("first_step", C.c_double),
                ("max_step", C.c_double), ("max_order", C.c_int32), ("tile_rows", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("outer_iters", C.c_int64), ("rkf_accepts", C.c_int64),
                ("rkf_retries", C.c_int64), ("be_steps", C.c_int64),
                ("newton_iters", C.c_int64), ("lu_factorisations", C.c_int64),
                ("lu_failures", C.c_int64), ("nan_reverts", C.c_int64),
                ("refine_sweeps", C.c_int64), ("cycles_rkf", C.c_int64),
                ("cycles_matrix", C.c_int64), ("cycles_lu", C.c_int64),
                ("cycles_solve", C.c_int64), ("cycles_lu_panel", C.c_int64),
                ("cycles_lu_rows", C.c_int64), ("cycles_lu_trailing", C.c_int64),
                ("cycles_solve_tri", C.c_int64),
                ("t_final", C.c_double),
                ("dt_be_final", C.c_double), ("status", C.c_int32), ("pad", C.c_int32),
                ("jac_evals", C.c_int64), ("rhs_evals", C.c_int64),
                ("order_final", C.c_int32), ("pad2", C.c_int32),
                ("cycles_total", C.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("pad")}


class Instance(C.Structure):
    _fields_ = [("model", C.c_void_p), ("k", C.c_void_p), ("x0", C.c_void_p),
                ("feed", C.c_void_p), ("atol", C.c_void_p), ("t", C.c_void_p),
                ("nt", C.c_int32), ("ncs", C.c_int32), ("cs", C.c_void_p),
                ("out", C.c_void_p)]


class LassieError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        lib_ = _lib
        msg = ""
        if lib_ is not None:
            msg = lib_.lassie_status_string(status).decode()
            last = lib_.lassie_last_error().decode()
            if last:
                msg += f" ({last})"
        super().__init__(f"{where}: status {status}: {msg}")
        self.status = status


_lib = None
_lock = threading.Lock()


def load():
    """Load the library (building it first if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import build as _build
        _build.build()  # incremental: a no-op when the library is up to date
        L = C.CDLL(LIB_PATH)
        vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        L.lassie_opts_default.argtypes = [C.POINTER(Opts)]
        L.lassie_opts_default.restype = None
        L.lassie_status_string.argtypes = [C.c_int]
        L.lassie_status_string.restype = C.c_char_p
        L.lassie_last_error.argtypes = []
        L.lassie_last_error.restype = C.c_char_p
        L.lassie_device_ok.argtypes = []
        L.lassie_device_ok.restype = C.c_int
        L.lassie_model_create_dense.argtypes = [i32, i32, vp, vp, C.POINTER(vp)]
        L.lassie_model_create_csr.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, C.POINTER(vp)]
        L.lassie_model_destroy.argtypes = [vp]
        L.lassie_model_destroy.restype = None
        L.lassie_model_info.argtypes = [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32),
                                        C.POINTER(i32)]
        L.lassie_solve.argtypes = [vp, vp, vp, vp, vp, vp, i32, vp, i32, C.POINTER(Opts), vp,
                                   C.POINTER(Stats)]
        L.lassie_solve_batch.argtypes = [vp, i32, C.POINTER(Opts), vp]
        L.lassie_batch_create.argtypes = [vp, i32, C.POINTER(Opts), C.POINTER(vp)]
        L.lassie_batch_run.argtypes = [vp, vp]
        L.lassie_batch_sync.argtypes = [vp]
        L.lassie_batch_read.argtypes = [vp, vp, vp]
        L.lassie_batch_launches.argtypes = [vp]
        L.lassie_batch_order_by_cost.argtypes = [vp]
        L.lassie_batch_bytes.argtypes = [vp, C.POINTER(i64), C.POINTER(i64)]
        L.lassie_batch_tile_rows.argtypes = [vp, vp]
        L.lassie_batch_destroy.argtypes = [vp]
        L.lassie_batch_destroy.restype = None
        L.lassie_rhs_device.argtypes = [vp, i32, vp, vp, vp, vp]
        L.lassie_rhs.argtypes = [vp, vp, vp, vp]
        L.lassie_newton_matrix.argtypes = [vp, vp, vp, dbl, vp]
        L.lassie_newton_matrix_device.argtypes = [vp, i32, dbl, vp, vp, vp, i32, vp]
        L.lassie_jacobian_nnz.argtypes = [vp, C.POINTER(C.c_int64)]
        L.lassie_jacobian_pattern.argtypes = [vp, vp, vp]
        L.lassie_lu_solve.argtypes = [i32, vp, vp, vp, i32]
        L.lassie_adjoint_batch.argtypes = [vp, i32, vp, C.POINTER(Opts), i32, i32, vp, vp, vp, vp]
        L.lassie_solve_noalloc.argtypes = [vp, vp, vp, vp, i32, C.POINTER(Opts), vp,
                                           C.POINTER(Stats), vp]
        L.lassie_tc_selftest.argtypes = [vp, vp, vp, vp, vp]
        L.lassie_tc_selftest_bf16.argtypes = [vp, vp, vp, vp, vp]
        for name in EXPORTS:
            f = getattr(L, name)
            if f.restype is C.c_int and name not in ("lassie_device_ok",):
                f.restype = C.c_int
        _lib = L
        return L


def check(status: int, where: str) -> None:
    if status != OK:
        raise LassieError(status, where)

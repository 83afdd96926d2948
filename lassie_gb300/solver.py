"""Python API over the C ABI: compile networks, integrate one model or a
batch of instances on the GPU, evaluate the RHS / Newton matrix / LU.

Mirrors the reference's engine entry (``Simulation<T>::run``,
``Simulation.cuh:230-981``): the same options (``rkf_step``, ``be_step``,
``newton_iter``, ``newton_tol``, ``stiffness_tol``, ``atol_vector``,
``cs_vector``, ``M_feed``) and the same trajectory layout (one row per
sampling time, one column per sampled species).
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _native as nat
from .model import Model

# fp64: the plain FP64 GPU form; mixed: FP32 factors + FP64 refinement;
# float: the reference's single-precision mode (-p float)
ENGINES = {"fp64": nat.PREC_FP64, "mixed": nat.PREC_MIXED, "float": nat.PREC_FLOAT}


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


class NativeModel:
    """A network compiled by the C ABI (``lassie_model_create_dense``)."""

    def __init__(self, left: np.ndarray, right: np.ndarray):
        L = nat.load()
        self._left = np.ascontiguousarray(left, dtype=np.int32)
        self._right = np.ascontiguousarray(right, dtype=np.int32)
        R, N = self._left.shape
        h = C.c_void_p()
        nat.check(L.lassie_model_create_dense(N, R, self._left.ctypes.data,
                                              self._right.ctypes.data, C.byref(h)),
                  "lassie_model_create_dense")
        self.handle = h
        self.n_species, self.n_reactions = N, R

    @classmethod
    def of(cls, m: Model) -> "NativeModel":
        return cls(m.left, m.right)

    def info(self) -> Tuple[int, int, int, int]:
        v = [C.c_int32() for _ in range(4)]
        nat.check(nat.load().lassie_model_info(self.handle, *[C.byref(x) for x in v]),
                  "lassie_model_info")
        return tuple(int(x.value) for x in v)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and nat._lib is not None:
            nat._lib.lassie_model_destroy(h)
            self.handle = None


ROOTS = {"pow": nat.ROOT_POW, "sqrt": nat.ROOT_SQRT}
# rank updates of the wide engine's factorisation: FP32 pipes ("off"),
# tensor cores with split TF32 operands ("tf32", the default, or True), or
# BF16 operands with FP32 accumulation ("bf16")
TENSOR_CORES = {False: 0, True: 1, "off": 0, "tf32": 1, "bf16": 2}


BDF_KEYS = ("rtol", "atol", "first_step", "max_step", "max_order")


def make_opts(m: Optional[Model] = None, engine: str = "mixed", max_steps: int = 0,
              deadline_s: float = 0.0, refine_max: int = 0, root: str = "pow",
              lu_reuse: bool = True, tensor_cores="tf32",
              bdf: Optional[Dict] = None, tile_rows: int = 0) -> nat.Opts:
    """Options of a solve.  ``bdf`` (a dict, possibly empty, of rtol, atol,
    first_step, max_step, max_order) selects the BDF controller with rtol/atol
    error control instead of LASSIE's loop; ``engine`` then picks its Newton
    iteration matrix (fp64: FP64 LU; mixed: FP32 Gauss-Jordan inverse)."""
    o = nat.Opts()
    nat.load().lassie_opts_default(C.byref(o))
    if m is not None:
        o.rkf_step = m.rkf_step
        o.be_step = m.be_step
        o.newton_tol = m.newton_tol
        o.stiffness_tol = m.stiffness_tol
        o.newton_iter = int(m.newton_iter)
    o.max_steps = int(max_steps)
    o.deadline_s = float(deadline_s)
    o.precision = ENGINES[engine]
    o.refine_max = int(refine_max)
    o.quarter_root = ROOTS[root]
    o.lu_reuse = 1 if lu_reuse else 0
    o.tensor_cores = TENSOR_CORES[tensor_cores]
    o.tile_rows = int(tile_rows)
    if bdf is not None:
        unknown = set(bdf) - set(BDF_KEYS)
        if unknown:
            raise ValueError(f"unknown BDF options {sorted(unknown)}")
        o.controller = nat.CTRL_BDF
        for key, val in bdf.items():
            setattr(o, key, int(val) if key == "max_order" else float(val))
    return o


class _Packed:
    """Keeps the contiguous arrays of one instance alive."""

    def __init__(self, m: Model, nm: NativeModel):
        N = m.n_species
        self.nm = nm
        self.k = np.ascontiguousarray(m.k[: m.n_reactions], np.float64)
        self.x0 = np.ascontiguousarray(m.x0[:N], np.float64)
        self.feed = None if m.feed is None else np.ascontiguousarray(m.feed[:N], np.float64)
        self.atol = None if m.atol is None else np.ascontiguousarray(m.atol[:N], np.float64)
        self.t = np.ascontiguousarray(m.t, np.float64)
        self.cs = None if m.cs is None else np.ascontiguousarray(m.cs, np.int32)
        ncs = N if self.cs is None else self.cs.shape[0]
        self.out = np.zeros((self.t.shape[0], ncs))

    def instance(self) -> nat.Instance:
        I = nat.Instance()
        I.model = self.nm.handle
        I.k, I.x0, I.feed, I.atol, I.t = (_p(self.k), _p(self.x0), _p(self.feed),
                                          _p(self.atol), _p(self.t))
        I.nt = self.t.shape[0]
        I.ncs = 0 if self.cs is None else self.cs.shape[0]
        I.cs = _p(self.cs)
        I.out = _p(self.out)
        return I


def simulate(m: Model, engine: str = "mixed", max_steps: int = 0, deadline_s: float = 0.0,
             nm: Optional[NativeModel] = None, root: str = "pow",
             lu_reuse: bool = True, tensor_cores="tf32",
             bdf: Optional[Dict] = None, refine_max: int = 0) -> Tuple[np.ndarray, Dict]:
    """Integrate one model on the GPU.  Returns (trajectory [nt, ncs], stats)."""
    nm = nm or NativeModel.of(m)
    pk = _Packed(m, nm)
    st = nat.Stats()
    o = make_opts(m, engine, max_steps, deadline_s, refine_max=refine_max, root=root,
                  lu_reuse=lu_reuse, tensor_cores=tensor_cores, bdf=bdf)
    rc = nat.load().lassie_solve(nm.handle, _p(pk.k), _p(pk.x0), _p(pk.feed), _p(pk.atol),
                                 _p(pk.t), pk.t.shape[0], _p(pk.cs),
                                 0 if pk.cs is None else pk.cs.shape[0], C.byref(o),
                                 _p(pk.out), C.byref(st))
    stats = st.as_dict()
    if rc not in (nat.OK, nat.ERR_MAX_STEPS, nat.ERR_DEADLINE, nat.ERR_STEP_TOO_SMALL):
        nat.check(rc, "lassie_solve")
    stats["status"] = rc
    return pk.out, stats


class Batch:
    """A device-resident batch (``lassie_batch_*``): inputs uploaded once,
    ``run()`` launches the persistent integrator on `stream`."""

    def __init__(self, models: Sequence[Model], engine: str = "mixed", max_steps: int = 0,
                 deadline_s: float = 0.0, native: Optional[Sequence[NativeModel]] = None,
                 refine_max: int = 0, root: str = "pow", lu_reuse: bool = True,
                 tensor_cores="tf32", bdf: Optional[Dict] = None, tile_rows: int = 0):
        L = nat.load()
        cache: Dict[int, NativeModel] = {}
        self.packs = []
        for q, m in enumerate(models):
            if native is not None:
                nm = native[q]
            else:
                key = id(m.left)
                nm = cache.get(key)
                if nm is None:
                    nm = cache[key] = NativeModel.of(m)
            self.packs.append(_Packed(m, nm))
        self.n = len(models)
        self._inst = (nat.Instance * max(self.n, 1))(*[p.instance() for p in self.packs])
        self.opts = make_opts(models[0] if self.n else None, engine, max_steps, deadline_s,
                              refine_max, root, lu_reuse, tensor_cores, bdf, tile_rows)
        h = C.c_void_p()
        nat.check(L.lassie_batch_create(C.cast(self._inst, C.c_void_p), self.n,
                                        C.byref(self.opts), C.byref(h)), "lassie_batch_create")
        self.handle = h

    def run(self, stream: int = 0) -> None:
        nat.check(nat.load().lassie_batch_run(self.handle, C.c_void_p(stream or None)),
                  "lassie_batch_run")

    def sync(self) -> None:
        nat.check(nat.load().lassie_batch_sync(self.handle), "lassie_batch_sync")

    def tile_rows(self) -> List[int]:
        """Rows per thread of each instance's factorisation tiles (8, 4 or 2),
        as fixed by the options or chosen by the autotuner."""
        rows = (C.c_int32 * max(self.n, 1))()
        nat.check(nat.load().lassie_batch_tile_rows(self.handle, C.cast(rows, C.c_void_p)),
                  "lassie_batch_tile_rows")
        return [int(rows[q]) for q in range(self.n)]

    def launches(self) -> int:
        return int(nat.load().lassie_batch_launches(self.handle))

    def order_by_cost(self) -> None:
        """Later runs take the instances longest first, by the last run's
        per-instance integration times (``lassie_batch_order_by_cost``); no
        result changes."""
        nat.check(nat.load().lassie_batch_order_by_cost(self.handle),
                  "lassie_batch_order_by_cost")

    def transfer_bytes(self) -> Tuple[int, int]:
        h2d, d2h = C.c_int64(), C.c_int64()
        nat.check(nat.load().lassie_batch_bytes(self.handle, C.byref(h2d), C.byref(d2h)),
                  "lassie_batch_bytes")
        return int(h2d.value), int(d2h.value)

    def read(self) -> Tuple[List[np.ndarray], List[Dict]]:
        stats = (nat.Stats * max(self.n, 1))()
        rc = nat.load().lassie_batch_read(self.handle, C.cast(self._inst, C.c_void_p),
                                          C.cast(stats, C.c_void_p))
        if rc not in (nat.OK, nat.ERR_MAX_STEPS, nat.ERR_DEADLINE, nat.ERR_STEP_TOO_SMALL):
            nat.check(rc, "lassie_batch_read")
        return [p.out for p in self.packs], [stats[q].as_dict() for q in range(self.n)]

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and nat._lib is not None:
            nat._lib.lassie_batch_destroy(h)
            self.handle = None


def simulate_batch(models: Sequence[Model], engine: str = "mixed", max_steps: int = 0,
                   deadline_s: float = 0.0, root: str = "pow",
                   lu_reuse: bool = True, bdf: Optional[Dict] = None,
                   tile_rows: int = 0) -> Tuple[List[np.ndarray], List[Dict]]:
    """Integrate independent instances in one persistent launch (host buffers
    in and out, ``lassie_solve_batch``)."""
    L = nat.load()
    cache: Dict[int, NativeModel] = {}
    packs = []
    for m in models:
        nm = cache.get(id(m.left))
        if nm is None:
            nm = cache[id(m.left)] = NativeModel.of(m)
        packs.append(_Packed(m, nm))
    n = len(models)
    inst = (nat.Instance * max(n, 1))(*[p.instance() for p in packs])
    stats = (nat.Stats * max(n, 1))()
    o = make_opts(models[0] if n else None, engine, max_steps, deadline_s, root=root,
                  lu_reuse=lu_reuse, bdf=bdf, tile_rows=tile_rows)
    rc = L.lassie_solve_batch(C.cast(inst, C.c_void_p), n, C.byref(o), C.cast(stats, C.c_void_p))
    if rc not in (nat.OK, nat.ERR_MAX_STEPS, nat.ERR_DEADLINE, nat.ERR_STEP_TOO_SMALL):
        nat.check(rc, "lassie_solve_batch")
    return [p.out for p in packs], [stats[q].as_dict() for q in range(n)]


def rhs(m: Model, x: np.ndarray, k: Optional[np.ndarray] = None,
        nm: Optional[NativeModel] = None) -> np.ndarray:
    """f(x) for one state (``lassie_rhs``)."""
    nm = nm or NativeModel.of(m)
    k = np.ascontiguousarray(m.k if k is None else k, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    dx = np.zeros(m.n_species)
    nat.check(nat.load().lassie_rhs(nm.handle, k.ctypes.data, x.ctypes.data, dx.ctypes.data),
              "lassie_rhs")
    return dx


def newton_matrix(m: Model, x: np.ndarray, h: float, k: Optional[np.ndarray] = None,
                  nm: Optional[NativeModel] = None) -> np.ndarray:
    """I - h*J(x) as a dense FP64 matrix (``lassie_newton_matrix``)."""
    nm = nm or NativeModel.of(m)
    k = np.ascontiguousarray(m.k if k is None else k, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    M = np.zeros((m.n_species, m.n_species))
    nat.check(nat.load().lassie_newton_matrix(nm.handle, k.ctypes.data, x.ctypes.data,
                                              float(h), M.ctypes.data),
              "lassie_newton_matrix")
    return M


def lu_solve(a: np.ndarray, b: np.ndarray, engine: str = "fp64") -> Tuple[np.ndarray, int]:
    """Factor and solve with the engine's per-CTA LU.  Returns (x, info);
    info > 0 is 1 + the column of an exactly zero pivot."""
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(a.shape[0])
    rc = nat.load().lassie_lu_solve(a.shape[0], a.ctypes.data, b.ctypes.data, x.ctypes.data,
                                    ENGINES[engine])
    if rc < 0:
        nat.check(rc, "lassie_lu_solve")
    return x, rc

"""Reaction-network model: LASSIE input-folder I/O and the sparse model compiler.

The input folder is the reference's drop-in format (``simulator.cu:79-152``):
mandatory ``left_side``, ``right_side`` (R rows x N tab-separated integers),
``c_vector`` (R lines), ``t_vector`` (lines), ``M_0`` (tab-separated), and the
optional ``cs_vector``, ``M_feed``, ``modelkind``, ``volume``, ``atol_vector``,
``be_step``, ``rkf_step``, ``newton_iter``, ``newton_tol``, ``stiffness_tol``
and ``alphabet`` (detected, unused).  Parsing follows ``Reader.h:23-134``:
every line read by ``getline`` yields one value, tokens split on TAB, numbers
parsed with ``strtod`` semantics (longest numeric prefix, 0 when none).
"""
from __future__ import annotations

import dataclasses
import os
import re
from typing import Dict, List, Optional, Sequence

import numpy as np

AVOGADRO = 6.022e23  # Simulation.cuh:985

MANDATORY = ("left_side", "right_side", "c_vector", "t_vector", "M_0")
OPTIONAL = ("cs_vector", "M_feed", "modelkind", "atol_vector", "alphabet",
            "be_step", "newton_iter", "newton_tol", "rkf_step",
            "stiffness_tol", "volume")

_STRTOD = re.compile(
    r"^[ \t\n\v\f\r]*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?"
    r"|inf(?:inity)?|nan))", re.IGNORECASE)


def strtod(text: str) -> float:
    """Value of the longest numeric prefix of ``text`` (C ``strtod``), else 0."""
    m = _STRTOD.match(text)
    if not m:
        return 0.0
    return float(m.group(1))


def _trunc_int(v: float) -> int:
    """``(int) strtod(...)``: truncation toward zero."""
    if v != v or v in (float("inf"), float("-inf")):
        return 0
    return int(v)


def _getline_lines(path: str) -> List[str]:
    """Lines as ``std::getline`` returns them (no extra empty last line)."""
    with open(path, "r", newline="") as f:
        data = f.read()
    if data == "":
        return []
    lines = data.split("\n")
    if data.endswith("\n"):
        lines.pop()
    return lines


def _tab_tokens(line: str) -> List[str]:
    """Tokens of ``getline(buf, token, '\\t')``: a trailing TAB adds nothing."""
    toks = line.split("\t")
    if toks and toks[-1] == "" and line.endswith("\t"):
        toks.pop()
    if line == "":
        return []
    return toks


def read_matrix(path: str) -> np.ndarray:
    """``Reader.h:104-124`` readMatrix.  Lines without tokens are skipped (the
    reference would index past the end of such a row)."""
    rows = []
    for line in _getline_lines(path):
        toks = _tab_tokens(line)
        if not toks:
            continue
        rows.append([_trunc_int(strtod(t)) for t in toks])
    if not rows:
        raise ValueError(f"{path}: empty stoichiometry matrix")
    width = len(rows[0])
    for r in rows:
        if len(r) != width:
            raise ValueError(f"{path}: ragged stoichiometry matrix")
    return np.asarray(rows, dtype=np.int32)


def read_by_line(path: str) -> np.ndarray:
    """``Reader.h:38-51`` readByLine: one value per line."""
    return np.asarray([strtod(l) for l in _getline_lines(path)], dtype=np.float64)


def read_by_tab(path: str) -> np.ndarray:
    """``Reader.h:53-69`` readByTab: TAB-separated values over all lines."""
    vals = []
    for line in _getline_lines(path):
        vals.extend(strtod(t) for t in _tab_tokens(line))
    return np.asarray(vals, dtype=np.float64)


def read_by_line_int(path: str) -> np.ndarray:
    """``Reader.h:89-102`` readByLineshort."""
    return np.asarray([_trunc_int(strtod(l)) for l in _getline_lines(path)],
                      dtype=np.int32)


def read_single(path: str) -> float:
    """``Reader.h:126-134`` readSingleValue: first line."""
    lines = _getline_lines(path)
    return strtod(lines[0]) if lines else 0.0


def read_type(path: str) -> int:
    """``Reader.h:23-36`` readType: 0 deterministic/concentration,
    1 stochastic/number, 2 otherwise."""
    lines = _getline_lines(path)
    first = lines[0] if lines else ""
    if first in ("deterministic", "concentration"):
        return 0
    if first in ("stochastic", "number"):
        return 1
    return 2


class InputError(Exception):
    """Input-folder error carrying the reference's process exit code."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


@dataclasses.dataclass
class Model:
    """A mass-action network plus one parameterisation and integration setup.

    ``left``/``right`` are the dense R x N reactant/product stoichiometries
    (``left_side``/``right_side``); ``k`` the R rate constants; ``x0`` and
    ``feed`` the N initial and constant (fed) amounts; ``t`` the sampling
    times; ``cs`` the sampled species.  Values are already deterministic
    (concentration) units; ``volume`` records a stochastic model's volume so
    outputs can be converted back (``Simulation.cuh:953-958``).
    """

    left: np.ndarray
    right: np.ndarray
    k: np.ndarray
    x0: np.ndarray
    t: np.ndarray
    cs: Optional[np.ndarray] = None
    feed: Optional[np.ndarray] = None
    atol: Optional[np.ndarray] = None
    rkf_step: float = 1e-3
    be_step: float = 0.01
    newton_iter: int = 10000
    newton_tol: float = 1e-6
    stiffness_tol: float = 1e-6
    modelkind: int = 0
    volume: float = 1.0

    @property
    def n_species(self) -> int:
        return int(self.left.shape[1])

    @property
    def n_reactions(self) -> int:
        return int(self.left.shape[0])

    def sampled(self) -> np.ndarray:
        if self.cs is None:
            return np.arange(self.n_species, dtype=np.int32)
        return np.asarray(self.cs, dtype=np.int32)

    def validate(self) -> None:
        R, N = self.left.shape
        if self.right.shape != (R, N):
            raise InputError(-4, "left_side and right_side differ in shape")
        if self.k.shape[0] < R:
            raise InputError(-4, "c_vector has fewer entries than reactions")
        if self.x0.shape[0] < N:
            raise InputError(-4, "M_0 has fewer entries than species")
        cs = self.sampled()
        if cs.size and (cs.min() < 0 or cs.max() >= N):
            raise InputError(-4, "cs_vector names a species out of range")


def load_folder(path: str) -> Model:
    """Read a LASSIE input folder (``simulator.cu:79-195``,
    ``Simulation.cuh:250-391``), applying the stochastic-to-deterministic
    conversion (``Simulation.cuh:983-1031``) when ``modelkind`` asks for it."""
    if not os.path.isdir(path):
        raise InputError(-1, "the input folder does not exist")
    present = {f for f in os.listdir(path) if f not in (".", "..", ".DS_Store")}
    missing = [f for f in MANDATORY if f not in present]
    if missing:
        raise InputError(-4, "missing mandatory files: " + ", ".join(missing))
    p = lambda f: os.path.join(path, f)  # noqa: E731
    left = read_matrix(p("left_side"))
    right = read_matrix(p("right_side"))
    k = read_by_line(p("c_vector"))
    t = read_by_line(p("t_vector"))
    x0 = read_by_tab(p("M_0"))
    N = left.shape[1]
    m = Model(left=left, right=right, k=k, x0=x0, t=t)
    if "be_step" in present:
        m.be_step = read_single(p("be_step"))
    if "rkf_step" in present:
        m.rkf_step = read_single(p("rkf_step"))
    if "newton_iter" in present:
        m.newton_iter = int(read_single(p("newton_iter")))
    if "newton_tol" in present:
        m.newton_tol = read_single(p("newton_tol"))
    if "stiffness_tol" in present:
        m.stiffness_tol = read_single(p("stiffness_tol"))
    if "atol_vector" in present:
        m.atol = read_by_line(p("atol_vector"))
    if "cs_vector" in present:
        m.cs = read_by_line_int(p("cs_vector"))
    if "M_feed" in present:
        m.feed = read_by_tab(p("M_feed"))
    if "modelkind" in present:
        m.modelkind = read_type(p("modelkind"))
    if m.modelkind == 2:
        raise InputError(-7, "the modelkind can be: deterministic/concentration "
                             "or stochastic/number")
    if m.modelkind:
        vol = read_single(p("volume")) if "volume" in present else 0.0
        if vol == 0:
            raise InputError(-8, "the modelkind is stochastic/number, but there "
                                 "is not volume file")
        m.volume = vol
        to_deterministic(m)
    if m.atol is not None and m.atol.shape[0] < N:
        raise InputError(-4, "atol_vector has fewer entries than species")
    if m.feed is not None and m.feed.shape[0] < N:
        raise InputError(-4, "M_feed has fewer entries than species")
    m.validate()
    return m


def to_deterministic(m: Model) -> None:
    """``Simulation.cuh:983-1031``: amounts / (V*N_A); a reaction with a
    reactant of stoichiometry >= 2 gets k*V*N_A/2, one with two or more
    reactant species k*V*N_A; three or more reactant species is an error."""
    conv = m.volume * AVOGADRO
    m.x0 = m.x0 / conv
    if m.feed is not None:
        m.feed = m.feed / conv
    k = m.k.copy()
    for i in range(k.shape[0]):
        row = m.left[i] if i < m.left.shape[0] else np.zeros(1, np.int32)
        nz = int(np.count_nonzero(row > 0))
        if nz >= 3:
            raise InputError(-12, "There are one or more reactions with higher "
                                  "order than the second one")
        if np.any(row >= 2):
            k[i] = (k[i] * conv) / 2.0
        elif nz > 1:
            k[i] = k[i] * conv
    m.k = k


def write_folder(m: Model, path: str, digits: int = 17) -> None:
    """Write ``m`` as a LASSIE input folder (deterministic units)."""
    os.makedirs(path, exist_ok=True)
    fmt = f"%.{digits}g"

    def wlines(name, vals, f=fmt):
        with open(os.path.join(path, name), "w") as fh:
            for v in vals:
                fh.write((f % v) + "\n")

    for name, mat in (("left_side", m.left), ("right_side", m.right)):
        with open(os.path.join(path, name), "w") as fh:
            for row in mat:
                fh.write("\t".join(str(int(v)) for v in row) + "\n")
    wlines("c_vector", m.k[: m.n_reactions])
    wlines("t_vector", m.t)
    with open(os.path.join(path, "M_0"), "w") as fh:
        fh.write("\t".join(fmt % v for v in m.x0[: m.n_species]) + "\n")
    if m.cs is not None:
        wlines("cs_vector", m.cs, "%d")
    if m.feed is not None:
        with open(os.path.join(path, "M_feed"), "w") as fh:
            fh.write("\t".join(fmt % v for v in m.feed[: m.n_species]) + "\n")
    if m.atol is not None:
        wlines("atol_vector", m.atol)
    defaults = Model(left=m.left, right=m.right, k=m.k, x0=m.x0, t=m.t)
    for name in ("be_step", "rkf_step", "newton_tol", "stiffness_tol"):
        if getattr(m, name) != getattr(defaults, name):
            wlines(name, [getattr(m, name)])
    if m.newton_iter != defaults.newton_iter:
        wlines("newton_iter", [m.newton_iter], "%d")


# --------------------------------------------------------------- compiler

@dataclasses.dataclass
class CompiledModel:
    """Sparse encodings of a network (``Simulation.cuh:397-418,1061-1130``),
    with int32 indices.

    ``rxn_ptr``/``rxn_species``/``rxn_stoich``: reactant CSR by reaction,
    species ascending.  ``sp_ptr``/``sp_rxn``/``sp_coef``: CSR of the net
    stoichiometry H = (B - A)^T by species, reactions ascending -- the order in
    which the reference sums each species' derivative (``kernels.cuh:16-47``).
    """

    n_species: int
    n_reactions: int
    rxn_ptr: np.ndarray
    rxn_species: np.ndarray
    rxn_stoich: np.ndarray
    sp_ptr: np.ndarray
    sp_rxn: np.ndarray
    sp_coef: np.ndarray


def compile_model(left: np.ndarray, right: np.ndarray) -> CompiledModel:
    left = np.asarray(left, dtype=np.int32)
    right = np.asarray(right, dtype=np.int32)
    R, N = left.shape
    rr, ss = np.nonzero(left)
    rxn_ptr = np.zeros(R + 1, np.int32)
    np.add.at(rxn_ptr, rr + 1, 1)
    rxn_ptr = np.cumsum(rxn_ptr).astype(np.int32)
    H = (right - left).T  # N x R
    si, rj = np.nonzero(H)
    sp_ptr = np.zeros(N + 1, np.int32)
    np.add.at(sp_ptr, si + 1, 1)
    sp_ptr = np.cumsum(sp_ptr).astype(np.int32)
    return CompiledModel(
        n_species=N, n_reactions=R,
        rxn_ptr=rxn_ptr, rxn_species=ss.astype(np.int32),
        rxn_stoich=left[rr, ss].astype(np.int32),
        sp_ptr=sp_ptr, sp_rxn=rj.astype(np.int32),
        sp_coef=H[si, rj].astype(np.int32))


def rhs_numpy(cm: CompiledModel, k: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Vectorised mass-action derivative (any summation order): for quick
    host-side checks only."""
    prop = np.array(k[: cm.n_reactions], dtype=np.float64, copy=True)
    r_of = np.repeat(np.arange(cm.n_reactions), np.diff(cm.rxn_ptr))
    np.multiply.at(prop, r_of, x[cm.rxn_species] ** cm.rxn_stoich)
    s_of = np.repeat(np.arange(cm.n_species), np.diff(cm.sp_ptr))
    dx = np.zeros(cm.n_species)
    np.add.at(dx, s_of, cm.sp_coef * prop[cm.sp_rxn])
    return dx

"""Seeded synthetic mass-action workloads.

Five workload shapes, each generated from ``numpy.random.default_rng(seed)``
with ``seed = 1000 * config + instance``:

* ``c1``: 64 species x 64 reactions; 1-2 distinct reactants (stoichiometry 1),
  0-2 products; k = 10^U(-3,0); x0 ~ U(0,1); t = linspace(0, 10, 100).
* ``c2``: 512 x 512 stiff; order 0/1/2 (order 2 is A+B or 2A), 1-2 products
  of stoichiometry 1-2; k = 10^U(-6,6); x0 = 10^U(-3,1); t = linspace(0,100,200).
* ``c3``: 4096 x 4096; exactly 2 reactants and 2 products (stoichiometry 1);
  k = 10^U(-4,2); x0 ~ U(0,1); t = linspace(0, 50, 100).
* ``c4``: batch of 2048 instances; N_i ~ U{32..512}, R_i = N_i, the c1
  structure; k = 10^U(-4,4) per instance; x0 ~ U(0,1); t = linspace(0,20,50).
* ``c5``: one 256 x 256 c1-structured model with k = 10^U(-3,3), 64 copies;
  targets from k * exp(N(0, 0.3^2)); 40 samples in (0, 10].

Products are drawn independently of the reactants, so a species may be both
consumed and produced by one reaction (its net coefficient is then B - A).

10^u and exp(x) are computed correctly rounded (``pow10``, ``exp_rn``) from
IEEE additions and multiplications only, so that a seed gives the same
network bit for bit on every machine: numpy's vectorised power differs from
the correctly rounded value on about 5 % of inputs on x86 (and differently
on Arm), which would change the rate constants in their last bits between
the machine that makes a fixture and the one that checks it.
"""
from __future__ import annotations

from typing import List, Optional, Tuple

import numpy as np

from .model import Model

# ------------------------------------------ correctly rounded 10^u and exp(x)
# Double-double arithmetic (error-free sums and products; Dekker's split, so
# that no fused operation is needed): exp(g) for |g| <= ln 2 / 2 by its Taylor
# series to 28 terms, 2^n by ldexp.  The double-double result carries about
# 104 correct bits, so rounding it to a double is correctly rounded except
# within 2^-104 of a tie, which the seeded inputs never come near.

_SPLIT = 134217729.0  # 2^27 + 1


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _split(a):
    c = _SPLIT * a
    hi = c - (c - a)
    return hi, a - hi


def _two_prod(a, b):
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl


def _dd_mul(ah, al, bh, bl):
    p, e = _two_prod(ah, bh)
    e = e + (ah * bl + al * bh)
    return _two_sum(p, e)


def _dd_add(ah, al, bh, bl):
    s, e = _two_sum(ah, bh)
    e = e + (al + bl)
    return _two_sum(s, e)


def _dd_const(num: str):
    """A decimal constant as an unevaluated double-double (hi, lo)."""
    from decimal import Decimal, getcontext
    getcontext().prec = 60
    d = Decimal(num)
    hi = float(d)
    return hi, float(d - Decimal(hi))


_LN2 = _dd_const("0.693147180559945309417232121458176568075500134360255254120680")
_LN10 = _dd_const("2.30258509299404568401799145468436420760110148862877297603333")
_INV_LN2 = _dd_const("1.44269504088896340735992468100189213742664595415298593413544")


def _inv_factorials(n: int):
    from decimal import Decimal, getcontext
    getcontext().prec = 60
    out, f = [], Decimal(1)
    for k in range(n + 1):
        if k:
            f *= k
        v = Decimal(1) / f
        hi = float(v)
        out.append((hi, float(v - Decimal(hi))))
    return out


_INV_FACT = _inv_factorials(28)


def _exp_dd(gh, gl):
    """exp(g) for a double-double g (any moderate size): g = n ln2 + r."""
    n = np.rint(gh * _INV_LN2[0])
    ph, pl = _dd_mul(n, np.zeros_like(n), _LN2[0], _LN2[1])
    rh, rl = _dd_add(gh, gl, -ph, -pl)
    # Horner: sum_k r^k / k!
    sh, sl = _INV_FACT[-1][0] + np.zeros_like(rh), _INV_FACT[-1][1] + np.zeros_like(rh)
    for k in range(len(_INV_FACT) - 2, -1, -1):
        sh, sl = _dd_mul(sh, sl, rh, rl)
        sh, sl = _dd_add(sh, sl, _INV_FACT[k][0], _INV_FACT[k][1])
    hi, lo = _two_sum(sh, sl)  # hi = the rounded sum
    return np.ldexp(hi, n.astype(np.int64))


def exp_rn(x) -> np.ndarray:
    """exp(x) correctly rounded (moderate |x|, normal results)."""
    x = np.asarray(x, np.float64)
    return _exp_dd(x, np.zeros_like(x))


def pow10(u) -> np.ndarray:
    """10^u correctly rounded (moderate |u|, normal results)."""
    u = np.asarray(u, np.float64)
    gh, gl = _dd_mul(u, np.zeros_like(u), _LN10[0], _LN10[1])
    return _exp_dd(gh, gl)


def _structure(rng: np.random.Generator, N: int, R: int, kind: str
               ) -> Tuple[np.ndarray, np.ndarray]:
    left = np.zeros((R, N), np.int32)
    right = np.zeros((R, N), np.int32)
    for j in range(R):
        if kind == "c1":
            nr = int(rng.integers(1, 3))
            sp = rng.choice(N, size=nr, replace=False)
            left[j, sp] = 1
            npd = int(rng.integers(0, 3))
            if npd:
                right[j, rng.choice(N, size=npd, replace=False)] = 1
        elif kind == "c2":
            order = int(rng.integers(0, 3))
            if order == 1:
                left[j, int(rng.integers(0, N))] = 1
            elif order == 2:
                if rng.random() < 0.5:
                    left[j, rng.choice(N, size=2, replace=False)] = 1
                else:
                    left[j, int(rng.integers(0, N))] = 2
            npd = int(rng.integers(1, 3))
            sp = rng.choice(N, size=npd, replace=False)
            right[j, sp] = rng.integers(1, 3, size=npd)
        elif kind == "c3":
            left[j, rng.choice(N, size=2, replace=False)] = 1
            right[j, rng.choice(N, size=2, replace=False)] = 1
        else:
            raise ValueError(kind)
    return left, right


def make_c1(instance: int = 0) -> Model:
    rng = np.random.default_rng(1000 * 1 + instance)
    N = R = 64
    left, right = _structure(rng, N, R, "c1")
    k = pow10(rng.uniform(-3.0, 0.0, R))
    x0 = rng.uniform(0.0, 1.0, N)
    return Model(left=left, right=right, k=k, x0=x0, t=np.linspace(0.0, 10.0, 100))


def make_c2(instance: int = 0) -> Model:
    rng = np.random.default_rng(1000 * 2 + instance)
    N = R = 512
    left, right = _structure(rng, N, R, "c2")
    k = pow10(rng.uniform(-6.0, 6.0, R))
    x0 = pow10(rng.uniform(-3.0, 1.0, N))
    return Model(left=left, right=right, k=k, x0=x0, t=np.linspace(0.0, 100.0, 200))


def make_c3(instance: int = 0) -> Model:
    rng = np.random.default_rng(1000 * 3 + instance)
    N = R = 4096
    left, right = _structure(rng, N, R, "c3")
    k = pow10(rng.uniform(-4.0, 2.0, R))
    x0 = rng.uniform(0.0, 1.0, N)
    return Model(left=left, right=right, k=k, x0=x0, t=np.linspace(0.0, 50.0, 100))


def make_c4_instance(instance: int) -> Model:
    rng = np.random.default_rng(1000 * 4 + instance)
    N = int(rng.integers(32, 513))
    left, right = _structure(rng, N, N, "c1")
    k = pow10(rng.uniform(-4.0, 4.0, N))
    x0 = rng.uniform(0.0, 1.0, N)
    return Model(left=left, right=right, k=k, x0=x0, t=np.linspace(0.0, 20.0, 50))


def make_sized(N: int, instance: int = 0) -> Model:
    """The batched workload's recipe (c1 structure, k = 10^U(-4,4), x0 ~
    U(0,1), t = linspace(0, 20, 50)) at a chosen size, seed (4, N, instance):
    networks above the batched engine's 512 species for the wide engine."""
    rng = np.random.default_rng((4, N, instance))
    left, right = _structure(rng, N, N, "c1")
    k = pow10(rng.uniform(-4.0, 4.0, N))
    x0 = rng.uniform(0.0, 1.0, N)
    return Model(left=left, right=right, k=k, x0=x0, t=np.linspace(0.0, 20.0, 50))


def c4_sizes(n_instances: int = 2048, first: int = 0) -> List[int]:
    """Species counts of the batched workload's instances (the first draw of
    each instance's generator), without building the networks."""
    return [int(np.random.default_rng(1000 * 4 + q).integers(32, 513))
            for q in range(first, first + n_instances)]


def make_c4(n_instances: int = 2048, first: int = 0) -> List[Model]:
    return [make_c4_instance(first + q) for q in range(n_instances)]


def make_c5(n_copies: int = 64) -> Tuple[List[Model], np.ndarray]:
    """Base model copies and the perturbed rate constants of each copy's
    target trajectory (``k * exp(N(0, 0.3^2))``)."""
    rng = np.random.default_rng(1000 * 5)
    N = R = 256
    left, right = _structure(rng, N, R, "c1")
    k = pow10(rng.uniform(-3.0, 3.0, R))
    x0 = rng.uniform(0.0, 1.0, N)
    t = np.linspace(0.0, 10.0, 41)[1:]
    base = [Model(left=left, right=right, k=k.copy(), x0=x0.copy(), t=t.copy())
            for _ in range(n_copies)]
    k_target = np.stack([k * exp_rn(rng.normal(0.0, 0.3, R)) for _ in range(n_copies)])
    return base, k_target


def shorten(m: Model, t_end: float, n_samples: int) -> Model:
    """Same network and parameters on a shorter horizon (parity tests at sizes
    the CPU oracle finishes in seconds)."""
    import dataclasses
    return dataclasses.replace(m, t=np.linspace(0.0, t_end, n_samples))


def make(config: str, instance: int = 0) -> Model:
    return {"c1": make_c1, "c2": make_c2, "c3": make_c3,
            "c4": make_c4_instance}[config](instance)


def tiny_network(kind: str, k: Optional[np.ndarray] = None) -> Model:
    """Closed-form known-answer networks (N <= 3)."""
    t = np.linspace(0.0, 2.0, 21)
    if kind == "decay":            # A -> 0,    x = x0 exp(-k t)
        left = np.array([[1]]); right = np.array([[0]])
        kk = np.array([0.7]); x0 = np.array([1.5])
    elif kind == "conversion":     # A -> B
        left = np.array([[1, 0]]); right = np.array([[0, 1]])
        kk = np.array([1.3]); x0 = np.array([1.0, 0.25])
    elif kind == "dimer":          # 2A -> B,   x_A = x0 / (1 + 2 k x0 t)
        left = np.array([[2, 0]]); right = np.array([[0, 1]])
        kk = np.array([0.5]); x0 = np.array([1.0, 0.0])
    elif kind == "bimolecular":    # A + B -> C
        left = np.array([[1, 1, 0]]); right = np.array([[0, 0, 1]])
        kk = np.array([0.8]); x0 = np.array([1.0, 0.6, 0.0])
    elif kind == "source":         # 0 -> A,    x = x0 + k t
        left = np.array([[0]]); right = np.array([[1]])
        kk = np.array([0.3]); x0 = np.array([0.2])
    elif kind == "reversible":     # A + B <-> C, conserves A+C and B+C
        left = np.array([[1, 1, 0], [0, 0, 1]])
        right = np.array([[0, 0, 1], [1, 1, 0]])
        kk = np.array([2.0, 0.5]); x0 = np.array([1.0, 0.8, 0.1])
    else:
        raise ValueError(kind)
    return Model(left=left.astype(np.int32), right=right.astype(np.int32),
                 k=kk if k is None else np.asarray(k, np.float64), x0=x0.astype(np.float64), t=t)

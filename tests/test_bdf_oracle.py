"""The standard controller's CPU restatement (oracle/lassie_oracle_bdf.c):
variable-order BDF with rtol/atol control.  Pinned against closed-form
solutions, against a tight-tolerance LSODA solution (scipy), and against
scipy's own BDF (the published algorithm it restates) for accuracy."""
import math

import os

import numpy as np
import pytest

from lassie_gb300 import synth
from oracle import oracle as O

RTOL, ATOL = 1e-6, 1e-9


def _tight(m, om):
    from scipy.integrate import solve_ivp
    sol = solve_ivp(lambda t, x: om.rhs(m.k, x), (m.t[0], m.t[-1]), m.x0, method="LSODA",
                    t_eval=m.t, rtol=1e-12, atol=1e-14,
                    jac=lambda t, x: om.jacobian_exact(m.k, x))
    assert sol.success
    return sol.y.T


def _scipy_bdf(m, om):
    from scipy.integrate import solve_ivp
    sol = solve_ivp(lambda t, x: om.rhs(m.k, x), (m.t[0], m.t[-1]), m.x0, method="BDF",
                    t_eval=m.t, rtol=RTOL, atol=ATOL,
                    jac=lambda t, x: om.jacobian_exact(m.k, x))
    assert sol.success
    return sol.y.T


def _err_over_tol(a, ref):
    return float(np.max(np.abs(a - ref) / (ATOL + RTOL * np.abs(ref))))


def test_closed_forms():
    # A -> 0: x = x0 exp(-k t)
    m = synth.tiny_network("decay")
    out, st, rc = O.solve_bdf(m, rtol=RTOL, atol=ATOL)
    assert rc == 0 and st["steps"] > 0
    ref = m.x0[0] * np.exp(-m.k[0] * m.t)
    assert np.max(np.abs(out[:, 0] - ref) / (ATOL + RTOL * ref)) < 50
    # 2A -> B: x_A = x0 / (1 + 2 k x0 t)
    m = synth.tiny_network("dimer")
    out, st, rc = O.solve_bdf(m, rtol=RTOL, atol=ATOL)
    assert rc == 0
    ref = m.x0[0] / (1 + 2 * m.k[0] * m.x0[0] * m.t)
    assert np.max(np.abs(out[:, 0] - ref) / (ATOL + RTOL * ref)) < 50
    # 0 -> A: linear, exact for every BDF order
    m = synth.tiny_network("source")
    out, st, rc = O.solve_bdf(m, rtol=RTOL, atol=ATOL)
    assert rc == 0
    assert np.allclose(out[:, 0], m.x0[0] + m.k[0] * m.t, rtol=1e-12, atol=1e-12)


SLOW = pytest.mark.skipif(not os.environ.get("LASSIE_SLOW_TESTS"),
                          reason="five minutes of scipy on 512 species; LASSIE_SLOW_TESTS=1 runs it")


@pytest.mark.parametrize("name", ["c1", "c5", "sized-100",
                                  pytest.param("c2-short", marks=SLOW)])
def test_accuracy_like_scipy_bdf(name):
    """Global error against LSODA at rtol 1e-12 is of the size scipy's BDF
    reaches at the same tolerances (both control the local error only).  On
    the stiff 512-species network (t in [0, 0.01]) this restatement's error is
    about 11x the tolerance, scipy's about 62x."""
    m = {"c1": synth.make_c1, "c5": lambda: synth.make_c5(1)[0][0],
         "sized-100": lambda: synth.make_sized(100, 3),
         "c2-short": lambda: synth.shorten(synth.make_c2(), 0.01, 6)}[name]()
    om = O.OracleModel(m.left, m.right)
    out, st, rc = O.solve_bdf(m, om=om, rtol=RTOL, atol=ATOL)
    assert rc == 0
    ref = _tight(m, om)
    mine, theirs = _err_over_tol(out, ref), _err_over_tol(_scipy_bdf(m, om), ref)
    assert mine < max(3 * theirs, 10.0), (mine, theirs)
    assert mine < 200


def test_conservation():
    m = synth.tiny_network("reversible")   # A + B <-> C keeps A + C and B + C
    out, _, rc = O.solve_bdf(m, rtol=RTOL, atol=ATOL)
    assert rc == 0
    a, b, c = out[:, 0], out[:, 1], out[:, 2]
    assert np.allclose(a + c, a[0] + c[0], rtol=1e-9, atol=1e-12)
    assert np.allclose(b + c, b[0] + c[0], rtol=1e-9, atol=1e-12)


def test_fed_species_constant():
    m = synth.make_sized(37, 0)
    m.feed = np.zeros(m.n_species)
    m.feed[[3, 17]] = [0.5, 2.0]
    out, _, rc = O.solve_bdf(m, rtol=RTOL, atol=ATOL)
    assert rc == 0
    cs = list(m.sampled())
    assert np.all(out[:, cs.index(3)] == 0.5) and np.all(out[:, cs.index(17)] == 2.0)


def test_order_cap():
    """Capping the order: the cap holds, lower orders take more steps, and the
    global error (local error control only) grows as the order falls: on C1
    about 4500, 470, 140, 56, 27 times the tolerance for caps 1..5."""
    m = synth.make_c1()
    ref = _tight(m, O.OracleModel(m.left, m.right))
    steps, errs = [], []
    for max_order in (1, 2, 3, 4, 5):
        out, st, rc = O.solve_bdf(m, rtol=RTOL, atol=ATOL, max_order=max_order)
        assert rc == 0 and st["order_final"] <= max_order
        steps.append(st["steps"])
        errs.append(_err_over_tol(out, ref))
    assert all(a > b for a, b in zip(steps, steps[1:])), steps
    assert errs[0] < 2e4 and errs[-1] < 100, errs


def test_step_options_and_errors():
    m = synth.make_c1()
    _, st_a, rc = O.solve_bdf(m, max_step=0.05)
    assert rc == 0
    _, st_b, rc = O.solve_bdf(m)
    assert rc == 0 and st_a["steps"] > st_b["steps"]
    _, st_c, rc = O.solve_bdf(m, first_step=1e-7)
    assert rc == 0
    _, _, rc = O.solve_bdf(m, rtol=0.0)
    assert rc == -20
    _, _, rc = O.solve_bdf(m, max_steps=5)
    assert rc == -21


def test_block_sum_mirror():
    rng = np.random.default_rng(5)
    for n in (1, 7, 33, 512, 777, 1500):
        v = rng.uniform(0, 1, n) * 10.0 ** rng.uniform(-5, 5, n)
        s = O.lib().lo_block_sum512(np.ascontiguousarray(v), n)
        assert math.isclose(s, math.fsum(v), rel_tol=1e-13)
    # the tree: with 512 values, lane pairs (l, l^16) add first
    v = np.zeros(512)
    v[0], v[16] = 1.0, 2.0 ** -53
    v[1] = 2.0 ** -53
    # ((1 + 2^-53) + ...) in the tree order differs from left-to-right only in
    # rounding; the result is one of the two neighbours of the exact sum
    s = O.lib().lo_block_sum512(v, 512)
    assert s in (1.0, 1.0 + 2.0 ** -52)


def test_fed_species_and_atol_vector_like_scipy():
    """Fed species held constant and per-species absolute tolerances: the
    restatement's error against LSODA at rtol 1e-12 (the same constraint
    applied there) is of the size of scipy's BDF with the same tolerances."""
    from scipy.integrate import solve_ivp
    m = synth.make_sized(60, 7)
    m.feed = np.zeros(m.n_species)
    m.feed[[5, 33]] = [0.8, 1.7]
    m.atol = np.full(m.n_species, 1e-10)
    m.atol[::4] = 1e-7
    om = O.OracleModel(m.left, m.right)
    fed = m.feed != 0
    x0 = np.where(fed, m.feed, m.x0)

    def f(t, x):
        d = om.rhs(m.k, x)
        d[fed] = 0.0
        return d

    def jac(t, x):
        J = om.jacobian_exact(m.k, x)
        J[fed, :] = 0.0
        return J

    ref = solve_ivp(f, (m.t[0], m.t[-1]), x0, method="LSODA", t_eval=m.t, rtol=1e-12,
                    atol=1e-14, jac=jac).y.T
    theirs = solve_ivp(f, (m.t[0], m.t[-1]), x0, method="BDF", t_eval=m.t, rtol=RTOL,
                       atol=m.atol, jac=jac).y.T
    out, st, rc = O.solve_bdf(m, rtol=RTOL)
    assert rc == 0
    cs = list(m.sampled())
    assert np.all(out[:, cs.index(5)] == 0.8) and np.all(out[:, cs.index(33)] == 1.7)
    tol = m.atol + RTOL * np.abs(ref)
    mine = float(np.max(np.abs(out - ref) / tol))
    other = float(np.max(np.abs(theirs - ref) / tol))
    assert mine < max(3 * other, 10.0), (mine, other)

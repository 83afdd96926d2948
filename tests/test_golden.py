"""The CPU oracle against golden vectors produced by the unmodified reference
binary (tests/golden/make_golden.py, run on the GPU machine).

Backward-Euler-dominated runs agree at every sample within rtol 1e-6 /
atol 1e-9 (Newton convergence absorbs rounding differences).  Runs that
accept many RKF45 steps part ways at the first step-size decision that
depends on the last bit of (atol/R)^(1/4): the reference computes it with
CUDA's pow(), which is not correctly rounded on every input, and its steps
are not restated here (the oracle offers sqrt(sqrt()), the C library's pow()
and the correctly rounded root; none of them is CUDA's).  LASSIE's loop
turns such a bit into a different step sequence, and its clock advances by
the next step (Simulation.cuh:753-767), so trajectories then move by up to
tens of percent.  Those cases are held to the oracle's own spread: sixteen
oracle runs whose quarter roots (eight seeds), Newton corrections (five
seeds) or LU rounding order (three variants) differ in the last bit give the
first sample at which any of them leaves the tolerance and their largest
excess over it; the reference must agree before that sample and stay within
twice that excess.  Measured (correctly rounded root): the reference's
excess is 0.5-1.02 of the spread's worst on every such case.

The GPU engine's default (pow) reproduces these cases bit for bit
(tests/test_gpu_golden.py).
"""
import glob
import os

import numpy as np
import pytest

from lassie_gb300.model import Model
from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL, ATOL = 1e-6, 1e-9

FULL_AGREEMENT = ("c2_t0012", "c4_i7_t05", "tiny_reversible_fed", "tiny_source")
WITHIN_SPREAD = ("c1", "c4_i2_t1", "tiny_bimolecular", "tiny_conversion", "tiny_decay",
                 "tiny_dimer", "tiny_reversible")
# linear invariants of the tiny networks: rows w with w . x constant
INVARIANTS = {
    "tiny_conversion": [[1, 1]],            # A -> B
    "tiny_dimer": [[1, 2]],                 # 2A -> B
    "tiny_bimolecular": [[1, 0, 1], [0, 1, 1]],  # A + B -> C
    "tiny_reversible": [[1, 0, 1], [0, 1, 1]],   # A + B <-> C
}


def load(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    m = Model(left=d["left"], right=d["right"], k=d["k"], x0=d["x0"], t=d["t"])
    if d["feed"].size:
        m.feed = d["feed"]
    return m, d


def cases():
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(HERE, "*.npz")))


def excess(a, b):
    return np.max(np.abs(a - b) - ATOL - RTOL * np.abs(b), axis=1)


def spread(m, root="rn"):
    """(unperturbed trajectory, its loop iterations, first divergence, worst
    excess, largest change of the loop-iteration count) over the sixteen
    perturbed oracle runs."""
    base, st, rc = O.solve(m, root=root)
    assert rc == 0
    runs = ([O.root_perturbation(2.0 ** -52, s) for s in range(1, 9)]
            + [O.solve_perturbation(2.0 ** -52, s) for s in range(1, 6)]
            + [O.lu_variant(v) for v in (1, 2, 3)])
    first, worst, dout = base.shape[0], 0.0, 0
    for ctx in runs:
        with ctx:
            p, sp, _ = O.solve(m, root=root)
        e = excess(p, base)
        if np.any(e > 0):
            first = min(first, int(np.argmax(e > 0)))
        worst = max(worst, float(e.max()))
        dout = max(dout, abs(sp["outer_iters"] - st["outer_iters"]))
    return base, st["outer_iters"], first, worst, dout


def test_fixture_set_complete():
    assert set(cases()) == set(WITHIN_SPREAD) | set(FULL_AGREEMENT)
    assert len(float_cases()) == len(cases())


@pytest.mark.parametrize("name", FULL_AGREEMENT)
def test_oracle_matches_reference_everywhere(name):
    m, d = load(name)
    out, st, rc = O.solve(m)
    assert rc == 0
    assert np.array_equal(d["ref_t"], m.t)
    ref = d["ref"]
    assert np.all(np.abs(out - ref) <= ATOL + RTOL * np.abs(ref))
    if "ref_outer_iters" in d.files:
        assert st["outer_iters"] == int(d["ref_outer_iters"])


@pytest.mark.parametrize("name", WITHIN_SPREAD)
def test_reference_within_the_oracles_spread(name):
    m, d = load(name)
    base, outer, first, worst, dout = spread(m)
    assert worst > 0, "the case no longer depends on last-bit decisions"
    e = excess(d["ref"], base)
    assert np.all(e[:first] <= 0), (first, e)
    assert e.max() <= 2 * worst, (float(e.max()), worst)
    # before the first divergence the two agree to a few ulps
    rel = np.abs(base[:first] - d["ref"][:first]) / np.maximum(np.abs(d["ref"][:first]), 1e-300)
    assert float(rel.max(initial=0.0)) < 1e-13
    if "ref_outer_iters" in d.files:
        # the reference's loop-iteration count within twice the spread's
        assert abs(int(d["ref_outer_iters"]) - outer) <= 2 * dout + 2


@pytest.mark.parametrize("name", sorted(INVARIANTS))
def test_oracle_and_reference_conserve_the_same_totals(name):
    """Whatever the step sequence, RKF45 and backward-Euler steps keep the
    linear invariants of the network: the oracle's and the reference's
    totals agree with the initial ones to rounding."""
    m, d = load(name)
    out, _, rc = O.solve(m, root="rn")
    assert rc == 0
    for w in INVARIANTS[name]:
        w = np.asarray(w, np.float64)
        t0 = float(w @ m.x0)
        assert np.allclose(out @ w, t0, rtol=1e-12, atol=1e-14)
        assert np.allclose(d["ref"] @ w, t0, rtol=1e-9, atol=1e-12)


def test_correctly_rounded_quarter_root():
    """lo_qroot_rn is x^(1/4) rounded to nearest: checked against exact
    rational arithmetic on the midpoints to the neighbouring doubles."""
    from fractions import Fraction
    L = O.lib()
    rng = np.random.default_rng(4)
    xs = np.concatenate([10.0 ** rng.uniform(-300, 300, 3000), rng.uniform(0, 4, 1000),
                         [1.0, 16.0, 81.0, 2.0 ** -1074, 1.7976931348623157e308]])
    for x in xs:
        y = L.lo_qroot_rn(float(x))
        lo = (Fraction(np.nextafter(y, 0.0)) + Fraction(y)) / 2
        hi = (Fraction(y) + Fraction(np.nextafter(y, np.inf))) / 2
        assert lo ** 4 < Fraction(float(x)) < hi ** 4, x
    assert L.lo_qroot_rn(0.0) == 0.0 and L.lo_qroot_rn(float("inf")) == float("inf")


# ------------------------------------------------ the reference's -p float
FLOAT_DIR = os.path.join(HERE, "float")
FRTOL, FATOL = 1e-5, 1e-9


def float_cases():
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(FLOAT_DIR, "*.npz")))


def fexcess(a, b):
    return np.max(np.abs(a - b) - FATOL - FRTOL * np.abs(b), axis=1)


@pytest.mark.parametrize("name", float_cases())
def test_float_oracle_against_the_reference_float_mode(name):
    """The oracle's float restatement (IEEE float division and powf) against
    the reference's -p float outputs (--use_fast_math division and pow):
    within the float tolerance before the first sample at which the float
    oracle's own spread (quarter root or Newton corrections moved by one
    float ulp) leaves it, and within twice the spread's excess after it
    (the spread is computed only when the reference leaves the tolerance
    somewhere)."""
    d = np.load(os.path.join(FLOAT_DIR, name + ".npz"))
    m = Model(left=d["left"], right=d["right"], k=d["k"], x0=d["x0"], t=d["t"])
    if d["feed"].size:
        m.feed = d["feed"]
    base, st, rc = O.solve(m, precision="float")
    assert rc == 0
    if np.all(fexcess(d["ref"], base) <= 0):
        return  # within the float tolerance at every sample: no spread needed
    first, worst = base.shape[0], 0.0
    for ctx in ([O.root_perturbation(2.0 ** -23, s) for s in range(1, 6)]
                + [O.solve_perturbation(2.0 ** -23, s) for s in range(1, 6)]):
        with ctx:
            p, _, _ = O.solve(m, precision="float")
        e = fexcess(p, base)
        if np.any(e > 0):
            first = min(first, int(np.argmax(e > 0)))
        worst = max(worst, float(e.max()))
    e = fexcess(d["ref"], base)
    assert np.all(e[:first] <= 0), (first, e)
    assert e.max() <= 2 * worst, (float(e.max()), worst)


# ------------------------------------------------ longer horizons
LONG_DIR = os.path.join(HERE, "long")
FIXTURES = os.path.join(os.path.dirname(HERE), "oracle_fixtures")


def long_cases():
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(LONG_DIR, "*.npz")))


@pytest.mark.parametrize("name", long_cases())
def test_stored_oracle_trajectory_matches_the_reference(name):
    """The reference binary's run (tests/golden/long/, make_golden.py --long)
    against the oracle's stored trajectory of the same network and samples
    (tests/oracle_fixtures/, make_oracle_fixtures.py): C2 over 8 893
    backward-Euler steps and C3 over 50 with 4096 x 4096 factorisations,
    within rtol 1e-6 / atol 1e-9 at every sample.  Nothing is integrated
    here: both runs take minutes to an hour."""
    d = np.load(os.path.join(LONG_DIR, name + ".npz"))
    f = np.load(os.path.join(FIXTURES, name + ".npz"))
    assert int(f["status"]) == 0
    assert np.array_equal(d["ref_t"], f["t"]) and np.array_equal(d["t"], f["t"])
    ref, out = d["ref"], f["out"]
    assert ref.shape == out.shape
    assert np.all(np.abs(out - ref) <= ATOL + RTOL * np.abs(ref)), \
        float(np.max(np.abs(out - ref) / np.maximum(np.abs(ref), ATOL)))

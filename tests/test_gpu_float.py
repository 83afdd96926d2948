"""The reference's single-precision mode (`-p float`, Simulation<float>)
against the reference binary's own -p float outputs.

tests/golden/float/*.npz hold the unmodified binary's -p float trajectories
(make_golden.py --float, run on the GPU machine).  The engine's float mode
(lassie_gb300/csrc/float_mode.cu) runs LASSIE's loop with float state and
the reference's double temporaries, compiled with the reference's device
flags, so the RKF45 steps and the small backward-Euler solves reproduce the
reference bit for bit, loop-iteration counts included.  The 512- and
84-species backward-Euler cases go through a float LU in place of cuSOLVER's
Sgetrf and agree within a float tolerance; the 363-species case parts at a
step decision that the float LU's last bits move, and is held to the spread
of the float oracle (tests/test_golden.py's float cases).
"""
import os
import subprocess

import numpy as np
import pytest

from lassie_gb300 import solver
from lassie_gb300.model import Model, write_folder
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "float")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# float state: about 7 significant digits
FRTOL, FATOL = 1e-5, 1e-9

BIT_EXACT = ("c1", "tiny_bimolecular", "tiny_conversion", "tiny_decay", "tiny_dimer",
             "tiny_reversible", "tiny_reversible_fed", "tiny_source")
WITHIN_TOL = ("c2_t0012", "c4_i2_t1")
DECISION_SENSITIVE = ("c4_i7_t05",)


def load(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    m = Model(left=d["left"], right=d["right"], k=d["k"], x0=d["x0"], t=d["t"])
    if d["feed"].size:
        m.feed = d["feed"]
    return m, d


def excess(a, b):
    return np.max(np.abs(a - b) - FATOL - FRTOL * np.abs(b), axis=1)


def float_spread(m):
    """First sample at which any of the float oracle's runs with the quarter
    root or the Newton corrections moved by one float ulp leaves the float
    tolerance of the unperturbed float oracle, and their largest excess."""
    base, _, rc = O.solve(m, precision="float")
    assert rc == 0
    first, worst = base.shape[0], 0.0
    runs = ([O.root_perturbation(2.0 ** -23, s) for s in range(1, 6)]
            + [O.solve_perturbation(2.0 ** -23, s) for s in range(1, 6)])
    for ctx in runs:
        with ctx:
            p, _, _ = O.solve(m, precision="float")
        e = excess(p, base)
        if np.any(e > 0):
            first = min(first, int(np.argmax(e > 0)))
        worst = max(worst, float(e.max()))
    return base, first, worst


def test_case_lists_cover_the_fixtures():
    import glob
    names = {os.path.basename(f)[:-4] for f in glob.glob(os.path.join(HERE, "*.npz"))}
    assert names == set(BIT_EXACT) | set(WITHIN_TOL) | set(DECISION_SENSITIVE)


@pytest.mark.parametrize("name", BIT_EXACT)
def test_float_mode_reproduces_the_reference_bit_for_bit(gpu, name):
    m, d = load(name)
    out, st = solver.simulate(m, engine="float", deadline_s=120)
    assert st["status"] == 0
    assert np.array_equal(out, d["ref"]), float(np.max(np.abs(out - d["ref"])))
    assert st["outer_iters"] == int(d["ref_outer_iters"])


@pytest.mark.parametrize("name", WITHIN_TOL)
def test_float_mode_backward_euler_cases_within_tolerance(gpu, name):
    m, d = load(name)
    out, st = solver.simulate(m, engine="float", deadline_s=300)
    assert st["status"] == 0
    assert np.all(excess(out, d["ref"]) <= 0), float(excess(out, d["ref"]).max())
    assert st["outer_iters"] == int(d["ref_outer_iters"])


@pytest.mark.parametrize("name", DECISION_SENSITIVE)
def test_float_mode_decision_sensitive_case_within_the_spread(gpu, name):
    m, d = load(name)
    base, first, worst = float_spread(m)
    assert worst > 0, "the case no longer depends on last-bit decisions"
    # the reference itself lies inside the float oracle's spread
    e_ref = excess(d["ref"], base)
    assert np.all(e_ref[:first] <= 0) and e_ref.max() <= 2 * worst
    out, st = solver.simulate(m, engine="float", deadline_s=300)
    assert st["status"] == 0
    e = excess(out, d["ref"])
    assert np.all(e[:first] <= 0), (e, first)
    assert e.max() <= 2 * worst, (float(e.max()), worst)


@pytest.mark.parametrize("name", BIT_EXACT)
def test_cli_p_float_against_the_reference(gpu, name, tmp_path):
    """`lassie in out -p float -dump-f64`: the drop-in command line's float
    mode."""
    m, d = load(name)
    inp, outp = str(tmp_path / "in"), str(tmp_path / "out")
    write_folder(m, inp)
    cli = os.path.join(ROOT, "lassie_gb300", "_native", "lassie")
    r = subprocess.run([cli, inp, outp, "-p", "float", "-dump-f64"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [[float(v) for v in ln.split("\t") if v.strip()]
            for ln in open(os.path.join(outp, "output", "Solution.f64")) if ln.strip()]
    sol = np.asarray(rows)
    assert np.array_equal(sol[:, 1:], d["ref"])


def test_float_mode_refuses_what_the_reference_float_mode_lacks(gpu):
    from lassie_gb300 import _native as nat
    from lassie_gb300 import synth
    m = synth.shorten(synth.make_c4_instance(0), 0.1, 2)
    with pytest.raises(nat.LassieError):
        solver.simulate(m, engine="float", bdf={})

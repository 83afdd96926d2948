"""Whole horizons against stored oracle trajectories
(tests/oracle_fixtures/, make_oracle_fixtures.py):

* the 256-species adjoint network over its whole horizon t in (0, 10]
  (40 samples, 1000 backward-Euler steps): the FP64 form bit for bit with
  the oracle's step counts; the mixed form within the oracle's spread (this
  network's RKF45 steps after backward-Euler stretches depend on last bits);
* the stiff 512-species network on t in [0, 0.1] (8 893 backward-Euler
  steps after three reverts take the step to 1e-5; its whole horizon would
  take the oracle days): the FP64 form bit for bit, the mixed form within
  rtol 1e-6 / atol 1e-9 with the oracle's step counts;
* the 4096-species network on t in [0, 0.5] (11 samples) on the wide
  engine, with each of its rank-update modes: within rtol 1e-6 / atol 1e-9
  with the oracle's backward-Euler steps.
"""
import os

import numpy as np
import pytest

from lassie_gb300 import solver, synth

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_fixtures")
RTOL, ATOL = 1e-6, 1e-9


def excess(a, b):
    return np.max(np.abs(a - b) - ATOL - RTOL * np.abs(b), axis=1)


def fixture(name):
    path = os.path.join(HERE, name + ".npz")
    if not os.path.exists(path):
        pytest.skip(f"{name}.npz not generated")
    return np.load(path)


def test_c5_full_horizon(gpu):
    d = fixture("c5_full")
    m = synth.make_c5(1)[0][0]
    assert np.array_equal(m.t, d["t"])
    out, st = solver.simulate(m, engine="fp64", root="sqrt", deadline_s=600)
    assert st["status"] == 0 == int(d["status"])
    assert np.array_equal(out, d["out"])
    assert (st["be_steps"], st["rkf_accepts"], st["newton_iters"]) == \
        (int(d["be_steps"]), int(d["rkf_accepts"]), int(d["newton_iters"]))
    mx, sx = solver.simulate(m, engine="mixed", root="sqrt", deadline_s=600)
    assert sx["status"] == 0
    e = excess(mx, d["out"])
    ok64 = np.all(e[:int(d["first_divergence"])] <= 0) and e.max() <= 2 * float(d["worst_excess"])
    oknw = (np.all(e[:int(d["first_divergence_normwise"])] <= 0)
            and e.max() <= 2 * float(d["worst_excess_normwise"]))
    assert ok64 or oknw, (float(e.max()), float(d["worst_excess"]), float(d["worst_excess_normwise"]))


def test_c2_to_a_tenth_time_unit(gpu):
    d = fixture("c2_t01")
    m = synth.shorten(synth.make_c2(), 0.1, 6)
    assert np.array_equal(m.t, d["t"])
    out, st = solver.simulate(m, engine="fp64", root="sqrt", deadline_s=1200)
    assert st["status"] == 0 == int(d["status"])
    assert np.array_equal(out, d["out"])
    assert st["be_steps"] == int(d["be_steps"])
    mx, sx = solver.simulate(m, engine="mixed", root="sqrt", deadline_s=1200)
    assert sx["status"] == 0
    assert np.all(excess(mx, d["out"]) <= 0), float(excess(mx, d["out"]).max())
    assert sx["be_steps"] == int(d["be_steps"])


@pytest.mark.parametrize("mode", ["tf32", "bf16", "off"])
def test_c3_to_half_time_unit(gpu, mode):
    """Rank updates on the tensor cores with split-TF32 (the default) or BF16
    operands, or on the FP32 pipes: the same trajectory and steps."""
    d = fixture("c3_t05")
    m = synth.shorten(synth.make_c3(), 0.5, 11)
    assert np.array_equal(m.t, d["t"])
    out, st = solver.simulate(m, engine="mixed", root="sqrt", deadline_s=1200, tensor_cores=mode,
                              refine_max=32 if mode == "bf16" else 0)
    assert st["status"] == 0 == int(d["status"])
    assert np.all(excess(out, d["out"]) <= 0), float(excess(out, d["out"]).max())
    assert st["be_steps"] == int(d["be_steps"])

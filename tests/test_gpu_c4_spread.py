"""The batched workload's sample against the oracle, instance by instance.

tests/oracle_fixtures/c4_spread.npz (make_c4_spread.py) holds, for every
13th instance of the 2048-instance workload on t in [0, 2] (152 instances,
at most 2500 loop iterations), the oracle's step counts and two spreads of
the oracle itself -- the first sample at which any of its perturbed runs
leaves rtol 1e-6 / atol 1e-9 of the unperturbed run, and their largest
excess over that tolerance:

* FP64 solvers: five one-ulp componentwise perturbations of the Newton
  corrections and three other LU rounding orders;
* solvers of the mixed form's accuracy class: five runs whose corrections
  move by +- 2^-53 * max|dx| per component.

Checks:

* The FP64 form reproduces the oracle, run here on the host's cores, bit for
  bit on every instance, trajectories and step counts.
* The mixed form, with factor reuse as shipped and without, agrees with the
  FP64 form within the tolerance before the first spread's first divergence
  and within twice its excess after it -- or, on instances that solvers of
  its own accuracy already move, within the second spread -- on every
  instance the oracle completes.  How many instances fall under each is
  printed.
"""
import os

import numpy as np
import pytest

from lassie_gb300 import solver, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
RTOL, ATOL = 1e-6, 1e-9


def excess(a, b):
    return np.max(np.abs(a - b) - ATOL - RTOL * np.abs(b), axis=1)


@pytest.fixture(scope="module")
def sample():
    f = np.load(os.path.join(HERE, "oracle_fixtures", "c4_spread.npz"))
    horizon, nsamp, cap = float(f["horizon"]), int(f["nsamp"]), int(f["cap"])
    models = [synth.shorten(synth.make_c4_instance(int(q)), horizon, nsamp) for q in f["index"]]
    b = solver.Batch(models, engine="fp64", max_steps=cap, deadline_s=900, root="sqrt")
    b.run(0)
    b.sync()
    outs, stats = b.read()
    oracle = O.solve_batch(models, threads=os.cpu_count() or 1, max_steps=cap)
    return f, models, cap, [o.copy() for o in outs], stats, oracle


def test_fp64_form_reproduces_the_oracle(gpu, sample):
    f, _, _, outs, stats, (oracle_out, oracle_stats, oracle_status) = sample
    keys = [str(k) for k in f["stat_keys"]]
    for j, (o, s) in enumerate(zip(outs, stats)):
        assert s["status"] == int(oracle_status[j]) == int(f["status"][j]), j
        assert [s[k] for k in keys] == [oracle_stats[j][k] for k in keys], j
        if s["status"] == 0:
            assert np.array_equal(o, oracle_out[j]), j


@pytest.mark.parametrize("lu_reuse", [True, False], ids=["reuse", "refactor"])
def test_mixed_form_within_the_oracles_spread(gpu, sample, lu_reuse):
    f, models, cap, ref, _, _ = sample
    b = solver.Batch(models, engine="mixed", max_steps=cap, deadline_s=900, root="sqrt",
                     lu_reuse=lu_reuse)
    b.run(0)
    b.sync()
    outs, stats = b.read()
    bad, fp64_spread, normwise_spread = [], 0, 0
    for j, (o, s) in enumerate(zip(outs, stats)):
        if int(f["status"][j]) != 0:
            continue  # capped by the loop-iteration limit in the oracle too
        e = excess(o, ref[j])

        def within(first, worst):
            return s["status"] == 0 and np.all(e[:first] <= 0) and e.max() <= 2 * worst

        if within(int(f["first_divergence"][j]), float(f["worst_excess"][j])):
            fp64_spread += 1
        elif within(int(f["first_divergence_normwise"][j]),
                    float(f["worst_excess_normwise"][j])):
            normwise_spread += 1
        else:
            bad.append((j, s["status"], float(e.max()), float(f["worst_excess"][j]),
                        float(f["worst_excess_normwise"][j])))
    print(f"lu_reuse={lu_reuse}: {fp64_spread} instances within the FP64 solvers' spread, "
          f"{normwise_spread} within the normwise solvers' spread, {len(bad)} outside")
    assert not bad, bad

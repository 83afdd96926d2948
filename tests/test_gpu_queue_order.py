"""lassie_batch_order_by_cost: a batch's later runs take the instances
longest first by the last run's per-instance integration times.  Each CTA
integrates its instance alone, so the order must change no trajectory and no
step count, in either controller."""
import numpy as np
import pytest

from lassie_gb300 import solver, synth

pytestmark = pytest.mark.gpu

COUNTERS = ("status", "outer_iters", "rkf_accepts", "rkf_retries", "be_steps", "newton_iters",
            "lu_factorisations", "lu_failures", "nan_reverts", "refine_sweeps")


def _models():
    return [synth.shorten(synth.make_c4_instance(q), 0.5, 4) for q in range(0, 320, 5)]


@pytest.mark.parametrize("engine", ["mixed", "fp64"])
@pytest.mark.parametrize("bdf", [None, {"rtol": 1e-6, "atol": 1e-9}], ids=["compat", "bdf"])
def test_cost_order_changes_no_result(gpu, engine, bdf):
    b = solver.Batch(_models(), engine=engine, max_steps=5000, deadline_s=300, bdf=bdf)
    b.order_by_cost()  # before any run: keeps the creation order
    b.run(0)
    b.sync()
    outs1, st1 = b.read()
    outs1 = [o.copy() for o in outs1]
    assert all(s["cycles_total"] > 0 for s in st1)
    b.order_by_cost()
    b.run(0)
    b.sync()
    outs2, st2 = b.read()
    for a, c, s, t in zip(outs1, outs2, st1, st2):
        assert np.array_equal(a, c)
        assert [s[k] for k in COUNTERS] == [t[k] for k in COUNTERS]

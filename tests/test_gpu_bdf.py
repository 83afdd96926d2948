"""The BDF controller on the GPU (bdf_integrate in compat_kernel<double>)
against its CPU restatement, bit for bit: trajectories at every sample and
the step statistics (accepted and rejected steps, Newton iterations,
Jacobian evaluations, factorisations, final order)."""
import numpy as np
import pytest

from lassie_gb300 import solver, synth
from lassie_gb300 import _native as nat
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _cases():
    for kind in ("decay", "conversion", "dimer", "bimolecular", "source", "reversible"):
        yield kind, synth.tiny_network(kind)
    yield "c1", synth.make_c1()
    yield "c5", synth.make_c5(1)[0][0]
    yield "sized-37", synth.make_sized(37, 0)
    yield "sized-100", synth.make_sized(100, 3)
    yield "sized-512", synth.shorten(synth.make_sized(512, 2), 0.5, 6)
    yield "c2-short", synth.shorten(synth.make_c2(), 0.01, 6)
    fed = synth.make_sized(64, 4)
    fed.feed = np.zeros(fed.n_species)
    fed.feed[[2, 40]] = [0.3, 1.5]
    yield "fed", fed


def _same(m, opts, out, st):
    ref, rst, rc = O.solve_bdf(m, **opts)
    assert rc == 0
    assert st["status"] == 0
    assert np.array_equal(out.view(np.int64), ref.view(np.int64)), \
        float(np.max(np.abs(out - ref) / (1e-9 + 1e-6 * np.abs(ref))))
    assert st["be_steps"] == rst["steps"]
    assert st["rkf_retries"] == rst["rejected"]
    assert st["lu_failures"] == rst["newton_failures"]
    assert st["newton_iters"] == rst["newton_iters"]
    assert st["jac_evals"] == rst["jac_evals"]
    assert st["lu_factorisations"] == rst["lu_factorisations"]
    assert st["rhs_evals"] == rst["rhs_evals"]
    assert st["order_final"] == rst["order_final"]


@pytest.mark.parametrize("name,m", list(_cases()), ids=[c[0] for c in _cases()])
def test_bdf_bit_exact(gpu, name, m):
    out, st = solver.simulate(m, engine="fp64", deadline_s=300, bdf={})
    _same(m, {}, out, st)


@pytest.mark.parametrize("opts", [
    {"rtol": 1e-8, "atol": 1e-12},
    {"rtol": 1e-4, "atol": 1e-7},
    {"max_order": 2},
    {"max_order": 1},
    {"max_step": 0.05},
    {"first_step": 1e-7},
], ids=lambda o: ",".join(f"{k}={v}" for k, v in o.items()))
def test_bdf_options_bit_exact(gpu, opts):
    m = synth.make_c1()
    out, st = solver.simulate(m, engine="mixed", deadline_s=300, bdf=opts)  # factors in FP64
    _same(m, opts, out, st)


def test_bdf_batch_of_uneven_sizes(gpu):
    """One persistent launch over instances of different sizes, each bit for
    bit its own oracle solve."""
    models = [synth.shorten(m, 1.0, 6) for m in synth.make_c4(8)]
    outs, stats = solver.simulate_batch(models, deadline_s=600, bdf={"rtol": 1e-6})
    for m, o, st in zip(models, outs, stats):
        _same(m, {"rtol": 1e-6}, o, st)


def test_bdf_atol_vector(gpu):
    m = synth.make_sized(50, 1)
    m.atol = np.full(m.n_species, 1e-10)
    m.atol[::3] = 1e-6
    out, st = solver.simulate(m, deadline_s=300, bdf={})
    _same(m, {}, out, st)


def test_bdf_limits(gpu):
    m = synth.make_c1()
    out, st = solver.simulate(m, max_steps=5, deadline_s=300, bdf={})
    assert st["status"] == nat.ERR_MAX_STEPS
    big = synth.make_sized(600, 0)
    with pytest.raises(nat.LassieError):
        solver.simulate(big, deadline_s=60, bdf={})
    with pytest.raises(ValueError):
        solver.make_opts(m, bdf={"rtoll": 1e-3})

"""The BDF controller on the GPU (bdf_integrate in compat_kernel): the FP64
form against its CPU restatement, bit for bit -- trajectories at every sample
and the step statistics (accepted and rejected steps, Newton iterations,
Jacobian evaluations, factorisations, final order); the mixed form against
the FP64 form and LSODA."""
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
    out, st = solver.simulate(m, engine="fp64", deadline_s=300, bdf=opts)
    _same(m, opts, out, st)


def test_bdf_batch_of_uneven_sizes(gpu):
    """One persistent launch over instances of different sizes, each bit for
    bit its own oracle solve."""
    models = [synth.shorten(m, 1.0, 6) for m in synth.make_c4(8)]
    outs, stats = solver.simulate_batch(models, engine="fp64", deadline_s=600,
                                        bdf={"rtol": 1e-6})
    for m, o, st in zip(models, outs, stats):
        _same(m, {"rtol": 1e-6}, o, st)


def test_bdf_atol_vector(gpu):
    m = synth.make_sized(50, 1)
    m.atol = np.full(m.n_species, 1e-10)
    m.atol[::3] = 1e-6
    out, st = solver.simulate(m, engine="fp64", deadline_s=300, bdf={})
    _same(m, {}, out, st)


@pytest.mark.parametrize("name", ["c1", "c5", "sized-300", "c2-short"])
def test_bdf_mixed_form(gpu, name):
    """Mixed form (FP32 Gauss-Jordan inverse as the Newton iteration matrix,
    FP64 residuals): its trajectory is as accurate as the FP64 form's
    against LSODA at rtol 1e-12, and the two agree to the tolerance scale."""
    from scipy.integrate import solve_ivp
    m = {"c1": synth.make_c1, "c5": lambda: synth.make_c5(1)[0][0],
         "sized-300": lambda: synth.make_sized(300, 5),
         "c2-short": lambda: synth.shorten(synth.make_c2(), 0.01, 6)}[name]()
    mixed, st_m = solver.simulate(m, engine="mixed", deadline_s=300, bdf={})
    fp64, st_d = solver.simulate(m, engine="fp64", deadline_s=300, bdf={})
    assert st_m["status"] == 0 and st_d["status"] == 0
    om = O.OracleModel(m.left, m.right)
    ref = solve_ivp(lambda t, x: om.rhs(m.k, x), (m.t[0], m.t[-1]), m.x0, method="LSODA",
                    t_eval=m.t, rtol=1e-12, atol=1e-14,
                    jac=lambda t, x: om.jacobian_exact(m.k, x)).y.T
    tol = 1e-9 + 1e-6 * np.abs(ref)
    err_m = float(np.max(np.abs(mixed - ref) / tol))
    err_d = float(np.max(np.abs(fp64 - ref) / tol))
    assert err_m < max(3 * err_d, 20.0), (err_m, err_d)
    assert float(np.max(np.abs(mixed - fp64) / tol)) < max(3 * err_d, 20.0)


def test_bdf_limits(gpu):
    m = synth.make_c1()
    out, st = solver.simulate(m, max_steps=5, deadline_s=300, bdf={})
    assert st["status"] == nat.ERR_MAX_STEPS
    big = synth.make_sized(600, 0)
    with pytest.raises(nat.LassieError):
        solver.simulate(big, deadline_s=60, bdf={})
    with pytest.raises(ValueError):
        solver.make_opts(m, bdf={"rtoll": 1e-3})

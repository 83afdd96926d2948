"""CUDA path vs the CPU oracle, through the C ABI.

The FP64 engine follows the oracle's arithmetic contract (same evaluation
order, explicit fma in the LU and solves, no contraction), so its outputs are
compared for exact equality.  The mixed engine (FP32 LU + FP64 refinement) is
compared at rtol 1e-6 / atol 1e-9, the spec parity tolerance.
"""
import numpy as np
import pytest

from lassie_gb300 import synth, solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-6, 1e-9


def within(a, b, rtol=RTOL, atol=ATOL):
    return bool(np.all(np.abs(a - b) <= atol + rtol * np.abs(b)))


def excess(a, b, rtol=RTOL, atol=ATOL):
    """Per sample: the largest amount by which |a - b| exceeds the tolerance."""
    return np.max(np.abs(a - b) - atol - rtol * np.abs(b), axis=1)


# Cases whose trajectory moves beyond rtol 1e-6 when the oracle's own Newton
# corrections are perturbed by one ulp: LASSIE's step-size controller turns
# last-bit differences into different step sequences (the reference binary
# differs from the oracle on them for the same reason).
DECISION_SENSITIVE = ("c4-2-short",)


def small_cases():
    yield "c1", synth.make_c1()
    yield "c4-2-short", synth.shorten(synth.make_c4_instance(2), 1.0, 11)
    yield "c4-33-short", synth.shorten(synth.make_c4_instance(33), 1.0, 11)
    yield "c4-5-short", synth.shorten(synth.make_c4_instance(5), 0.3, 4)
    yield "c2-short", synth.shorten(synth.make_c2(), 0.012, 3)
    for kind in ("decay", "conversion", "dimer", "bimolecular", "source", "reversible"):
        yield kind, synth.tiny_network(kind)


@pytest.mark.parametrize("name,m", list(small_cases()), ids=[c[0] for c in small_cases()])
def test_rhs_bit_exact(gpu, name, m):
    om = O.OracleModel(m.left, m.right)
    rng = np.random.default_rng(7)
    for _ in range(3):
        x = rng.uniform(0, 2, m.n_species)
        assert np.array_equal(solver.rhs(m, x), om.rhs(m.k, x))


@pytest.mark.parametrize("name,m", list(small_cases()), ids=[c[0] for c in small_cases()])
def test_newton_matrix_bit_exact(gpu, name, m):
    om = O.OracleModel(m.left, m.right)
    x = np.random.default_rng(3).uniform(0, 2, m.n_species)
    h = 0.01
    J = om.jacobian(m.k, x)
    M_ref = np.eye(m.n_species) - h * J
    assert np.array_equal(solver.newton_matrix(m, x, h), M_ref)


def _newton_batch_cases():
    base, _ = synth.make_c5(1)
    yield "c5-256", base[0], 300
    yield "sized-37", synth.make_sized(37, 0), 64
    yield "sized-601", synth.make_sized(601, 1), 3
    for kind in ("decay", "dimer", "bimolecular", "reversible"):
        yield kind, synth.tiny_network(kind), 5


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("name,m,n_inst", list(_newton_batch_cases()),
                         ids=[c[0] for c in _newton_batch_cases()])
def test_newton_matrix_device_batch_bit_exact(gpu, name, m, n_inst, precision):
    """lassie_newton_matrix_device: I - h*J(x_b) for every parameterisation
    equals the oracle's Jacobian formed in FP64 (FP32 output: that matrix
    rounded once).  Odd N covers the unaligned row heads and tails."""
    torch = pytest.importorskip("torch")
    from lassie_gb300 import _native as nat
    nm = solver.NativeModel.of(m)
    om = O.OracleModel(m.left, m.right)
    N, R = m.n_species, m.n_reactions
    rng = np.random.default_rng(N + n_inst)
    x = rng.uniform(0, 2, (n_inst, N))
    k = 10.0 ** rng.uniform(-3, 3, (n_inst, R))
    h = 0.0123
    dt = torch.float64 if precision == 0 else torch.float32
    M_t = torch.full((n_inst, N, N), float("nan"), dtype=dt, device="cuda")
    x_t, k_t = torch.tensor(x, device="cuda"), torch.tensor(k, device="cuda")
    nat.check(nat.load().lassie_newton_matrix_device(nm.handle, n_inst, h, k_t.data_ptr(),
                                                     x_t.data_ptr(), M_t.data_ptr(),
                                                     precision, None),
              "lassie_newton_matrix_device")
    torch.cuda.synchronize()
    M = M_t.cpu().numpy()
    for b in sorted({0, n_inst // 2, n_inst - 1}):
        ref = np.eye(N) - h * om.jacobian(k[b], x[b])
        if precision == 1:
            ref = ref.astype(np.float32)
        assert np.array_equal(M[b], ref), (name, b)


def test_device_kernels_at_4096_species(gpu):
    """The largest network of the workloads (4096 species, 4096 reactions):
    batched RHS and Newton matrix (FP64 and FP32) bit for bit against the
    oracle for two parameterisations (2 x 128 MB of FP64 matrices)."""
    torch = pytest.importorskip("torch")
    from lassie_gb300 import _native as nat
    m = synth.make_c3()
    nm = solver.NativeModel.of(m)
    om = O.OracleModel(m.left, m.right)
    N, R, n_inst = m.n_species, m.n_reactions, 2
    rng = np.random.default_rng(4096)
    x = rng.uniform(0, 2, (n_inst, N))
    k = 10.0 ** rng.uniform(-4, 2, (n_inst, R))
    x_t, k_t = torch.tensor(x, device="cuda"), torch.tensor(k, device="cuda")
    L = nat.load()
    dx_t = torch.empty((n_inst, N), dtype=torch.float64, device="cuda")
    nat.check(L.lassie_rhs_device(nm.handle, n_inst, k_t.data_ptr(), x_t.data_ptr(),
                                  dx_t.data_ptr(), None), "lassie_rhs_device")
    h = 0.01
    for precision, dt in ((0, torch.float64), (1, torch.float32)):
        M_t = torch.full((n_inst, N, N), float("nan"), dtype=dt, device="cuda")
        nat.check(L.lassie_newton_matrix_device(nm.handle, n_inst, h, k_t.data_ptr(),
                                                x_t.data_ptr(), M_t.data_ptr(), precision, None),
                  "lassie_newton_matrix_device")
        torch.cuda.synchronize()
        for b in range(n_inst):
            ref = np.eye(N) - h * om.jacobian(k[b], x[b])
            if precision == 1:
                ref = ref.astype(np.float32)
            assert np.array_equal(M_t[b].cpu().numpy(), ref), (precision, b)
        del M_t
    dx = dx_t.cpu().numpy()
    for b in range(n_inst):
        assert np.array_equal(dx[b].view(np.int64), om.rhs(k[b], x[b]).view(np.int64))


def test_newton_matrix_device_empty_and_args(gpu):
    from lassie_gb300 import _native as nat
    m = synth.tiny_network("dimer")
    nm = solver.NativeModel.of(m)
    L = nat.load()
    assert L.lassie_newton_matrix_device(nm.handle, 0, 0.1, None, None, None, 0, None) == 0
    assert L.lassie_newton_matrix_device(nm.handle, 1, 0.1, None, None, None, 0, None) == -20
    assert L.lassie_newton_matrix_device(nm.handle, 0, 0.1, None, None, None, 7, None) == -20
    import ctypes as C
    nnz = C.c_int64(0)
    assert L.lassie_jacobian_nnz(nm.handle, C.byref(nnz)) == 0
    om = O.OracleModel(m.left, m.right)
    J = om.jacobian(m.k, np.full(m.n_species, 0.7))
    assert nnz.value >= int(np.count_nonzero(J))


@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 64, 100, 257, 512])
def test_lu_fp64_bit_exact(gpu, n):
    rng = np.random.default_rng(n)
    a = rng.normal(size=(n, n)) + np.eye(n) * 0.1
    b = rng.normal(size=n)
    lu, piv, rc = O.lu_factor(a)
    assert rc == 0
    ref = O.lu_solve(lu, piv, b)
    x, info = solver.lu_solve(a, b, "fp64")
    assert info == 0
    assert np.array_equal(x, ref)


@pytest.mark.parametrize("n", [8, 64, 300])
def test_lu_mixed_close(gpu, n):
    rng = np.random.default_rng(n + 1)
    a = rng.normal(size=(n, n)) + np.eye(n) * n
    b = rng.normal(size=n)
    x, info = solver.lu_solve(a, b, "mixed")
    assert info == 0
    ref = np.linalg.solve(a, b)
    assert np.allclose(x, ref, rtol=1e-4, atol=1e-5)


def test_lu_singular_reports_column(gpu):
    a = np.eye(6)
    a[:, 3] = 0.0
    x, info = solver.lu_solve(a, np.ones(6), "fp64")
    assert info == 4
    _, _, rc = O.lu_factor(a)
    assert rc == 4


@pytest.mark.parametrize("name,m", list(small_cases()), ids=[c[0] for c in small_cases()])
def test_solve_fp64_bit_exact(gpu, name, m):
    ref, st_ref, rc = O.solve(m, max_steps=2_000_000)
    assert rc == 0
    out, st = solver.simulate(m, engine="fp64", deadline_s=120, root="sqrt")
    assert st["status"] == 0
    assert st["be_steps"] == st_ref["be_steps"]
    assert st["rkf_accepts"] == st_ref["rkf_accepts"]
    assert st["newton_iters"] == st_ref["newton_iters"]
    assert np.array_equal(out, ref), float(np.max(np.abs(out - ref)))


@pytest.mark.parametrize("name,m", [c for c in small_cases() if c[0] not in DECISION_SENSITIVE],
                         ids=[c[0] for c in small_cases() if c[0] not in DECISION_SENSITIVE])
@pytest.mark.parametrize("lu_reuse", [True, False], ids=["reuse", "refactor"])
def test_solve_mixed_within_tolerance(gpu, name, m, lu_reuse):
    ref, st_ref, rc = O.solve(m, max_steps=2_000_000)
    out, st = solver.simulate(m, engine="mixed", deadline_s=120, root="sqrt", lu_reuse=lu_reuse)
    assert st["status"] == 0
    assert within(out, ref), float(np.max(excess(out, ref)))
    # the same step sequence as the oracle
    assert (st["be_steps"], st["rkf_accepts"]) == (st_ref["be_steps"], st_ref["rkf_accepts"])
    if not lu_reuse:
        assert st["lu_factorisations"] == st["be_steps"]


@pytest.mark.parametrize("name,m", [c for c in small_cases() if c[0] in DECISION_SENSITIVE],
                         ids=list(DECISION_SENSITIVE))
def test_solve_mixed_decision_sensitive(gpu, name, m):
    """On a decision-sensitive case the mixed form is held to the oracle's own
    spread: five oracle runs whose Newton corrections are perturbed by one
    ulp give the first sample that leaves the tolerance and the largest
    excess; the mixed form must agree within tolerance before that sample
    and stay within twice that excess."""
    ref, _, rc = O.solve(m, max_steps=2_000_000)
    assert rc == 0
    firsts, worst = [], 0.0
    for seed in range(1, 6):
        with O.solve_perturbation(2.0 ** -52, seed):
            p, _, _ = O.solve(m, max_steps=2_000_000)
        e = excess(p, ref)
        firsts.append(int(np.argmax(e > 0)) if np.any(e > 0) else len(e))
        worst = max(worst, float(e.max()))
    assert worst > 0, "the case is not decision-sensitive any more"
    out, st = solver.simulate(m, engine="mixed", deadline_s=120, root="sqrt")
    assert st["status"] == 0
    e = excess(out, ref)
    assert np.all(e[:min(firsts)] <= 0), (e, firsts)
    assert e.max() <= 2 * worst, (float(e.max()), worst)


def test_batch_equals_single(gpu):
    models = [synth.shorten(synth.make_c4_instance(q), 0.2, 3) for q in range(6)]
    outs, stats = solver.simulate_batch(models, engine="fp64", deadline_s=120, root="sqrt")
    for m, o, s in zip(models, outs, stats):
        ref, _, _ = O.solve(m)
        assert s["status"] == 0
        assert np.array_equal(o, ref)


def _rhs_batch_models():
    base, _ = synth.make_c5(1)
    yield "c5-256", base[0]
    yield "sized-37", synth.make_sized(37, 0)
    yield "sized-601", synth.make_sized(601, 1)
    yield "c2-512", synth.make_c2()
    for kind in ("dimer", "source", "reversible"):
        yield kind, synth.tiny_network(kind)


@pytest.mark.parametrize("name,m", list(_rhs_batch_models()), ids=[c[0] for c in _rhs_batch_models()])
def test_rhs_device_batch_bits(gpu, name, m):
    """lassie_rhs_device against the oracle bit for bit, the sign of zero
    included: every third state has a quarter of its species at 0, so some
    sums consist of -0.0 terms only (the oracle's 0.0 + -0.0 is +0.0)."""
    torch = pytest.importorskip("torch")
    from lassie_gb300 import _native as nat
    nm = solver.NativeModel.of(m)
    om = O.OracleModel(m.left, m.right)
    n_inst = 97
    rng = np.random.default_rng(m.n_species)
    x = rng.uniform(0, 2, (n_inst, m.n_species))
    x[::3, rng.random(m.n_species) < 0.25] = 0.0
    k = 10.0 ** rng.uniform(-3, 3, (n_inst, m.n_reactions))
    dx_t = torch.full((n_inst, m.n_species), float("nan"), dtype=torch.float64, device="cuda")
    x_t, k_t = torch.tensor(x, device="cuda"), torch.tensor(k, device="cuda")
    nat.check(nat.load().lassie_rhs_device(nm.handle, n_inst, k_t.data_ptr(), x_t.data_ptr(),
                                           dx_t.data_ptr(), None), "lassie_rhs_device")
    torch.cuda.synchronize()
    dx = dx_t.cpu().numpy()
    for b in range(n_inst):
        ref = om.rhs(k[b], x[b])
        assert np.array_equal(dx[b].view(np.int64), ref.view(np.int64)), (name, b)


@pytest.mark.parametrize("n_inst", [1, 7, 1000])
def test_rhs_device_batch_bit_exact(gpu, n_inst):
    """lassie_rhs_device (one warp per parameterisation) on device buffers,
    against the oracle's RHS for every instance."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    base, _ = synth.make_c5(1)
    m = base[0]
    nm = solver.NativeModel.of(m)
    om = O.OracleModel(m.left, m.right)
    rng = np.random.default_rng(n_inst)
    x = rng.uniform(0, 2, (n_inst, m.n_species))
    k = 10.0 ** rng.uniform(-3, 3, (n_inst, m.n_reactions))
    dx_t = torch.zeros((n_inst, m.n_species), dtype=torch.float64, device="cuda")
    x_t = torch.tensor(x, device="cuda")
    k_t = torch.tensor(k, device="cuda")
    from lassie_gb300 import _native as nat
    nat.check(nat.load().lassie_rhs_device(nm.handle, n_inst, k_t.data_ptr(), x_t.data_ptr(),
                                           dx_t.data_ptr(), None), "lassie_rhs_device")
    torch.cuda.synchronize()
    dx = dx_t.cpu().numpy()
    for b in range(0, n_inst, max(1, n_inst // 50)):
        assert np.array_equal(dx[b], om.rhs(k[b], x[b])), b

"""The wide engine (one network above 512 species over the whole GPU,
blocked Gauss-Jordan inverse + FP64 refinement) against the CPU oracle,
through the C ABI.

Cases: the batched workload's recipe at 600 and 777 species on t in
[0, 0.2] (backward-Euler steps with the reference's stiffness switch; the
oracle finishes them in seconds), and the 4096-species workload on t in
[0, 0.02] against a stored oracle trajectory (two 4096 x 4096
factorisations take the oracle about two minutes).  All three are
insensitive to last-bit differences of the linear solve (checked with the
oracle's perturbation probe), so the mixed form is held to rtol 1e-6 /
atol 1e-9 at every sample and to the oracle's step counts.
"""
import os

import numpy as np
import pytest

from lassie_gb300 import _native as nat
from lassie_gb300 import solver, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-6, 1e-9
HERE = os.path.dirname(os.path.abspath(__file__))


def within(a, b, rtol=RTOL, atol=ATOL):
    return bool(np.all(np.abs(a - b) <= atol + rtol * np.abs(b)))


CASES = [(600, 1), (777, 0)]


@pytest.mark.parametrize("N,inst", CASES, ids=[f"n{n}-{i}" for n, i in CASES])
@pytest.mark.parametrize("lu_reuse", [True, False], ids=["reuse", "refactor"])
def test_wide_mixed_matches_oracle(gpu, N, inst, lu_reuse):
    m = synth.shorten(synth.make_sized(N, inst), 0.2, 5)
    ref, st_ref, rc = O.solve(m)
    assert rc == 0
    out, st = solver.simulate(m, engine="mixed", deadline_s=300, root="sqrt", lu_reuse=lu_reuse)
    assert st["status"] == 0
    assert within(out, ref), float(np.max(np.abs(out - ref) - RTOL * np.abs(ref)))
    assert (st["be_steps"], st["rkf_accepts"], st["newton_iters"]) == \
        (st_ref["be_steps"], st_ref["rkf_accepts"], st_ref["newton_iters"])


def test_wide_fp64_matches_oracle(gpu):
    """The FP64 form of the wide engine (Gauss-Jordan inverse in FP64, no
    refinement) rounds differently from the oracle's LU, by far less than
    the parity tolerance."""
    m = synth.shorten(synth.make_sized(600, 1), 0.2, 5)
    ref, st_ref, rc = O.solve(m)
    out, st = solver.simulate(m, engine="fp64", deadline_s=300, root="sqrt")
    assert st["status"] == 0
    assert within(out, ref, rtol=1e-10, atol=1e-13)
    assert st["be_steps"] == st_ref["be_steps"]


def test_wide_c3_matches_stored_oracle_trajectory(gpu):
    d = np.load(os.path.join(HERE, "oracle_fixtures", "c3_t002.npz"))
    m = synth.shorten(synth.make_c3(), 0.02, 3)
    assert np.array_equal(m.t, d["t"])
    # the rank-32 updates on the FP32 pipes (the tensor-core forms below)
    out, st = solver.simulate(m, engine="mixed", deadline_s=300, root="sqrt", tensor_cores="off")
    assert st["status"] == 0 and int(d["status"]) == 0
    assert within(out, d["out"]), float(np.max(np.abs(out - d["out"]) - RTOL * np.abs(d["out"])))
    assert st["be_steps"] == int(d["be_steps"])
    assert st["newton_iters"] == int(d["newton_iters"])


# BF16 factors are good to about 2^-9, so the refinement may take more
# sweeps than the default cap of 8
TC_MODES = [("tf32", 0), ("bf16", 32)]


@pytest.mark.parametrize("N,inst", CASES[:1], ids=["n600-1"])
@pytest.mark.parametrize("mode,refine_max", TC_MODES, ids=[m for m, _ in TC_MODES])
def test_wide_tensor_cores_match_oracle(gpu, N, inst, mode, refine_max):
    """Rank-32 updates on the tensor cores (tcgen05; TF32 products of split
    operands, or BF16 operands with FP32 accumulation): the refinement
    brings the solves to the FP64 solution, so the trajectory meets the same
    bar as the FP32-pipe factorisation."""
    m = synth.shorten(synth.make_sized(N, inst), 0.2, 5)
    ref, st_ref, rc = O.solve(m)
    out, st = solver.simulate(m, engine="mixed", deadline_s=300, root="sqrt", tensor_cores=mode,
                              refine_max=refine_max)
    assert st["status"] == 0
    assert within(out, ref), float(np.max(np.abs(out - ref) - RTOL * np.abs(ref)))
    assert (st["be_steps"], st["rkf_accepts"], st["newton_iters"]) == \
        (st_ref["be_steps"], st_ref["rkf_accepts"], st_ref["newton_iters"])


@pytest.mark.parametrize("mode,refine_max", TC_MODES, ids=[m for m, _ in TC_MODES])
def test_wide_c3_tensor_cores_match_stored_oracle_trajectory(gpu, mode, refine_max):
    d = np.load(os.path.join(HERE, "oracle_fixtures", "c3_t002.npz"))
    m = synth.shorten(synth.make_c3(), 0.02, 3)
    out, st = solver.simulate(m, engine="mixed", deadline_s=300, root="sqrt", tensor_cores=mode,
                              refine_max=refine_max)
    assert st["status"] == 0
    assert within(out, d["out"]), float(np.max(np.abs(out - d["out"]) - RTOL * np.abs(d["out"])))
    assert st["newton_iters"] == int(d["newton_iters"])


def test_wide_networks_do_not_batch(gpu):
    big = synth.shorten(synth.make_sized(600, 1), 0.1, 2)
    small = synth.shorten(synth.make_c4_instance(0), 0.1, 2)
    with pytest.raises(nat.LassieError) as e:
        solver.simulate_batch([big, small], engine="mixed")
    assert e.value.status == nat.ERR_TOO_LARGE


@pytest.mark.parametrize("tensor_cores", [False, True], ids=["fp32-pipes", "tensor-cores"])
def test_wide_c3_full_horizon_conserves_total_amount(gpu, tensor_cores):
    """The whole 4096-species workload (t in [0, 50], 100 samples) through
    lassie_solve: every reaction turns 2 molecules into 2, so sum(x) is a
    linear invariant of both step types (w^T M = w^T makes every Newton
    correction conserve it, converged or not); it holds at every sample to
    FP64 rounding over the ~6000 steps, and every species stays finite and
    non-negative.  (A revert of negative species would break the invariant;
    this trajectory has none.)"""
    m = synth.make_c3()
    out, st = solver.simulate(m, engine="mixed", deadline_s=600, root="sqrt",
                              tensor_cores=tensor_cores)
    assert st["status"] == 0 and st["nan_reverts"] == 0 and st["lu_failures"] == 0
    assert st["be_steps"] > 1000
    assert np.all(np.isfinite(out)) and np.all(out >= 0)
    total = out.sum(axis=1)
    assert np.all(np.abs(total - m.x0.sum()) <= 1e-10 * m.x0.sum()), \
        float(np.max(np.abs(total - m.x0.sum())))


def test_wide_two_level_tournament(gpu):
    """4200 species: the first panel's 4200 candidate rows make 33 groups of
    128 and 1056 survivors, more than one CTA holds (1024), so the FP32 pivot
    search takes a second tournament level (the FP64 form, 512 a CTA, takes
    three).  The FP64 form (Gauss-Jordan in FP64, no refinement) and the
    mixed form agree within rtol 1e-6 / atol 1e-9 with the same step
    counts."""
    m = synth.shorten(synth.make_sized(4200, 0), 0.02, 3)
    o64, s64 = solver.simulate(m, engine="fp64", deadline_s=900, root="sqrt")
    omx, smx = solver.simulate(m, engine="mixed", deadline_s=900, root="sqrt")
    assert s64["status"] == 0 == smx["status"]
    assert s64["lu_factorisations"] >= 1 and smx["lu_factorisations"] >= 1
    assert within(omx, o64), float(np.max(np.abs(omx - o64) - RTOL * np.abs(o64)))
    assert (s64["be_steps"], s64["rkf_accepts"]) == (smx["be_steps"], smx["rkf_accepts"])
    print(f"4200 species: {s64['be_steps']} backward-Euler steps, "
          f"{s64['lu_factorisations']} FP64 and {smx['lu_factorisations']} FP32 inversions")

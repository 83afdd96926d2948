"""The oracle's own spread on a sample of the 2048-instance workload.

LASSIE's loop (Simulation.cuh:737-909) turns last-bit differences of the
Newton corrections into different step sequences: the RKF45 accept test
compares |w1 - w2| / dt, a difference of nearly equal numbers, with
atol = 1e-12, and the Newton loop stops on an absolute norm.  Two valid FP64
implementations of the same loop -- the reference binary with cuSOLVER and
this oracle -- therefore part ways on some instances.  For every instance of
the sample this script runs the oracle once as is and eight more times with
a linear solve that differs from it in the last bits only:

  * five runs whose Newton corrections are scaled componentwise by
    (1 +- 2^-52) with seeded signs (seeds 1..5);
  * three runs with another rounding order of the LU (the triangular solves,
    the Schur update, or both, without fma).

Per instance it stores the unperturbed run's step counts and a digest of
its trajectory, and over the eight other runs the first sample at which any
of them leaves rtol 1e-6 / atol 1e-9 of the unperturbed trajectory and the
largest excess over that tolerance.

A second spread (``--normwise``, added to the same file) models solvers of
the mixed form's accuracy class: five runs whose Newton corrections move by
+- 2^-53 * max|dx| per component (an iterative refinement that stops on a
normwise bound is accurate to about that).  The GPU test holds the mixed
form to the first spread, or where that fails to the second, and reports
which.  Perturbed normwise runs often end in the reference's permanent
dt/10 reverts and run to the iteration cap, so ``--only=j,...`` probes just
the sample positions that leave the first spread (the others keep a zero
spread and must then agree within the tolerance).

Sample: every 13th instance of the workload (152 instances, seeds
1000*4 + 13*j), shortened to t in [0, 2] with 5 samples, at most 2500 loop
iterations (the benchmark's FP64-form comparison).  About 50 minutes on 7
cores:

    python tests/oracle_fixtures/make_c4_spread.py [processes]
    python tests/oracle_fixtures/make_c4_spread.py [processes] --normwise [--only=60,87,121]
"""
from __future__ import annotations

import hashlib
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

STRIDE, COUNT, HORIZON, NSAMP, CAP = 13, 152, 2.0, 5, 2500
RTOL, ATOL = 1e-6, 1e-9
ULP_SEEDS = (1, 2, 3, 4, 5)
LU_VARIANTS = (1, 2, 3)
STAT_KEYS = ("be_steps", "rkf_accepts", "newton_iters", "nan_reverts", "rkf_retries")


def sample_model(j: int):
    from lassie_gb300 import synth
    return synth.shorten(synth.make_c4_instance(STRIDE * j), HORIZON, NSAMP)


def digest(out: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(out, np.float64).tobytes()).hexdigest()


def excess(a, b):
    """Per sample, the largest amount by which |a - b| exceeds the tolerance."""
    return np.max(np.abs(a - b) - ATOL - RTOL * np.abs(b), axis=1)


def one(j: int):
    from oracle import oracle as O
    m = sample_model(j)
    ref, st, rc = O.solve(m, max_steps=CAP)
    nt = ref.shape[0]
    first, worst, moved = nt, 0.0, 0
    for kind, arg in [("ulp", s) for s in ULP_SEEDS] + [("lu", v) for v in LU_VARIANTS]:
        ctx = O.solve_perturbation(2.0 ** -52, arg) if kind == "ulp" else O.lu_variant(arg)
        with ctx:
            p, sp, _ = O.solve(m, max_steps=CAP)
        e = excess(p, ref)
        if np.any(e > 0):
            first = min(first, int(np.argmax(e > 0)))
        worst = max(worst, float(e.max()))
        moved += int(tuple(sp[k] for k in STAT_KEYS) != tuple(st[k] for k in STAT_KEYS))
    return (j, m.n_species, rc, digest(ref), [st[k] for k in STAT_KEYS], first, worst, moved)


NORMWISE_EPS = 2.0 ** -53


def normwise_run(task):
    """One run of the normwise spread: seed 0 is the unperturbed oracle."""
    from oracle import oracle as O
    j, seed = task
    m = sample_model(j)
    if seed == 0:
        out, _, _ = O.solve(m, max_steps=CAP)
    else:
        with O.normwise_perturbation(NORMWISE_EPS, seed):
            out, _, _ = O.solve(m, max_steps=CAP)
    return j, seed, out


def main_normwise(procs: int, only) -> int:
    """The normwise spread of the instances in `only` (sample positions; all
    when empty).  Instances not probed keep first divergence 0 and excess 0,
    so the GPU test holds them to the tolerance itself when they leave the
    FP64 solvers' spread."""
    path = os.path.join(HERE, "c4_spread.npz")
    f = dict(np.load(path))
    js = list(only) if only else list(range(COUNT))
    tasks = [(j, sd) for j in js for sd in (0,) + ULP_SEEDS]
    with mp.get_context("spawn").Pool(procs) as pool:
        runs = pool.map(normwise_run, tasks, chunksize=1)
    outs = {(j, sd): o for j, sd, o in runs}
    first = np.zeros(COUNT, np.int32)
    worst = np.zeros(COUNT, np.float64)
    for j in js:
        ref = outs[(j, 0)]
        fj, wj = ref.shape[0], 0.0
        for sd in ULP_SEEDS:
            e = excess(outs[(j, sd)], ref)
            if np.any(e > 0):
                fj = min(fj, int(np.argmax(e > 0)))
            wj = max(wj, float(e.max()))
        first[j], worst[j] = fj, wj
    f["first_divergence_normwise"] = first
    f["worst_excess_normwise"] = worst
    f["normwise_eps"] = NORMWISE_EPS
    f["normwise_probed"] = np.array(sorted(js), np.int32)
    np.savez_compressed(path, **f)
    print(f"normwise spread of {len(js)} instances: {sum(1 for j in js if worst[j] > 0)} move")
    return 0


def main(procs: int) -> int:
    t0 = time.time()
    # larger networks first, so the pool's tail is short
    sizes = [sample_model(j).n_species for j in range(COUNT)]
    order = sorted(range(COUNT), key=lambda j: -sizes[j])
    with mp.get_context("spawn").Pool(procs) as pool:
        rows = sorted(pool.map(one, order, chunksize=1))
    np.savez_compressed(
        os.path.join(HERE, "c4_spread.npz"),
        index=np.array([STRIDE * r[0] for r in rows], np.int32),
        n_species=np.array([r[1] for r in rows], np.int32),
        status=np.array([r[2] for r in rows], np.int32),
        digest=np.array([r[3] for r in rows]),
        stats=np.array([r[4] for r in rows], np.int64),
        stat_keys=np.array(STAT_KEYS),
        first_divergence=np.array([r[5] for r in rows], np.int32),
        worst_excess=np.array([r[6] for r in rows], np.float64),
        runs_with_other_steps=np.array([r[7] for r in rows], np.int32),
        horizon=HORIZON, nsamp=NSAMP, cap=CAP)
    sens = sum(1 for r in rows if r[6] > 0)
    print(f"{COUNT} instances, {sens} decision-sensitive, {time.time() - t0:.0f} s")
    return 0


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    procs = int(args[0]) if args else (os.cpu_count() or 1)
    only = [int(a) for o in sys.argv[1:] if o.startswith("--only=") for a in o[7:].split(",")]
    sys.exit(main_normwise(procs, only) if "--normwise" in sys.argv else main(procs))

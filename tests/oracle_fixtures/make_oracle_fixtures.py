"""Fixtures computed by the CPU oracle (oracle/) for cases too slow to run
inside the test suite.  The GPU machine's tests must not spend minutes in
the oracle, so the trajectories are stored:

  * c3_t002: the 4096-species workload on t in [0, 0.02] (two
    backward-Euler steps with 4096 x 4096 LU factorisations, about two
    minutes on one core);
  * c3_t05: the same network on t in [0, 0.5] (11 samples, about fifty
    backward-Euler steps, tens of minutes);
  * c2_t01: the stiff 512-species network on t in [0, 0.1] (6 samples;
    three negative-species reverts take the backward-Euler step to 1e-5, so
    8 893 steps with a 512 x 512 LU each, fifteen minutes -- its whole
    horizon t in [0, 100] would take the oracle days on one core);
  * c5_full: the 256-species adjoint network (base rate constants) over its
    whole horizon, 40 samples in (0, 10].

    python tests/oracle_fixtures/make_oracle_fixtures.py [name ...]

Each fixture holds the sampling times, the oracle's trajectory and status
and its step counts; the network and its parameters are regenerated from
their seed by lassie_gb300.synth.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lassie_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402


def c3_short():
    return synth.shorten(synth.make_c3(), 0.02, 3)


def c3_t05():
    return synth.shorten(synth.make_c3(), 0.5, 11)


def c5_full():
    return synth.make_c5(1)[0][0]


def c2_t01():
    return synth.shorten(synth.make_c2(), 0.1, 6)


CASES = {"c3_t002": c3_short, "c3_t05": c3_t05, "c2_t01": c2_t01, "c5_full": c5_full}
# cases whose fixture also holds the oracle's spread: the first sample at
# which any run with a last-bit different solve leaves rtol 1e-6 /
# atol 1e-9, and the largest excess (FP64 solvers: five one-ulp
# perturbations and three LU rounding orders; normwise: five runs with
# corrections moved by 2^-53 max|dx|)
SPREAD = ("c5_full",)
# a perturbed run may take the reference's permanent dt/10 reverts and run
# far longer than the unperturbed one: it stops at this many times the
# unperturbed run's loop iterations
SPREAD_CAP = 4


def spread(m, base, runs, cap):
    """A perturbed run stops after `cap` loop iterations; its unreached
    samples stay 0 and count as leaving the tolerance there."""
    first, worst = base.shape[0], 0.0
    for ctx in runs:
        with ctx:
            p, _, _ = O.solve(m, max_steps=cap)
        e = np.max(np.abs(p - base) - 1e-9 - 1e-6 * np.abs(base), axis=1)
        if np.any(e > 0):
            first = min(first, int(np.argmax(e > 0)))
        worst = max(worst, float(e.max()))
    return first, worst


def main():
    names = sys.argv[1:] or list(CASES)
    for name in names:
        make = CASES[name]
        m = make()
        t0 = time.time()
        out, st, rc = O.solve(m)
        extra = {}
        if name in SPREAD:
            cap = SPREAD_CAP * st["outer_iters"]
            f1, w1 = spread(m, out, [O.solve_perturbation(2.0 ** -52, q) for q in range(1, 6)]
                            + [O.lu_variant(v) for v in (1, 2, 3)], cap)
            f2, w2 = spread(m, out, [O.normwise_perturbation(2.0 ** -53, q) for q in range(1, 6)],
                            cap)
            extra = dict(first_divergence=f1, worst_excess=w1, first_divergence_normwise=f2,
                         worst_excess_normwise=w2)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), t=m.t, out=out, status=rc,
                            be_steps=st["be_steps"], rkf_accepts=st["rkf_accepts"],
                            newton_iters=st["newton_iters"], nan_reverts=st["nan_reverts"],
                            seconds=time.time() - t0, **extra)
        print(name, rc, st, "%.1fs" % (time.time() - t0), flush=True)


if __name__ == "__main__":
    main()

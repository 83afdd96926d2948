"""Generate the golden fixtures from the reference LASSIE binary.

Runs ``oracle/_ref/lassie_ref_f64`` (the unmodified reference sources built
by ``oracle/build_ref.sh`` with 17-digit Solution output) on seeded small
models and stores inputs and outputs as ``tests/golden/<case>.npz``.  The
reference binary needs a CUDA GPU, so this runs on the GPU machine:

    python tests/golden/make_golden.py <out_dir> [--float]

(--float: the reference's -p float runs, stored under tests/golden/float/;
--long: two longer horizons, stored under tests/golden/long/).

Each fixture holds the dense stoichiometries, rate constants, initial state,
sampling times, the reference's trajectory (``ref``), its number of loop
iterations (``ref_outer_iters``, the lines of its ProgressSimulation) and
its integration time.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lassie_gb300 import synth  # noqa: E402
from lassie_gb300.model import write_folder  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "lassie_ref_f64")


def long_cases():
    """Longer horizons, stored under tests/golden/long/ (--long): the same
    networks and samples as tests/oracle_fixtures/c2_t01.npz and
    c3_t05.npz, so that the stored oracle trajectories are checked against
    the reference without running either."""
    yield "c2_t01", synth.shorten(synth.make_c2(), 0.1, 6)
    yield "c3_t05", synth.shorten(synth.make_c3(), 0.5, 11)


def cases():
    yield "c1", synth.make_c1()
    for kind in ("decay", "conversion", "dimer", "bimolecular", "source", "reversible"):
        yield "tiny_" + kind, synth.tiny_network(kind)
    yield "c4_i2_t1", synth.shorten(synth.make_c4_instance(2), 1.0, 11)
    yield "c4_i7_t05", synth.shorten(synth.make_c4_instance(7), 0.5, 6)
    yield "c2_t0012", synth.shorten(synth.make_c2(), 0.012, 3)
    fed = synth.tiny_network("reversible")
    fed.feed = np.array([0.0, 0.8, 0.0])
    yield "tiny_reversible_fed", fed


def read_solution(path: str, ncols: int) -> np.ndarray:
    rows = []
    with open(path) as f:
        for line in f:
            vals = [float(v) for v in line.strip().split("\t") if v != ""]
            if vals:
                rows.append(vals)
    return np.asarray(rows)


def main(out_dir: str, precision: str = "double", long: bool = False) -> int:
    """precision "float": the reference's -p float runs (Simulation<float>);
    long: the longer-horizon cases instead of the standard set."""
    os.makedirs(out_dir, exist_ok=True)
    status = 0
    extra = ["-p", "float"] if precision == "float" else []
    for name, m in (long_cases() if long else cases()):
        with tempfile.TemporaryDirectory() as tmp:
            inp, outp = os.path.join(tmp, "in"), os.path.join(tmp, "out")
            write_folder(m, inp)
            t0 = time.time()
            r = subprocess.run([REF, inp, outp] + extra, stdout=subprocess.PIPE,
                               stderr=subprocess.PIPE, text=True, timeout=1200)
            wall = time.time() - t0
            mt = re.search(r"LASSIE_REF integration_ms ([0-9.eE+-]+)", r.stderr)
            sol_path = os.path.join(outp, "output", "Solution")
            sol = read_solution(sol_path, m.n_species + 1) if os.path.exists(sol_path) else None
            # the reference writes one ProgressSimulation line per loop
            # iteration (Simulation.cuh:671-673)
            prog = os.path.join(outp, "output", "ProgressSimulation")
            outer = sum(1 for ln in open(prog) if ln.strip()) if os.path.exists(prog) else -1
        if r.returncode != 0 or sol is None:
            print(f"{name}: reference failed rc={r.returncode}\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
            status = 1
            continue
        np.savez_compressed(
            os.path.join(out_dir, name + ".npz"), left=m.left, right=m.right, k=m.k,
            x0=m.x0, t=m.t, feed=(m.feed if m.feed is not None else np.zeros(0)),
            ref_t=sol[:, 0], ref=sol[:, 1:], wall_s=wall, ref_outer_iters=outer,
            integration_ms=float(mt.group(1)) if mt else -1.0)
        print(f"{name}: N={m.n_species} nt={m.t.shape[0]} wall={wall:.2f}s "
              f"integration_ms={mt.group(1) if mt else '?'}")
    return status


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a not in ("--float", "--long")]
    prec = "float" if "--float" in sys.argv[1:] else "double"
    long = "--long" in sys.argv[1:]
    sub = "float" if prec == "float" else ("long" if long else "")
    default = os.path.join(ROOT, "tests", "golden", sub)
    sys.exit(main(args[0] if args else default, prec, long))

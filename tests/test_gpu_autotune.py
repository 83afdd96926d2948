"""The factorisation autotuner (lassie_opts.tile_rows = 0).

At batch creation the trailing-update tile rows of the per-CTA
factorisations (8, 4 or 2 rows per thread) are timed on the device per
network-size band and the fastest is stored per instance.  Every choice
gives the same factors bit for bit, so the trajectories do not depend on
the choice: checked here for both forms against each fixed choice (and, for
the FP64 form, against the oracle), on networks from every size band.  The
choice itself is cached per process, so a second batch repeats it."""
import numpy as np
import pytest

from lassie_gb300 import solver, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _models():
    # one network per size band (<= 32, 64, 128, 256, 512 species)
    sizes = (24, 50, 100, 200, 400)
    return [synth.shorten(synth.make_sized(n, 3), 0.2, 3) for n in sizes]


@pytest.mark.parametrize("engine", ["fp64", "mixed"])
def test_tile_rows_leave_trajectories_bit_identical(gpu, engine):
    models = _models()
    runs = {}
    for rows in (0, 8, 4, 2):
        b = solver.Batch(models, engine=engine, deadline_s=300, root="sqrt", tile_rows=rows)
        b.run(0)
        b.sync()
        outs, stats = b.read()
        assert all(s["status"] == 0 for s in stats)
        runs[rows] = ([o.copy() for o in outs], b.tile_rows(), [s["be_steps"] for s in stats])
    if engine == "fp64":
        for m, o in zip(models, runs[8][0]):
            ref, _, rc = O.solve(m)
            assert rc == 0 and np.array_equal(o, ref)
    for rows in (0, 4, 2):
        for a, c in zip(runs[rows][0], runs[8][0]):
            assert np.array_equal(a, c), rows
        assert runs[rows][2] == runs[8][2]
    for rows in (8, 4, 2):
        assert runs[rows][1] == [rows] * len(models)
    assert set(runs[0][1]) <= {8, 4, 2}


def test_autotuned_choice_repeats(gpu):
    models = _models()
    first = solver.Batch(models, engine="mixed", deadline_s=300).tile_rows()
    again = solver.Batch(models, engine="mixed", deadline_s=300).tile_rows()
    assert first == again
    # instances of one size band share the band's choice
    same_band = [synth.shorten(synth.make_sized(n, 1), 0.2, 3) for n in (130, 250)]
    rows = solver.Batch(same_band, engine="mixed", deadline_s=300).tile_rows()
    assert rows[0] == rows[1]

"""A batch run (queue reset + one persistent launch) captured in a CUDA graph
and replayed gives the same trajectories and counters as a direct run."""
import numpy as np
import pytest

from lassie_gb300 import solver, synth

pytestmark = pytest.mark.gpu


def test_batch_run_replays_from_a_cuda_graph(gpu):
    torch = pytest.importorskip("torch")
    models = [synth.shorten(m, 0.5, 3) for m in synth.make_c4(24)]
    b = solver.Batch(models, engine="mixed", deadline_s=120)
    s = torch.cuda.Stream()
    b.run(s.cuda_stream)
    torch.cuda.synchronize()
    ref, st_ref = b.read()
    ref = [r.copy() for r in ref]
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.run(s.cuda_stream)
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        out, st = b.read()
        for r, o in zip(ref, out):
            assert np.array_equal(r, o)
        assert [x["be_steps"] for x in st] == [x["be_steps"] for x in st_ref]
        assert all(x["status"] == 0 for x in st)

"""lassie_solve_noalloc: the integrator for callers that cannot allocate
device memory (hosts running under another framework's memory pool that owns
all device memory, plugins barred from allocating after start-up, real-time
loops that must not wait on the allocator).  Its working memory is a static
device arena inside the library, so the caller only provides device buffers
for the inputs and the trajectory.

Checked through the C ABI against lassie_solve (which allocates) on two
calls in a row -- the second call finds the first call's data in the arena --
within the parity tolerance of the other GPU tests; the FP64 form also bit
for bit against the oracle.  A second call leaves the device's free memory
unchanged.  Collected last, so that a run stopping at the first failure has
run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from lassie_gb300 import _native as nat
from lassie_gb300 import solver, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-6, 1e-9


def _device(a, torch):
    return torch.tensor(np.ascontiguousarray(a, np.float64), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("engine", ["mixed", "fp64"])
def test_noalloc_matches_solve_on_two_calls(gpu, engine):
    torch = pytest.importorskip("torch")
    L = nat.load()
    m = synth.shorten(synth.make_c4_instance(2), 1.0, 11)  # 84 species, BE and RKF45 steps
    assert m.n_species <= 128
    nm = solver.NativeModel.of(m)
    ref, st_ref = solver.simulate(m, engine=engine, nm=nm, root="sqrt")
    assert st_ref["status"] == 0
    oracle_ref = None
    if engine == "fp64":
        oracle_ref, _, rc = O.solve(m)
        assert rc == 0
    dk, dx0, dt = _device(m.k, torch), _device(m.x0, torch), _device(m.t, torch)
    nt, N = m.t.shape[0], m.n_species
    free = []
    for call in range(2):
        dout = torch.full((nt, N), -1.0, dtype=torch.float64, device="cuda")
        st = nat.Stats()
        o = solver.make_opts(m, engine, root="sqrt")
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        rc = L.lassie_solve_noalloc(nm.handle, dk.data_ptr(), dx0.data_ptr(), dt.data_ptr(), nt,
                                    C.byref(o), dout.data_ptr(), C.byref(st), None)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        assert rc == 0, (call, rc, L.lassie_last_error())
        out = dout.cpu().numpy()
        assert np.all(np.abs(out - ref) <= ATOL + RTOL * np.abs(ref)), call
        assert st.be_steps == st_ref["be_steps"] and st.rkf_accepts == st_ref["rkf_accepts"]
        if oracle_ref is not None:
            assert np.array_equal(out, oracle_ref), call
            assert np.array_equal(out, ref), call
    # the second call (set-up done by the first) allocates nothing
    assert free[2] == free[3], free


def test_noalloc_without_stats_or_samples(gpu):
    torch = pytest.importorskip("torch")
    L = nat.load()
    m = synth.tiny_network("dimer")
    nm = solver.NativeModel.of(m)
    dk, dx0 = _device(m.k, torch), _device(m.x0, torch)
    rc = L.lassie_solve_noalloc(nm.handle, dk.data_ptr(), dx0.data_ptr(), None, 0,
                                C.byref(solver.make_opts(m)), None, None, None)
    assert rc == 0, L.lassie_last_error()


def test_noalloc_rejects_networks_beyond_the_arena(gpu):
    torch = pytest.importorskip("torch")
    L = nat.load()
    q = next(q for q in range(100) if synth.make_c4_instance(q).n_species > 128)
    m = synth.shorten(synth.make_c4_instance(q), 0.1, 2)
    nm = solver.NativeModel.of(m)
    dk, dx0, dt = _device(m.k, torch), _device(m.x0, torch), _device(m.t, torch)
    dout = torch.zeros((2, m.n_species), dtype=torch.float64, device="cuda")
    rc = L.lassie_solve_noalloc(nm.handle, dk.data_ptr(), dx0.data_ptr(), dt.data_ptr(), 2,
                                C.byref(solver.make_opts(m)), dout.data_ptr(), None, None)
    assert rc == nat.ERR_TOO_LARGE

"""The tensor-core (tcgen05) tile product behind the wide engine's rank-32
updates: one 128 x 32 by 32 x 128 product through TF32 MMAs on split
operands, against an FP64 product on the host.  The split keeps the error
near FP32 rounding: below 1e-6 of sum |a||b| per entry."""
import numpy as np
import pytest

from lassie_gb300 import _native as nat

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1])
def test_tc_tile_product_matches_fp64(gpu, seed):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(128, 32)).astype(np.float32)
    b = (rng.normal(size=(32, 128)) * 10.0 ** rng.uniform(-3, 3, size=(32, 1))).astype(np.float32)
    da = torch.tensor(a, device="cuda")
    db = torch.tensor(b, device="cuda")
    dd = torch.full((128, 128), float("nan"), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.check(nat.load().lassie_tc_selftest(da.data_ptr(), db.data_ptr(), dd.data_ptr(),
                                            st.data_ptr(), None), "lassie_tc_selftest")
    torch.cuda.synchronize()
    assert int(st.item()) == 1
    d = dd.cpu().numpy().astype(np.float64)
    ref = a.astype(np.float64) @ b.astype(np.float64)
    scale = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64)
    err = np.abs(d - ref) / scale
    assert np.all(np.isfinite(d))
    assert err.max() < 1e-6, float(err.max())

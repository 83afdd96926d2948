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


def _bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("seed", [0, 1])
def test_tc_tile_product_bf16(gpu, seed):
    """kind::f16 MMAs on BF16 operands with FP32 accumulation: the products
    of the BF16-rounded operands are exact, their FP32 sum is good to a few
    FP32 roundings of sum |a||b|; against the unrounded FP64 product the
    error is the BF16 rounding of the operands (about 2^-8 of sum |a||b|)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(128, 32)).astype(np.float32)
    b = (rng.normal(size=(32, 128)) * 10.0 ** rng.uniform(-3, 3, size=(32, 1))).astype(np.float32)
    da = torch.tensor(a, device="cuda")
    db = torch.tensor(b, device="cuda")
    dd = torch.full((128, 128), float("nan"), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.check(nat.load().lassie_tc_selftest_bf16(da.data_ptr(), db.data_ptr(), dd.data_ptr(),
                                                 st.data_ptr(), None), "lassie_tc_selftest_bf16")
    torch.cuda.synchronize()
    assert int(st.item()) == 1
    d = dd.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(d))
    scale = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64)
    ref16 = _bf16(a) @ _bf16(b)
    assert (np.abs(d - ref16) / scale).max() < 1e-6
    ref = a.astype(np.float64) @ b.astype(np.float64)
    err = (np.abs(d - ref) / scale).max()
    assert 1e-5 < err < 2.0 ** -7, err

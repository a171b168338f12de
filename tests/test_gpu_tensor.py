"""Split-BF16 tensor-core path (tcgen05): the single-tile product first, then whole transforms
whose first pass runs on the tensor cores, against the FP64 oracle at the split-BF16 tolerance."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TC_TOL = 2e-6  # split-BF16 tolerance (FP32 accumulation of three BF16 parts per operand)


@pytest.fixture(scope="module")
def F():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import fft_gb300
    return fft_gb300


def test_tile_product(F):
    rng = np.random.default_rng(1)
    a = rng.uniform(-1, 1, (128, 32)).astype(np.float32)
    bt = rng.uniform(-1, 1, (32, 32)).astype(np.float32)
    d, flags = F.diag_tc_tile(a, bt)
    assert flags == 0
    ref = a.astype(np.float64) @ bt.astype(np.float64).T
    assert rel_l2(d, ref) <= TC_TOL, rel_l2(d, ref)
    # layout check with an exact case: B = identity gives A back to ~2^-24
    d, flags = F.diag_tc_tile(a, np.eye(32, dtype=np.float32))
    assert flags == 0 and np.max(np.abs(d - a)) <= 1e-6 * np.max(np.abs(a))


SIZES = [16, 64, 112, 480, 1000, 1024, 1920, 4096, 16384, 7, 3, 240, 2187, 15625]


@pytest.mark.parametrize("n", SIZES)
def test_tensor_core_transforms(F, n):
    import torch
    rng = np.random.default_rng(n)
    b = 37
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(np.complex64)
    p = F.Plan(n, "f32", "complex", b, precision="split_bf16")
    assert "precision=split_bf16" in p.tuning()["choice"]
    xi = torch.from_numpy(x).cuda()
    y = torch.empty_like(xi)
    z = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), y.data_ptr(), 0)
    p.exec(True, y.data_ptr(), z.data_ptr(), 0)
    torch.cuda.synchronize()
    ref = oracle.batch(x.astype(np.complex128), n, real=False, inverse=False)
    assert rel_l2(y.cpu().numpy(), ref) <= TC_TOL, rel_l2(y.cpu().numpy(), ref)
    assert rel_l2(z.cpu().numpy() / n, x) <= 2 * TC_TOL
    import ctypes
    flags = ctypes.c_uint(9)
    assert F.lib().ssfft_plan_error(p.handle, ctypes.byref(flags)) == 0 and flags.value == 0


def test_tensor_core_uneven_batch(F):
    import torch
    rng = np.random.default_rng(8)
    sizes = [64, 80, 100, 480, 1024, 3840, 16384, 7, 250] * 2
    x = (rng.uniform(-1, 1, sum(sizes)) + 1j * rng.uniform(-1, 1, sum(sizes))).astype(np.complex64)
    m = F.Multi(sizes, "f32", precision="split_bf16")
    xi = torch.from_numpy(x).cuda()
    a = torch.empty_like(xi)
    m.exec(False, xi.data_ptr(), a.data_ptr(), 0)
    torch.cuda.synchronize()
    got = a.cpu().numpy()
    off = 0
    for n in sizes:
        ref = oracle.fft(x[off:off + n].astype(np.complex128))
        assert rel_l2(got[off:off + n], ref) <= TC_TOL, n
        off += n

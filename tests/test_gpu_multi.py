"""Uneven-size batches (ssfft_multi_*): every transform of a mixed-size list equals the FP64
oracle within the FP32 tolerance, and the CUDA-graph submission equals the plain per-size
launches bit for bit."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def F():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fft_gb300
    fft_gb300.lib()
    return fft_gb300


def test_fast_sizes_count(F):
    assert len(F.fast_sizes(64, 16384)) == 175


def test_multi_matches_oracle_and_plain(F):
    rng = np.random.default_rng(21)
    pool = F.fast_sizes(64, 16384)
    lg = rng.uniform(np.log(64), np.log(16384), 300)
    sizes = [min(pool, key=lambda s, v=v: abs(np.log(s) - v)) for v in lg] + [7, 97, 100]
    total = sum(sizes)
    x = (rng.uniform(-1, 1, total) + 1j * rng.uniform(-1, 1, total)).astype(np.complex64)
    m = F.Multi(sizes, "f32")
    assert m.info()["total_elements"] == total
    xi = torch.from_numpy(x).cuda()
    a = torch.empty_like(xi)
    b = torch.empty_like(xi)
    for inverse in (False, True):
        m.exec(inverse, xi.data_ptr(), a.data_ptr(), 0)
        m.exec_plain(inverse, xi.data_ptr(), b.data_ptr(), 0)
        torch.cuda.synchronize()
        ga, gb = a.cpu().numpy(), b.cpu().numpy()
        assert np.array_equal(ga, gb)
        off = 0
        for n in sizes:
            ref = oracle.fft(x[off:off + n].astype(np.complex128), inverse)
            assert rel_l2(ga[off:off + n], ref) <= 1e-6, (n, inverse)
            off += n
    m.close()

"""Uneven-size batches (ssfft_multi_*): every transform of a mixed-size list equals the FP64
oracle within the FP32 (FP64) tolerance, and the work-item queue kernels (one CUDA graph) equal
the plain per-size launches bit for bit -- the same schedules and tables, so the same roundings --
as does the per-size graph design kept behind the debug switch multi_mode=1."""
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


def _uneven(F, rng, count, lo=64, hi=16384):
    pool = F.fast_sizes(lo, hi)
    lg = rng.uniform(np.log(lo), np.log(hi), count)
    return [min(pool, key=lambda s, v=v: abs(np.log(s) - v)) for v in lg]


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_queue_equals_plain_and_oracle_both_dtypes(F, dt):
    """A larger list (every class shape; partial work items) in FP32 and FP64, twice in a row
    through the same captured graph."""
    rng = np.random.default_rng(31 if dt == "f32" else 32)
    sizes = _uneven(F, rng, 2000 if dt == "f32" else 600, 64, 16384 if dt == "f32" else 8192)
    cdt = np.complex64 if dt == "f32" else np.complex128
    total = sum(sizes)
    x = (rng.uniform(-1, 1, total) + 1j * rng.uniform(-1, 1, total)).astype(cdt)
    m = F.Multi(sizes, dt)
    info = m.info()
    assert 1 <= info["launches"] < info["distinct_sizes"]
    xi = torch.from_numpy(x).cuda()
    a = torch.empty_like(xi)
    b = torch.empty_like(xi)
    tol = 1e-6 if dt == "f32" else 1e-14
    starts = np.concatenate([[0], np.cumsum(sizes)])
    for inverse in (False, True):
        m.exec_plain(inverse, xi.data_ptr(), b.data_ptr(), 0)
        for _ in range(2):
            a.fill_(0)
            m.exec(inverse, xi.data_ptr(), a.data_ptr(), 0)
            torch.cuda.synchronize()
            assert torch.equal(a, b)
        ga = a.cpu().numpy()
        for i in range(0, len(sizes), 17):
            n, o = sizes[i], starts[i]
            ref = oracle.fft(x[o:o + n].astype(np.complex128), inverse)
            assert rel_l2(ga[o:o + n], ref) <= tol, (n, inverse)
    m.close()


def test_per_size_graph_mode_still_matches(F, monkeypatch):
    rng = np.random.default_rng(41)
    sizes = _uneven(F, rng, 400)
    total = sum(sizes)
    x = (rng.uniform(-1, 1, total) + 1j * rng.uniform(-1, 1, total)).astype(np.complex64)
    xi = torch.from_numpy(x).cuda()
    a, b = torch.empty_like(xi), torch.empty_like(xi)
    monkeypatch.setenv("SSFFT_DEBUG", "multi_mode=1")
    m1 = F.Multi(sizes, "f32")
    monkeypatch.delenv("SSFFT_DEBUG")
    m2 = F.Multi(sizes, "f32")
    assert m1.info()["launches"] == m1.info()["distinct_sizes"]
    m1.exec(False, xi.data_ptr(), a.data_ptr(), 0)
    m2.exec(False, xi.data_ptr(), b.data_ptr(), 0)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    m1.close()
    m2.close()

"""Two-CTA cluster (pair) kernel for long complex FP32 transforms (an option; SSFFT_DEBUG=pair_min=<n> turns
it on by size): the planner's splits, explicit splits, the single-CTA schedule of the same sizes,
uneven batches that mix pair and single-CTA sizes, and option validation -- all against the
oracle."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu
F32_TOL = 1e-6


@pytest.fixture(scope="module")
def F():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import fft_gb300
    return fft_gb300


def _complex_case(F, n, batch, expect_pair=True, **opts):
    import torch
    rng = np.random.default_rng(n + batch)
    x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
    if expect_pair is not None:
        F.schedule_options(**opts)
        name = F.schedule_name(n, "f32", "complex", batch)
        F.schedule_options()
        assert name.startswith("ssfft_cl::pair<") == expect_pair, name
    p = F.Plan(n, "f32", "complex", batch, **opts)
    xi = torch.from_numpy(x).cuda()
    y = torch.empty_like(xi)
    z = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), y.data_ptr(), 0)
    p.exec(True, y.data_ptr(), z.data_ptr(), 0)
    torch.cuda.synchronize()
    xd = x.astype(np.complex128)
    ref = oracle.batch(xd, n, real=False, inverse=False)
    assert rel_l2(y.cpu().numpy(), ref) <= F32_TOL, rel_l2(y.cpu().numpy(), ref)
    refi = oracle.batch(ref, n, real=False, inverse=True)
    assert rel_l2(z.cpu().numpy(), refi) <= F32_TOL
    assert np.array_equal(xi.cpu().numpy(), x), "input left untouched"


@pytest.mark.parametrize("n", [9000, 10000, 12288, 13824, 15000, 15552, 16000, 16384])
def test_default_pair_splits(F, n, monkeypatch):
    monkeypatch.setenv("SSFFT_DEBUG", "pair_min=8193")  # the planner's split where the pair kernel is on
    _complex_case(F, n, 37)


@pytest.mark.parametrize("radices,split", [([16, 8, 16, 8], 2), ([32, 32, 16], 1), ([16, 32, 32], 1),
                                           ([32, 16, 32], 2), ([8, 8, 16, 16], 2)])
def test_explicit_splits_16384(F, radices, split):
    _complex_case(F, 16384, 19, radices=radices, cluster_split=split)


@pytest.mark.parametrize("n,radices,split", [(15360, [8, 15, 16, 8], 2), (8192, [8, 16, 4, 16], 2),
                                             (4000, [10, 20, 20], 1), (12000, [12, 10, 10, 10], 2)])
def test_explicit_splits_other_sizes(F, n, radices, split):
    _complex_case(F, n, 11, radices=radices, cluster_split=split)


@pytest.mark.parametrize("n", [12288, 16384])
def test_single_cta_schedule_of_pair_sizes(F, n):
    _complex_case(F, n, 9, expect_pair=False, cluster_split=-1)


def test_pair_register_cap(F, monkeypatch):
    monkeypatch.setenv("SSFFT_DEBUG", "pair_min=8193")
    _complex_case(F, 16384, 23, min_ctas_per_sm=3)


def test_uneven_batch_with_pair_sizes(F, monkeypatch):
    import torch
    monkeypatch.setenv("SSFFT_DEBUG", "pair_min=8193")
    sizes = [16384, 64, 9000, 4096, 12288, 15000, 16384, 100, 13824, 10000] * 3
    rng = np.random.default_rng(5)
    total = sum(sizes)
    x = (rng.uniform(-1, 1, total) + 1j * rng.uniform(-1, 1, total)).astype(np.complex64)
    m = F.Multi(sizes, "f32")
    xi = torch.from_numpy(x).cuda()
    y = torch.empty_like(xi)
    for inv in (False, True):
        m.exec(inv, xi.data_ptr(), y.data_ptr(), 0)
        torch.cuda.synchronize()
        got = y.cpu().numpy()
        off = 0
        for n in sizes:
            ref = oracle.fft(x[off:off + n].astype(np.complex128), inv)
            assert rel_l2(got[off:off + n], ref) <= F32_TOL, (n, inv)
            off += n


def test_pair_autotune(F, monkeypatch):
    monkeypatch.setenv("SSFFT_DEBUG", "pair_min=8193")
    _complex_case(F, 16384, 64, expect_pair=None, autotune=1)


def test_invalid_pair_options_refused(F):
    with pytest.raises(F.SsfftError):
        F.Plan(16384, "f32", "complex", 4, cluster_split=2)  # no radices
    with pytest.raises(F.SsfftError):
        F.Plan(10000, "f32", "complex", 4, radices=[25, 16, 25], cluster_split=1)  # odd first phase
    with pytest.raises(F.SsfftError):
        F.Plan(16384, "f32", "complex", 4, radices=[16, 16, 8, 8], cluster_split=4)  # empty second phase

"""Schedule options and the autotuner: every candidate shape and radix order gives the oracle's
result, tuned choices are cached, invalid options are refused."""
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


def _real_case(F, n, batch, **opts):
    import torch
    rng = np.random.default_rng(n)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    p = F.Plan(n, "f32", "real", batch, **opts)
    xi = torch.from_numpy(x).cuda()
    spec = torch.empty((batch, n // 2), dtype=torch.complex64, device="cuda")
    back = torch.empty((batch, n), dtype=torch.float32, device="cuda")
    p.exec(False, xi.data_ptr(), spec.data_ptr(), 0)
    p.exec(True, spec.data_ptr(), back.data_ptr(), 0)
    torch.cuda.synchronize()
    ref = oracle.batch(x.astype(np.float64), n, real=True, inverse=False)
    assert rel_l2(spec.cpu().numpy(), ref) <= F32_TOL
    assert rel_l2(back.cpu().numpy() / n, x) <= F32_TOL
    return p


@pytest.mark.parametrize("radices", [[16, 8, 15], [15, 8, 16], [8, 15, 16], [16, 12, 10], [15, 16, 8]])
def test_explicit_radix_orders(F, radices):
    p = _real_case(F, 3840, 64, radices=radices)
    assert p.describe()["radices"] == radices


@pytest.mark.parametrize("opts", [dict(cta_threads=64), dict(cta_threads=512), dict(values_per_thread=8),
                                  dict(values_per_thread=32), dict(min_ctas_per_sm=4),
                                  dict(prefetch_quarter_waves=-1), dict(prefetch_quarter_waves=8)])
def test_explicit_shapes(F, opts):
    for n in (480, 1920):
        _real_case(F, n, 100, **opts)


def test_invalid_options_refused(F):
    with pytest.raises(F.SsfftError):
        F.Plan(3840, "f32", "real", 4, radices=[16, 8, 16])
    with pytest.raises(F.SsfftError):
        F.Plan(1024, "f32", "complex", 4, values_per_thread=64)
    with pytest.raises(F.SsfftError):
        F.Plan(1024, "f32", "complex", 4, autotune=3)


def test_autotune_matches_oracle_and_caches(F, tmp_path, monkeypatch):
    import torch
    for n, kind, dt in ((3840, "real", "f32"), (1000, "complex", "f32"), (1024, "complex", "f64"),
                        (960, "real_halfshift", "f32")):
        p = F.Plan(n, dt, kind, 2048, autotune=2)
        t = p.tuning()
        assert t["choice"].startswith("radices=")
        rng = np.random.default_rng(3)
        if kind == "complex":
            cdt = np.complex64 if dt == "f32" else np.complex128
            x = (rng.uniform(-1, 1, (2048, n)) + 1j * rng.uniform(-1, 1, (2048, n))).astype(cdt)
            xi = torch.from_numpy(x).cuda()
            y = torch.empty_like(xi)
            p.exec(False, xi.data_ptr(), y.data_ptr(), 0)
            torch.cuda.synchronize()
            ref = oracle.batch(x[:64].astype(np.complex128), n, real=False, inverse=False)
            tol = F32_TOL if dt == "f32" else 1e-14
            assert rel_l2(y[:64].cpu().numpy(), ref) <= tol
        else:
            x = rng.standard_normal((2048, n)).astype(np.float32)
            xi = torch.from_numpy(x).cuda()
            y = torch.empty((2048, n // 2), dtype=torch.complex64, device="cuda")
            p.exec(False, xi.data_ptr(), y.data_ptr(), 0)
            torch.cuda.synchronize()
            ref = oracle.batch(x[:64].astype(np.float64), n, real=True, inverse=False,
                               modified=kind == "real_halfshift")
            assert rel_l2(y[:64].cpu().numpy(), ref) <= F32_TOL
        # a second plan of the same shape takes the cached choice without timing anything
        q = F.Plan(n, dt, kind, 2048, autotune=2)
        assert q.tuning()["choice"] == t["choice"] and q.tuning()["log"] == []


def test_multi_autotuned_equals_plain(F):
    import torch
    rng = np.random.default_rng(5)
    sizes = [64, 100, 480, 1000, 3840, 16384, 7] * 3
    x = (rng.uniform(-1, 1, sum(sizes)) + 1j * rng.uniform(-1, 1, sum(sizes))).astype(np.complex64)
    m = F.Multi(sizes, "f32", autotune=1)
    xi = torch.from_numpy(x).cuda()
    a = torch.empty_like(xi)
    m.exec(False, xi.data_ptr(), a.data_ptr(), 0)
    torch.cuda.synchronize()
    got = a.cpu().numpy()
    off = 0
    for n in sizes:
        ref = oracle.fft(x[off:off + n].astype(np.complex128))
        assert rel_l2(got[off:off + n], ref) <= F32_TOL, n
        off += n


@pytest.mark.parametrize("n", [12, 36, 64, 96, 100, 1000, 1024, 3840, 8192])
@pytest.mark.parametrize("fuse", [1, -1])
def test_fused_split_on_and_off(F, n, fuse):
    """The RealFFT split fused into the last forward / first inverse pass (mirror-paired
    butterflies, odd and even unit counts) and the unfused kernels give the oracle's result."""
    _real_case(F, n, 33, fuse_split=fuse)


@pytest.mark.parametrize("n,kind,batch", [(2048, "real", 8192), (1024, "real", 8192), (16384, "complex", 512),
                                          (3840, "real", 4096)])
def test_autotuned_directions_match_oracle(F, n, kind, batch):
    """The tuner keeps the fastest forward and the fastest inverse candidate (the two directions may
    run different shapes and register caps): both directions and a round trip against the oracle."""
    import torch
    p = F.Plan(n, "f32", kind, batch, autotune=2)
    rng = np.random.default_rng(n)
    if kind == "complex":
        x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
        xi = torch.from_numpy(x).cuda()
        y = torch.empty_like(xi)
        z = torch.empty_like(xi)
    else:
        x = rng.standard_normal((batch, n)).astype(np.float32)
        xi = torch.from_numpy(x).cuda()
        y = torch.empty((batch, n // 2), dtype=torch.complex64, device="cuda")
        z = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), y.data_ptr(), 0)
    p.exec(True, y.data_ptr(), z.data_ptr(), 0)
    torch.cuda.synchronize()
    ys = y[:32].cpu().numpy()
    ref = oracle.batch(x[:32].astype(np.float64 if kind == "real" else np.complex128), n, real=kind == "real",
                       inverse=False)
    assert rel_l2(ys, ref) <= F32_TOL
    refi = oracle.batch(ref, n, real=kind == "real", inverse=True)
    assert rel_l2(z[:32].cpu().numpy(), refi) <= F32_TOL
    assert rel_l2(z[:32].cpu().numpy() / n, x[:32]) <= F32_TOL

"""The continuous-batching server (ssfft_server_*): results equal per-request execution, a
request's result is bit-identical alone and in a mix of other requests, budget admission, and
the synthetic open-loop load generator's statistics."""
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


def make_request(rng, n, kind, inverse, frames):
    if kind == "complex":
        x = (rng.standard_normal((frames, n)) + 1j * rng.standard_normal((frames, n))).astype(np.complex64)
        out = np.empty_like(x)
    elif not inverse:
        x = rng.standard_normal((frames, n)).astype(np.float32)
        out = np.empty((frames, n // 2), np.complex64)
    else:
        x = (rng.standard_normal((frames, n // 2)) + 1j * rng.standard_normal((frames, n // 2))).astype(np.complex64)
        out = np.empty((frames, n), np.float32)
    return x, out


def expected(x, n, kind, inverse):
    if kind == "complex":
        return np.stack([oracle.fft(r.astype(np.complex128), inverse) for r in x])
    if not inverse:
        return np.stack([oracle.rfft(r.astype(np.float64), kind == "real_halfshift") for r in x])
    return np.stack([oracle.irfft(r.astype(np.complex128), n, kind == "real_halfshift") for r in x])


SHAPES = [(256, "complex"), (480, "real"), (1920, "real"), (3840, "real"), (1000, "complex"), (65536, "real"),
          (4096, "real_halfshift"), (20000, "complex")]


def test_server_matches_oracle_and_isolation(F):
    rng = np.random.default_rng(3)
    srv = F.Server(hbm_budget_bytes=256 << 20, waves=3, max_requests_per_wave=16)
    reqs = []
    for i in range(40):
        n, kind = SHAPES[i % len(SHAPES)]
        inverse = bool(i % 3 == 1)
        x, out = make_request(rng, n, kind, inverse, 1 + (i * 7) % 9)
        t = srv.submit(n, kind, inverse, x, out, frames=x.shape[0])
        reqs.append((t, n, kind, inverse, x, out))
    srv.drain()
    for t, n, kind, inverse, x, out in reqs:
        ref = expected(x, n, kind, inverse)
        assert rel_l2(out, ref) <= 1e-6, (n, kind, inverse, rel_l2(out, ref))
    st = srv.stats()
    assert st["completed"] == 40 and st["failed"] == 0
    assert st["p99_latency_us"] >= st["p50_latency_us"] > 0
    # the same requests alone, one at a time: bit-identical results
    alone = F.Server(hbm_budget_bytes=256 << 20, waves=1, max_requests_per_wave=1)
    for t, n, kind, inverse, x, out in reqs[:16]:
        o2 = np.empty_like(out)
        tk = alone.submit(n, kind, inverse, x, o2, frames=x.shape[0])
        alone.wait(tk)
        assert np.array_equal(o2, out), (n, kind, inverse)
    alone.close()
    srv.close()


def test_plain_mode_matches_batched(F):
    rng = np.random.default_rng(8)
    plain = F.Server(hbm_budget_bytes=128 << 20, coalesce=False)
    batched = F.Server(hbm_budget_bytes=128 << 20, waves=4)
    for i in range(12):
        n, kind = SHAPES[i % len(SHAPES)]
        x, o1 = make_request(rng, n, kind, False, 3)
        o2 = np.empty_like(o1)
        t1 = plain.submit(n, kind, False, x, o1, frames=3)
        t2 = batched.submit(n, kind, False, x, o2, frames=3)
        plain.wait(t1)
        batched.wait(t2)
        assert np.array_equal(o1, o2)
    plain.close()
    batched.close()


def test_budget_rejects_oversized_request(F):
    srv = F.Server(hbm_budget_bytes=1 << 20)
    x = np.zeros((64, 65536), np.float32)
    out = np.zeros((64, 32768), np.complex64)
    with pytest.raises(F.SsfftError) as e:
        srv.submit(65536, "real", False, x, out, frames=64)
    assert e.value.status == 6
    srv.close()


def test_loadgen_reports_latency_and_throughput(F):
    srv = F.Server(hbm_budget_bytes=2 << 30, waves=4)
    st = srv.loadgen(offered_rate=20000, duration_s=0.5, seed=5, n_min=256, n_max=4096)
    assert st["failed"] == 0 and st["completed"] == st["submitted"] > 0
    assert 0 < st["p50_latency_us"] <= st["p99_latency_us"]
    assert st["frames"] > 0 and st["flops"] > 0
    srv.close()


def _pinned_like(a):
    """A page-locked (and, under unified addressing, device-mapped) copy of a numpy array."""
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t, t.numpy()


def test_in_place_requests_match_copy_path_and_oracle(F):
    """Requests in pinned host buffers are served in place (the kernels read and write the host
    buffers, no copies): mixed single-CTA shapes, both directions, in place and copied requests in
    the same waves; every result equals the oracle and, bit for bit, the copied result."""
    rng = np.random.default_rng(17)
    shapes = [(256, "complex"), (480, "real"), (1920, "real"), (3840, "real"), (1000, "complex"),
              (4096, "real_halfshift"), (98, "real"), (7, "complex"), (16384, "complex"), (32768, "real")]
    srv = F.Server(hbm_budget_bytes=256 << 20, waves=3, max_requests_per_wave=24)
    keep, jobs = [], []
    for i in range(48):
        n, kind = shapes[i % len(shapes)]
        inverse = bool(i % 3 == 1)
        x, out = make_request(rng, n, kind, inverse, 1 + (i * 5) % 7)
        tx, px = _pinned_like(x)
        to, po = _pinned_like(out)
        keep += [tx, to]
        t1 = srv.submit(n, kind, inverse, px, po, frames=x.shape[0])
        o2 = np.empty_like(out)
        t2 = srv.submit(n, kind, inverse, x, o2, frames=x.shape[0])   # pageable: copy path
        jobs.append((t1, t2, n, kind, inverse, x, po, o2))
    srv.drain()
    st = srv.stats()
    assert st["failed"] == 0 and st["completed"] == 96
    assert st["in_place"] == 48, st["in_place"]
    for t1, t2, n, kind, inverse, x, po, o2 in jobs:
        assert np.array_equal(po, o2), (n, kind, inverse)
        ref = expected(x, n, kind, inverse)
        assert rel_l2(po, ref) <= 1e-6, (n, kind, inverse, rel_l2(po, ref))
    srv.close()


def test_plain_server_never_in_place(F):
    rng = np.random.default_rng(18)
    plain = F.Server(hbm_budget_bytes=64 << 20, coalesce=False)
    x, out = make_request(rng, 480, "real", False, 2)
    tx, px = _pinned_like(x)
    to, po = _pinned_like(out)
    plain.wait(plain.submit(480, "real", False, px, po, frames=2))
    assert plain.stats()["in_place"] == 0
    assert rel_l2(po, expected(x, 480, "real", False)) <= 1e-6
    plain.close()


def test_completion_by_callbacks_matches(F, monkeypatch):
    """Waves complete through a polling completion thread; the callback form kept behind the
    debug switch serve_hostfunc=1 gives the same results."""
    rng = np.random.default_rng(19)
    monkeypatch.setenv("SSFFT_DEBUG", "serve_hostfunc=1")
    cb = F.Server(hbm_budget_bytes=128 << 20, waves=2)
    monkeypatch.delenv("SSFFT_DEBUG")
    poll = F.Server(hbm_budget_bytes=128 << 20, waves=2)
    for i in range(8):
        n, kind = SHAPES[i % len(SHAPES)]
        x, o1 = make_request(rng, n, kind, bool(i % 2), 2)
        o2 = np.empty_like(o1)
        t1 = cb.submit(n, kind, bool(i % 2), x, o1, frames=2)
        t2 = poll.submit(n, kind, bool(i % 2), x, o2, frames=2)
        cb.wait(t1)
        poll.wait(t2)
        assert np.array_equal(o1, o2)
    assert cb.stats()["failed"] == 0 and poll.stats()["failed"] == 0
    cb.close()
    poll.close()

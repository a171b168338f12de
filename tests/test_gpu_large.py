"""GPU parity for the multi-pass (four-step) path: transforms longer than one CTA holds, through
the C ABI, against the FP64 oracle (oracle/ssfft_oracle.c) and size-independent properties.

Tolerances: relL2 <= 1e-6 (FP32) up to 2^16 points, <= 5e-6 at 2^24 and the other large single
transforms, <= 1e-14 for FP64; Bluestein lengths (a prime factor above 1024): <= 2e-6 (FP32),
<= 1e-13 (FP64), two M-point transforms and two chirp products deep."""
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


def c2c(F, x, inverse=False):
    b, n = x.shape
    p = F.Plan(n, "f32" if x.dtype == np.complex64 else "f64", "complex", b)
    xi = torch.from_numpy(x).cuda()
    xo = torch.empty_like(xi)
    p.exec(inverse, xi.data_ptr(), xo.data_ptr(), 0)
    torch.cuda.synchronize()
    d = p.describe()
    return xo, xi, d


@pytest.mark.parametrize("n,dt,tol", [
    (16384 * 2, "f32", 1e-6), (65536, "f32", 1e-6), (3 ** 10, "f32", 1e-6), (2 ** 12 * 3 ** 2 * 5, "f32", 1e-6),
    (5 ** 7, "f32", 1e-6), (7 * 2 ** 13, "f32", 1e-6), (16384, "f64", 1e-14), (65536, "f64", 1e-14),
    (3 ** 10, "f64", 1e-14),
])
def test_large_c2c_vs_oracle(F, n, dt, tol):
    rng = np.random.default_rng(n)
    b = 3
    cdt = np.complex64 if dt == "f32" else np.complex128
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(cdt)
    for inv in (False, True):
        xo, xi, d = c2c(F, x, inv)
        assert d["launches"] >= 2
        got = xo.cpu().numpy()
        ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
        assert rel_l2(got, ref) <= tol, (n, dt, inv, rel_l2(got, ref))
        assert np.array_equal(xi.cpu().numpy(), x), "input was changed"


@pytest.mark.parametrize("n", [2 ** 24, 3 ** 15, 2 ** 12 * 3 ** 4 * 5 ** 2])
def test_config_large_single_f32(F, n):
    """One FP32 transform each at 2^24, 3^15 and 2^12 3^4 5^2, U[-1,1): oracle comparison (FP64
    oracle on the same FP32 inputs), then the round trip ifft(fft(x)) = N x and Parseval."""
    rng = np.random.default_rng(n % 1000)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)[None, :]
    xo, xi, d = c2c(F, x, False)
    got = xo.cpu().numpy()[0]
    ref = oracle.fft(x[0].astype(np.complex128))
    err = rel_l2(got, ref)
    assert err <= 5e-6, err
    # Parseval: sum |X|^2 = N sum |x|^2
    px = np.sum(np.abs(x[0].astype(np.complex128)) ** 2) * n
    assert abs(np.sum(np.abs(got.astype(np.complex128)) ** 2) - px) / px < 1e-5
    del ref
    back = torch.empty_like(xo)
    p = F.Plan(n, "f32", "complex", 1)
    p.exec(True, xo.data_ptr(), back.data_ptr(), 0)
    torch.cuda.synchronize()
    assert rel_l2(back.cpu().numpy()[0], n * x[0].astype(np.complex128)) <= 5e-6


@pytest.mark.parametrize("n,dt", [(65536, "f32"), (2 * 3 ** 10, "f32"), (40960 * 2, "f64")])
@pytest.mark.parametrize("kind", ["real", "real_halfshift"])
def test_large_real_vs_oracle(F, n, dt, kind):
    rng = np.random.default_rng(n + len(kind))
    b = 2
    mod = kind == "real_halfshift"
    rdt = np.float32 if dt == "f32" else np.float64
    cdt = np.complex64 if dt == "f32" else np.complex128
    tol = 1e-6 if dt == "f32" else 1e-14
    x = rng.standard_normal((b, n)).astype(rdt)
    p = F.Plan(n, dt, kind, b)
    assert p.describe()["launches"] >= 3
    xi = torch.from_numpy(x).cuda()
    spec = torch.empty((b, n // 2), dtype=torch.complex64 if dt == "f32" else torch.complex128, device="cuda")
    p.exec(False, xi.data_ptr(), spec.data_ptr(), 0)
    back = torch.empty_like(xi)
    p.exec(True, spec.data_ptr(), back.data_ptr(), 0)
    torch.cuda.synchronize()
    s = spec.cpu().numpy()
    ref = np.stack([oracle.rfft(r.astype(np.float64), mod) for r in x])
    assert rel_l2(s, ref) <= tol, rel_l2(s, ref)
    refb = np.stack([oracle.irfft(r.astype(np.complex128), n, mod) for r in s.astype(cdt)])
    assert rel_l2(back.cpu().numpy(), refb) <= tol
    assert np.array_equal(xi.cpu().numpy(), x)


def test_large_batch_and_host_path(F):
    rng = np.random.default_rng(1)
    n, b = 2 ** 17, 5
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(np.complex64)
    p = F.Plan(n, "f32", "complex", b)
    out = np.empty_like(x)
    p.exec_host(False, x, out)
    ref = np.stack([oracle.fft(r.astype(np.complex128)) for r in x])
    assert rel_l2(out, ref) <= 1e-6


def test_linearity_large(F):
    rng = np.random.default_rng(2)
    n = 2 ** 20
    a = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)[None]
    c = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)[None]
    fa = c2c(F, a)[0].cpu().numpy().astype(np.complex128)
    fc = c2c(F, c)[0].cpu().numpy().astype(np.complex128)
    fac = c2c(F, (a + c).astype(np.complex64))[0].cpu().numpy().astype(np.complex128)
    assert rel_l2(fac, fa + fc) <= 2e-6


# Bluestein lengths: a prime factor above 1024 (which no pass takes, and which a direct pass would
# run in O(p^2)), in and beyond one CTA
@pytest.mark.parametrize("n,dt,tol", [(17 * 1031, "f32", 2e-6), (2 * 20011, "f32", 2e-6), (10007, "f64", 1e-13),
                                      (3 * 4099, "f64", 1e-13), (12289, "f32", 2e-6), (1031, "f64", 1e-13)])
def test_bluestein_c2c_vs_oracle(F, n, dt, tol):
    rng = np.random.default_rng(n)
    cdt = np.complex64 if dt == "f32" else np.complex128
    x = (rng.uniform(-1, 1, (2, n)) + 1j * rng.uniform(-1, 1, (2, n))).astype(cdt)
    y, xi, d = c2c(F, x)
    assert d["radices"] == []  # no pass schedule: Bluestein
    got = y.cpu().numpy()
    if dt == "f32":
        ref = oracle.fft(x[0].astype(np.complex128))
        assert rel_l2(got[0], ref) <= tol, rel_l2(got[0], ref)
        ref1 = oracle.fft(x[1].astype(np.complex128))
        assert rel_l2(got[1], ref1) <= tol
    else:
        # At these prime lengths the reference's own FFT<double> (its generic step evaluates
        # cos/sin of phases up to 2 pi p) carries ~1e-12 error, so the FP64 result is held to
        # 1e-13 against an exact DFT (numpy's FFT in FP64) and to the reference's accuracy
        # against the oracle.
        exact = np.fft.fft(x.astype(np.complex128), axis=1)
        assert rel_l2(got, exact) <= tol, rel_l2(got, exact)
        ref = oracle.fft(x[0].astype(np.complex128))
        assert rel_l2(got[0], ref) <= 5e-11, rel_l2(got[0], ref)
    # inverse (unnormalised) brings it back
    z, _, _ = c2c(F, got, inverse=True)
    assert rel_l2(z.cpu().numpy() / n, x) <= 2 * tol


@pytest.mark.parametrize("n", [2 * 20011 * 2, 2 * 1031])
def test_bluestein_real_vs_oracle(F, n):
    rng = np.random.default_rng(5)
    x = rng.standard_normal((1, n)).astype(np.float32)
    p = F.Plan(n, "f32", "real", 1)
    xi = torch.from_numpy(x).cuda()
    s = torch.empty((1, n // 2), dtype=torch.complex64, device="cuda")
    b = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), s.data_ptr(), 0)
    p.exec(True, s.data_ptr(), b.data_ptr(), 0)
    torch.cuda.synchronize()
    ref = oracle.rfft(x[0].astype(np.float64))
    assert rel_l2(s.cpu().numpy()[0], ref) <= 2e-6, rel_l2(s.cpu().numpy()[0], ref)
    assert rel_l2(b.cpu().numpy() / n, x) <= 4e-6


# Lengths the reference accepts that need the path beyond one CTA in a special form: odd real
# lengths (packed rows: the last real is neither read nor written, signalsmith-fft.h:446-502) and
# half-shift lengths with a prime factor above 1024 (Bluestein with the rotations on its chirp
# kernels).  Batches of several transforms, so odd rows start at odd offsets.
@pytest.mark.parametrize("n,dt,kind,b,tol", [
    (40001, "f32", "real", 3, 1e-6), (40001, "f32", "real_halfshift", 2, 1e-6), (35055, "f32", "real", 3, 2e-6),
    (20003, "f64", "real", 2, 1e-13), (35054, "f32", "real_halfshift", 2, 2e-6), (2 * 20011 * 2, "f32", "real_halfshift", 1, 2e-6),
    (20014, "f64", "real_halfshift", 1, 5e-11)])
def test_reference_lengths_beyond_one_cta(F, n, dt, kind, b, tol):
    rng = np.random.default_rng(n + b)
    mod = kind == "real_halfshift"
    rdt = np.float32 if dt == "f32" else np.float64
    cdt = np.complex64 if dt == "f32" else np.complex128
    h = n // 2
    x = rng.standard_normal((b, n)).astype(rdt)
    p = F.Plan(n, dt, kind, b)
    xi = torch.from_numpy(x).cuda()
    spec = torch.full((b, h), complex(5, 5), dtype=torch.complex64 if dt == "f32" else torch.complex128,
                      device="cuda")
    p.exec(False, xi.data_ptr(), spec.data_ptr(), 0)
    back = torch.full_like(xi, 7.0)
    p.exec(True, spec.data_ptr(), back.data_ptr(), 0)
    torch.cuda.synchronize()
    s = spec.cpu().numpy()
    ref = np.stack([oracle.rfft(r.astype(np.float64), mod) for r in x])
    assert rel_l2(s, ref) <= tol, rel_l2(s, ref)
    bk = back.cpu().numpy()
    refb = np.stack([oracle.irfft(r.astype(np.complex128), n, mod) for r in s.astype(cdt)])
    assert rel_l2(bk[:, :2 * h], refb) <= tol, rel_l2(bk[:, :2 * h], refb)
    if n & 1:
        assert np.all(bk[:, 2 * h:] == 7.0), "the last real of an odd row is not written"
    assert np.array_equal(xi.cpu().numpy(), x)

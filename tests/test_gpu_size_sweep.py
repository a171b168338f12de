"""Many lengths through the planner's whole decision space (radix lists, composite and large
radices, fused RealFFT split, direct prime passes, multi-pass, Bluestein), against an exact DFT
(numpy's FFT in FP64; the oracle pins the reference's own results elsewhere).  Seeded random
lengths plus the boundaries of each path."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

F32_TOL, F64_TOL = 2e-6, 1e-13  # FP32: a few passes deep incl. Bluestein; FP64: exact-DFT reference


def _lengths():
    rng = np.random.default_rng(2024)
    fixed = [1, 2, 3, 4, 5, 7, 11, 13, 16, 17, 31, 32, 64, 97, 127, 128, 255, 256, 257, 1000, 1021, 1024, 1031,
             2048, 4095, 4096, 4097, 8191, 8192, 8193, 12289, 16383, 16384, 16385, 20000, 32768, 65537]
    rand = sorted(set(int(v) for v in np.exp(rng.uniform(np.log(2), np.log(70000), 60))))
    return sorted(set(fixed + rand))


LENGTHS = _lengths()


@pytest.fixture(scope="module")
def F():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fft_gb300
    return fft_gb300


@pytest.mark.parametrize("n", LENGTHS)
def test_complex_f32(F, n):
    rng = np.random.default_rng(n)
    b = 2
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(np.complex64)
    p = F.Plan(n, "f32", "complex", b)
    xi = torch.from_numpy(x).cuda()
    y = torch.empty_like(xi)
    z = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), y.data_ptr(), 0)
    p.exec(True, y.data_ptr(), z.data_ptr(), 0)
    torch.cuda.synchronize()
    exact = np.fft.fft(x.astype(np.complex128), axis=1)
    assert rel_l2(y.cpu().numpy(), exact) <= F32_TOL, (n, p.describe())
    assert rel_l2(z.cpu().numpy() / n, x) <= 2 * F32_TOL, n


# even real lengths (odd ones follow the reference's floor(n/2) convention, not a DFT, and are
# checked against the oracle and the golden vectors in test_gpu_parity.py)
@pytest.mark.parametrize("n", sorted(set(2 * (v // 2) for v in LENGTHS if v >= 2)))
def test_real_f32(F, n):
    rng = np.random.default_rng(n + 1)
    b = 2
    x = rng.standard_normal((b, n)).astype(np.float32)
    p = F.Plan(n, "f32", "real", b)
    h = n // 2
    xi = torch.from_numpy(x).cuda()
    s = torch.empty((b, h), dtype=torch.complex64, device="cuda")
    p.exec(False, xi.data_ptr(), s.data_ptr(), 0)
    torch.cuda.synchronize()
    got = s.cpu().numpy()
    full = np.fft.fft(x[:, :2 * h].astype(np.float64).reshape(b, h, 2) @ np.array([1, 1j]), axis=1)  # z = x0 + i x1
    # RealFFT bins from the packed complex transform (reference layout, DC + Nyquist in bin 0)
    k = np.arange(h)
    zc = np.conj(full[:, (-k) % h])
    odd = (full + zc) / 2
    even = (full - zc) / 2 * (-1j * np.exp(-2j * np.pi * k / (2 * h)))
    ref = odd + even
    ref[:, 0] = (full[:, 0].real + full[:, 0].imag) + 1j * (full[:, 0].real - full[:, 0].imag)
    assert rel_l2(got, ref) <= F32_TOL, (n, p.describe())


@pytest.mark.parametrize("n", [v for v in LENGTHS if v <= 20000])
def test_complex_f64(F, n):
    rng = np.random.default_rng(n + 2)
    x = (rng.uniform(-1, 1, (1, n)) + 1j * rng.uniform(-1, 1, (1, n)))
    p = F.Plan(n, "f64", "complex", 1)
    xi = torch.from_numpy(x).cuda()
    y = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), y.data_ptr(), 0)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), np.fft.fft(x, axis=1)) <= F64_TOL, (n, p.describe())

"""GPU parity tests: the sm_103a kernels, called through the C ABI (libssfft.so via ctypes, device
buffers from torch), against the reference's golden vectors and the CPU oracle, plus the
reference test suite's own checks (tests/00-fft.cpp, tests/01-real.cpp) restated on the device.

Tolerances (relative L2 error against the FP64 oracle): 1e-14 for FP64 (1e-13 for the direct
O(p^2) prime passes), 1e-6 for FP32."""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F32_TOL = 1e-6
F64_TOL = 1e-14


def f64_tol(n):
    m = n
    for p in (2, 3, 5):
        while m % p == 0:
            m //= p
    return F64_TOL if m == 1 else 1e-13


@pytest.fixture(scope="module")
def F():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fft_gb300
    fft_gb300.lib()
    _prewarm(fft_gb300)
    return fft_gb300


def _prewarm(F):
    """Compile the many single-transform plans of the golden tests concurrently (NVRTC runs
    outside the library's lock; ctypes releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    keys = [(n, dt, "complex", 1) for n in COMPLEX_SIZES for dt in ("f32", "f64")]
    keys += [(n, dt, k, 1) for n in range(2, 100) for dt in ("f32", "f64") for k in ("real", "real_halfshift")]
    torch.cuda.init()
    dev = torch.cuda.current_device()

    def make(k):
        torch.cuda.set_device(dev)
        F.Plan(*k).destroy()

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(make, keys))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def run_complex(F, x, inverse, batch=None):
    """x: (b, n) complex numpy -> numpy result through ssfft_exec."""
    b, n = x.shape
    dt = "f32" if x.dtype == np.complex64 else "f64"
    p = F.Plan(n, dt, "complex", b)
    xi = dev(x)
    xo = torch.empty_like(xi)
    p.exec(inverse, xi.data_ptr(), xo.data_ptr(), torch.cuda.current_stream().cuda_stream, batch)
    torch.cuda.synchronize()
    return xo.cpu().numpy(), xi.cpu().numpy()


COMPLEX_SIZES = [1, 2, 4, 8, 16, 32, 64, 128, 256, 3, 6, 9, 12, 18, 24, 5, 10, 15, 20, 25,
                 7, 14, 21, 28, 49, 11, 13, 17, 19, 22, 23, 480, 1024]


@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_complex_golden(F, golden, dt):
    """FP64: within 1e-14 of the reference's FFT<double> output.  FP32: within 1e-6 of the FP64
    oracle on the same inputs, and within 3e-6 of the reference's own FFT<float> output (which
    carries up to ~1e-6 error of its own: float-rounded phases, signalsmith-fft.h:123)."""
    for n in COMPLEX_SIZES:
        x = golden[f"c2c_{dt}_{n}_in"][None, :]
        for d, inv in (("fwd", False), ("inv", True)):
            got, xin = run_complex(F, x, inv)
            ref = golden[f"c2c_{dt}_{n}_{d}"]
            if dt == "f64":
                assert rel_l2(got[0], ref) <= f64_tol(n), (n, d, rel_l2(got[0], ref))
            else:
                exact = oracle.fft(x[0].astype(np.complex128), inv)
                assert rel_l2(got[0], exact) <= F32_TOL, (n, d, rel_l2(got[0], exact))
                assert rel_l2(got[0], ref) <= 3 * F32_TOL, (n, d, rel_l2(got[0], ref))
            assert np.array_equal(xin, x), "input was changed"


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("kind", ["real", "real_halfshift"])
def test_real_golden(F, golden, dt, kind):
    mod = kind == "real_halfshift"
    for n in list(range(2, 100)) + [480, 960, 1920, 3840]:
        key = f"r_{dt}_m{int(mod)}_{n}"
        if key + "_in" not in golden:
            continue
        # FP32 against the reference's own RealFFT<float> output: both carry ~1e-7 error
        tol = f64_tol(n // 2) if dt == "f64" else 3 * F32_TOL
        x = golden[key + "_in"]
        p = F.Plan(n, dt, kind, 1)
        h = n // 2
        cdt = torch.complex64 if dt == "f32" else torch.complex128
        xi = dev(x)
        # the output buffer has n complex slots; the second half must stay untouched
        # (tests/01-real.cpp:49-52, :70-73)
        out = torch.full((n,), complex(52, 21), dtype=cdt, device="cuda")
        p.exec(False, xi.data_ptr(), out.data_ptr(), 0)
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        assert rel_l2(o[:h], golden[key + "_fwd"]) <= tol, (n, "fwd", rel_l2(o[:h], golden[key + "_fwd"]))
        assert np.all(o[h:] == complex(52, 21))
        s = golden[key + "_spec"]
        si = dev(s)
        ro = torch.full((n + 1,), 7.0, dtype=xi.dtype, device="cuda")
        p.exec(True, si.data_ptr(), ro.data_ptr(), 0)
        torch.cuda.synchronize()
        r = ro.cpu().numpy()
        assert rel_l2(r[:2 * h], golden[key + "_inv"]) <= tol, (n, "inv")
        assert np.all(r[2 * h:] == 7.0)


def test_individual_bins_and_linearity(F):
    """tests/00-fft.cpp:19-99 on the device, FP64 and FP32, all bins of each size at once."""
    for dt, cdt in (("f64", np.complex128), ("f32", np.complex64)):
        for n in COMPLEX_SIZES:
            i = np.arange(n)
            x = np.exp(2j * np.pi * np.outer(np.arange(n), i) / n).astype(cdt)  # row b = bin b
            got, _ = run_complex(F, x, False)
            exp = n * np.eye(n)
            for b in range(n):
                assert oracle.close_enough(got[b], exp[b]), (dt, n, b)
            rng = np.random.default_rng(n)
            a = (rng.uniform(-0.5, 0.5, (1, n)) + 1j * rng.uniform(-0.5, 0.5, (1, n))).astype(cdt)
            c = (rng.uniform(-0.5, 0.5, (1, n)) + 1j * rng.uniform(-0.5, 0.5, (1, n))).astype(cdt)
            fa, fc, fac = run_complex(F, a, False)[0], run_complex(F, c, False)[0], run_complex(F, a + c, False)[0]
            assert oracle.close_enough(fac, fa + fc)


def test_round_trip_is_n_times_input(F):
    """ifft(fft(x)) == N x (tests/00-fft.cpp:101-145)."""
    rng = np.random.default_rng(3)
    for n in COMPLEX_SIZES + [4096, 8192]:
        x = (rng.uniform(-0.5, 0.5, (2, n)) + 1j * rng.uniform(-0.5, 0.5, (2, n))).astype(np.complex128)
        spec, _ = run_complex(F, x, False)
        back, _ = run_complex(F, spec, True)
        assert rel_l2(back, n * x) <= 1e-13, n


@pytest.mark.parametrize("n", [256, 768, 1000, 1024, 2048, 3072, 4096, 4608, 4800, 5000, 5120, 6000, 6144, 6400, 7680,
                               8000, 8192, 9216, 15000, 15360, 16200, 16384, 2187, 6561])
def test_complex_f32_vs_oracle(F, n):
    rng = np.random.default_rng(n)
    b = 6
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(np.complex64)
    for inv in (False, True):
        got, _ = run_complex(F, x, inv)
        ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
        assert rel_l2(got, ref) <= F32_TOL, (n, inv, rel_l2(got, ref))


@pytest.mark.parametrize("n", [10240, 12288, 15360, 16384])
def test_real_f32_mid_lengths_vs_oracle(F, n):
    """RealFFT<float> lengths whose half runs the mid-length schedules (16 values a thread, the
    largest radix in the middle pass, 2-3 CTAs per SM) or the fused 32-32-8 list: forward and
    inverse of 40 frames against the oracle."""
    rng = np.random.default_rng(n + 11)
    b, h = 40, n // 2
    x = rng.standard_normal((b, n)).astype(np.float32)
    p = F.Plan(n, "f32", "real", b)
    xi = dev(x)
    s = torch.empty((b, h), dtype=torch.complex64, device="cuda")
    back = torch.empty_like(xi)
    st = torch.cuda.current_stream().cuda_stream
    p.exec(False, xi.data_ptr(), s.data_ptr(), st)
    p.exec(True, s.data_ptr(), back.data_ptr(), st)
    torch.cuda.synchronize()
    ref = np.stack([oracle.rfft(r.astype(np.float64)) for r in x])
    assert rel_l2(s.cpu().numpy(), ref) <= F32_TOL
    sb = s.cpu().numpy()
    refi = np.stack([oracle.irfft(r.astype(np.complex128), n) for r in sb])
    assert rel_l2(back.cpu().numpy(), refi) <= F32_TOL


@pytest.mark.parametrize("n", [20480, 24576])
def test_real_f32_long_staged_vs_oracle(F, n):
    """RealFFT<float> lengths whose half (10240, 12288 points) the planner stages by default (split
    and pre-twiddle as separate steps) unless the staged kernel spills (then the fused plain
    kernel runs): more frames than resident CTAs, forward and inverse against the oracle on a
    sample of frames, the plan's error flag zero, and an input off a 16-byte boundary (the plain
    kernel of the same radix order) giving the same spectrum."""
    import ctypes
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    b, h = 2 * sms + 7, n // 2
    rng = np.random.default_rng(n + 21)
    x = rng.standard_normal((b, n)).astype(np.float32)
    p = F.Plan(n, "f32", "real", b)
    st = torch.cuda.current_stream().cuda_stream
    xi = dev(x)
    s = torch.empty((b, h), dtype=torch.complex64, device="cuda")
    back = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), s.data_ptr(), st)
    p.exec(True, s.data_ptr(), back.data_ptr(), st)
    torch.cuda.synchronize()
    rows = list(range(0, b, 37)) + [b - 1]
    ref = np.stack([oracle.rfft(x[r].astype(np.float64)) for r in rows])
    assert rel_l2(s.cpu().numpy()[rows], ref) <= F32_TOL
    sb = s.cpu().numpy()
    refi = np.stack([oracle.irfft(sb[r].astype(np.complex128), n) for r in rows])
    assert rel_l2(back.cpu().numpy()[rows], refi) <= F32_TOL
    flags = ctypes.c_uint(99)
    assert F.lib().ssfft_plan_error(p.handle, ctypes.byref(flags)) == 0 and flags.value == 0
    buf = torch.zeros(b * n + 2, dtype=torch.float32, device="cuda")
    buf[2:] = xi.reshape(-1)
    s2 = torch.empty_like(s)
    assert F.lib().ssfft_exec(p.handle, 0, F._vp(buf.data_ptr() + 8), F._vp(s2.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert rel_l2(s2.cpu().numpy()[rows], ref) <= F32_TOL


def test_config_fp64_1024_x256(F):
    """FFT<double> N=1024, 256 transforms, forward then inverse, U[-1,1) (relL2 <= 1e-14)."""
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (256, 1024)) + 1j * rng.uniform(-1, 1, (256, 1024))
    got, _ = run_complex(F, x, False)
    ref = np.stack([oracle.fft(r) for r in x])
    assert rel_l2(got, ref) <= F64_TOL
    back, _ = run_complex(F, got, True)
    refb = np.stack([oracle.fft(r, True) for r in ref])
    assert rel_l2(back, refb) <= F64_TOL
    assert rel_l2(back, 1024 * x) <= F64_TOL


@pytest.mark.parametrize("n", [480, 960, 1920, 3840])
@pytest.mark.parametrize("kind", ["real", "real_halfshift"])
def test_config_realfft_f32_frames(F, n, kind):
    """RealFFT<float> frames: N(0,1) noise + 3 sinusoids, forward and inverse vs the oracle."""
    rng = np.random.default_rng(n)
    frames = 512
    t = np.arange(n)
    x = rng.standard_normal((frames, n))
    for _ in range(3):
        f = rng.uniform(0, n / 2, (frames, 1))
        a = rng.uniform(0.1, 2, (frames, 1))
        ph = rng.uniform(0, 2 * np.pi, (frames, 1))
        x += a * np.sin(2 * np.pi * f * t / n + ph)
    x32 = x.astype(np.float32)
    mod = kind == "real_halfshift"
    p = F.Plan(n, "f32", kind, frames)
    xi = dev(x32)
    spec = torch.empty((frames, n // 2), dtype=torch.complex64, device="cuda")
    p.exec(False, xi.data_ptr(), spec.data_ptr(), 0)
    back = torch.empty_like(xi)
    p.exec(True, spec.data_ptr(), back.data_ptr(), 0)
    torch.cuda.synchronize()
    ref = np.stack([oracle.rfft(r.astype(np.float64), mod) for r in x32])
    s = spec.cpu().numpy()
    assert rel_l2(s, ref) <= F32_TOL, rel_l2(s, ref)
    refb = np.stack([oracle.irfft(r.astype(np.complex128), n, mod) for r in s])
    assert rel_l2(back.cpu().numpy(), refb) <= F32_TOL
    assert rel_l2(back.cpu().numpy(), n * x32.astype(np.float64)) <= 2e-6


@pytest.mark.parametrize("n", [480, 960, 1920, 3840])
def test_config_realfft_f32_full_16384_frames(F, n):
    """The headline configuration at its full size: 16384 frames of N(0,1) noise + 3 sinusoids
    (the bench's own generator), forward and inverse.  Every 64th frame (256 frames) against the
    FP64 oracle at the FP32 bar; every frame through size-independent properties: the round trip
    ifft(fft(x)) = N x and Parseval's identity for the packed spectrum."""
    import os
    import bench
    frames = 16384
    x32 = bench.frames_for(n, frames, 1000 + n)
    p = F.Plan(n, "f32", "real", frames)
    xi = dev(x32)
    spec = torch.empty((frames, n // 2), dtype=torch.complex64, device="cuda")
    back = torch.empty_like(xi)
    p.exec(False, xi.data_ptr(), spec.data_ptr(), 0)
    p.exec(True, spec.data_ptr(), back.data_ptr(), 0)
    torch.cuda.synchronize()
    s = spec.cpu().numpy()
    b = back.cpu().numpy()
    pick = np.arange(0, frames, 64)
    threads = os.cpu_count() or 1
    ref = oracle.batch(x32[pick].astype(np.float64), n, real=True, inverse=False, threads=threads)
    assert rel_l2(s[pick], ref) <= F32_TOL, rel_l2(s[pick], ref)
    refb = oracle.batch(s[pick].astype(np.complex128), n, real=True, inverse=True, threads=threads)
    assert rel_l2(b[pick], refb) <= F32_TOL, rel_l2(b[pick], refb)
    assert rel_l2(b, n * x32.astype(np.float64)) <= 2e-6
    s64 = s.astype(np.complex128)
    energy_bins = (s64[:, 0].real ** 2 + s64[:, 0].imag ** 2 + 2 * np.sum(np.abs(s64[:, 1:]) ** 2, axis=1)) / n
    energy_time = np.sum(x32.astype(np.float64) ** 2, axis=1)
    assert np.max(np.abs(energy_bins - energy_time) / energy_time) <= 1e-5


def test_partial_batch_and_host_path(F):
    rng = np.random.default_rng(9)
    n, b = 240, 37
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(np.complex64)
    p = F.Plan(n, "f32", "complex", b)
    xi = dev(x)
    xo = torch.zeros_like(xi)
    p.exec(False, xi.data_ptr(), xo.data_ptr(), 0, batch=20)
    torch.cuda.synchronize()
    o = xo.cpu().numpy()
    ref = np.stack([oracle.fft(r.astype(np.complex128)) for r in x])
    assert rel_l2(o[:20], ref[:20]) <= F32_TOL
    assert np.all(o[20:] == 0)
    host_out = np.empty_like(x)
    p.exec_host(False, x, host_out)
    assert rel_l2(host_out, ref) <= F32_TOL


def test_in_place_single_kernel(F):
    rng = np.random.default_rng(4)
    x = (rng.uniform(-1, 1, (8, 1024)) + 1j * rng.uniform(-1, 1, (8, 1024))).astype(np.complex64)
    p = F.Plan(1024, "f32", "complex", 8)
    xi = dev(x)
    p.exec(False, xi.data_ptr(), xi.data_ptr(), 0)
    torch.cuda.synchronize()
    ref = np.stack([oracle.fft(r.astype(np.complex128)) for r in x])
    assert rel_l2(xi.cpu().numpy(), ref) <= F32_TOL


def test_reference_shaped_api(F):
    """FFT / RealFFT / ModifiedRealFFT objects: host arrays and device tensors."""
    rng = np.random.default_rng(2)
    f = F.FFT(1000, 1, dtype="f64")
    assert f.size() == 1024
    x = rng.standard_normal(1024) + 1j * rng.standard_normal(1024)
    assert rel_l2(f.fft(x), oracle.fft(x)) <= F64_TOL
    assert rel_l2(f.ifft(x), oracle.fft(x, True)) <= F64_TOL
    r = F.RealFFT(480, dtype="f64")
    xr = rng.standard_normal(480)
    assert rel_l2(r.fft(xr), oracle.rfft(xr)) <= F64_TOL
    m = F.ModifiedRealFFT(480, dtype="f64")
    assert rel_l2(m.fft(xr), oracle.rfft(xr, True)) <= F64_TOL
    s = m.fft(xr)
    assert rel_l2(m.ifft(s), oracle.irfft(s, 480, True)) <= F64_TOL
    t = torch.from_numpy(xr).cuda()
    assert rel_l2(F.rfft(t).cpu().numpy(), oracle.rfft(xr)) <= F64_TOL


LONG_STAGED = [8192, 9600, 10240, 10800, 11520, 12288, 13824, 14400, 15000, 15360, 16000, 16384]


@pytest.mark.parametrize("staging", [0, 1])
@pytest.mark.parametrize("n", LONG_STAGED)
def test_long_staged_kernels_match_oracle(F, n, staging):
    """Long complex FP32 transforms on the bulk-copy staged kernel: the planner's default (staging
    where it measured faster and the kernel does not spill, the plain kernel otherwise) and
    staging forced wherever the input fits (plan option staging=1).  The whole input is staged
    where it fits beside the work buffer, the first pass's leading rows otherwise (the rest copied
    into the work buffer once the previous group's last pass has read it).  More transforms than
    resident CTAs, so every persistent CTA walks several groups and issues the next group's
    copies; forward and inverse against the oracle on a sample of the transforms, the plan's
    error flag zero."""
    import ctypes
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    b = 2 * sms + 7
    rng = np.random.default_rng(n + 5)
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(np.complex64)
    p = F.Plan(n, "f32", "complex", b, staging=staging)
    name = p.kernel(False)
    if staging == 1:
        assert "batch_staged" in name, name
    xi = dev(x)
    xo = torch.empty_like(xi)
    rows = list(range(0, b, 17)) + [b - 1]
    for inv in (False, True):
        p.exec(inv, xi.data_ptr(), xo.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        got = xo.cpu().numpy()[rows]
        ref = np.stack([oracle.fft(x[r].astype(np.complex128), inv) for r in rows])
        assert rel_l2(got, ref) <= F32_TOL, (n, inv, name, rel_l2(got, ref))
    flags = ctypes.c_uint(99)
    assert F.lib().ssfft_plan_error(p.handle, ctypes.byref(flags)) == 0 and flags.value == 0, name
    p.destroy()


@pytest.mark.parametrize("n", [8748, 9600, 10800, 12288, 16384])
def test_long_staged_unaligned_input_runs_plain_kernel_of_same_order(F, n):
    """A staged plan given an input off a 16-byte boundary runs the plain kernel with the plan's own
    radix order (its pass tables follow that order; 8748 / 9600 / 12288 stage with a list other
    than the planner's plain default)."""
    rng = np.random.default_rng(n + 3)
    b = 9
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(np.complex64)
    p = F.Plan(n, "f32", "complex", b)
    buf = torch.zeros(b * n + 1, dtype=torch.complex64, device="cuda")
    buf[1:] = dev(x).reshape(-1)
    out = torch.empty((b, n), dtype=torch.complex64, device="cuda")
    for inv in (False, True):
        assert F.lib().ssfft_exec(p.handle, int(inv), F._vp(buf.data_ptr() + 8), F._vp(out.data_ptr()), None) == 0
        torch.cuda.synchronize()
        ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
        assert rel_l2(out.cpu().numpy(), ref) <= F32_TOL, (n, inv, p.kernel(inv))


def test_staged_kernels_report_no_error(F, monkeypatch):
    """The bulk-copy staged kernels (SSFFT_DEBUG=staged=1 when the plan is made) bound their waits and
    report a per-plan flag; after normal runs (aligned and misaligned inputs, partial last
    group) it must read zero, and the results match the oracle."""
    rng = np.random.default_rng(12)
    n, b = 1920, 301
    x = rng.standard_normal((b, n)).astype(np.float32)
    monkeypatch.setenv("SSFFT_DEBUG", "staged=1")
    assert "batch_staged" in F.schedule_name(n, "f32", "real", b)
    p = F.Plan(n, "f32", "real", b)
    monkeypatch.delenv("SSFFT_DEBUG")
    xi = dev(x)
    out = torch.empty((b, n // 2), dtype=torch.complex64, device="cuda")
    p.exec(False, xi.data_ptr(), out.data_ptr(), 0)
    # an 8-byte-offset view (aligned for float pairs, not for 16-byte bulk copies) runs the
    # unstaged kernel of the same schedule
    buf = torch.zeros(b * n + 2, dtype=torch.float32, device="cuda")
    buf[2:] = xi.reshape(-1)
    out2 = torch.empty_like(out)
    ctypes_ok = F.lib().ssfft_exec(p.handle, 0, F._vp(buf.data_ptr() + 8), F._vp(out2.data_ptr()), None)
    torch.cuda.synchronize()
    assert ctypes_ok == 0
    import ctypes
    flags = ctypes.c_uint(99)
    assert F.lib().ssfft_plan_error(p.handle, ctypes.byref(flags)) == 0 and flags.value == 0
    ref = np.stack([oracle.rfft(r.astype(np.float64)) for r in x])
    assert rel_l2(out.cpu().numpy(), ref) <= F32_TOL
    assert np.array_equal(out.cpu().numpy(), out2.cpu().numpy())

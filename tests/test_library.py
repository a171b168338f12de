"""Host-side checks of libssfft.so that need no GPU: it loads, exports every entry point that
include/ssfft.h declares, reproduces the reference's size helpers bit for bit, rejects invalid
arguments with status codes, and its planner's kernels compile for sm_103a."""
import ctypes
import os
import re

import numpy as np
import pytest

import fft_gb300 as F
from conftest import ROOT


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ssfft.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ssfft_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(F.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_size_helpers_bit_exact(golden):
    idx = golden["size_index"]
    for name in ("size_minimum", "size_maximum", "real_size_minimum", "real_size_maximum"):
        got = np.array([getattr(F, name)(int(i)) for i in idx])
        assert np.array_equal(got, golden[name]), name
    # documented quirks of RealFFT (signalsmith-fft.h:403-408)
    assert F.real_size_maximum(480) == 512 and F.real_size_minimum(480) == 514


def _smooth_table(limit: int) -> np.ndarray:
    """Every 2^a 3^b 5^c <= limit, ascending (brute force)."""
    out = []
    a = 1
    while a <= limit:
        b = a
        while b <= limit:
            c = b
            while c <= limit:
                out.append(c)
                c *= 5
            b *= 3
        a *= 2
    return np.array(sorted(out), dtype=np.int64)


def test_smooth_size_helpers_against_brute_force():
    """Opt-in 5-smooth helpers (no reference counterpart: the reference never picks a 5,
    signalsmith-fft.h:317-348) against a brute-force table for every n in 1..2^20."""
    lib = F.lib()
    top = 1 << 20
    tab = _smooth_table(4 * top)
    n = np.arange(1, top + 1, dtype=np.int64)
    want_min = tab[np.searchsorted(tab, n, side="left")]
    want_max = tab[np.searchsorted(tab, n, side="right") - 1]
    fmin, fmax = lib.ssfft_size_minimum_smooth, lib.ssfft_size_maximum_smooth
    rmin, rmax = lib.ssfft_real_size_minimum_smooth, lib.ssfft_real_size_maximum_smooth
    got_min = np.fromiter((fmin(int(i)) for i in n), dtype=np.int64, count=top)
    got_max = np.fromiter((fmax(int(i)) for i in n), dtype=np.int64, count=top)
    assert np.array_equal(got_min, want_min)
    assert np.array_equal(got_max, want_max)
    # real lengths: even m with m/2 5-smooth
    half_up = (n + 1) // 2
    want_rmin = 2 * tab[np.searchsorted(tab, half_up, side="left")]
    half_dn = n // 2
    want_rmax = np.where(half_dn >= 1, 2 * tab[np.maximum(np.searchsorted(tab, half_dn, side="right") - 1, 0)], 0)
    sample = n[::7]
    got_rmin = np.array([rmin(int(i)) for i in sample], dtype=np.int64)
    got_rmax = np.array([rmax(int(i)) for i in sample], dtype=np.int64)
    assert np.array_equal(got_rmin, want_rmin[::7])
    assert np.array_equal(got_rmax, want_rmax[::7])
    assert fmin(0) == 0 and fmax(0) == 0 and rmin(0) == 0 and rmax(1) == 0 and rmin(1) == 2
    # large arguments: exact and no overflow
    for m in ((1 << 62) + 1, (1 << 63) - 1, 3 ** 39 + 2):
        odd = [3 ** b * 5 ** c for b in range(41) for c in range(28) if 3 ** b * 5 ** c < (1 << 66)]
        up = min(f << max(0, (m - 1) // f).bit_length() if f < m else f for f in odd)
        assert fmin(m) == (up if up < (1 << 64) else 0), m
        lo = max(f << ((m // f).bit_length() - 1) for f in odd if f <= m)
        assert fmax(m) == lo, m
    assert fmin(2 ** 63) == 2 ** 63
    assert fmin(2 ** 64 - 1) == 0  # no 5-smooth size >= 2^64 - 1 fits in size_t
    # the Python and drop-in names
    assert F.FFT.sizeMinimumSmooth(481) == 486 and F.FFT.sizeMaximumSmooth(481) == 480
    assert F.RealFFT.sizeMinimumSmooth(961) == 972 and F.RealFFT.sizeMaximumSmooth(961) == 960


def test_status_strings():
    lib = F.lib()
    for code in range(10):
        assert lib.ssfft_status_string(code)


def test_invalid_arguments_rejected_without_gpu():
    lib = F.lib()
    h = ctypes.c_void_p()
    assert lib.ssfft_plan_create(ctypes.byref(h), 0, 0, 0, 1) == 1          # n == 0
    assert lib.ssfft_plan_create(ctypes.byref(h), 1, 0, 1, 1) == 1          # real n < 2
    assert lib.ssfft_plan_create(ctypes.byref(h), 64, 7, 0, 1) == 2         # bad dtype
    assert lib.ssfft_plan_create(ctypes.byref(h), 64, 0, 9, 1) == 2         # bad kind
    assert lib.ssfft_plan_create(None, 64, 0, 0, 1) == 2
    assert lib.ssfft_exec(None, 0, None, None, None) == 2
    assert lib.ssfft_plan_destroy(None) == 2


@pytest.mark.parametrize("n,dt,kind,batch", [
    (480, "f32", "real", 16384), (960, "f32", "real", 16384), (1920, "f32", "real", 16384),
    (3840, "f32", "real", 16384), (1024, "f64", "complex", 256), (16384, "f32", "complex", 4),
    (8192, "f64", "complex", 2), (97, "f32", "complex", 1), (3840, "f32", "real_halfshift", 8),
])
def test_plan_kernels_compile_for_sm103a(n, dt, kind, batch):
    assert F.jit_check(n, dt, kind, batch, "sm_103a") > 0


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 30, 98, 512])
def test_small_and_odd_kernels_compile_for_sm103a(n):
    """Degenerate shapes (a single bin, no split pairs, odd real lengths, direct passes) compile
    under NVRTC too: it refuses constructs the host compiler accepts (zero-length arrays)."""
    for dt in ("f32", "f64"):
        for kind in ("complex", "real", "real_halfshift"):
            if kind != "complex" and n < 2:
                continue
            assert F.jit_check(n, dt, kind, 3, "sm_103a") > 0, (n, dt, kind)


@pytest.mark.parametrize("n, dt, kind", [(1024, "f32", "complex"), (3840, "f32", "real"), (1024, "f64", "complex")])
def test_staged_kernels_compile_for_sm103a(n, dt, kind, monkeypatch):
    """The bulk-copy staged variant (opt-in) and the failure-detection launch use it."""
    monkeypatch.setenv("SSFFT_DEBUG", "staged=1")
    assert "batch_staged" in F.schedule_name(n, dt, kind, 64)
    assert F.jit_check(n, dt, kind, 64, "sm_103a") > 0
    monkeypatch.delenv("SSFFT_DEBUG")
    assert "batch_staged" not in F.schedule_name(n, dt, kind, 64)


def test_schedules_respect_register_and_thread_budget():
    for n in list(range(1, 300)) + [480, 960, 1920, 3840, 4096, 8192, 16384, 15360, 3 ** 8]:
        info = F.schedule_info(n, "f32", "complex", 1000)
        assert info["threads"] * info["per_cta"] <= 1024
        assert info["smem_bytes"] <= 227 * 1024
        r = info["radices"]
        assert int(np.prod(r)) == n


def _minb(name: str) -> int:
    # batch<T, N, THREADS, PER_CTA, STRIDE, KIND, INV, ODD, EMAX, MINB, FUSE, radices...>
    return int(name.split("<", 1)[1].split(", ")[9])


def test_planner_policies_for_long_and_mid_transforms(monkeypatch):
    """The measured planner rules stay in force: register caps of two CTAs per SM (32 values a
    thread, <= 256 threads) and of five CTAs per SM (16 values, one transform per 256-thread CTA),
    fusable RealFFT lists, the smallest radix in the middle of long three-pass lists, and the
    cluster kernel off unless asked for."""
    assert _minb(F.schedule_name(8192, "f32", "complex", 4096)) == 2
    assert _minb(F.schedule_name(4096, "f32", "complex", 4096)) == 5
    assert _minb(F.schedule_name(8192, "f32", "real", 4096)) == 5
    assert _minb(F.schedule_name(2048, "f32", "complex", 4096)) == 1  # 128-thread CTAs: no cap
    assert _minb(F.schedule_name(4096, "f64", "complex", 4096)) == 1  # FP64: no cap
    assert F.schedule_info(16384, "f32", "real", 64)["radices"] == [32, 32, 8]
    assert ", true, 32, 32, 8>" in F.schedule_name(16384, "f32", "real", 64)  # split fused
    assert F.schedule_info(16384, "f32", "complex", 64)["radices"] == [32, 16, 32]
    assert F.schedule_info(15360, "f32", "real", 64)["radices"] == [16, 24, 20]
    # the headline RealFFT schedules
    assert F.schedule_info(3840, "f32", "real", 16384)["radices"] == [16, 15, 8]
    assert F.schedule_info(480, "f32", "real", 16384)["radices"] == [16, 15]
    assert not F.schedule_name(16384, "f32", "complex", 64).startswith("ssfft_cl::pair<")
    monkeypatch.setenv("SSFFT_DEBUG", "pair_min=8193")
    assert F.schedule_name(16384, "f32", "complex", 64).startswith("ssfft_cl::pair<")
    assert not F.schedule_name(8192, "f32", "complex", 64).startswith("ssfft_cl::pair<")


def test_fp64_tables_hold_every_twiddle_power():
    """FP64 passes load every power W^m .. W^{(R-1)m} (their bound is FP64 arithmetic); FP32
    register butterflies store the power-of-two rows and form the rest by products."""
    assert F.schedule_info(1024, "f64", "complex", 1)["radices"] == [16, 8, 8]
    assert F.schedule_info(1024, "f32", "complex", 1)["radices"] == [16, 8, 8]
    # passes 2 and 3 (radix 8 after 16 and 128 points): 7 rows (FP64) or 3 rows (FP32)
    assert F.schedule_tables(1024, "f64", "complex", 1)["tw"].size == 2 * 7 * (16 + 128)
    assert F.schedule_tables(1024, "f32", "complex", 1)["tw"].size == 2 * 3 * (16 + 128)


def test_large_spec_describes_multipass_plans_only():
    """ssfft_diag_large_spec: launch records of a multi-pass or Bluestein plan (no GPU); one-CTA
    lengths are refused."""
    spec, blob = F.large_spec(1 << 21, "f32", "complex")
    assert spec["N"] == 1 << 21 and len(spec["passes"]) == 3 and len(blob) > 0
    p0, p2 = spec["passes"][0], spec["passes"][-1]
    assert p0["fwd"].startswith("ssfft_cl::strided<float") and p0["inv"] != p0["fwd"]
    assert p0["U0"] * 128 == 1 << 21 and p2["out_es"] == (1 << 21) // 128
    spec, _ = F.large_spec(40000, "f64", "real")
    assert spec["real"] == 1 and spec["split_fwd"].startswith("ssfft_cl::real_split<double")
    spec, blob = F.large_spec(20011, "f32", "complex")  # a prime above 1024: Bluestein
    assert spec["M"] >= 2 * 20011 - 1 and spec["blue"][0] == "ssfft_cl::blue_pre<float, false>"
    assert len(blob) >= spec["off_bhat"] + 8 * spec["M"]
    with pytest.raises(F.SsfftError):
        F.large_spec(1024, "f32", "complex")  # one CTA


def test_cluster_split_options_in_the_planner():
    """The two-CTA cluster schedule from explicit options (no GPU): a valid split runs the pair
    kernel with its phases, an odd first phase or a split with no second phase is refused, and
    cluster_split=-1 keeps the one-CTA kernel."""
    try:
        F.schedule_options(radices=[16, 8, 16, 8], cluster_split=2)
        name = F.schedule_name(16384, "f32", "complex", 8)
        assert name.startswith("ssfft_cl::pair<float, 128, 128,") and "Radices<16, 8>, ssfft_cl::Radices<16, 8>>" in name
        assert F.jit_check(16384, "f32", "complex", 8) > 0
        F.schedule_options(radices=[25, 16, 25], cluster_split=1)
        with pytest.raises(F.SsfftError):
            F.schedule_name(10000, "f32", "complex", 8)
        F.schedule_options(cluster_split=-1)
        assert F.schedule_name(16384, "f32", "complex", 8).startswith(("ssfft_cl::batch<", "ssfft_cl::batch_staged<"))
        F.schedule_options(cluster_split=-1, staging=-1)
        assert F.schedule_name(16384, "f32", "complex", 8).startswith("ssfft_cl::batch<")
    finally:
        F.schedule_options()


def test_long_staging_in_the_planner():
    """Long FP32 transforms (complex, and RealFFT halves) stage their input by default where the
    plain kernel runs one CTA per SM and the staged one keeps 224-384 threads (the whole input when it fits beside the
    work buffer, else the first pass's leading rows); the plan option staging=-1 keeps the plain
    kernel and staging=1 stages wherever the input fits.  (No GPU: the build-time spill check is
    covered by the GPU parity tests.)"""
    try:
        name = F.schedule_name(16384, "f32", "complex", 4096)
        args = name[name.index("<") + 1:-1].split(", ")
        assert name.startswith("ssfft_cl::batch_staged<float, 16384,") and int(args[2]) == 256, name
        assert 0 < int(args[9]) < 32, name  # leading rows of the radix-32 first pass
        assert F.schedule_name(10240, "f32", "complex", 4096).startswith("ssfft_cl::batch_staged<float, 10240, 320,")
        assert ", 0, 16, 16, 40>" in F.schedule_name(10240, "f32", "complex", 4096)  # whole input staged
        # two CTAs per SM for the plain kernel (8192), or too few threads staged (10000): plain
        assert F.schedule_name(8192, "f32", "complex", 4096).startswith("ssfft_cl::batch<")
        assert F.schedule_name(10000, "f32", "complex", 4096).startswith("ssfft_cl::batch<")
        # FP64 and short transforms keep the plain kernel
        assert F.schedule_name(8192, "f64", "complex", 64).startswith("ssfft_cl::batch<")
        assert not F.schedule_name(32768, "f32", "real", 64).startswith("ssfft_cl::batch_staged")
        assert F.schedule_name(20480, "f32", "real", 64).startswith("ssfft_cl::batch_staged")  # half 10240
        assert not F.schedule_name(16384, "f32", "real", 64).startswith("ssfft_cl::batch_staged")  # 2 CTAs / SM
        assert not F.schedule_name(20480, "f32", "real_halfshift", 64).startswith("ssfft_cl::batch_staged")
        assert F.schedule_name(4096, "f32", "complex", 64).startswith("ssfft_cl::batch<")
        assert F.jit_check(16384, "f32", "complex", 4096) > 0
        F.schedule_options(staging=-1)
        assert F.schedule_name(16384, "f32", "complex", 4096).startswith("ssfft_cl::batch<")
        F.schedule_options(staging=1)
        assert F.schedule_name(4096, "f32", "complex", 64).startswith("ssfft_cl::batch_staged<")
        with pytest.raises(F.SsfftError):
            F.schedule_options(staging=2)
    finally:
        F.schedule_options()


def test_long_schedules_respect_shared_memory_and_thread_bounds():
    """Every FP32 length of 8192-16384 complex points (and the RealFFT lengths of those halves)
    gets a schedule within the device's limits: shared memory within 227 KiB, at most 1024
    threads per CTA; a staged one keeps one transform per CTA and 224-384 threads, and a
    leading-row staging keeps at least half the first pass's rows and fewer than all."""
    smooth = []
    for n in range(8192, 16385):
        m = n
        for p in (2, 3, 5):
            while m % p == 0:
                m //= p
        if m == 1:
            smooth.append(n)
    for kind, lengths in (("complex", smooth), ("real", [2 * n for n in smooth if n % 2 == 0])):
        for n in lengths:
            info = F.schedule_info(n, "f32", kind, 4096)
            name = F.schedule_name(n, "f32", kind, 4096, 0)
            assert info["smem_bytes"] <= 227 * 1024, (n, kind, info)
            assert info["threads"] * info["per_cta"] <= 1024, (n, kind, info)
            if "batch_staged" in name:
                args = name[name.index("<") + 1:-1].split(", ")
                assert info["per_cta"] == 1 and 224 <= info["threads"] <= 384, (n, kind, name)
                k = int(args[9])
                r0 = int(args[10])
                assert k == 0 or (2 * k >= r0 and k < r0), (n, kind, name)

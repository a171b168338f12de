"""Run the exact kernel source (fft_gb300/csrc/ssfft_codelets.cuh) on the CPU through the CUDA
emulation shim in tests/emu/, with the schedules and FP64 tables libssfft.so's planner picks, and
compare with the oracle.  This checks the kernels' index arithmetic, butterflies, twiddle layout,
real split/merge (including the reference's pair-overwrite order) and partial CTAs without a GPU.
The GPU parity tests (test_gpu_parity.py) repeat the comparison on the device."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import fft_gb300 as F
import oracle
from conftest import ROOT, rel_l2

# (n, dtype, kind, plan batch, exec batch)
CASES = [
    (1, "f64", "complex", 1, 1), (2, "f64", "complex", 3, 3), (3, "f32", "complex", 2, 2),
    (8, "f64", "complex", 1, 1), (16, "f32", "complex", 5, 5), (23, "f64", "complex", 1, 1),
    (49, "f64", "complex", 2, 2), (60, "f32", "complex", 100, 100), (96, "f64", "complex", 3, 3),
    (240, "f32", "complex", 2, 2), (1024, "f64", "complex", 2, 2), (1920, "f32", "complex", 1, 1),
    (4096, "f32", "complex", 1, 1), (50, "f64", "complex", 3, 3), (36, "f32", "complex", 5, 5),
    (18, "f64", "complex", 2, 2), (2880, "f32", "complex", 3, 3), (200, "f64", "real", 3, 3),
    (81, "f64", "complex", 3, 3), (2187, "f32", "complex", 2, 2), (486, "f64", "real", 2, 2),
    (2, "f64", "real", 1, 1), (3, "f64", "real", 2, 2), (7, "f32", "real", 1, 1), (10, "f64", "real", 4, 4),
    (98, "f32", "real", 3, 3), (480, "f32", "real", 5, 5), (3840, "f32", "real", 2, 2),
    (64, "f32", "complex", 300, 300), (1024, "f64", "complex", 7, 7), (480, "f32", "real", 40, 40),
    (3840, "f32", "real", 5, 5), (960, "f32", "real_halfshift", 9, 9),
    (1920, "f32", "real", 3, 3), (1000, "f64", "real", 2, 2), (64, "f32", "real", 50, 50), (30, "f64", "real", 3, 3),
    (96, "f64", "real", 4, 4), (100, "f32", "real", 7, 7), (8192, "f32", "real", 1, 1), (36, "f32", "real", 9, 9),
    (18, "f64", "real", 2, 2), (12, "f32", "real", 3, 3),
    # large composite radices 18, 20, 24, 25 (where they save a pass)
    (480, "f32", "complex", 3, 3), (15625, "f32", "complex", 1, 1), (11250, "f32", "complex", 1, 1), (7500, "f64", "complex", 1, 1),
    (13824, "f32", "complex", 1, 1), (960, "f64", "real", 2, 2),
    # radix 27, 32, 36, 40, 45 for long transforms
    (16384, "f32", "complex", 1, 1), (13500, "f32", "complex", 1, 1), (15552, "f32", "complex", 1, 1),
    (13122, "f32", "complex", 1, 1), (12800, "f32", "complex", 1, 1), (15000, "f32", "complex", 1, 1),
    (8100, "f64", "complex", 1, 1), (8748, "f32", "complex", 1, 1), (9720, "f32", "complex", 1, 1),
    (10240, "f32", "complex", 1, 1), (11664, "f32", "complex", 1, 1),
    # mid-length schedules (16 values a thread, largest radix in the middle pass)
    (5120, "f32", "complex", 2, 2), (6000, "f32", "complex", 1, 1), (7680, "f32", "complex", 1, 1),
    (12288, "f32", "real", 1, 1), (10800, "f32", "complex", 2, 2), (9600, "f32", "complex", 1, 1),
    (20480, "f32", "real", 2, 2),
    # one persistent CTA walking three groups of the leading-row staged kernel (the copies of the
    # next group's rows issued from the first and the last pass)
    (16384, "f32", "complex", 3, 3), (15000, "f32", "complex", 3, 3),
    (2, "f64", "real_halfshift", 1, 1), (4, "f64", "real_halfshift", 2, 2), (9, "f64", "real_halfshift", 1, 1),
    (12, "f32", "real_halfshift", 2, 2), (98, "f64", "real_halfshift", 1, 1), (960, "f32", "real_halfshift", 2, 2),
]
# split-BF16 tensor-core first pass (complex FP32): the emulated MMA decodes the same shared-memory
# descriptors and core-matrix layout the device reads
TC_CASES = [(64, "f32", "complex", 40, 40), (1920, "f32", "complex", 3, 3), (16, "f32", "complex", 200, 200),
            (112, "f32", "complex", 5, 5), (7, "f32", "complex", 130, 130), (4096, "f32", "complex", 1, 1),
            (480, "f32", "complex", 9, 9), (3, "f32", "complex", 1, 1)]
TC_TOL = 2e-6
# two-CTA cluster (pair) schedules: (n, plan batch, exec batch, radices, phase-A radix count);
# the default complex cases above of 8192+ points run the bulk-copy kernel.
PAIR_CASES = [(16384, 1, 1, [16, 8, 16, 8], 2), (12288, 2, 2, [32, 16, 24], 1), (9216, 1, 1, [16, 6, 12, 8], 2),
              (15360, 1, 1, [8, 15, 16, 8], 2), (8192, 3, 3, [8, 16, 4, 16], 2), (4000, 2, 2, [10, 20, 20], 1)]
# transforms at scattered offsets (the offset-table launches of uneven batches): (case, variant);
# "offs" compiles the plain kernel of the case (not the staged one this module's plans pick)
OFFS_CASES = [((240, "f32", "complex", 2, 2), "offs"), ((64, "f32", "complex", 300, 300), "offs"),
              ((1920, "f32", "complex", 1, 1), "offs"), ((4096, "f32", "complex", 1, 1), "offs"),
              ((16384, "f32", "complex", 1, 1), "pair16384"), ((1024, "f64", "complex", 7, 7), "offs"),
              ((5120, "f32", "complex", 2, 2), "offs"), ((7680, "f32", "complex", 1, 1), "offs")]
VARIANTS = {"default": {"fuse_split": 1}, "tc": {"precision": "split_bf16"}, "offs": {}}
for _c in PAIR_CASES:
    VARIANTS[f"pair{_c[0]}"] = ({"cluster_split": _c[4], "radices": _c[3]} if _c[3] else {})


def tc_matrix(r0):
    """The radix-r0 DFT as the tensor-core pass's 32 x 32 real matrix, transposed (row = output
    column): [Re y_k | Im y_k] from [Re x_r | Im x_r], y_k = sum_r x_r exp(-2 pi i r k / r0)."""
    bt = np.zeros((32, 32))
    for k in range(r0):
        for r in range(r0):
            c, s = np.cos(2 * np.pi * r * k / r0), np.sin(2 * np.pi * r * k / r0)
            bt[k, r], bt[k, 16 + r], bt[16 + k, r], bt[16 + k, 16 + r] = c, s, -s, c
    return bt.astype(np.float32)



@pytest.fixture(scope="module", autouse=True)
def staged_schedules():
    """The emulator covers both the plain and the bulk-copy staged kernels: plans made while this
    module runs may pick the staged kernel (SSFFT_DEBUG=staged=1); the setting is restored afterwards."""
    old = os.environ.get("SSFFT_DEBUG")
    os.environ["SSFFT_DEBUG"] = "staged=1"
    yield
    if old is None:
        os.environ.pop("SSFFT_DEBUG", None)
    else:
        os.environ["SSFFT_DEBUG"] = old


@pytest.fixture(scope="module")
def emulator(staged_schedules, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("emu")
    lines = []
    index = {}
    cases = [(c, "default") for c in CASES] + [(c, "tc") for c in TC_CASES]
    cases += [((c[0], "f32", "complex", c[1], c[2]), f"pair{c[0]}") for c in PAIR_CASES]
    cases += [(c, "offs") for c, v in OFFS_CASES if v == "offs"]
    for case, var in cases:
        (n, dt, kind, pb, _) = case
        # offset-table launches run the plain kernel (the library routes them off the staged one)
        os.environ["SSFFT_DEBUG"] = "staged=0" if var == "offs" else "staged=1"
        F.schedule_options(**VARIANTS[var])
        for inv in (False, True):
            # a RealFFT plan may run a different radix order per direction (fused split)
            F.schedule_direction(inv)
            info = F.schedule_info(n, dt, kind, pb)
            name = F.schedule_name(n, dt, kind, pb, inv)
            index[(n, dt, kind, pb, inv, var)] = (len(lines), info)
            cluster = 2 if name.startswith("ssfft_cl::pair<") else 1
            lines.append(f'{{"{n}-{dt}-{kind}-{int(inv)}", &{name}, {info["threads"] * info["per_cta"]}, '
                         f'{info["smem_bytes"]}, {cluster}}},')
        F.schedule_options()
        F.schedule_direction(False)
    os.environ["SSFFT_DEBUG"] = "staged=1"
    (d / "emu_cases.inc").write_text("\n".join(lines) + "\n")
    exe = d / "emu"
    cmd = ["g++", "-std=c++20", "-O1", "-pthread", "-w", "-I", str(d), "-I", os.path.join(ROOT, "tests", "emu"),
           "-I", os.path.join(ROOT, "fft_gb300", "csrc"), os.path.join(ROOT, "tests", "emu", "emu_main.cpp"),
           "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe, index, d


def _run(emulator, n, dt, kind, pb, eb, inv, x, tc=False, var=None):
    exe, index, d = emulator
    var = var or ("tc" if tc else "default")
    ci, info = index[(n, dt, kind, pb, inv, var)]
    F.schedule_options(**VARIANTS[var])
    F.schedule_direction(inv)
    sdt = np.float32 if dt == "f32" else np.float64
    real = kind != "complex"
    h2 = 2 * (n // 2)
    if not real:
        in_dist = out_dist = 2 * n
    elif not inv:
        in_dist, out_dist = n, h2
    else:
        in_dist, out_dist = h2, n
    xin = np.ascontiguousarray(x).view(sdt).reshape(eb, in_dist)
    out = np.full((eb, out_dist), np.nan, dtype=sdt)
    tabs = F.schedule_tables(n, dt, kind, pb)
    blob = np.array([tabs[k].size for k in ("tw", "roots", "rtw", "rot")], dtype=np.uint64).tobytes()
    blob += b"".join(tabs[k].astype(sdt).tobytes() for k in ("tw", "roots", "rtw", "rot"))
    name = F.schedule_name(n, dt, kind, pb, inv)
    if "batch_tc" in name:
        blob += tc_matrix(info["radices"][0]).tobytes()
    F.schedule_options()
    F.schedule_direction(False)
    fi, fo, ft = d / f"in{ci}", d / f"out{ci}", d / f"tab{ci}"
    fi.write_bytes(xin.tobytes())
    fo.write_bytes(out.tobytes())
    ft.write_bytes(blob)
    groups = -(-eb // info["per_cta"])
    # persistent (staged) kernels: fewer CTAs than groups, so each CTA walks several groups;
    # cluster (pair) kernels: two CTAs per transform
    grid = max(1, groups // 2) if "batch_staged" in name else 2 * eb if name.startswith("ssfft_cl::pair<") else groups
    in_bytes = in_dist * np.dtype(sdt).itemsize
    subprocess.run([str(exe), str(ci), str(grid), str(fi), str(fo), str(ft), str(eb), str(in_dist), str(out_dist),
                    str(np.dtype(sdt).itemsize), str(in_bytes)], check=True, timeout=300)
    return np.frombuffer(fo.read_bytes(), dtype=sdt).reshape(eb, out_dist)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-{c[2]}")
def test_emulated_kernel_matches_oracle(emulator, case):
    n, dt, kind, pb, eb = case
    rng = np.random.default_rng(n * 7 + len(kind))
    tol = 1e-6 if dt == "f32" else 1e-13
    cdt = np.complex64 if dt == "f32" else np.complex128
    rdt = np.float32 if dt == "f32" else np.float64
    if kind == "complex":
        x = (rng.uniform(-1, 1, (eb, n)) + 1j * rng.uniform(-1, 1, (eb, n))).astype(cdt)
        for inv in (False, True):
            got = _run(emulator, n, dt, kind, pb, eb, inv, x).view(cdt)
            ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
            assert rel_l2(got, ref) <= tol, (inv, rel_l2(got, ref))
    else:
        mod = kind == "real_halfshift"
        h = n // 2
        x = rng.standard_normal((eb, n)).astype(rdt)
        got = _run(emulator, n, dt, kind, pb, eb, False, x).view(cdt)
        ref = np.stack([oracle.rfft(r.astype(np.float64), mod) for r in x])
        assert got.shape == ref.shape
        assert rel_l2(got, ref) <= tol, rel_l2(got, ref)
        s = (rng.standard_normal((eb, h)) + 1j * rng.standard_normal((eb, h))).astype(cdt)
        got = _run(emulator, n, dt, kind, pb, eb, True, s)
        ref = np.stack([oracle.irfft(r.astype(np.complex128), n, mod) for r in s])
        assert rel_l2(got[:, :2 * h], ref) <= tol, rel_l2(got[:, :2 * h], ref)
        if n % 2:
            assert np.all(np.isnan(got[:, 2 * h:])), "odd real length: last sample must be left alone"


@pytest.mark.parametrize("case", TC_CASES, ids=lambda c: f"tc-{c[0]}")
def test_emulated_tensor_core_kernel_matches_oracle(emulator, case):
    n, dt, kind, pb, eb = case
    F.schedule_options(precision="split_bf16")
    name = F.schedule_name(n, dt, kind, pb)
    F.schedule_options()
    assert "batch_tc" in name
    rng = np.random.default_rng(n * 11)
    x = (rng.uniform(-1, 1, (eb, n)) + 1j * rng.uniform(-1, 1, (eb, n))).astype(np.complex64)
    for inv in (False, True):
        got = _run(emulator, n, dt, kind, pb, eb, inv, x, tc=True).view(np.complex64)
        ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
        assert rel_l2(got, ref) <= TC_TOL, (inv, rel_l2(got, ref))


@pytest.mark.parametrize("case", PAIR_CASES, ids=lambda c: f"pair-{c[0]}")
def test_emulated_pair_kernel_matches_oracle(emulator, case):
    """Two-CTA cluster kernel: both CTAs of a cluster run at once, the second phase reads half of
    each row from the other CTA's shared memory."""
    n, pb, eb, rad, split = case
    var = f"pair{n}"
    F.schedule_options(**VARIANTS[var])
    name = F.schedule_name(n, "f32", "complex", pb)
    F.schedule_options()
    assert name.startswith("ssfft_cl::pair<"), name
    rng = np.random.default_rng(n * 13)
    x = (rng.uniform(-1, 1, (eb, n)) + 1j * rng.uniform(-1, 1, (eb, n))).astype(np.complex64)
    for inv in (False, True):
        got = _run(emulator, n, "f32", "complex", pb, eb, inv, x, var=var).view(np.complex64)
        ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
        assert rel_l2(got, ref) <= 1e-6, (inv, rel_l2(got, ref))




@pytest.mark.parametrize("case,var", OFFS_CASES, ids=lambda c: str(c[0]) if isinstance(c, tuple) else c)
def test_emulated_offset_table(emulator, case, var):
    """Each transform read and written at its own offset (odd gaps between them): every transform
    matches the oracle and nothing outside the transforms is written."""
    exe, index, d = emulator
    n, dt, kind, pb, eb = case
    sdt = np.float32 if dt == "f32" else np.float64
    cdt = np.complex64 if dt == "f32" else np.complex128
    ci, info = index[(n, dt, kind, pb, False, var)]
    os.environ["SSFFT_DEBUG"] = "staged=0" if var == "offs" else "staged=1"
    F.schedule_options(**VARIANTS[var])
    name = F.schedule_name(n, dt, kind, pb)
    tabs = F.schedule_tables(n, dt, kind, pb)
    F.schedule_options()
    os.environ["SSFFT_DEBUG"] = "staged=1"
    assert "batch_staged" not in name, name
    gap = 3
    offs = np.array([g * (n + gap) + 1 for g in range(eb)], dtype=np.int64)  # complex units
    total = int(offs[-1]) + n + gap
    rng = np.random.default_rng(n + eb)
    x = (rng.uniform(-1, 1, (eb, n)) + 1j * rng.uniform(-1, 1, (eb, n))).astype(cdt)
    buf = np.full(total, np.nan, dtype=cdt)
    for g in range(eb):
        buf[offs[g]:offs[g] + n] = x[g]
    blob = np.array([tabs[k].size for k in ("tw", "roots", "rtw", "rot")], dtype=np.uint64).tobytes()
    blob += b"".join(tabs[k].astype(sdt).tobytes() for k in ("tw", "roots", "rtw", "rot"))
    fi, fo, ft, fs = d / f"oin{ci}", d / f"oout{ci}", d / f"otab{ci}", d / f"offs{ci}"
    fi.write_bytes(buf.tobytes())
    fo.write_bytes(np.full(total, np.nan, dtype=cdt).tobytes())
    ft.write_bytes(blob)
    fs.write_bytes((2 * offs).tobytes())  # scalars
    groups = -(-eb // info["per_cta"])
    grid = 2 * eb if name.startswith("ssfft_cl::pair<") else groups
    subprocess.run([str(exe), str(ci), str(grid), str(fi), str(fo), str(ft), str(eb), str(2 * n), str(2 * n),
                    str(np.dtype(sdt).itemsize), str(2 * n * np.dtype(sdt).itemsize), str(fs)], check=True, timeout=300)
    out = np.frombuffer(fo.read_bytes(), dtype=cdt)
    inside = np.zeros(total, dtype=bool)
    for g in range(eb):
        inside[offs[g]:offs[g] + n] = True
        ref = oracle.fft(x[g].astype(np.complex128))
        assert rel_l2(out[offs[g]:offs[g] + n], ref) <= (1e-6 if dt == "f32" else 1e-13), g
    assert np.all(np.isnan(out[~inside])), "nothing written outside the transforms"

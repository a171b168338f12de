"""Run the multi-pass (four-step) pass kernels (ssfft_cl::strided, the exact source in
fft_gb300/csrc/ssfft_codelets.cuh) on the CPU through the CUDA emulation shim in tests/emu/, with
the launch records and table bytes libssfft.so's planner produces (ssfft_diag_large_spec), pass
by pass, and compare with the oracle.  This checks the passes' strides, segment loads and stores,
inter-pass twiddles and the inverse conjugation without a GPU; test_gpu_large.py repeats the
comparison on the device."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import fft_gb300 as F
import oracle
from conftest import ROOT, rel_l2

# (n, dtype, kind, transforms): two passes (FP32 above 16384 points, FP64 above 8192) and three
# passes; RealFFT lengths add the split kernel (and the half-shift rotations)
CASES = [(20000, "f32", "complex", 2), (32768, "f32", "complex", 1), (10000, "f64", "complex", 2),
         (1 << 21, "f32", "complex", 1), (2 * 3 ** 9, "f32", "complex", 1), (40000, "f32", "real", 2),
         (40000, "f32", "real_halfshift", 1), (20000, "f64", "real", 1), (20000, "f64", "real_halfshift", 1)]


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("emu_strided")
    lines, splits, specs = [], [], {}
    for n, dt, kind, _ in CASES:
        spec, blob = F.large_spec(n, dt, kind)
        specs[(n, dt, kind)] = (spec, blob, len(lines), len(splits))
        for p in spec["passes"]:
            for key in ("fwd", "inv"):
                lines.append(f'{{"{n}-{dt}-{key}", &{p[key]}, {p["cta"]}, {p["smem"]}}},')
        if spec["real"]:
            splits += [f'{{"{n}-{dt}-{kind}-fwd", &{spec["split_fwd"]}}},',
                       f'{{"{n}-{dt}-{kind}-inv", &{spec["split_inv"]}}},']
    (d / "emu_strided_cases.inc").write_text("\n".join(lines) + "\n")
    (d / "emu_split_cases.inc").write_text("\n".join(splits) + "\n")
    exe = d / "emu_strided"
    cmd = ["g++", "-std=c++20", "-O2", "-pthread", "-w", "-I", str(d), "-I", os.path.join(ROOT, "tests", "emu"),
           "-I", os.path.join(ROOT, "fft_gb300", "csrc"), os.path.join(ROOT, "tests", "emu", "emu_strided_main.cpp"),
           "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe, specs, d


def _transform(emulator, n, dt, kind, x, inverse):
    """x: [transforms, complex points] (the reals viewed as pairs for a RealFFT forward, the
    bins for its inverse); returns the same shape, as the library's launch sequence does."""
    exe, specs, d = emulator
    spec, blob, first, first_split = specs[(n, dt, kind)]
    sdt = np.float32 if dt == "f32" else np.float64
    nb, N = x.shape
    ft = d / f"tab-{n}-{dt}-{kind}"
    ft.write_bytes(blob)
    fi, fo = d / f"in-{n}-{dt}", d / f"out-{n}-{dt}"
    cur = np.ascontiguousarray(x).view(sdt).reshape(-1)

    def split(inv, src, buf):
        fi.write_bytes(src.tobytes())
        fo.write_bytes(buf.tobytes())
        blocks = -(-(N // 2 + 1) // 256)
        args = [f"s{first_split + int(inv)}", blocks, fi, fo, ft, nb, N, spec["off_rtw"]]
        subprocess.run([str(exe)] + [str(a) for a in args], check=True, timeout=600)
        return np.frombuffer(fo.read_bytes(), dtype=sdt).copy()

    if spec["real"] and inverse:
        cur = split(True, cur, np.full_like(cur, np.nan))
    for i, p in enumerate(spec["passes"]):
        fi.write_bytes(cur.tobytes())
        fo.write_bytes(np.full_like(cur, np.nan).tobytes())
        grid = nb * p["U1"] * (-(-p["U0"] // p["G"]))
        case = first + 2 * i + (1 if inverse else 0)
        args = [f"p{case}", grid, fi, fo, ft, nb, N, p["U0"], p["U1"], p["is0"], p["is1"], p["in_es"], p["os0"],
                p["os1"], p["out_es"], p["off_tw"], p["off_roots"], p["off_twlo"], p["off_twhi"], spec["off_rot"]]
        subprocess.run([str(exe)] + [str(a) for a in args], check=True, timeout=600)
        cur = np.frombuffer(fo.read_bytes(), dtype=sdt).copy()
    if spec["real"] and not inverse:
        cur = split(False, cur, cur)
    cdt = np.complex64 if dt == "f32" else np.complex128
    return cur.view(cdt).reshape(nb, N)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-{c[2]}")
def test_emulated_multipass_matches_oracle(emulator, case):
    n, dt, kind, nb = case
    rng = np.random.default_rng(n % 1009)
    cdt = np.complex64 if dt == "f32" else np.complex128
    rdt = np.float32 if dt == "f32" else np.float64
    tol = 1e-6 if dt == "f32" else 1e-13
    if kind == "complex":
        x = (rng.uniform(-1, 1, (nb, n)) + 1j * rng.uniform(-1, 1, (nb, n))).astype(cdt)
        for inv in (False, True):
            got = _transform(emulator, n, dt, kind, x, inv)
            assert np.all(np.isfinite(got)), "every output element written"
            ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
            assert rel_l2(got, ref) <= tol, (inv, rel_l2(got, ref))
    else:
        mod = kind == "real_halfshift"
        x = rng.standard_normal((nb, n)).astype(rdt)
        got = _transform(emulator, n, dt, kind, x.view(cdt), False)
        ref = np.stack([oracle.rfft(r.astype(np.float64), mod) for r in x])
        assert rel_l2(got, ref) <= tol, rel_l2(got, ref)
        s = (rng.standard_normal((nb, n // 2)) + 1j * rng.standard_normal((nb, n // 2))).astype(cdt)
        back = _transform(emulator, n, dt, kind, s, True).view(rdt)
        ref = np.stack([oracle.irfft(r.astype(np.complex128), n, mod) for r in s])
        assert rel_l2(back, ref) <= tol, rel_l2(back, ref)

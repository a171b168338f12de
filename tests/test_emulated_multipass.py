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

# (n, dtype, transforms): two passes (FP32 above 16384 points, FP64 above 8192) and three passes
CASES = [(20000, "f32", 2), (32768, "f32", 1), (10000, "f64", 2), (1 << 21, "f32", 1), (2 * 3 ** 9, "f32", 1)]


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("emu_strided")
    lines, specs = [], {}
    for n, dt, _ in CASES:
        spec, blob = F.large_spec(n, dt, "complex")
        specs[(n, dt)] = (spec, blob, len(lines))
        for p in spec["passes"]:
            for key in ("fwd", "inv"):
                lines.append(f'{{"{n}-{dt}-{key}", &{p[key]}, {p["cta"]}, {p["smem"]}}},')
    (d / "emu_strided_cases.inc").write_text("\n".join(lines) + "\n")
    exe = d / "emu_strided"
    cmd = ["g++", "-std=c++20", "-O2", "-pthread", "-w", "-I", str(d), "-I", os.path.join(ROOT, "tests", "emu"),
           "-I", os.path.join(ROOT, "fft_gb300", "csrc"), os.path.join(ROOT, "tests", "emu", "emu_strided_main.cpp"),
           "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe, specs, d


def _transform(emulator, n, dt, x, inverse):
    exe, specs, d = emulator
    spec, blob, first = specs[(n, dt)]
    sdt = np.float32 if dt == "f32" else np.float64
    nb = x.shape[0]
    ft = d / f"tab-{n}-{dt}"
    ft.write_bytes(blob)
    cur = np.ascontiguousarray(x).view(sdt).reshape(-1)
    for i, p in enumerate(spec["passes"]):
        fi, fo = d / f"in-{n}-{dt}", d / f"out-{n}-{dt}"
        fi.write_bytes(cur.tobytes())
        fo.write_bytes(np.full_like(cur, np.nan).tobytes())
        grid = nb * p["U1"] * (-(-p["U0"] // p["G"]))
        case = first + 2 * i + (1 if inverse else 0)
        args = [case, grid, fi, fo, ft, nb, n, p["U0"], p["U1"], p["is0"], p["is1"], p["in_es"], p["os0"], p["os1"],
                p["out_es"], p["off_tw"], p["off_roots"], p["off_twlo"], p["off_twhi"], spec["off_rot"]]
        subprocess.run([str(exe)] + [str(a) for a in args], check=True, timeout=600)
        cur = np.frombuffer(fo.read_bytes(), dtype=sdt).copy()
    cdt = np.complex64 if dt == "f32" else np.complex128
    return cur.view(cdt).reshape(nb, n)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}")
def test_emulated_multipass_matches_oracle(emulator, case):
    n, dt, nb = case
    rng = np.random.default_rng(n % 1009)
    cdt = np.complex64 if dt == "f32" else np.complex128
    x = (rng.uniform(-1, 1, (nb, n)) + 1j * rng.uniform(-1, 1, (nb, n))).astype(cdt)
    tol = 1e-6 if dt == "f32" else 1e-13
    for inv in (False, True):
        got = _transform(emulator, n, dt, x, inv)
        assert np.all(np.isfinite(got)), "every output element written"
        ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
        assert rel_l2(got, ref) <= tol, (inv, rel_l2(got, ref))

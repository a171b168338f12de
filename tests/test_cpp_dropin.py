"""Compile the C++ drop-in tests (tests/cpp/dropin_tests.cpp, the reference suite's checks written
against include/signalsmith-fft.h) against libssfft.so; run them on the GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CUDA = os.path.dirname(os.path.dirname(os.path.realpath(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")))


def build_dropin(tmp_path):
    exe = tmp_path / "dropin_tests"
    lib_dir = os.path.join(ROOT, "fft_gb300")
    lib64 = os.path.join(CUDA, "lib64")
    cmd = ["g++", "-std=c++11", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "dropin_tests.cpp"),
           "-L", lib_dir, "-lssfft", "-L", lib64, "-lcudart", f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{lib64}",
           "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_dropin_header_compiles_cxx11(tmp_path):
    """The drop-in header builds as C++11 with warnings, like the reference's test build."""
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    build_dropin(tmp_path)


@pytest.mark.gpu
def test_dropin_reference_suite_on_gpu(tmp_path, golden):
    """The reference suite's checks, plus the setSize family's return values against the table
    the reference produced (RealFFT returns the half size) and plan reuse on an unchanged size."""
    exe = build_dropin(tmp_path)
    cases = tmp_path / "setsize.txt"
    cases.write_text("\n".join(" ".join(str(int(v)) for v in row) for row in golden["setsize_returns"]) + "\n")
    r = subprocess.run([str(exe), str(cases)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]


def test_golden_setsize_table_is_the_reference_contract(golden):
    """The fixture's RealFFT rows return the half size (reference :434) and FFT rows the size."""
    t = golden["setsize_returns"]
    assert len(t) >= 30
    for cls, first, n, r_set, size1, r_min, r_max, size2 in t:
        if cls == 0:
            assert r_set == n and size1 == n and r_max == size2
        else:
            assert r_set == n // 2 and size1 == 2 * (n // 2) and size2 == 2 * r_max

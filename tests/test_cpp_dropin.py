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
def test_dropin_reference_suite_on_gpu(tmp_path):
    exe = build_dropin(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]

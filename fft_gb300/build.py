"""Build recipe for libssfft.so (the GB300 transform library) -- no cmake, no torch extension.

Steps:
1. embed ``csrc/ssfft_codelets.cuh`` (the size-specialised kernel templates compiled at plan
   time by NVRTC) into ``csrc/ssfft_codelets_src.inc`` as a C++ raw string;
2. compile every ``csrc/*.cu`` host translation unit with nvcc for sm_103a, in parallel;
3. link ``fft_gb300/libssfft.so`` against NVRTC (driver entry points are resolved at run time).

``python -m fft_gb300.build`` runs it; ``__graft_entry__.build()`` calls :func:`build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libssfft.so")
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["ssfft_plan.cu", "ssfft_jit.cu", "ssfft_stage.cu", "ssfft_large.cu", "ssfft_serve.cu", "ssfft_multi.cu", "ssfft_noalloc.cu", "ssfft_tune.cu"]


def cuda_root() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _embed_codelets() -> None:
    src = open(os.path.join(CSRC, "ssfft_codelets.cuh")).read()
    delim = "SSFFTSRC"
    assert f"){delim}\"" not in src
    text = f'R"{delim}({src}){delim}"\n'
    out = os.path.join(CSRC, "ssfft_codelets_src.inc")
    if not os.path.exists(out) or open(out).read() != text:
        with open(out, "w") as f:
            f.write(text)


def _compile(src: str, obj: str, nvcc: str) -> None:
    cmd = [nvcc, *ARCH_FLAGS, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")


def _stale(objs: list[str]) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "ssfft.h"),
                                                                 __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link libssfft.so if any source is newer; returns its path."""
    _embed_codelets()
    objdir = os.path.join(HERE, "_build")
    os.makedirs(objdir, exist_ok=True)
    objs = [os.path.join(objdir, s.replace(".cu", ".o")) for s in SOURCES]
    if not force and not _stale(objs):
        return LIB
    root = cuda_root()
    nvcc = os.path.join(root, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, s, o, nvcc) for s, o in zip(SOURCES, objs)]
        for f in futs:
            f.result()
    lib64 = os.path.join(root, "lib64")
    if not os.path.isdir(lib64):
        lib64 = os.path.join(root, "lib")
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs, "-L" + lib64, "-lnvrtc", "-Xlinker", "-rpath=" + lib64]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)

"""Generate tests/golden/reference_vectors.npz from the UNMODIFIED reference implementation.

Run where the reference source is checked out, naming its directory (required):

    REF_DIR=<reference checkout> python tests/golden/make_golden.py

It builds oracle/_ref/libssref.so (the reference header behind the C shim in
oracle/ref_shim.cpp, via ``make -C oracle ref``) and records, on seeded inputs:

* complex FFT<double>/FFT<float> forward and inverse outputs at the reference tests' sizes
  (tests/00-fft.cpp:8-16) plus 480 and 1024;
* RealFFT / ModifiedRealFFT <double>/<float> forward outputs and inverse outputs (of an
  independent seeded spectrum) at every size 2..99 (tests/01-real.cpp:17 covers the even ones;
  odd sizes pin the reference's floor(n/2) behaviour) plus the mixed-radix frame sizes
  480, 960, 1920, 3840;
* FFT::sizeMinimum/sizeMaximum and RealFFT::sizeMinimum/sizeMaximum for 1..4096;
* the return values of setSize / setSizeMinimum / setSizeMaximum and size() of FFT, RealFFT and
  ModifiedRealFFT objects (signalsmith-fft.h:356-369, :416-444) at SETSIZE_CASES.

The fixture is what pins the oracle (tests/test_oracle.py) and the GPU path
(tests/test_gpu_parity.py) on hosts that have no reference checkout.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

COMPLEX_SIZES = [1, 2, 4, 8, 16, 32, 64, 128, 256, 3, 6, 9, 12, 18, 24, 5, 10, 15, 20, 25,
                 7, 14, 21, 28, 49, 11, 13, 17, 19, 22, 23, 480, 1024]
REAL_SIZES = list(range(2, 100)) + [480, 960, 1920, 3840]
SEED = 20241203
# (first size, size set) pairs: unchanged, grown, shrunk, odd real lengths, zero
SETSIZE_CASES = [(8, 8), (8, 480), (480, 3840), (3840, 7), (7, 6), (6, 7), (1, 2), (2, 1), (16, 0), (0, 5),
                 (100, 1025), (1030, 1030), (4096, 999)]


def main() -> None:
    ref_dir = os.environ.get("REF_DIR")
    if not ref_dir:
        raise SystemExit("set REF_DIR to the reference checkout (the directory holding signalsmith-fft.h)")
    oracle.build(reference=ref_dir)
    rng = np.random.Generator(np.random.PCG64(SEED))
    out: dict[str, np.ndarray] = {}
    for n in COMPLEX_SIZES:
        x = rng.uniform(-0.5, 0.5, n) + 1j * rng.uniform(-0.5, 0.5, n)
        for name, dt in (("f64", np.complex128), ("f32", np.complex64)):
            xi = x.astype(dt)
            out[f"c2c_{name}_{n}_in"] = xi
            out[f"c2c_{name}_{n}_fwd"] = oracle.fft(xi, False, kind="reference")
            out[f"c2c_{name}_{n}_inv"] = oracle.fft(xi, True, kind="reference")
    for n in REAL_SIZES:
        x = rng.standard_normal(n)
        h = n // 2
        spec = rng.standard_normal(h) + 1j * rng.standard_normal(h)
        for name, rdt, cdt in (("f64", np.float64, np.complex128), ("f32", np.float32, np.complex64)):
            if name == "f64" or n <= 100 or n in (480, 960, 1920, 3840):
                for mod in (0, 1):
                    key = f"r_{name}_m{mod}_{n}"
                    xi = x.astype(rdt)
                    si = spec.astype(cdt)
                    out[key + "_in"] = xi
                    out[key + "_fwd"] = oracle.rfft(xi, bool(mod), kind="reference")
                    out[key + "_spec"] = si
                    out[key + "_inv"] = oracle.irfft(si, n, bool(mod), kind="reference")
    idx = np.arange(1, 4097, dtype=np.int64)
    out["size_index"] = idx
    out["size_minimum"] = np.array([oracle.size_minimum(int(i), "reference") for i in idx], dtype=np.int64)
    out["size_maximum"] = np.array([oracle.size_maximum(int(i), "reference") for i in idx], dtype=np.int64)
    out["real_size_minimum"] = np.array([oracle.real_size_minimum(int(i), "reference") for i in idx], dtype=np.int64)
    out["real_size_maximum"] = np.array([oracle.real_size_maximum(int(i), "reference") for i in idx], dtype=np.int64)
    ref = oracle.lib("reference")
    f = ref.ref_setsize_returns
    f.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    f.restype = ctypes.c_int
    rows = []
    for cls in (0, 1, 2):
        for first, n in SETSIZE_CASES:
            r = (ctypes.c_size_t * 5)()
            assert f(cls, first, n, r) == 0
            rows.append([cls, first, n, *r])
    out["setsize_returns"] = np.array(rows, dtype=np.int64)
    out["meta_seed"] = np.array([SEED], dtype=np.int64)
    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()

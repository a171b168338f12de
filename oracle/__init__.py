"""CPU oracle for the Signalsmith FFT transform path -- TEST INFRASTRUCTURE ONLY.

Two CPU implementations sit behind one numpy-level interface:

* ``port``      -- ``oracle/liboracle.so``, the plain-C restatement of the reference header
  signalsmith-fft.h in ``oracle/ssfft_oracle.c`` (builds on any host; it is what the GPU
  host runs as checker).
* ``port_native`` -- ``oracle/liboracle_native.so``, the same source built for speed (host vector
  ISA, FP contraction allowed): the CPU baseline's timing build, never a checker.
* ``reference`` -- ``oracle/_ref/libssref.so``, the unmodified reference header compiled behind a
  C shim (``oracle/ref_shim.cpp``); only exists where the reference checkout was available.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm use
this package.  The GPU library in ``fft_gb300/`` never imports it.

Conventions follow the reference API: complex transforms are unnormalised
(``ifft(fft(x)) == n*x``, signalsmith-fft.h:374-386); ``rfft`` maps n reals to n/2 complex bins
with {DC, Nyquist} packed into bin 0 (signalsmith-fft.h:446-473); ``irfft`` maps n/2 bins back to
2*(n/2) reals scaled by n (signalsmith-fft.h:475-502).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
NATIVE_SO = os.path.join(HERE, "liboracle_native.so")
REF_SO = os.path.join(HERE, "_ref", "libssref.so")
_lock = threading.Lock()
_libs: dict = {}

_c_size = ctypes.c_size_t
_c_int = ctypes.c_int
_vp = ctypes.c_void_p


def build(reference: str | None = None) -> None:
    """Compile liboracle.so; with `reference` (the directory of a reference checkout, holding
    signalsmith-fft.h) also the reference shim oracle/_ref/libssref.so."""
    subprocess.run(["make", "-s", "-C", HERE, "all", "native"], check=True)
    if reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={reference}"], check=True)


def reference_dir() -> str | None:
    """The reference checkout used to build the shim: $REF_DIR, else a checkout named `reference`
    beside this repository, if it holds signalsmith-fft.h; None otherwise (e.g. on hosts that only
    carry this repository)."""
    cands = [os.environ.get("REF_DIR"), os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.exists(os.path.join(c, "signalsmith-fft.h")):
            return c
    return None


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def _bind(lib, prefix: str):
    for sfx in ("f64", "f32"):
        f = getattr(lib, f"{prefix}fft_{sfx}")
        f.argtypes = [_c_size, _c_int, _vp, _vp]
        f.restype = _c_int
        f = getattr(lib, f"{prefix}rfft_{sfx}")
        f.argtypes = [_c_size, _c_int, _c_int, _vp, _vp]
        f.restype = _c_int
        f = getattr(lib, f"{prefix}batch_{sfx}")
        f.argtypes = [_c_int, _c_int, _c_int, _c_size, _c_size, _vp, _vp, _c_int, _c_size]
        f.restype = _c_int
    for name in ("size_minimum", "size_maximum", "real_size_minimum", "real_size_maximum"):
        f = getattr(lib, f"{prefix}{name}")
        f.argtypes = [_c_size]
        f.restype = _c_size
    return lib


def lib(kind: str = "port"):
    """Load (building if needed) the ``port`` or ``reference`` shared library."""
    with _lock:
        if kind in _libs:
            return _libs[kind]
        if kind == "port":
            if not os.path.exists(PORT_SO):
                build()
            l = _bind(ctypes.CDLL(PORT_SO), "oracle_")
        elif kind == "port_native":
            # the same restatement built for speed (timing legs only; never a checker)
            if not os.path.exists(NATIVE_SO):
                build()
            l = _bind(ctypes.CDLL(NATIVE_SO), "oracle_")
        elif kind == "reference":
            if not os.path.exists(REF_SO):
                raise FileNotFoundError("oracle/_ref/libssref.so was not built (no reference checkout here)")
            l = _bind(ctypes.CDLL(REF_SO), "ref_")
        else:
            raise ValueError(kind)
        _libs[kind] = l
        return l


def _prefix(kind: str) -> str:
    return "ref_" if kind == "reference" else "oracle_"


def native_flags() -> str:
    """Compiler command line of the timing build (liboracle_native.so)."""
    r = subprocess.run(["make", "-s", "-C", HERE, "flags"], capture_output=True, text=True)
    return r.stdout.strip()


def _sfx(dtype) -> str:
    dt = np.dtype(dtype)
    if dt in (np.dtype(np.complex128), np.dtype(np.float64)):
        return "f64"
    if dt in (np.dtype(np.complex64), np.dtype(np.float32)):
        return "f32"
    raise TypeError(f"unsupported dtype {dt}")


def fft(x: np.ndarray, inverse: bool = False, kind: str = "port") -> np.ndarray:
    """Complex FFT of a 1-D complex64/complex128 array (FFT<float>/FFT<double>)."""
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    l = lib(kind)
    f = getattr(l, f"{_prefix(kind)}fft_{_sfx(x.dtype)}")
    rc = f(x.size, int(bool(inverse)), x.ctypes.data, out.ctypes.data)
    if rc:
        raise ValueError(f"oracle rejected size {x.size}")
    return out


def ifft(x: np.ndarray, kind: str = "port") -> np.ndarray:
    return fft(x, True, kind)


def rfft(x: np.ndarray, modified: bool = False, kind: str = "port") -> np.ndarray:
    """RealFFT<V>::fft (or ModifiedRealFFT): n reals -> n//2 complex."""
    x = np.ascontiguousarray(x)
    n = x.size
    cdt = np.complex128 if x.dtype == np.float64 else np.complex64
    out = np.empty(n // 2, dtype=cdt)
    l = lib(kind)
    f = getattr(l, f"{_prefix(kind)}rfft_{_sfx(x.dtype)}")
    rc = f(n, int(bool(modified)), 0, x.ctypes.data, out.ctypes.data)
    if rc:
        raise ValueError(f"oracle rejected real size {n}")
    return out


def irfft(spec: np.ndarray, n: int, modified: bool = False, kind: str = "port") -> np.ndarray:
    """RealFFT<V>::ifft: n//2 complex -> 2*(n//2) reals (unnormalised)."""
    spec = np.ascontiguousarray(spec)
    assert spec.size == n // 2
    rdt = np.float64 if spec.dtype == np.complex128 else np.float32
    out = np.empty(2 * (n // 2), dtype=rdt)
    l = lib(kind)
    f = getattr(l, f"{_prefix(kind)}rfft_{_sfx(spec.dtype)}")
    rc = f(n, int(bool(modified)), 1, spec.ctypes.data, out.ctypes.data)
    if rc:
        raise ValueError(f"oracle rejected real size {n}")
    return out


def batch(x: np.ndarray, n: int, *, real: bool, inverse: bool, modified: bool = False,
          threads: int = 1, repeats: int = 1, out: np.ndarray | None = None, kind: str = "port") -> np.ndarray:
    """Run ``repeats`` passes over a batch of independent transforms on ``threads`` host threads,
    one plan instance per thread.  ``x`` is a 2-D array [batch, per-transform elements]."""
    x = np.ascontiguousarray(x)
    b = x.shape[0]
    if real and not inverse:
        shape, dt = (b, n // 2), (np.complex128 if x.dtype == np.float64 else np.complex64)
    elif real and inverse:
        shape, dt = (b, 2 * (n // 2)), (np.float64 if x.dtype == np.complex128 else np.float32)
    else:
        shape, dt = (b, n), x.dtype
    if out is None:
        out = np.empty(shape, dtype=dt)
    l = lib(kind)
    f = getattr(l, f"{_prefix(kind)}batch_{_sfx(x.dtype)}")
    rc = f(int(real), int(modified), int(inverse), n, b, x.ctypes.data, out.ctypes.data, int(threads), int(repeats))
    if rc:
        raise RuntimeError(f"oracle batch failed rc={rc}")
    return out


def size_minimum(n: int, kind: str = "port") -> int:
    return int(getattr(lib(kind), f"{_prefix(kind)}size_minimum")(n))


def size_maximum(n: int, kind: str = "port") -> int:
    return int(getattr(lib(kind), f"{_prefix(kind)}size_maximum")(n))


def real_size_minimum(n: int, kind: str = "port") -> int:
    return int(getattr(lib(kind), f"{_prefix(kind)}real_size_minimum")(n))


def real_size_maximum(n: int, kind: str = "port") -> int:
    return int(getattr(lib(kind), f"{_prefix(kind)}real_size_maximum")(n))


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """True relative L2 error ||a-b|| / ||b|| computed in float64 (b is the reference)."""
    a = np.asarray(a).astype(np.complex128 if np.iscomplexobj(a) else np.float64).ravel()
    b = np.asarray(b).astype(np.complex128 if np.iscomplexobj(b) else np.float64).ravel()
    den = np.sqrt(np.sum(np.abs(b) ** 2))
    num = np.sqrt(np.sum(np.abs(a - b) ** 2))
    if den == 0:
        return float(num)
    return float(num / den)


def close_enough(a: np.ndarray, b: np.ndarray) -> bool:
    """The reference tests' closeness check (tests/tests-common.h:17-33):
    sqrt(sum|a-b|^2 / sum(|a^2|^2 + |b^2|^2)) < 1e-6; note the energy term is |a|^4."""
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    if a.size != b.size:
        return False
    err = np.sum(np.abs(a - b) ** 2)
    energy = np.sum(np.abs(a * a) ** 2 + np.abs(b * b) ** 2)
    if energy == 0:
        return True
    return bool(np.sqrt(err / energy) < 1e-6)

"""fft_gb300 -- Python binding of libssfft.so, the GB300 Signalsmith-FFT transform library.

The product is the C ABI in ``include/ssfft.h`` (and the C++ drop-in header
``include/signalsmith-fft.h`` on top of it).  This module binds that ABI with ctypes so tests,
benchmarks and Python callers can drive it; device buffers may come from PyTorch (any object
with ``data_ptr()``), but no PyTorch operator runs on the transform path.  If the library is
missing the import of the binding fails loudly: there is no CPU fallback.

Mirrors the reference API (signalsmith-fft.h):

* ``FFT(size, fast_direction)`` / ``RealFFT`` / ``ModifiedRealFFT`` with ``set_size``,
  ``set_size_minimum``, ``set_size_maximum``, ``size``, ``fft``, ``ifft`` -- unnormalised, out
  of place, real spectra with {DC, Nyquist} in bin 0;
* ``size_minimum`` / ``size_maximum`` (and the RealFFT variants), bit-exact with the reference.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libssfft.so")

F32, F64 = 0, 1
COMPLEX, REAL, REAL_HALFSHIFT = 0, 1, 2

STATUS = {
    0: "success", 1: "invalid size", 2: "invalid value", 3: "CUDA error", 4: "allocation failed",
    5: "unsupported", 6: "exceeds HBM budget", 7: "timed out", 8: "not ready", 9: "shut down",
}


class SsfftError(RuntimeError):
    def __init__(self, status: int, what: str = "", detail: str = ""):
        self.status = status
        msg = f"{what}: {STATUS.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


_lib = None
_lib_lock = threading.Lock()
_sz = ctypes.c_size_t
_int = ctypes.c_int
_vp = ctypes.c_void_p


class PlanOptions(ctypes.Structure):
    """ssfft_plan_options (0 = planner default)."""
    _fields_ = [("autotune", ctypes.c_int), ("cta_threads", ctypes.c_int), ("values_per_thread", ctypes.c_int),
                ("min_ctas_per_sm", ctypes.c_int), ("radices", ctypes.c_int * 24), ("precision", ctypes.c_int),
                ("prefetch_quarter_waves", ctypes.c_int), ("fuse_split", ctypes.c_int),
                ("cluster_split", ctypes.c_int), ("staging", ctypes.c_int)]


PRECISION = {"fp32": 0, "split_bf16": 1}


def _options(autotune=0, radices=None, cta_threads=0, values_per_thread=0, min_ctas_per_sm=0, precision="fp32",
             prefetch_quarter_waves=0, fuse_split=0, cluster_split=0, staging=0):
    o = PlanOptions()
    o.staging = int(staging)
    o.prefetch_quarter_waves = int(prefetch_quarter_waves)
    o.fuse_split = int(fuse_split)
    o.cluster_split = int(cluster_split)
    o.autotune, o.cta_threads = int(autotune), int(cta_threads)
    o.values_per_thread, o.min_ctas_per_sm = int(values_per_thread), int(min_ctas_per_sm)
    for i, r in enumerate(radices or []):
        o.radices[i] = int(r)
    o.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
    return o


def schedule_options(**opts) -> None:
    """Options (as for Plan) that schedule_info / schedule_name / schedule_tables / jit_check
    apply in this thread; no arguments restores the planner defaults."""
    if opts:
        o = _options(**opts)
        check(lib().ssfft_schedule_options(ctypes.byref(o)), "schedule_options")
    else:
        check(lib().ssfft_schedule_options(None), "schedule_options")


def schedule_direction(inverse: bool) -> None:
    """Direction whose schedule schedule_info / schedule_tables report in this thread."""
    check(lib().ssfft_schedule_direction(int(bool(inverse))), "schedule_direction")


def diag_tc_tile(a: np.ndarray, bt: np.ndarray) -> tuple:
    """D = A B for one 128 x 32 x 32 FP32 tile through the split-BF16 tensor-core path (GPU).
    ``bt`` is B transposed.  Returns (D, error flag)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    bt = np.ascontiguousarray(bt, dtype=np.float32)
    assert a.shape == (128, 32) and bt.shape == (32, 32)
    d = np.zeros((128, 32), dtype=np.float32)
    flags = ctypes.c_uint(0)
    check(lib().ssfft_diag_tc_tile(_vp(a.ctypes.data), _vp(bt.ctypes.data), _vp(d.ctypes.data), ctypes.byref(flags)),
          "diag_tc_tile")
    return d, flags.value


def _declare(l):
    l.ssfft_status_string.argtypes = [_int]
    l.ssfft_status_string.restype = ctypes.c_char_p
    l.ssfft_last_cuda_error.restype = ctypes.c_char_p
    for name in ("ssfft_size_minimum", "ssfft_size_maximum", "ssfft_real_size_minimum", "ssfft_real_size_maximum",
                 "ssfft_size_minimum_smooth", "ssfft_size_maximum_smooth", "ssfft_real_size_minimum_smooth",
                 "ssfft_real_size_maximum_smooth"):
        getattr(l, name).argtypes = [_sz]
        getattr(l, name).restype = _sz
    l.ssfft_plans_created.argtypes = []
    l.ssfft_plans_created.restype = _sz
    l.ssfft_plan_create.argtypes = [ctypes.POINTER(_vp), _sz, _int, _int, _sz]
    l.ssfft_plan_destroy.argtypes = [_vp]
    l.ssfft_plan_create_ex.argtypes = [ctypes.POINTER(_vp), _sz, _int, _int, _sz, ctypes.POINTER(PlanOptions)]
    l.ssfft_plan_tuning.argtypes = [_vp, ctypes.c_char_p, _sz, ctypes.c_char_p, _sz]
    l.ssfft_plan_size.argtypes = [_vp]
    l.ssfft_plan_size.restype = _sz
    l.ssfft_plan_batch.argtypes = [_vp]
    l.ssfft_plan_batch.restype = _sz
    l.ssfft_plan_device_bytes.argtypes = [_vp]
    l.ssfft_plan_device_bytes.restype = _sz
    l.ssfft_plan_describe.argtypes = [_vp, ctypes.POINTER(_int), ctypes.POINTER(_int), _int, ctypes.POINTER(_int),
                                      ctypes.POINTER(_int), ctypes.POINTER(_int)]
    l.ssfft_plan_kernel.argtypes = [_vp, _int, ctypes.c_char_p, _sz]
    l.ssfft_exec.argtypes = [_vp, _int, _vp, _vp, _vp]
    l.ssfft_exec_batch.argtypes = [_vp, _int, _vp, _vp, _sz, _vp]
    l.ssfft_exec_host.argtypes = [_vp, _int, _vp, _vp]
    l.ssfft_plan_error.argtypes = [_vp, ctypes.POINTER(ctypes.c_uint)]
    l.ssfft_jit_check.argtypes = [_sz, _int, _int, _sz, ctypes.c_char_p, ctypes.POINTER(_sz)]
    l.ssfft_schedule_info.argtypes = [_sz, _int, _int, _sz, ctypes.POINTER(_int), _int, ctypes.POINTER(_int),
                                      ctypes.POINTER(_int), ctypes.POINTER(_int), ctypes.POINTER(_sz)]
    l.ssfft_schedule_name.argtypes = [_sz, _int, _int, _sz, _int, ctypes.c_char_p, _sz]
    dp = ctypes.POINTER(ctypes.c_double)
    szp = ctypes.POINTER(_sz)
    l.ssfft_schedule_tables.argtypes = [_sz, _int, _int, _sz, dp, szp, dp, szp, dp, szp, dp, szp]
    l.ssfft_diag_staged_timeout.argtypes = [_sz, ctypes.c_uint, ctypes.POINTER(ctypes.c_uint)]
    l.ssfft_schedule_options.argtypes = [ctypes.POINTER(PlanOptions)]
    l.ssfft_schedule_direction.argtypes = [_int]
    l.ssfft_diag_tc_tile.argtypes = [_vp, _vp, _vp, ctypes.POINTER(ctypes.c_uint)]
    for name in ("ssfft_plan_create", "ssfft_plan_create_ex", "ssfft_plan_tuning", "ssfft_plan_destroy", "ssfft_plan_describe",
                 "ssfft_plan_kernel", "ssfft_exec", "ssfft_exec_batch",
                 "ssfft_exec_host", "ssfft_plan_error", "ssfft_diag_staged_timeout", "ssfft_schedule_options", "ssfft_schedule_direction",
                 "ssfft_diag_tc_tile", "ssfft_jit_check", "ssfft_schedule_info", "ssfft_schedule_name",
                 "ssfft_schedule_tables"):
        getattr(l, name).restype = _int
    return l


def lib():
    """The loaded libssfft.so (raises if it was not built -- there is no fallback)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: run `python -m fft_gb300.build` (no CPU fallback exists)")
            _lib = _declare(ctypes.CDLL(LIB_PATH))
        return _lib


def check(status: int, what: str = "ssfft") -> None:
    if status != 0:
        detail = lib().ssfft_last_cuda_error().decode(errors="replace") if status == 3 else ""
        raise SsfftError(status, what, detail)


def _dtype_code(dtype) -> int:
    if dtype in ("f32", "float32", np.float32, np.complex64, F32):
        return F32
    if dtype in ("f64", "float64", np.float64, np.complex128, F64):
        return F64
    s = str(dtype)
    if "float32" in s or "complex64" in s:
        return F32
    if "float64" in s or "complex128" in s:
        return F64
    raise TypeError(f"unsupported dtype {dtype}")


def _kind_code(kind) -> int:
    if kind in ("complex", "c2c", COMPLEX):
        return COMPLEX
    if kind in ("real", "r2c", REAL):
        return REAL
    if kind in ("real_halfshift", "halfshift", "modified", REAL_HALFSHIFT):
        return REAL_HALFSHIFT
    raise ValueError(f"unknown kind {kind}")


# ------------------------------------------------------------------ size helpers

def size_minimum(n: int) -> int:
    """FFT<V>::sizeMinimum (signalsmith-fft.h:327-337)."""
    return int(lib().ssfft_size_minimum(n))


def size_maximum(n: int) -> int:
    """FFT<V>::sizeMaximum (signalsmith-fft.h:338-348)."""
    return int(lib().ssfft_size_maximum(n))


def real_size_minimum(n: int) -> int:
    """RealFFT<V>::sizeMinimum (signalsmith-fft.h:403-405)."""
    return int(lib().ssfft_real_size_minimum(n))


def real_size_maximum(n: int) -> int:
    """RealFFT<V>::sizeMaximum (signalsmith-fft.h:406-408)."""
    return int(lib().ssfft_real_size_maximum(n))


def size_minimum_smooth(n: int) -> int:
    """Smallest 2^a 3^b 5^c >= n (opt-in; the reference's sizeMinimum never picks a 5)."""
    return int(lib().ssfft_size_minimum_smooth(n))


def size_maximum_smooth(n: int) -> int:
    """Largest 2^a 3^b 5^c <= n (opt-in; the reference's sizeMaximum never picks a 5)."""
    return int(lib().ssfft_size_maximum_smooth(n))


def real_size_minimum_smooth(n: int) -> int:
    """Smallest even m >= n whose half is 2^a 3^b 5^c."""
    return int(lib().ssfft_real_size_minimum_smooth(n))


def real_size_maximum_smooth(n: int) -> int:
    """Largest even m <= n whose half is 2^a 3^b 5^c (0 when n < 2)."""
    return int(lib().ssfft_real_size_maximum_smooth(n))


def plans_created() -> int:
    """Plans this process has created so far (monotonic)."""
    return int(lib().ssfft_plans_created())


def schedule_info(n: int, dtype="f32", kind="complex", batch: int = 1) -> dict:
    """The single-CTA schedule the planner picks for (n, dtype, kind, batch), without a GPU."""
    rad = (_int * 32)()
    np_, th, pc = _int(), _int(), _int()
    smem = _sz()
    check(lib().ssfft_schedule_info(n, _dtype_code(dtype), _kind_code(kind), batch, rad, 32, ctypes.byref(np_),
                                    ctypes.byref(th), ctypes.byref(pc), ctypes.byref(smem)), "schedule_info")
    return {"radices": list(rad[:np_.value]), "threads": th.value, "per_cta": pc.value, "smem_bytes": smem.value}


def schedule_name(n: int, dtype="f32", kind="complex", batch: int = 1, inverse: bool = False) -> str:
    """The kernel template instantiation a single-CTA plan runs."""
    buf = ctypes.create_string_buffer(1024)
    check(lib().ssfft_schedule_name(n, _dtype_code(dtype), _kind_code(kind), batch, int(bool(inverse)), buf, 1024),
          "schedule_name")
    return buf.value.decode()


def schedule_tables(n: int, dtype="f32", kind="complex", batch: int = 1) -> dict:
    """FP64 tables (pass twiddles, direct-pass roots, real split twiddles, half-shift rotations)
    of a single-CTA plan, as interleaved re/im float64 arrays."""
    cnt = [_sz() for _ in range(4)]
    null = ctypes.POINTER(ctypes.c_double)()
    args = []
    for c in cnt:
        args += [null, ctypes.byref(c)]
    check(lib().ssfft_schedule_tables(n, _dtype_code(dtype), _kind_code(kind), batch, *args), "schedule_tables")
    arrs = [np.zeros(c.value, dtype=np.float64) for c in cnt]
    args = []
    for a, c in zip(arrs, cnt):
        args += [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(c)]
    check(lib().ssfft_schedule_tables(n, _dtype_code(dtype), _kind_code(kind), batch, *args), "schedule_tables")
    return dict(zip(("tw", "roots", "rtw", "rot"), arrs))


def diag_staged_timeout(n: int = 1024, spin_limit: int = 1000) -> int:
    """Run the staged kernel once with a lost input copy (GPU); returns the error flag it raised."""
    flags = ctypes.c_uint(0)
    check(lib().ssfft_diag_staged_timeout(n, spin_limit, ctypes.byref(flags)), "ssfft_diag_staged_timeout")
    return flags.value


def large_spec(n: int, dtype="f32", kind="complex") -> tuple:
    """The multi-pass plan of n points (no GPU): (launch records as a dict, table bytes)."""
    import json as _json
    nb = _sz()
    l = lib()
    l.ssfft_diag_large_spec.argtypes = [_sz, _int, _int, ctypes.c_char_p, _sz, _vp, ctypes.POINTER(_sz)]
    l.ssfft_diag_large_spec.restype = _int
    buf = ctypes.create_string_buffer(1 << 16)
    check(l.ssfft_diag_large_spec(n, _dtype_code(dtype), _kind_code(kind), buf, 1 << 16, None, ctypes.byref(nb)),
          f"large_spec(n={n})")
    blob = (ctypes.c_ubyte * nb.value)()
    check(l.ssfft_diag_large_spec(n, _dtype_code(dtype), _kind_code(kind), None, 0, ctypes.cast(blob, _vp),
                                  ctypes.byref(nb)), f"large_spec(n={n})")
    return _json.loads(buf.value.decode()), bytes(blob)


def jit_check(n: int, dtype="f32", kind="complex", batch: int = 1, arch: str = "sm_103a") -> int:
    """Compile (no GPU needed) the kernels a plan would use; returns the cubin size."""
    nbytes = _sz()
    check(lib().ssfft_jit_check(n, _dtype_code(dtype), _kind_code(kind), batch, arch.encode(), ctypes.byref(nbytes)),
          f"jit_check(n={n})")
    return nbytes.value


# ------------------------------------------------------------------ plans

class Plan:
    """One ``ssfft_plan_t``: ``batch`` transforms of size ``n`` (complex or real).

    Keyword options map onto ``ssfft_plan_options`` (0 = planner default): ``autotune`` (1, 2),
    ``radices`` (explicit pass order), ``cta_threads``, ``values_per_thread``,
    ``min_ctas_per_sm`` (register cap), ``precision`` ("fp32" / "split_bf16"),
    ``prefetch_quarter_waves``, ``fuse_split`` (1 / -1), ``cluster_split`` (-1 never, k > 0
    with ``radices``: the first k radices as the first phase of the two-CTA cluster kernel) and
    ``staging`` (bulk-copy input staging: -1 never, 1 wherever the input fits)."""

    def __init__(self, n: int, dtype="f32", kind="complex", batch: int = 1, *, autotune: int = 0, radices=None,
                 cta_threads: int = 0, values_per_thread: int = 0, min_ctas_per_sm: int = 0, precision="fp32",
                 prefetch_quarter_waves: int = 0, fuse_split: int = 0, cluster_split: int = 0, staging: int = 0):
        self.n = int(n)
        self.dtype = _dtype_code(dtype)
        self.kind = _kind_code(kind)
        self.batch = max(1, int(batch))
        h = _vp()
        opt = _options(autotune, radices, cta_threads, values_per_thread, min_ctas_per_sm, precision,
                       prefetch_quarter_waves, fuse_split, cluster_split, staging)
        check(lib().ssfft_plan_create_ex(ctypes.byref(h), self.n, self.dtype, self.kind, self.batch,
                                         ctypes.byref(opt)),
              f"plan_create(n={n}, kind={kind}, batch={batch})")
        self._h = h

    def tuning(self) -> dict:
        """Schedule options in force and the autotuner's candidate timings (if it ran)."""
        a = ctypes.create_string_buffer(256)
        b = ctypes.create_string_buffer(16384)
        check(lib().ssfft_plan_tuning(self._h, a, 256, b, 16384), "plan_tuning")
        return {"choice": a.value.decode(), "log": [x for x in b.value.decode().splitlines() if x]}

    def kernel(self, inverse: bool = False) -> str:
        """Kernel template the plan launches ("multi-pass" beyond one CTA)."""
        b = ctypes.create_string_buffer(1024)
        check(lib().ssfft_plan_kernel(self._h, int(bool(inverse)), b, 1024), "plan_kernel")
        return b.value.decode()

    @property
    def handle(self):
        return self._h

    def destroy(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().ssfft_plan_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def describe(self) -> dict:
        np_, th, pc, nl = _int(), _int(), _int(), _int()
        rad = (_int * 32)()
        check(lib().ssfft_plan_describe(self._h, ctypes.byref(np_), rad, 32, ctypes.byref(th), ctypes.byref(pc),
                                        ctypes.byref(nl)), "plan_describe")
        return {"radices": list(rad[:np_.value]), "threads": th.value, "per_cta": pc.value, "launches": nl.value,
                "device_bytes": int(lib().ssfft_plan_device_bytes(self._h))}

    def exec(self, inverse: bool, d_in: int, d_out: int, stream: int = 0, batch: int | None = None) -> None:
        """Run on device pointers (ints), asynchronously on ``stream`` (a cudaStream_t value)."""
        b = self.batch if batch is None else int(batch)
        check(lib().ssfft_exec_batch(self._h, int(bool(inverse)), _vp(d_in), _vp(d_out), b, _vp(stream)), "exec")

    def exec_host(self, inverse: bool, h_in: np.ndarray, h_out: np.ndarray) -> None:
        """Run on host arrays (synchronous; copies overlap with compute inside the library)."""
        assert h_in.flags.c_contiguous and h_out.flags.c_contiguous
        check(lib().ssfft_exec_host(self._h, int(bool(inverse)), _vp(h_in.ctypes.data), _vp(h_out.ctypes.data)),
              "exec_host")

    def in_elems(self, inverse: bool) -> int:
        """Scalars of the input of one transform."""
        if self.kind == COMPLEX:
            return 2 * self.n
        return 2 * (self.n // 2) if inverse else self.n

    def out_elems(self, inverse: bool) -> int:
        if self.kind == COMPLEX:
            return 2 * self.n
        return self.n if inverse else 2 * (self.n // 2)


_plan_cache: dict = {}
_plan_cache_lock = threading.Lock()


def get_plan(n: int, dtype="f32", kind="complex", batch: int = 1) -> Plan:
    key = (int(n), _dtype_code(dtype), _kind_code(kind), int(batch))
    with _plan_cache_lock:
        p = _plan_cache.get(key)
        if p is None:
            p = Plan(n, dtype, kind, batch)
            _plan_cache[key] = p
        return p


def clear_plan_cache() -> None:
    with _plan_cache_lock:
        for p in _plan_cache.values():
            p.destroy()
        _plan_cache.clear()


# ------------------------------------------------------------------ torch-tensor helpers

def _torch():
    import torch
    return torch


def _stream_handle(stream=None) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def fft(x, inverse: bool = False, out=None, stream=None):
    """Complex FFT over the last dimension of a CUDA complex64/complex128 tensor (unnormalised)."""
    torch = _torch()
    assert x.is_cuda and x.dtype in (torch.complex64, torch.complex128)
    x = x.contiguous()
    n = x.shape[-1]
    batch = x.numel() // n if n else 0
    if out is None:
        out = torch.empty_like(x)
    if batch == 0:
        return out
    p = get_plan(n, "f32" if x.dtype == torch.complex64 else "f64", "complex", batch)
    p.exec(inverse, x.data_ptr(), out.data_ptr(), _stream_handle(stream), batch)
    return out


def ifft(x, out=None, stream=None):
    return fft(x, True, out, stream)


def rfft(x, modified: bool = False, out=None, stream=None):
    """RealFFT<V>::fft over the last dimension: n reals -> n//2 complex (bin 0 = {DC, Nyquist})."""
    torch = _torch()
    assert x.is_cuda and x.dtype in (torch.float32, torch.float64)
    x = x.contiguous()
    n = x.shape[-1]
    batch = x.numel() // n
    cdt = torch.complex64 if x.dtype == torch.float32 else torch.complex128
    if out is None:
        out = torch.empty(*x.shape[:-1], n // 2, dtype=cdt, device=x.device)
    p = get_plan(n, "f32" if x.dtype == torch.float32 else "f64", "real_halfshift" if modified else "real", batch)
    p.exec(False, x.data_ptr(), out.data_ptr(), _stream_handle(stream), batch)
    return out


def irfft(spec, n: int, modified: bool = False, out=None, stream=None):
    """RealFFT<V>::ifft: n//2 complex -> 2*(n//2) reals (unnormalised)."""
    torch = _torch()
    assert spec.is_cuda and spec.dtype in (torch.complex64, torch.complex128)
    spec = spec.contiguous()
    assert spec.shape[-1] == n // 2
    batch = spec.numel() // (n // 2)
    rdt = torch.float32 if spec.dtype == torch.complex64 else torch.float64
    if out is None:
        out = torch.empty(*spec.shape[:-1], n, dtype=rdt, device=spec.device)
    p = get_plan(n, "f32" if rdt == torch.float32 else "f64", "real_halfshift" if modified else "real", batch)
    p.exec(True, spec.data_ptr(), out.data_ptr(), _stream_handle(stream), batch)
    return out


# ------------------------------------------------------------------ reference-shaped API

class FFT:
    """signalsmith::FFT<V> (signalsmith-fft.h:69-387) on the GPU.

    ``fft``/``ifft`` accept CUDA tensors (device path) or numpy arrays (host path through
    ``ssfft_exec_host``); both are out of place and unnormalised like the reference."""

    _dtype = "f32"

    def __init__(self, size: int, fast_direction: int = 0, dtype="f32"):
        self._dtype = dtype
        self._size = 0
        self._plan = None
        if fast_direction > 0:
            size = size_minimum(size)
        elif fast_direction < 0:
            size = size_maximum(size)
        self.set_size(size)

    sizeMinimum = staticmethod(size_minimum)
    sizeMaximum = staticmethod(size_maximum)
    sizeMinimumSmooth = staticmethod(size_minimum_smooth)
    sizeMaximumSmooth = staticmethod(size_maximum_smooth)

    def set_size(self, size: int) -> int:
        if size != self._size:
            self._size = int(size)
            self._plan = Plan(self._size, self._dtype, "complex", 1) if size else None
        return self._size

    def set_size_minimum(self, size: int) -> int:
        return self.set_size(size_minimum(size))

    def set_size_maximum(self, size: int) -> int:
        return self.set_size(size_maximum(size))

    def size(self) -> int:
        return self._size

    def _run(self, x, out, inverse: bool):
        if isinstance(x, np.ndarray):
            cdt = np.complex64 if _dtype_code(self._dtype) == F32 else np.complex128
            xin = np.ascontiguousarray(x, dtype=cdt)
            res = np.empty_like(xin) if out is None else out
            self._plan.exec_host(inverse, xin, res)
            return res
        return fft(x, inverse, out)

    def fft(self, x, out=None):
        return self._run(x, out, False)

    def ifft(self, x, out=None):
        return self._run(x, out, True)


class RealFFT:
    """signalsmith::RealFFT<V> (signalsmith-fft.h:393-503) on the GPU."""

    modified = False

    def __init__(self, size: int, fast_direction: int = 0, dtype="f32"):
        self._dtype = dtype
        self._n = 0
        self._plan = None
        if fast_direction > 0:
            size = real_size_minimum(size)
        elif fast_direction < 0:
            size = real_size_maximum(size)
        self.set_size(size)

    sizeMinimum = staticmethod(real_size_minimum)
    sizeMaximum = staticmethod(real_size_maximum)
    sizeMinimumSmooth = staticmethod(real_size_minimum_smooth)
    sizeMaximumSmooth = staticmethod(real_size_maximum_smooth)

    def set_size(self, size: int) -> int:
        """Returns the complex half size, size // 2, as the reference's RealFFT::setSize does
        (``return complexFft.setSize(size/2)``, signalsmith-fft.h:434); an unchanged size keeps
        the plan."""
        size = int(size)
        if size != self._n or self._plan is None:
            self._n = size
            kind = "real_halfshift" if self.modified else "real"
            self._plan = Plan(self._n, self._dtype, kind, 1) if size // 2 else None
        return self._n // 2

    def set_size_minimum(self, size: int) -> int:
        return self.set_size(real_size_minimum(size))

    def set_size_maximum(self, size: int) -> int:
        return self.set_size(real_size_maximum(size))

    def size(self) -> int:
        return 2 * (self._n // 2)

    def fft(self, x, out=None):
        if isinstance(x, np.ndarray):
            rdt = np.float32 if _dtype_code(self._dtype) == F32 else np.float64
            cdt = np.complex64 if rdt == np.float32 else np.complex128
            xin = np.ascontiguousarray(x, dtype=rdt)
            res = np.empty(self._n // 2, dtype=cdt) if out is None else out
            self._plan.exec_host(False, xin, res)
            return res
        return rfft(x, self.modified, out)

    def ifft(self, spec, out=None):
        if isinstance(spec, np.ndarray):
            cdt = np.complex64 if _dtype_code(self._dtype) == F32 else np.complex128
            rdt = np.float32 if cdt == np.complex64 else np.float64
            sin = np.ascontiguousarray(spec, dtype=cdt)
            res = np.empty(self._n, dtype=rdt) if out is None else out
            self._plan.exec_host(True, sin, res)
            return res
        return irfft(spec, self._n, self.modified, out)


class ModifiedRealFFT(RealFFT):
    """signalsmith::ModifiedRealFFT<V> (signalsmith-fft.h:505-508): bins at k + 1/2."""

    modified = True


# ------------------------------------------------------------------ serving

class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_waves_in_flight", ctypes.c_int),
                ("max_requests_per_wave", ctypes.c_int), ("coalesce", ctypes.c_int)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("dtype", ctypes.c_int), ("inverse", ctypes.c_int), ("n", ctypes.c_size_t),
                ("frames", ctypes.c_size_t), ("h_in", ctypes.c_void_p), ("h_out", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("waves", ctypes.c_uint64), ("launches", ctypes.c_uint64), ("p50_latency_us", ctypes.c_double),
                ("p99_latency_us", ctypes.c_double), ("mean_latency_us", ctypes.c_double),
                ("max_latency_us", ctypes.c_double), ("span_seconds", ctypes.c_double), ("frames", ctypes.c_double),
                ("flops", ctypes.c_double), ("in_place", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class LoadgenConfig(ctypes.Structure):
    _fields_ = [("offered_rate", ctypes.c_double), ("duration_s", ctypes.c_double), ("seed", ctypes.c_uint64),
                ("n_min", ctypes.c_size_t), ("n_max", ctypes.c_size_t), ("max_frames", ctypes.c_int),
                ("real_fraction", ctypes.c_double)]


def _declare_server(l):
    if getattr(l, "_server_declared", False):
        return l
    l.ssfft_server_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(ServerConfig)]
    l.ssfft_server_prepare.argtypes = [_vp, _sz, _int, _int]
    l.ssfft_server_submit.argtypes = [_vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]
    l.ssfft_server_wait.argtypes = [_vp, ctypes.c_uint64, ctypes.c_double]
    l.ssfft_server_drain.argtypes = [_vp, ctypes.c_double]
    l.ssfft_server_get_stats.argtypes = [_vp, ctypes.POINTER(ServerStats), _int]
    l.ssfft_server_destroy.argtypes = [_vp]
    l.ssfft_server_loadgen.argtypes = [_vp, ctypes.POINTER(LoadgenConfig), ctypes.POINTER(ServerStats)]
    for name in ("ssfft_server_create", "ssfft_server_prepare", "ssfft_server_submit", "ssfft_server_wait",
                 "ssfft_server_drain", "ssfft_server_get_stats", "ssfft_server_destroy", "ssfft_server_loadgen"):
        getattr(l, name).restype = _int
    l._server_declared = True
    return l


class Server:
    """Continuous-batching request server (ssfft_server_* in include/ssfft.h)."""

    def __init__(self, hbm_budget_bytes: int = 1 << 30, waves: int = 8, max_requests_per_wave: int = 256,
                 coalesce: bool = True):
        l = _declare_server(lib())
        cfg = ServerConfig(hbm_budget_bytes, waves, max_requests_per_wave, int(bool(coalesce)))
        h = _vp()
        check(l.ssfft_server_create(ctypes.byref(h), ctypes.byref(cfg)), "server_create")
        self._h = h
        self._keep = {}

    def prepare(self, n: int, dtype="f32", kind="complex") -> None:
        check(lib().ssfft_server_prepare(self._h, n, _dtype_code(dtype), _kind_code(kind)), "server_prepare")

    def submit(self, n: int, kind, inverse: bool, h_in: np.ndarray, h_out: np.ndarray, frames: int = 1,
               dtype="f32") -> int:
        """Queue a request on host arrays (kept alive until the request completes)."""
        r = Request(_kind_code(kind), _dtype_code(dtype), int(bool(inverse)), n, frames, h_in.ctypes.data,
                    h_out.ctypes.data)
        t = ctypes.c_uint64()
        check(lib().ssfft_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)), "server_submit")
        self._keep[t.value] = (h_in, h_out)
        return t.value

    def wait(self, ticket: int, timeout: float = 60.0) -> None:
        check(lib().ssfft_server_wait(self._h, ticket, timeout), "server_wait")
        self._keep.pop(ticket, None)

    def drain(self, timeout: float = 600.0) -> None:
        check(lib().ssfft_server_drain(self._h, timeout), "server_drain")
        self._keep.clear()

    def stats(self, reset: bool = False) -> dict:
        st = ServerStats()
        check(lib().ssfft_server_get_stats(self._h, ctypes.byref(st), int(reset)), "server_stats")
        return st.as_dict()

    def loadgen(self, offered_rate: float, duration_s: float, seed: int = 1, n_min: int = 256, n_max: int = 65536,
                max_frames: int = 64, real_fraction: float = 0.7) -> dict:
        cfg = LoadgenConfig(offered_rate, duration_s, seed, n_min, n_max, max_frames, real_fraction)
        st = ServerStats()
        check(lib().ssfft_server_loadgen(self._h, ctypes.byref(cfg), ctypes.byref(st)), "server_loadgen")
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().ssfft_server_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ uneven-size batches

def fast_sizes(lo: int, hi: int) -> list:
    """The 2^a 3^b 5^c sizes in [lo, hi], ascending."""
    out = []
    a = 1
    while a <= hi:
        b = a
        while b <= hi:
            c = b
            while c <= hi:
                if c >= lo:
                    out.append(c)
                c *= 5
            b *= 3
        a *= 2
    return sorted(out)


class Multi:
    """ssfft_multi_*: one submission of complex transforms of uneven sizes stored back to back
    (a CUDA graph of work-item queue kernels, one per class of CTA shapes)."""

    def __init__(self, sizes, dtype="f32", autotune: int = 0, precision="fp32"):
        l = lib()
        if not getattr(l, "_multi_declared", False):
            l.ssfft_multi_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(_sz), _sz, _int]
            l.ssfft_multi_create_ex.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(_sz), _sz, _int,
                                                ctypes.POINTER(PlanOptions)]
            l.ssfft_multi_exec.argtypes = [_vp, _int, _vp, _vp, _vp]
            l.ssfft_multi_exec_plain.argtypes = [_vp, _int, _vp, _vp, _vp]
            l.ssfft_multi_info.argtypes = [_vp, ctypes.POINTER(_sz), ctypes.POINTER(_sz)]
            l.ssfft_multi_launches.argtypes = [_vp]
            l.ssfft_multi_launches.restype = _sz
            l.ssfft_multi_destroy.argtypes = [_vp]
            for name in ("ssfft_multi_create", "ssfft_multi_create_ex", "ssfft_multi_exec", "ssfft_multi_exec_plain", "ssfft_multi_info",
                         "ssfft_multi_destroy"):
                getattr(l, name).restype = _int
            l._multi_declared = True
        self.sizes = [int(n) for n in sizes]
        arr = (_sz * len(self.sizes))(*self.sizes)
        h = _vp()
        opt = _options(autotune, precision=precision)
        check(l.ssfft_multi_create_ex(ctypes.byref(h), arr, len(self.sizes), _dtype_code(dtype), ctypes.byref(opt)),
              "multi_create")
        self._h = h

    def exec(self, inverse: bool, d_in: int, d_out: int, stream: int = 0) -> None:
        check(lib().ssfft_multi_exec(self._h, int(bool(inverse)), _vp(d_in), _vp(d_out), _vp(stream)), "multi_exec")

    def exec_plain(self, inverse: bool, d_in: int, d_out: int, stream: int = 0) -> None:
        check(lib().ssfft_multi_exec_plain(self._h, int(bool(inverse)), _vp(d_in), _vp(d_out), _vp(stream)),
              "multi_exec_plain")

    def info(self) -> dict:
        a, b = _sz(), _sz()
        check(lib().ssfft_multi_info(self._h, ctypes.byref(a), ctypes.byref(b)), "multi_info")
        return {"distinct_sizes": a.value, "total_elements": b.value,
                "launches": int(lib().ssfft_multi_launches(self._h))}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().ssfft_multi_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

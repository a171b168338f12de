"""Run the transform path beyond one CTA -- the multi-pass (four-step) pass kernels
(ssfft_cl::strided), the RealFFT split kernel and Bluestein's element-wise kernels, the exact
source in fft_gb300/csrc/ssfft_codelets.cuh -- on the CPU through the CUDA emulation shim in
tests/emu/, with the launch records and table bytes libssfft.so's planner produces
(ssfft_diag_large_spec), launch by launch in the library's order, and compare with the oracle.
This checks the passes' strides, segment loads and stores, inter-pass twiddles, the split and
pre-twiddle, Bluestein's chirp tables and its composition with the M-point plans, and the inverse
conjugations without a GPU; test_gpu_large.py repeats the comparisons on the device."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import fft_gb300 as F
import oracle
from conftest import ROOT, rel_l2

# (n, dtype, kind, transforms): two passes (FP32 above 16384 points, FP64 above 8192) and three
# passes; RealFFT lengths add the split kernel (and the half-shift rotations); lengths with a
# prime factor above 1024 run Bluestein's algorithm over multi-pass M-point plans
CASES = [(20000, "f32", "complex", 2), (32768, "f32", "complex", 1), (10000, "f64", "complex", 2),
         (1 << 21, "f32", "complex", 1), (2 * 3 ** 9, "f32", "complex", 1), (40000, "f32", "real", 2),
         (40000, "f32", "real_halfshift", 1), (20000, "f64", "real", 1), (20000, "f64", "real_halfshift", 1),
         (17527, "f32", "complex", 1), (10007, "f64", "complex", 1), (35054, "f32", "real", 1),
         (20014, "f64", "real", 1),
         # the reference accepts every length: odd real lengths beyond one CTA (packed rows, the
         # last real neither read nor written) and half-shift lengths that need Bluestein
         (40001, "f32", "real", 3), (40001, "f32", "real_halfshift", 2), (20003, "f64", "real", 2),
         (35054, "f32", "real_halfshift", 1), (35055, "f32", "real", 2), (20014, "f64", "real_halfshift", 1)]


class Emu:
    """The emulator binary, its case tables and the planner's records of every case."""

    def __init__(self, d):
        self.d, self.passes, self.splits, self.blues, self.packs, self.specs = d, [], [], [], [], {}

    def add_plan(self, n, dt, kind):
        key = (n, dt, kind)
        if key in self.specs:
            return self.specs[key]
        spec, blob = F.large_spec(n, dt, kind)
        rec = {"spec": spec, "blob": blob, "pass0": len(self.passes), "split0": len(self.splits),
               "blue0": len(self.blues), "pack0": len(self.packs)}
        for p in spec["passes"]:
            for k in ("fwd", "inv"):
                self.passes.append(f'{{"{n}-{dt}-{k}", &{p[k]}, {p["cta"]}, {p["smem"]}}},')
        if spec["real"]:
            self.splits += [f'{{"{n}-{dt}-{kind}-fwd", &{spec["split_fwd"]}}},',
                            f'{{"{n}-{dt}-{kind}-inv", &{spec["split_inv"]}}},']
        if "M" in spec:
            self.blues += [f'{{"{n}-{dt}-blue{i}", &{name}}},' for i, name in enumerate(spec["blue"])]
        if spec.get("odd"):
            self.packs += [f'{{"{n}-{dt}-pack", &{spec["pack"]}}},', f'{{"{n}-{dt}-unpack", &{spec["unpack"]}}},']
        self.specs[key] = rec
        if "M" in spec:
            rec["inner"] = self.add_plan(spec["M"], dt, "complex")
        return rec

    def build(self):
        for name, lines in (("emu_strided_cases.inc", self.passes), ("emu_split_cases.inc", self.splits),
                            ("emu_blue_cases.inc", self.blues), ("emu_pack_cases.inc", self.packs)):
            (self.d / name).write_text("\n".join(lines) + "\n")
        self.exe = self.d / "emu_strided"
        cmd = ["g++", "-std=c++20", "-O2", "-pthread", "-w", "-I", str(self.d), "-I",
               os.path.join(ROOT, "tests", "emu"), "-I", os.path.join(ROOT, "fft_gb300", "csrc"),
               os.path.join(ROOT, "tests", "emu", "emu_strided_main.cpp"), "-o", str(self.exe)]
        subprocess.run(cmd, check=True)

    def run(self, args):
        subprocess.run([str(self.exe)] + [str(a) for a in args], check=True, timeout=600)

    def file(self, name, data):
        f = self.d / name
        f.write_bytes(data.tobytes() if hasattr(data, "tobytes") else bytes(data))
        return f


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    e = Emu(tmp_path_factory.mktemp("emu_strided"))
    for n, dt, kind, _ in CASES:
        e.add_plan(n, dt, kind)
    e.build()
    return e


def _sdt(dt):
    return np.float32 if dt == "f32" else np.float64


def _passes(e, rec, cur, nb, inverse, table):
    """The multi-pass launches of `rec` over nb transforms (flat scalars in, flat scalars out)."""
    spec = rec["spec"]
    N = spec["N"]
    for i, p in enumerate(spec["passes"]):
        fi, fo = e.file("pin", cur), e.file("pout", np.full_like(cur, np.nan))
        grid = nb * p["U1"] * (-(-p["U0"] // p["G"]))
        e.run([f"p{rec['pass0'] + 2 * i + int(inverse)}", grid, fi, fo, table, nb, N, p["U0"], p["U1"], p["is0"],
               p["is1"], p["in_es"], p["os0"], p["os1"], p["out_es"], p["off_tw"], p["off_roots"], p["off_twlo"],
               p["off_twhi"], spec["off_rot"]])
        cur = np.frombuffer(fo.read_bytes(), dtype=cur.dtype).copy()
    return cur


def _split(e, rec, inverse, src, buf, nb, table):
    N = rec["spec"]["N"]
    fi, fo = e.file("sin", src), e.file("sbuf", buf)
    e.run([f"s{rec['split0'] + int(inverse)}", -(-(N // 2 + 1) // 256), fi, fo, table, nb, N, rec["spec"]["off_rtw"]])
    return np.frombuffer(fo.read_bytes(), dtype=buf.dtype).copy()


def _pack(e, rec, src, dst, nb, n, unpack):
    """Odd real lengths: rows of n reals to rows of N complex (or back)."""
    N = rec["spec"]["N"]
    fi, fo = e.file("kin", src), e.file("kout", dst)
    e.run([f"k{rec['pack0'] + int(unpack)}", -(-N // 256), fi, fo, nb, n, N])
    return np.frombuffer(fo.read_bytes(), dtype=dst.dtype).copy()


def _bluestein(e, rec, cur, nb, cin, cout, dt, rot_in=-1, rot_out=-1):
    """Bluestein's launches in the library's order: chirp product, M-point forward, product with
    the spectrum of b, M-point inverse, final chirp product scaled by 1/M (with the half-shift
    rotation on the input of a forward, on the output of an inverse)."""
    spec, inner = rec["spec"], rec["inner"]
    N, M = spec["N"], spec["M"]
    sdt = _sdt(dt)
    eb = 2 * np.dtype(sdt).itemsize
    blob = bytearray(rec["blob"])
    # the spectrum of b, as the plan takes it on the device: one forward M-point transform
    b = np.frombuffer(bytes(blob[spec["off_bhat"]:spec["off_bhat"] + M * eb]), dtype=sdt).copy()
    inner_tab = e.file("itab", inner["blob"])
    bhat = _passes(e, inner, b, 1, False, inner_tab)
    blob[spec["off_bhat"]:spec["off_bhat"] + M * eb] = bhat.tobytes()
    table = e.file("btab", blob)
    gm, gn = -(-M // 256), -(-N // 256)
    out = np.full(nb * N * 2, np.nan, dtype=sdt)
    work = np.full(nb * M * 2, np.nan, dtype=sdt)

    def blue(i, grid, o, w):
        fi, fo, fw = e.file("bin", cur), e.file("bout", o), e.file("bwork", w)
        e.run([f"b{rec['blue0'] + i}", grid, nb, fi, fo, fw, table, N, M, N, spec["off_chirp"], spec["off_bhat"],
               rot_in if i in (0, 1) else -1, rot_out if i in (3, 4) else -1])
        return (np.frombuffer(fo.read_bytes(), dtype=sdt).copy(), np.frombuffer(fw.read_bytes(), dtype=sdt).copy())

    _, work = blue(1 if cin else 0, gm, out, work)
    work = _passes(e, inner, work, nb, False, inner_tab)
    _, work = blue(2, gm, out, work)
    work = _passes(e, inner, work, nb, True, inner_tab)
    out, _ = blue(4 if cout else 3, gn, out, work)
    return out


def _transform(e, n, dt, kind, x, inverse):
    """x: [transforms, n] reals for a RealFFT forward, [transforms, N] bins for its inverse,
    [transforms, n] complex points otherwise; returns [transforms, N] complex (forward), [transforms,
    n] reals (RealFFT inverse; for odd n the last real of a row is the prefilled NaN, unwritten) or
    complex points, launched as the library launches it."""
    rec = e.specs[(n, dt, kind)]
    spec = rec["spec"]
    sdt = _sdt(dt)
    real = bool(spec["real"])
    odd = bool(spec.get("odd"))
    N = spec["N"]
    nb = x.shape[0]
    cur = np.ascontiguousarray(x).view(sdt).reshape(-1)
    table = e.file("tab", rec["blob"])
    if real and not inverse and odd:
        cur = _pack(e, rec, cur, np.full(nb * 2 * N, np.nan, dtype=sdt), nb, n, False)
    if real and inverse:
        cur = _split(e, rec, True, cur, np.full_like(cur, np.nan), nb, table)
    if "M" in spec:
        mod = bool(spec.get("modified"))
        cur = _bluestein(e, rec, cur, nb, inverse and not real, inverse, dt,
                         spec["off_brot"] if mod and not inverse else -1, spec["off_brot"] if mod and inverse else -1)
    else:
        cur = _passes(e, rec, cur, nb, inverse, table)
    if real and not inverse:
        cur = _split(e, rec, False, cur, cur, nb, table)
    cdt = np.complex64 if dt == "f32" else np.complex128
    if real and inverse:
        if odd:
            return _pack(e, rec, cur, np.full(nb * n, np.nan, dtype=sdt), nb, n, True).reshape(nb, n)
        return cur.reshape(nb, n)
    return cur.view(cdt).reshape(nb, -1)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-{c[2]}")
def test_emulated_path_beyond_one_cta_matches_oracle(emu, case):
    n, dt, kind, nb = case
    rng = np.random.default_rng(n % 1009)
    cdt = np.complex64 if dt == "f32" else np.complex128
    rdt = _sdt(dt)
    blue = "M" in emu.specs[(n, dt, kind)]["spec"]
    # Bluestein's chirp products and its two M-point transforms add error: 2e-6 FP32, 5e-11 FP64
    # against the oracle (whose own FP64 error at prime lengths is ~1e-12)
    tol = (2e-6 if blue else 1e-6) if dt == "f32" else (5e-11 if blue else 1e-13)
    if kind == "complex":
        x = (rng.uniform(-1, 1, (nb, n)) + 1j * rng.uniform(-1, 1, (nb, n))).astype(cdt)
        for inv in (False, True):
            got = _transform(emu, n, dt, kind, x, inv)
            assert np.all(np.isfinite(got)), "every output element written"
            ref = np.stack([oracle.fft(r.astype(np.complex128), inv) for r in x])
            assert rel_l2(got, ref) <= tol, (inv, rel_l2(got, ref))
    else:
        mod = kind == "real_halfshift"
        x = rng.standard_normal((nb, n)).astype(rdt)
        got = _transform(emu, n, dt, kind, x, False)
        assert np.all(np.isfinite(got)), "every bin written"
        ref = np.stack([oracle.rfft(r.astype(np.float64), mod) for r in x])
        assert rel_l2(got, ref) <= tol, rel_l2(got, ref)
        s = (rng.standard_normal((nb, n // 2)) + 1j * rng.standard_normal((nb, n // 2))).astype(cdt)
        back = _transform(emu, n, dt, kind, s, True)
        h2 = 2 * (n // 2)
        assert np.all(np.isfinite(back[:, :h2])) and np.all(np.isnan(back[:, h2:])), "2*(n//2) reals written"
        ref = np.stack([oracle.irfft(r.astype(np.complex128), n, mod) for r in s])
        assert rel_l2(back[:, :h2], ref) <= tol, rel_l2(back[:, :h2], ref)

"""The uneven-batch work-item queue kernel (ssfft_cl::queue), run on the CPU through the CUDA
emulation shim in tests/emu/ with the classes, items and FP64 tables libssfft.so's planner makes
(ssfft_diag_multi_spec), against the FP64 oracle.  Checks the class kernels' dispatch, the item
layout (partial items, CTAs wider than their transforms), the per-size offset tables and that a
class launch writes only its own transforms.  The GPU tests (test_gpu_multi.py) repeat the
comparison on the device."""
import ctypes
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import fft_gb300 as F
import oracle
from conftest import ROOT, rel_l2

# (dtype, sizes with repeat counts): every class shape the planner forms for uneven batches,
# with partial items (counts that do not fill the transforms per CTA) and single transforms
CASES = {
    "f32": [(64, 45), (72, 9), (100, 13), (243, 5), (256, 3), (625, 6), (1000, 2), (1024, 3), (1458, 2),
            (2048, 2), (3840, 1), (4096, 2), (3645, 1), (6561, 1), (8192, 1), (12288, 1), (15552, 1), (16384, 1)],
    "f64": [(64, 10), (96, 7), (243, 2), (1024, 3), (2187, 1), (4096, 1), (8192, 1)],
}


def spec_of(sizes, dt, qmax=16384, members=16):
    """The queue spec of an uneven list; every size up to qmax in a class (the library's default
    keeps sizes above 4096 out of the classes; the kernel must be right for any class)."""
    old = os.environ.get("SSFFT_DEBUG")
    os.environ["SSFFT_DEBUG"] = f"queue_max_n={qmax},queue_members={members}"
    try:
        return _spec(sizes, dt)
    finally:
        if old is None:
            os.environ.pop("SSFFT_DEBUG", None)
        else:
            os.environ["SSFFT_DEBUG"] = old


def _spec(sizes, dt):
    l = F.lib()
    l.ssfft_diag_multi_spec.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.c_size_t, ctypes.c_int,
                                        ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_size_t)]
    l.ssfft_diag_multi_spec.restype = ctypes.c_int
    arr = (ctypes.c_size_t * len(sizes))(*sizes)
    buf = ctypes.create_string_buffer(1 << 22)
    nb = ctypes.c_size_t()
    code = 0 if dt == "f32" else 1
    assert l.ssfft_diag_multi_spec(arr, len(sizes), code, buf, 1 << 22, None, ctypes.byref(nb)) == 0
    blob = np.zeros(nb.value, dtype=np.uint8)
    assert l.ssfft_diag_multi_spec(arr, len(sizes), code, None, 0, blob.ctypes.data, ctypes.byref(nb)) == 0
    return json.loads(buf.value.decode()), blob


def uneven_list(dt, seed=5):
    rng = np.random.default_rng(seed)
    sizes = [n for n, c in CASES[dt] for _ in range(c)]
    rng.shuffle(sizes)
    return sizes


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("emuq")
    lines, index = [], {}
    for dt in CASES:
        spec, _ = spec_of(uneven_list(dt), dt)
        sb = 4 if dt == "f32" else 8
        for ci, c in enumerate(spec["classes"]):
            for inv in (False, True):
                index[(dt, ci, inv)] = len(lines)
                lines.append(f'{{&{c["inv" if inv else "fwd"]}, {c["cta"]}, {c["smem"]}, {sb}}},')
    (d / "emu_queue_cases.inc").write_text("\n".join(lines) + "\n")
    exe = d / "emuq"
    cmd = ["g++", "-std=c++20", "-O1", "-pthread", "-w", "-I", str(d), "-I", os.path.join(ROOT, "tests", "emu"),
           "-I", os.path.join(ROOT, "fft_gb300", "csrc"), os.path.join(ROOT, "tests", "emu", "emu_queue_main.cpp"),
           "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe, index, d


def test_default_queue_keeps_long_sizes_out_of_classes():
    """By default sizes above 1024 points run as launches of their own, and a class holds at most
    four sizes."""
    sizes = uneven_list("f32")
    spec, _ = _spec(sizes, "f32")
    assert sorted(spec["own_launch"]) == sorted({n for n in sizes if n > 1024})
    assert all(m["n"] <= 1024 for c in spec["classes"] for m in c["members"])
    assert all(len(c["members"]) <= 4 for c in spec["classes"])


def test_queue_classes_cover_every_transform_once():
    """Every transform of the list is in exactly one item of one class, and items never exceed
    their member's transforms per CTA (host only)."""
    for dt in CASES:
        sizes = uneven_list(dt)
        spec, _ = spec_of(sizes, dt)
        seen = {}
        for c in spec["classes"]:
            assert c["cta"] % 128 == 0 and c["cta"] <= 1024
            for m in c["members"]:
                assert m["threads"] * m["per_cta"] <= c["cta"]
            for k, cnt, first in c["items"]:
                m = c["members"][k]
                assert 1 <= cnt <= m["per_cta"]
                for g in range(first, first + cnt):
                    key = (m["n"], g)
                    assert key not in seen
                    seen[key] = True
            # queue order: longest transforms first
            ns = [c["members"][k]["n"] for k, _, _ in c["items"]]
            assert ns == sorted(ns, reverse=True)
        counts = {}
        for n in sizes:
            counts[n] = counts.get(n, 0) + 1
        assert len(seen) == len(sizes)
        assert all(sum(1 for (n2, _) in seen if n2 == n) == c for n, c in counts.items())


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("inv", [False, True])
def test_emulated_queue_kernels_match_oracle(emulator, dt, inv):
    exe, index, d = emulator
    sizes = uneven_list(dt)
    spec, blob = spec_of(sizes, dt)
    sdt, cdt = (np.float32, np.complex64) if dt == "f32" else (np.float64, np.complex128)
    rng = np.random.default_rng(11 + inv)
    total = sum(sizes)
    x = (rng.uniform(-1, 1, total) + 1j * rng.uniform(-1, 1, total)).astype(cdt)
    starts = np.concatenate([[0], np.cumsum(sizes)])[:-1]
    by_size = {}
    for i, n in enumerate(sizes):
        by_size.setdefault(n, []).append(2 * int(starts[i]))  # scalar offsets, in list order
    ntab = spec["tables"][0][0] // 8 if spec["tables"] else 0
    tables = blob[:ntab * 8].view(np.float64).astype(sdt)
    sentinel = np.array(complex(3.0, -7.0), dtype=cdt)
    (d / "tab.bin").write_bytes(tables.tobytes())
    (d / "in.bin").write_bytes(x.tobytes())
    covered = np.zeros(total, dtype=bool)
    tol = 1e-6 if dt == "f32" else 1e-13
    worst = 0.0
    for ci, c in enumerate(spec["classes"]):
        mem = []
        for m in c["members"]:
            mem += [m["n"], m["tw"][0], m["roots"][0], m["threads"]]
        ok, ot = spec["tables"][ci]
        nit = c["nitems"]
        kidx = blob[ok:ok + 4 * nit].view(np.int32)
        toff = blob[ot:ot + 4 * nit * c["cta"]].view(np.int32).reshape(nit, c["cta"])
        # the tables are the items: item b runs member k on its transforms first.., one thread group each
        for b, (k, cnt, first) in enumerate(c["items"]):
            assert kidx[b] == k
            th = c["members"][k]["threads"]
            n = c["members"][k]["n"]
            for t in range(c["cta"]):
                g = t // th
                want = by_size[n][first + g] // 2 if g < cnt else -1
                assert toff[b, t] == want, (ci, b, t)
        (d / "kidx.bin").write_bytes(kidx.tobytes())
        (d / "toff.bin").write_bytes(toff.tobytes())
        (d / "mem.bin").write_bytes(np.array(mem, dtype=np.int64).tobytes())
        (d / "out.bin").write_bytes(np.full(total, sentinel).tobytes())
        r = subprocess.run([str(exe), str(index[(dt, ci, inv)]), str(d / "kidx.bin"), str(d / "toff.bin"),
                            str(d / "mem.bin"), str(d / "tab.bin"), str(d / "in.bin"), str(d / "out.bin"), "3"],
                           capture_output=True, text=True, timeout=900)
        assert r.returncode == 0, r.stderr[-2000:]
        y = np.frombuffer((d / "out.bin").read_bytes(), dtype=cdt)
        mine = np.zeros(total, dtype=bool)
        for m in c["members"]:
            for o in by_size[m["n"]]:
                mine[o // 2:o // 2 + m["n"]] = True
        assert np.all(y[~mine] == sentinel), f"class {ci} wrote outside its transforms"
        for m in c["members"]:
            n = m["n"]
            for o in by_size[n]:
                got = y[o // 2:o // 2 + n]
                ref = oracle.fft(x[o // 2:o // 2 + n].astype(np.complex128), inv)
                err = rel_l2(got, ref)
                worst = max(worst, err)
                assert err <= tol, (dt, n, inv, err)
        covered |= mine
    assert covered.all()

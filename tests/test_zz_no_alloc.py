"""The allocation-free entry point ssfft_fft_noalloc_f32, called through the C ABI.

It exists for callers that cannot allocate device memory when they need a transform (a real-time
thread that must not enter the allocator, a host framework that owns all device memory); its
only working memory is a fixed array inside the library.  Checked against the plan-based entry
point (ssfft_plan_create + ssfft_exec) within the FP32 tolerance of the other parity tests, on two
calls in a row (the shared scratch array keeps the previous call's contents), against the FP64
oracle, and the device's free memory must not change across calls once the first call has done
its set-up.

This file is collected last on purpose, so that a run stopping at its first failure has already
run every other test."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

F32_TOL = 1e-6


@pytest.fixture(scope="module")
def F():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fft_gb300
    l = fft_gb300.lib()
    l.ssfft_fft_noalloc_f32.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                        ctypes.c_void_p]
    l.ssfft_fft_noalloc_f32.restype = ctypes.c_int
    l.ssfft_fft_noalloc_max_size.restype = ctypes.c_size_t
    return fft_gb300


def noalloc(F, xi, out, inverse):
    rc = F.lib().ssfft_fft_noalloc_f32(xi.data_ptr(), out.data_ptr(), xi.numel(), int(inverse), None)
    assert rc == 0, F.lib().ssfft_last_cuda_error()


@pytest.mark.parametrize("n", [1, 2, 3, 16, 1920, 4096, 3 ** 7, 1000, 2 ** 17, 2 ** 20])
def test_noalloc_matches_plan_entry_point_twice(F, n):
    rng = np.random.default_rng(n)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    xi = torch.from_numpy(x).cuda()
    for inverse in (False, True):
        plan = F.Plan(n, "f32", "complex", 1)
        ref = torch.empty_like(xi)
        plan.exec(inverse, xi.data_ptr(), ref.data_ptr(), 0)
        torch.cuda.synchronize()
        r = ref.cpu().numpy()
        for _ in range(2):
            out = torch.full_like(xi, complex(7, 7))
            noalloc(F, xi, out, inverse)
            torch.cuda.synchronize()
            assert rel_l2(out.cpu().numpy(), r) <= F32_TOL, (n, inverse, rel_l2(out.cpu().numpy(), r))
        assert np.array_equal(xi.cpu().numpy(), x), "input was changed"


@pytest.mark.parametrize("n", [2, 3, 5, 2 * 3 * 5 * 1024, 3 ** 9, 5 ** 6, 2 ** 20])
def test_noalloc_matches_fp64_oracle(F, n):
    """The same entry point against the FP64 oracle (the reference's algorithm on the CPU), so a
    mistake shared with the plan-based path cannot hide; sizes cover every radix it uses."""
    import oracle
    rng = np.random.default_rng(7 * n + 1)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    xi = torch.from_numpy(x).cuda()
    for inverse in (False, True):
        ref = oracle.fft(x.astype(np.complex128), inverse)
        out = torch.empty_like(xi)
        noalloc(F, xi, out, inverse)
        torch.cuda.synchronize()
        err = rel_l2(out.cpu().numpy(), ref)
        assert err <= F32_TOL, (n, inverse, err)


def test_noalloc_allocates_nothing_per_call(F):
    """Once the first call on the device has done its set-up (which also loads every kernel of
    the entry point), later calls of any size -- radices 2, 3, 4 and 5 -- leave the device's
    free memory unchanged."""
    sizes = [2 ** 16, 2 * 3 * 5 * 1024, 3 ** 9, 5 ** 6, 2 ** 15 * 2, 1]
    bufs = [(torch.randn(n, dtype=torch.complex64, device="cuda"),
             torch.empty(n, dtype=torch.complex64, device="cuda")) for n in sizes]
    noalloc(F, bufs[0][0], bufs[0][1], False)   # first call on the device does the set-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        for xi, out in bufs:
            noalloc(F, xi, out, False)
            noalloc(F, xi, out, True)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_its_scratch(F):
    l = F.lib()
    mx = l.ssfft_fft_noalloc_max_size()
    assert mx == 2 ** 20
    x = torch.zeros(8, dtype=torch.complex64, device="cuda")
    y = torch.zeros(8, dtype=torch.complex64, device="cuda")
    assert l.ssfft_fft_noalloc_f32(x.data_ptr(), y.data_ptr(), mx + 1, 0, None) == 1      # invalid size
    assert l.ssfft_fft_noalloc_f32(x.data_ptr(), y.data_ptr(), 0, 0, None) == 1
    assert l.ssfft_fft_noalloc_f32(x.data_ptr(), y.data_ptr(), 7, 0, None) == 5         # prime 7: unsupported
    assert l.ssfft_fft_noalloc_f32(x.data_ptr(), x.data_ptr(), 8, 0, None) == 2         # in place refused
    # partial overlap of the two ranges is refused too (either order)
    assert l.ssfft_fft_noalloc_f32(x.data_ptr(), x.data_ptr() + 8, 4, 0, None) == 2
    assert l.ssfft_fft_noalloc_f32(x.data_ptr() + 8, x.data_ptr(), 4, 0, None) == 2
    # adjacent, non-overlapping halves of one buffer are fine
    assert l.ssfft_fft_noalloc_f32(x.data_ptr(), x.data_ptr() + 32, 4, 0, None) == 0
    torch.cuda.synchronize()

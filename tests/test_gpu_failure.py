"""Failure detection of the staged (bulk-copy) kernel, without a GPU fault.

The staged kernel waits on an mbarrier for each group's input copy with a bounded number of
try_wait attempts; when they run out it raises the plan's error flag and returns, so the context
stays usable.  ``ssfft_diag_staged_timeout`` makes that wait run out on purpose: the barrier is
told to expect the group's bytes but the copy is never issued (nothing is in flight when the
kernel returns).
"""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_lost_copy_raises_flag_and_context_survives():
    torch = pytest.importorskip("torch")
    import fft_gb300 as ff
    assert ff.diag_staged_timeout(1024, 500) == 1
    assert ff.diag_staged_timeout(256, 50) == 1
    # long transforms: whole input staged (12288), leading rows staged with the rest copied into
    # the work buffer behind a second barrier (16384)
    assert ff.diag_staged_timeout(12288, 200) == 1
    assert ff.diag_staged_timeout(16384, 200) == 1
    # the context is still usable: an ordinary transform runs and is correct
    rng = np.random.default_rng(7)
    x = (rng.standard_normal((8, 1024)) + 1j * rng.standard_normal((8, 1024))).astype(np.complex64)
    got = ff.fft(torch.from_numpy(x).cuda()).cpu().numpy()
    want = oracle.batch(x.astype(np.complex128), 1024, real=False, inverse=False)
    assert rel_l2(got, want) < 1e-6


def test_diag_rejects_bad_arguments():
    import fft_gb300 as ff
    with pytest.raises(ff.SsfftError):
        ff.diag_staged_timeout(8, 10)
    with pytest.raises(ff.SsfftError):
        ff.diag_staged_timeout(32768, 10)

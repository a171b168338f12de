"""Pin the CPU oracle (oracle/ssfft_oracle.c, a C restatement of signalsmith-fft.h) against the
golden vectors that tests/golden/make_golden.py produced by running the unmodified reference,
and -- where the reference checkout exists -- against the reference itself on fresh inputs."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

COMPLEX_SIZES = [1, 2, 4, 8, 16, 32, 64, 128, 256, 3, 6, 9, 12, 18, 24, 5, 10, 15, 20, 25,
                 7, 14, 21, 28, 49, 11, 13, 17, 19, 22, 23, 480, 1024]


@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_complex_matches_golden(golden, dt):
    worst = 0.0
    for n in COMPLEX_SIZES:
        x = golden[f"c2c_{dt}_{n}_in"]
        for d in ("fwd", "inv"):
            got = oracle.fft(x, d == "inv")
            ref = golden[f"c2c_{dt}_{n}_{d}"]
            # same operation order as the reference: bit-identical here, tight bound elsewhere
            worst = max(worst, rel_l2(got, ref))
    assert worst <= (1e-15 if dt == "f64" else 1e-7), worst


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("mod", [0, 1])
def test_real_matches_golden(golden, dt, mod):
    worst = 0.0
    for n in list(range(2, 100)) + [480, 960, 1920, 3840]:
        key = f"r_{dt}_m{mod}_{n}"
        if key + "_in" not in golden:
            continue
        got = oracle.rfft(golden[key + "_in"], bool(mod))
        worst = max(worst, rel_l2(got, golden[key + "_fwd"]))
        got = oracle.irfft(golden[key + "_spec"], n, bool(mod))
        worst = max(worst, rel_l2(got, golden[key + "_inv"]))
    assert worst <= (1e-15 if dt == "f64" else 1e-7), worst


def test_bit_exact_on_this_host(golden):
    """x86-64 without FMA contraction reproduces the reference bit for bit."""
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("bit-exactness is pinned on the host that generated the fixtures")
    for n in (7, 49, 480, 1024):
        x = golden[f"c2c_f64_{n}_in"]
        assert np.array_equal(oracle.fft(x), golden[f"c2c_f64_{n}_fwd"])


def test_size_helpers_match_golden(golden):
    idx = golden["size_index"]
    for name in ("size_minimum", "size_maximum", "real_size_minimum", "real_size_maximum"):
        got = np.array([getattr(oracle, name)(int(i)) for i in idx])
        assert np.array_equal(got, golden[name]), name


def test_reference_tests_restated():
    """The reference's own checks (tests/00-fft.cpp, tests/01-real.cpp) on the oracle."""
    rng = np.random.default_rng(5)
    for n in COMPLEX_SIZES[:31]:
        # individual bins: e^{2 pi i n b / N} -> N delta[k - b]   (tests/00-fft.cpp:19-60)
        i = np.arange(n)
        for b in range(n):
            x = np.exp(2j * np.pi * i * b / n)
            exp = np.zeros(n, complex)
            exp[b] = n
            assert oracle.close_enough(oracle.fft(x), exp)
        # inverse round trip = N x   (tests/00-fft.cpp:101-145)
        x = rng.uniform(-0.5, 0.5, n) + 1j * rng.uniform(-0.5, 0.5, n)
        assert oracle.close_enough(oracle.ifft(oracle.fft(x)), n * x)
    # sizes rule (tests/00-fft.cpp:168-186)
    for i in range(1, 1000):
        for v in (oracle.size_minimum(i), oracle.size_maximum(i)):
            m, threes = v, 0
            while m % 2 == 0:
                m //= 2
            while m % 3 == 0:
                m //= 3
                threes += 1
            assert m == 1 and threes <= 2
        assert oracle.size_minimum(i) >= i >= oracle.size_maximum(i)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference checkout not built here")
def test_port_equals_reference_fresh_inputs():
    rng = np.random.default_rng(11)
    for n in (5, 12, 97, 240, 960, 4096, 3 * 2 ** 12):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        for inv in (False, True):
            assert np.array_equal(oracle.fft(x, inv), oracle.fft(x, inv, kind="reference"))
    for n in (2, 9, 100, 480, 3840):
        x = rng.standard_normal(n)
        for mod in (False, True):
            assert np.array_equal(oracle.rfft(x, mod), oracle.rfft(x, mod, kind="reference"))

"""The merge's exact fixed-point amplitude accumulator (sfci_gb300/csrc/common.cuh),
compiled for the host, against exact rational arithmetic.

The merge sums each determinant's terms as integers in units of 2^-64 (a
low and a high addend per term, kept in two words without carries between
them) and converts the sum back to double once.  So a merged amplitude must
equal the correctly rounded (nearest, ties to even) value of the exact sum of
the terms, each rounded to the nearest point of the 2^-64 grid (ties to even),
whatever the order of the terms."""
import ctypes as C
import math
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "sfci_gb300", "csrc")
FRAC = 64


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    d = tmp_path_factory.mktemp("fx")
    so = str(d / "gen_host.so")
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + CSRC, "-I/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "native", "gen_host.cpp"), os.path.join(CSRC, "ham.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(so)
    L.gh_fx_sum.restype = C.c_double
    L.gh_fx_sum.argtypes = [np.ctypeslib.ndpointer(np.float64), C.c_long, C.POINTER(C.c_int)]
    L.gh_fx_roundtrip.restype = C.c_double
    L.gh_fx_roundtrip.argtypes = [C.c_double, C.POINTER(C.c_int)]
    L.gh_fx32_sum.restype = C.c_double
    L.gh_fx32_sum.argtypes = [np.ctypeslib.ndpointer(np.float64), C.c_long, C.POINTER(C.c_int)]
    L.gh_above_cut.argtypes = [np.ctypeslib.ndpointer(np.float64), C.c_long, C.c_double,
                               np.ctypeslib.ndpointer(np.uint8)]
    return L


def to_grid(x):
    """x * 2^64 rounded to the nearest integer, ties to even (Python's round of a Fraction)."""
    return round(Fraction(x) * (1 << FRAC))


def exact(terms):
    return float(Fraction(sum(to_grid(float(t)) for t in terms), 1 << FRAC))


def fsum(L, terms):
    bad = C.c_int(0)
    a = np.ascontiguousarray(terms, dtype=np.float64)
    return L.gh_fx_sum(a, len(a), C.byref(bad)), bad.value


def f32sum(L, terms):
    big = C.c_int(0)
    a = np.ascontiguousarray(terms, dtype=np.float64)
    return L.gh_fx32_sum(a, len(a), C.byref(big)), big.value


def test_random_sums_are_correctly_rounded(fx):
    rng = np.random.default_rng(7)
    for trial in range(400):
        n = int(rng.integers(1, 40))
        mag = np.exp2(rng.uniform(-67, 23.9, n))
        terms = mag * rng.choice([-1.0, 1.0], n)
        got, bad = fsum(fx, terms)
        assert bad == 0
        assert got == exact(terms), (trial, terms)
        rng.shuffle(terms)
        assert fsum(fx, terms)[0] == got  # order-independent


def test_cancellation_and_sign_changes(fx):
    rng = np.random.default_rng(8)
    for _ in range(200):
        x = rng.uniform(-10, 10, 8)
        terms = np.concatenate([x, -x[::-1], [rng.uniform(-1e-9, 1e-9)]])
        got, _ = fsum(fx, terms)
        assert got == exact(terms)
    assert fsum(fx, np.array([1.0, -1.0]))[0] == 0.0
    assert fsum(fx, np.array([3.5, -1.25, -2.25]))[0] == 0.0


def test_rounding_ties_to_even(fx):
    # 2^53 + 1 (in units of 2^-72 * 2^k) sits halfway between two doubles
    for k in (0, 5, 20, 30):
        ulp = math.ldexp(1.0, k - FRAC)
        big = math.ldexp(1.0, 53 + k - FRAC)
        for extra, want in ((1, big), (3, big + 4 * ulp)):
            # big + extra*ulp built from exactly representable pieces
            got, _ = fsum(fx, np.array([big, extra * ulp]))
            assert got == want, (k, extra)
        got, _ = fsum(fx, np.array([-big, -ulp]))
        assert got == -big


def test_rounding_to_the_grid(fx):
    bad = C.c_int(0)
    g = math.ldexp(1.0, -64)  # the grid unit
    assert fx.gh_fx_roundtrip(math.ldexp(1.0, -66), C.byref(bad)) == 0.0   # 1/4 unit
    assert fx.gh_fx_roundtrip(math.ldexp(1.0, -65), C.byref(bad)) == 0.0   # 1/2 unit: tie to even 0
    assert fx.gh_fx_roundtrip(0.75 * g, C.byref(bad)) == g
    assert fx.gh_fx_roundtrip(g, C.byref(bad)) == g
    assert fx.gh_fx_roundtrip(-1.5 * g, C.byref(bad)) == -2 * g             # tie to even 2
    assert fx.gh_fx_roundtrip(2.5 * g, C.byref(bad)) == 2 * g               # tie to even 2
    assert fx.gh_fx_roundtrip(-2.75 * g, C.byref(bad)) == -3 * g
    for x in (1e-5, -0.3, 123.456, -7.5e6, 5e-300, 0.0, -0.0, 1e-19, -3.3e-20):
        assert fx.gh_fx_roundtrip(x, C.byref(bad)) == exact([x])
    assert bad.value == 0


def test_no_drift_over_many_same_sign_terms(fx):
    """10^4 small terms of one sign on one key (a hot determinant near the cut):
    with each term rounded to nearest the error grows like sqrt(n) * 2^-66, far
    below the n * 2^-65 a truncation toward zero would accumulate."""
    rng = np.random.default_rng(12)
    n = 10000
    for sign in (1.0, -1.0):
        terms = sign * rng.uniform(1e-10, 1e-9, n)
        got, bad = fsum(fx, terms)
        assert bad == 0
        ref = math.fsum(terms)
        assert abs(got - ref) < 2e-18, (got, ref, got - ref)       # truncation: ~2.7e-16
        assert abs(got - ref) <= 1e-12 * abs(ref)
        f32, big = f32sum(fx, terms)
        assert big == 0 and f32 == got


def test_range_flag(fx):
    for x in (math.ldexp(1.0, 24), -2e7, float("inf"), float("nan")):
        bad = C.c_int(0)
        assert fx.gh_fx_roundtrip(x, C.byref(bad)) == 0.0
        assert bad.value == 1
    bad = C.c_int(0)
    fx.gh_fx_roundtrip(math.ldexp(1.0, 24) * (1 - 2 ** -53), C.byref(bad))
    assert bad.value == 0


def test_many_terms_on_one_accumulator(fx):
    """Up to the 2^19 terms one accumulator may receive, at the largest allowed
    magnitude and mixed signs, the split words do not overflow."""
    n = 1 << 19
    big = math.ldexp(1.0, 24) * (1 - 2 ** -53)
    for sign in (1.0, -1.0):
        terms = np.full(n, sign * big)
        got, bad = fsum(fx, terms)
        assert bad == 0
        assert got == sign * float(Fraction(to_grid(big)) * n / (1 << FRAC))
    rng = np.random.default_rng(3)
    terms = rng.uniform(-1, 1, n) * np.exp2(rng.uniform(-60, 23, n))
    got, _ = fsum(fx, terms)
    assert got == float(Fraction(sum(to_grid(float(t)) for t in terms), 1 << FRAC))


@pytest.fixture(scope="module")
def fx32(fx):
    return fx


def test_digit_form_sums_exactly(fx32):
    """The warp tables' narrow form (four words of signed base-2^21 digits) gives
    the same exact, correctly rounded sums as the wide form."""
    rng = np.random.default_rng(11)
    for trial in range(300):
        n = int(rng.integers(1, 60))
        terms = np.exp2(rng.uniform(-70, 17.9, n)) * rng.choice([-1.0, 1.0], n)
        got, big = f32sum(fx32, terms)
        assert big == 0
        assert got == exact(terms), (trial, terms)
        rng.shuffle(terms)
        assert f32sum(fx32, terms)[0] == got
    x = rng.uniform(-5, 5, 9)
    assert f32sum(fx32, np.concatenate([x, -x]))[0] == 0.0


def test_digit_form_capacity_and_range(fx32):
    n = 1 << 11  # terms one warp-table slot may receive
    big = math.ldexp(1.0, 18) * (1 - 2 ** -53)
    for sign in (1.0, -1.0):
        got, flag = f32sum(fx32, np.full(n, sign * big))
        assert flag == 0
        assert got == sign * float(Fraction(to_grid(big)) * n / (1 << FRAC))
    for x in (math.ldexp(1.0, 18), -3e5, float("inf"), float("nan")):
        assert f32sum(fx32, np.array([x]))[1] == 1


def test_integer_magnitude_cut(fx):
    """The prunes and compactions test |a| > cut as an integer compare of the bits of
    |a| against those of the cut (cut_key / above_cut).  For every finite amplitude,
    signed zeros, subnormals, infinities and values one ulp either side of the cut
    included, it must agree with the floating-point compare; a negative cut keeps
    everything."""
    rng = np.random.default_rng(7)
    for cut in (1e-5, 1e-8, 0.0, 5e-324, 1.0, 1e300, -1.0):
        mags = 10.0 ** rng.uniform(-330, 308, 20000)
        x = np.concatenate([mags * rng.choice([-1.0, 1.0], mags.size),
                            [0.0, -0.0, 5e-324, -5e-324, np.inf, -np.inf, 2.2e-308, -1.1e-308]])
        if cut >= 0:
            near = [cut, np.nextafter(cut, np.inf), np.nextafter(cut, 0.0) if cut > 0 else 0.0]
            x = np.concatenate([x, near, [-v for v in near]])
        x = np.ascontiguousarray(x, np.float64)
        out = np.zeros(x.size, np.uint8)
        fx.gh_above_cut(x, x.size, cut, out)
        np.testing.assert_array_equal(out.astype(bool), np.abs(x) > cut)

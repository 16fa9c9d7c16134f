"""The SpMSpV device-memory plan (csrc/plan.h) on the host: fewest generation
passes first, then the largest level-2 groups, every buffer within the budget."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "sfci_gb300", "csrc")
_u = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
DIVS = (16, 24, 32, 48, 64)


@pytest.fixture(scope="module")
def pl(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("pl") / "plan.so")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I" + CSRC, os.path.join(ROOT, "tests", "native",
                                                                                    "plan_host.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(so)
    L.pl_plan.argtypes = [_u, C.c_uint, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, _u]
    L.pl_passes.argtypes = [_u, C.c_uint, C.c_uint64]
    L.pl_class.argtypes = [_u, C.c_uint64, C.c_uint, C.c_uint, _u, C.c_int]
    return L


def _plan(pl, sizes, avail, cap, partition=True):
    binoff = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    out = np.zeros(4, np.uint64)
    ok = pl.pl_plan(binoff, len(sizes), int(binoff[-1]), int(avail), int(cap), int(max(sizes)), int(partition), out)
    return bool(ok), [int(x) for x in out], binoff


def _check_fits(sizes, avail, C1, C2, SC, passes, partition=True):
    assert C1 + (C2 if partition else 0) + 2 * SC <= avail
    assert C1 >= max(sizes) and C2 >= max(sizes)
    # the greedy grouping: every pass fits C1
    n, acc = 1, 0
    for s in sizes:
        if acc + s > C1:
            n, acc = n + 1, 0
        acc += s
    assert n == passes


def test_benchmark_shape_takes_two_passes(pl):
    """512 level-1 bins of 3.07e10 terms in all (56 spin orbitals, Nd = 1e6), output
    capacity 6e7, 90% of 293 GB of free memory: two passes, where a fixed 1/16
    level-2 buffer would need three."""
    sizes = [60_000_000] * 512
    avail = int(0.9 * 293e9) // 16
    ok, (C1, C2, SC, passes), binoff = _plan(pl, sizes, avail, 60_000_000)
    assert ok and passes == 2
    _check_fits(sizes, avail, C1, C2, SC, passes)
    fixed_c2 = avail // 16
    fixed_c1 = avail - fixed_c2 - 2 * (60_000_000 + fixed_c2)
    assert pl.pl_passes(binoff, 512, fixed_c1) == 3
    # the largest level-2 buffer among the two-pass plans
    for d in DIVS:
        c2 = avail // d
        c1 = avail - c2 - 2 * (60_000_000 + c2)
        if pl.pl_passes(binoff, 512, c1) == 2:
            assert C2 == c2
            break


def test_everything_fits_in_one_pass(pl):
    sizes = [1000 + 7 * i for i in range(512)]
    T = sum(sizes)
    avail = 50 * T
    ok, (C1, C2, SC, passes), _ = _plan(pl, sizes, avail, 5000)
    assert ok and passes == 1 and C1 == T
    assert C2 == min(T, max(avail // 16, 1 << 20))


def test_without_partition_levels_one_group_buffer(pl):
    sizes = [10_000] * 64
    T = sum(sizes)
    avail = 4 * T
    ok, (C1, C2, SC, passes), _ = _plan(pl, sizes, avail, 1000, partition=False)
    assert ok
    assert C2 == max(10_000, min(T, avail // 6))
    _check_fits(sizes, avail, C1, C2, SC, passes, partition=False)


def test_budget_below_one_bin_is_refused(pl):
    sizes = [5_000_000] * 8
    ok, _, _ = _plan(pl, sizes, 4_000_000, 1000)
    assert not ok


@pytest.mark.parametrize("seed", range(6))
def test_random_plans_fit_and_minimise_passes(pl, seed):
    rng = np.random.default_rng(seed)
    nb = int(rng.choice([64, 256, 512]))
    sizes = [int(x) for x in rng.integers(1 << 18, 1 << 22, size=nb)]
    T = sum(sizes)
    avail = int(T * rng.uniform(0.4, 3.0)) + (1 << 22)
    cap = int(rng.integers(1, 1 << 20))
    ok, (C1, C2, SC, passes), binoff = _plan(pl, sizes, avail, min(cap, T))
    if not ok:
        return
    _check_fits(sizes, avail, C1, C2, SC, passes)
    for d in DIVS:
        c2 = max(max(sizes), min(T, max(avail // d, 1 << 20)))
        sc = min(cap, T) + min(c2, T)
        c1 = T if T + c2 + 2 * sc <= avail else avail - c2 - 2 * sc
        if avail >= c2 + 2 * sc + max(sizes) and c1 >= max(sizes):
            assert pl.pl_passes(binoff, nb, c1) >= passes


def _class_plan(pl, hh, c1, nop_max, run_cap=2048):
    out = np.zeros(4 * 512, np.uint64)
    n = pl.pl_class(np.asarray(hh, np.uint64), int(c1), nop_max, run_cap, out, 512)
    return [tuple(int(x) for x in out[4 * i:4 * i + 4]) for i in range(n)]


@pytest.mark.parametrize("seed,scale,frac", [(0, 1e9, 1 / 24), (1, 1e6, 1 / 5), (2, 3e10, 1 / 60), (3, 1e4, 1.0)])
def test_class_passes_cover_every_class_in_aligned_fitting_blocks(pl, seed, scale, frac):
    """Class passes (plan_class_passes): every class with terms lies in exactly one
    pass, in order; a pass is whole aligned blocks of 2^k classes, holds at most
    c1 terms unless it is a single block, and its runs (occupied pairs x blocks)
    fit the generator's table."""
    rng = np.random.default_rng(seed)
    hh = (rng.uniform(0.7, 1.3, 256) * scale).astype(np.uint64)
    hh[rng.integers(0, 256, 5)] = 0  # a few empty classes
    c1 = int(max(int(hh.sum() * frac), int(hh.max())))
    nop_max = 45
    passes = _class_plan(pl, hh, c1, nop_max)
    covered = np.zeros(256, bool)
    prev = 0
    for lo, hi, terms, k in passes:
        assert lo >= prev and lo % (1 << k) == 0 and hi % (1 << k) == 0 and hi > lo
        assert terms == int(hh[lo:hi].sum()) > 0
        assert terms <= c1 or hi - lo == (1 << k)
        assert nop_max * ((hi - lo) >> k) <= 2048
        covered[lo:hi] = True
        prev = hi
    assert covered[hh > 0].all()
    # close to the fewest passes the capacity allows
    assert len(passes) <= 2 * max(1, -(-int(hh.sum()) // c1)) + 1

"""The screen's term groups (csrc/screen.cuh) compiled for the host.

The groups name the double-excitation terms of gen.cuh's index space that the
screen keeps or skips together.  Checked here on the CPU:

* per determinant, group g's (class, p, q, r, size) against the Python model of
  the groups that the GPU screen tests build their expected products from;
* the groups tile the double-excitation terms in index order, each term maps
  back to its group, and each term's excitation removes p and q and adds r;
* the group of every term, taken from its target key alone, against the C
  group_of_term (the map the kept-term compaction relies on);
* pair unranking, the k-th set bit and the k-th occupied / empty orbital
  against brute-force scans.

Cases cover closed- and open-shell determinants, a spin with one electron (no
same-spin groups), a full spin shell (no holes) and 128-bit keys.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from test_gpu_screen import det_groups, group_of_target

CSRC = os.path.join(ROOT, "sfci_gb300", "csrc")


@pytest.fixture(scope="module")
def sh(tmp_path_factory):
    d = tmp_path_factory.mktemp("sh")
    so = str(d / "screen_host.so")
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + CSRC, "-I/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "native", "gen_host.cpp"), os.path.join(CSRC, "ham.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(so)
    L.gh_groups.restype = C.c_long
    L.gh_groups.argtypes = [np.ctypeslib.ndpointer(np.uint64), C.c_int, np.ctypeslib.ndpointer(np.int32), C.c_long,
                            np.ctypeslib.ndpointer(np.uint64), np.ctypeslib.ndpointer(np.uint32), C.c_long,
                            C.POINTER(C.c_long), C.POINTER(C.c_long)]
    L.gh_screen_index_checks.restype = C.c_long
    L.gh_screen_index_checks.argtypes = [C.c_uint, C.c_uint64]
    return L


def random_det(rng, N, na, nb):
    a = rng.choice(np.arange(0, N, 2), na, replace=False)
    b = rng.choice(np.arange(1, N, 2), nb, replace=False)
    d = 0
    for o in list(a) + list(b):
        d |= 1 << int(o)
    return d


def run_groups(sh, d, N, tcap):
    W = 1 if N <= 64 else 2
    kw = np.array([d & (2 ** 64 - 1), d >> 64] if W == 2 else [d], np.uint64)
    cap = 200000
    rows = np.zeros(6 * cap, np.int32)
    tk = np.zeros(W * max(tcap, 1), np.uint64)
    tg = np.zeros(max(tcap, 1), np.uint32)
    nt, bad = C.c_long(0), C.c_long(0)
    ng = sh.gh_groups(kw, N, rows, cap, tk, tg, tcap, C.byref(nt), C.byref(bad))
    assert 0 <= ng <= cap
    return rows[:6 * ng].reshape(ng, 6), tk, tg, nt.value, bad.value


CASES = [  # (N, alpha electrons, beta electrons, determinants, check every term's group in Python)
    (56, 7, 7, 2, True),
    (40, 6, 4, 2, True),
    (24, 1, 5, 1, True),   # one spin-0 electron: no spin-0 same-spin groups
    (20, 10, 3, 1, True),  # full spin-0 shell: no spin-0 holes
    (128, 10, 10, 1, False),
]


@pytest.mark.parametrize("N,na,nb,ndet,per_term", CASES)
def test_groups_match_model(sh, N, na, nb, ndet, per_term):
    rng = np.random.default_rng(N * 1000 + na * 10 + nb)
    for _ in range(ndet):
        d = random_det(rng, N, na, nb)
        rows, tk, tg, nt, bad = run_groups(sh, d, N, 400000 if per_term else 0)
        assert bad == 0
        model = det_groups(d, N)
        assert len(model) == len(rows)
        got = [tuple(int(x) for x in r[[0, 1, 2, 3, 5]]) for r in rows]
        assert got == model
        if not per_term:
            continue
        assert 0 < nt <= 400000
        assert nt == int(rows[:, 5].sum())
        want = np.array([group_of_target(d, int(k), N) for k in tk[:nt]], np.int64)
        np.testing.assert_array_equal(tg[:nt].astype(np.int64), want)


def test_index_helpers(sh):
    assert sh.gh_screen_index_checks(1 << 22, 12345) == 0

"""The device excitation decoder (csrc/gen.cuh) compiled for the host, against the
reference's DiagCal_bit / OffDiagGen_bit_e outputs stored in the golden fixtures.

Each connected determinant must appear exactly once with the sum of the
reference's raw terms for it (direct + exchange, one- + two-body pieces)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, SYSTEMS

CSRC = os.path.join(ROOT, "sfci_gb300", "csrc")


@pytest.fixture(scope="module")
def gh(tmp_path_factory):
    d = tmp_path_factory.mktemp("gh")
    so = str(d / "gen_host.so")
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + CSRC, "-I/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "native", "gen_host.cpp"), os.path.join(CSRC, "ham.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(so)
    L.gh_load.argtypes = [C.c_char_p, C.c_int]
    L.gh_terms.restype = C.c_long
    L.gh_terms.argtypes = [np.ctypeslib.ndpointer(np.uint64), np.ctypeslib.ndpointer(np.uint64),
                           np.ctypeslib.ndpointer(np.float64), C.c_long]
    return L


@pytest.mark.parametrize("name", SYSTEMS)
def test_decoder_matches_reference(gh, golden_in, name):
    g, path = golden_in(name)
    N = 2 * int(g["M"])
    assert gh.gh_load(path.encode(), N) == 0
    cap = 200000
    for t in range(3):
        det = np.array([g["off%d_det" % t]], np.uint64)
        k = np.zeros(cap, np.uint64)
        a = np.zeros(cap)
        n = gh.gh_terms(det, k, a, cap)
        assert 0 < n <= cap
        k, a = k[:n], a[:n]
        # term 0 is the diagonal, the rest are distinct connected determinants
        diag_ref = g["diag_vals"][list(g["diag_dets"]).index(det[0])]
        assert abs(a[0] - diag_ref) <= 1e-12 * max(1.0, abs(diag_ref))
        ko, ao = k[1:], a[1:]
        assert np.unique(ko).size == ko.size
        rk, ra = g["off%d_keys" % t], g["off%d_amps" % t]
        order = np.argsort(ko)
        ko, ao = ko[order], ao[order]
        # the reference emits every connected determinant here (dense integrals)
        assert np.array_equal(ko, rk), "connected set differs"
        scale = np.max(np.abs(ra))
        assert np.max(np.abs(ao - ra)) <= 1e-13 * scale + 1e-15


def _double_term_check(gh, det, words):
    gh.gh_double_term_mismatches.restype = C.c_long
    gh.gh_double_term_mismatches.argtypes = [np.ctypeslib.ndpointer(np.uint64), C.c_int]
    return gh.gh_double_term_mismatches(det, words)


@pytest.mark.parametrize("name", SYSTEMS)
def test_branch_free_doubles_match(gh, golden_in, name):
    """The generation kernel computes doubles on one branch-free path; its keys and
    elements must equal the class-by-class decoder's bit for bit."""
    g, path = golden_in(name)
    assert gh.gh_load(path.encode(), 2 * int(g["M"])) == 0
    for t in range(3):
        assert _double_term_check(gh, np.array([g["off%d_det" % t]], np.uint64), 1) == 0


def test_branch_free_doubles_two_word_keys(gh, tmp_path):
    from sfci_gb300 import fcidump as fd
    M, ne = 40, 10
    p = str(tmp_path / "d_IN")
    fd.uhf_to_in_file(p, M, ne, 3, 4)
    assert gh.gh_load(p.encode(), 2 * M) == 0
    rng = np.random.default_rng(5)
    for _ in range(3):
        occ = list(rng.choice(np.arange(0, 2 * M, 2), ne // 2, replace=False)) + \
              list(rng.choice(np.arange(1, 2 * M, 2), ne // 2, replace=False))
        lo = sum(1 << int(b) for b in occ if b < 64)
        hi = sum(1 << int(b - 64) for b in occ if b >= 64)
        assert _double_term_check(gh, np.array([lo, hi], np.uint64), 2) == 0

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

"""The drivers' small host linear algebra (csrc/hostla.h), compiled for the host:
the tridiagonal eigensolver of the subspace Lanczos iteration (Sturm bisection +
inverse iteration) against scipy's, and the pivoted-QR least squares of the
linear Krylov driver against numpy's."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "sfci_gb300", "csrc")
_f = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


@pytest.fixture(scope="module")
def hl(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("hl") / "hostla.so")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I" + CSRC,
           os.path.join(ROOT, "tests", "native", "hostla_host.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(so)
    L.hl_tri_lowest.argtypes = [C.c_int, _f, _f, C.c_int, _f, _f]
    L.hl_lstsq.argtypes = [C.c_int, C.c_int, _f, _f, _f]
    return L


def _lowest(hl, a, b, nev):
    m = a.size
    th = np.zeros(nev)
    v = np.zeros(nev * m)
    hl.hl_tri_lowest(m, np.ascontiguousarray(a), np.ascontiguousarray(np.append(b, 0.0)), nev, th, v)
    return th, v.reshape(nev, m)


def _check_pairs(a, b, th, V, tol):
    import scipy.linalg as sl
    ref, X = sl.eigh_tridiagonal(a, b)
    nev = th.size
    scale = max(1.0, np.max(np.abs(ref)))
    assert np.allclose(th, ref[:nev], rtol=0, atol=tol * scale)
    T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    for k in range(nev):
        assert abs(np.linalg.norm(V[k]) - 1.0) < 1e-12
        assert np.linalg.norm(T @ V[k] - th[k] * V[k]) < 100 * tol * scale
    assert np.allclose(V @ V.T, np.eye(nev), atol=1e-8)


@pytest.mark.parametrize("m", [1, 2, 5, 50, 300])
def test_tridiagonal_lowest_pairs(hl, m):
    rng = np.random.default_rng(m)
    a = rng.normal(size=m) * 3.0
    b = rng.normal(size=max(m - 1, 0))
    nev = min(m, 10)
    th, V = _lowest(hl, a, b, nev)
    _check_pairs(a, b, th, V, 1e-13)


def test_tridiagonal_close_pairs(hl):
    """Wilkinson's W21+: its top eigenvalues come in pairs agreeing to ~1e-14;
    the negated matrix puts them lowest."""
    a = -np.abs(np.arange(-10, 11)).astype(float)
    b = -np.ones(20)
    th, V = _lowest(hl, a, b, 6)
    _check_pairs(a, b, th, V, 1e-12)


def test_tridiagonal_lanczos_shaped(hl):
    """A Lanczos-like T: the lowest eigenvalues well separated, the rest dense."""
    rng = np.random.default_rng(7)
    m = 200
    a = np.concatenate([[-20.0, -15.0, -12.0], rng.uniform(0, 5, m - 3)])
    b = rng.uniform(0.01, 1.0, m - 1)
    th, V = _lowest(hl, a, b, 8)
    _check_pairs(a, b, th, V, 1e-13)


@pytest.mark.parametrize("m,n", [(2, 1), (6, 5), (31, 30), (10, 3)])
def test_least_squares_full_rank(hl, m, n):
    rng = np.random.default_rng(m * 100 + n)
    A = rng.normal(size=(m, n))
    e = rng.normal(size=m)
    y = np.zeros(n)
    hl.hl_lstsq(m, n, np.ascontiguousarray(A.T.reshape(-1)), e, y)
    ref = np.linalg.lstsq(A, e, rcond=None)[0]
    assert np.allclose(y, ref, rtol=1e-10, atol=1e-12)


def test_least_squares_rank_deficient(hl):
    """A repeated column: the basic solution leaves one of the pair at zero and
    reaches the least-squares residual."""
    rng = np.random.default_rng(3)
    A = rng.normal(size=(8, 4))
    A[:, 3] = A[:, 1]
    e = rng.normal(size=8)
    y = np.zeros(4)
    hl.hl_lstsq(8, 4, np.ascontiguousarray(A.T.reshape(-1)), e, y)
    ref = np.linalg.lstsq(A, e, rcond=None)[0]
    assert abs(np.linalg.norm(A @ y - e) - np.linalg.norm(A @ ref - e)) < 1e-10
    assert y[1] == 0.0 or y[3] == 0.0

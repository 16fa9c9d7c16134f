"""The C-ABI library: builds, loads, exports every declared entry point, and
rejects bad input before touching the GPU.  No device compute here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

import sfci_gb300 as sg


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(sfci_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = sg.load_library()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_gsaes_matches_scipy():
    import scipy.linalg as sl
    rng = np.random.default_rng(3)
    for n in (1, 3, 20, 40):
        A = rng.normal(size=(n, n))
        K = A + A.T
        B = rng.normal(size=(n, n))
        S = B @ B.T + n * np.eye(n)
        ev, X = sg.gsaes(K, S)
        ref = sl.eigh(K, S, eigvals_only=True)
        assert np.max(np.abs(ev - ref)) < 1e-11 * max(1.0, np.max(np.abs(ref)))
        assert np.max(np.abs(X.T @ S @ X - np.eye(n))) < 1e-10
        assert np.max(np.abs(K @ X - (S @ X) * ev)) < 1e-9


def test_gsaes_rejects_indefinite_overlap():
    with pytest.raises(sg.SfciError) as e:
        sg.gsaes(np.eye(2), np.array([[1.0, 2.0], [2.0, 1.0]]))
    assert e.value.status == "SFCI_ERR_NUMERIC"


def _create(path, norb, ne):
    L = sg.load_library()
    h = C.c_void_p()
    st = L.sfci_ctx_create(path.encode(), norb, ne, None, C.byref(h))
    return st, L


def test_missing_file_is_io_error(tmp_path):
    st, L = _create(str(tmp_path / "nope_IN"), 20, 10)
    assert L.sfci_status_name(st).decode() == "SFCI_ERR_IO"


def test_bad_sizes_rejected(tmp_path):
    p = tmp_path / "x_IN"
    p.write_text("0\n0\n0\n0\n0\n0\n0\n")
    for norb, ne in ((130, 4), (7, 2), (8, 8), (8, -1)):
        st, L = _create(str(p), norb, ne)
        assert L.sfci_status_name(st).decode() == "SFCI_ERR_ARG", (norb, ne)


def test_asymmetric_integrals_rejected(tmp_path):
    # (mn|pq) and (nm|pq) share a table slot; different values must be refused
    p = tmp_path / "asym_IN"
    p.write_text("2\n1.0 2 4 2 4\n2.0 4 2 2 4\n0\n0\n0\n0\n0\n0\n")
    st, L = _create(str(p), 4, 2)
    assert L.sfci_status_name(st).decode() == "SFCI_ERR_UNSUPPORTED"
    assert b"contradicts" in L.sfci_last_error()


def test_repeated_entry_rejected(tmp_path):
    p = tmp_path / "rep_IN"
    p.write_text("2\n1.0 2 4 3 5\n1.0 2 4 3 5\n0\n0\n0\n0\n0\n0\n")
    st, L = _create(str(p), 4, 2)
    assert L.sfci_status_name(st).decode() == "SFCI_ERR_UNSUPPORTED"


def test_keys_roundtrip_helpers():
    ints = [0, 1, (1 << 64) + 5, (1 << 127) | 3]
    k = sg.keys_from_ints(ints, 2)
    assert sg.ints_from_keys(k) == ints


def test_tag_keys_checks_instance_and_tag_bits():
    k = sg.keys_from_ints([(1 << 119) | 7, 3], 2)
    t = sg.tag_keys(k, 31)
    assert sg.ints_from_keys(t) == [(31 << 123) | (1 << 119) | 7, (31 << 123) | 3]
    assert sg.ints_from_keys(sg.tag_keys(k, 0)) == sg.ints_from_keys(k)
    assert sg.tag_keys(np.zeros((0, 2), np.uint64), 5).shape == (0, 2)
    for bad in (-1, 32):
        with pytest.raises(ValueError):
            sg.tag_keys(k, bad)
    with pytest.raises(ValueError):
        sg.tag_keys(t, 1)


def test_solver_entry_points_reject_null_arguments():
    """Argument checks of the linear-solver and subspace entry points run before
    any device call."""
    L = sg.load_library()
    name = lambda st: L.sfci_status_name(st).decode()
    d = C.c_double()
    n = C.c_uint64()
    assert name(L.sfci_spmspv_linear(None, None, None, 0.0, None, 1, None)) == "SFCI_ERR_ARG"
    assert name(L.sfci_res_norm(None, None, None, None, 0.0, C.byref(d))) == "SFCI_ERR_ARG"
    assert name(L.sfci_krylov_linear(None, None, None, 0.0, 5, 1, None)) == "SFCI_ERR_ARG"
    assert name(L.sfci_shift_invert(None, None, 0.0, 5, 1, C.byref(d))) == "SFCI_ERR_ARG"
    assert name(L.sfci_cisd(None, None, 0, 1, None, None, None, C.byref(n))) == "SFCI_ERR_ARG"
    assert name(L.sfci_fci(None, 1, None, None, None, C.byref(n))) == "SFCI_ERR_ARG"
    assert name(L.sfci_ctx_set_screen_guard(None, 1e-6)) == "SFCI_ERR_ARG"
    assert name(L.sfci_ctx_set_screen_floor(None, 1e-8)) == "SFCI_ERR_ARG"


def test_vec_create_rejects_oversized_capacity_without_a_device_call():
    """A capacity beyond 2^40 entries is SFCI_ERR_ARG before the context is read
    (the placeholder context address is never dereferenced)."""
    L = sg.load_library()
    h = C.c_void_p()
    st = L.sfci_vec_create(C.c_void_p(16), (1 << 40) + 1, C.byref(h))
    assert L.sfci_status_name(st).decode() == "SFCI_ERR_ARG" and not h.value
    assert L.sfci_status_name(L.sfci_vec_create(None, 1, C.byref(h))).decode() == "SFCI_ERR_ARG"


def test_dot_noalloc_rejects_bad_arguments_without_a_device_call():
    """sfci_dot_noalloc checks its arguments before any CUDA call: null pointers,
    a key width other than 1 or 2 words, and sizes beyond the fixed scratch
    array's 16,777,216 entries are SFCI_ERR_ARG (the pointers below are never
    dereferenced)."""
    L = sg.load_library()
    f = L.sfci_dot_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p,
                  C.c_void_p]
    name = lambda st: L.sfci_status_name(st).decode()
    p = 16  # a non-null placeholder address
    cases = [
        (p, p, 10, p, p, 10, 1, None),            # null d_out
        (None, p, 10, p, p, 10, 1, p),            # null x keys with nx > 0
        (p, None, 10, p, p, 10, 1, p),            # null x amplitudes
        (p, p, 10, None, p, 10, 1, p),            # null y keys with ny > 0
        (p, p, 10, p, None, 10, 2, p),            # null y amplitudes
        (p, p, 10, p, p, 10, 3, p),               # three-word keys
        (p, p, 10, p, p, 10, 0, p),               # zero-word keys
        (p, p, 1 << 24, p, p, 1, 1, p),           # nx + ny = 2^24 + 1
        (p, p, (1 << 24) + 1, p, p, 0, 1, p),     # nx alone beyond the limit
        (p, p, 0, p, p, (1 << 24) + 1, 2, p),     # ny alone beyond the limit
    ]
    for c in cases:
        st = f(c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], None)
        assert name(st) == "SFCI_ERR_ARG", c
    st = f(p, p, 1 << 24, p, p, 1, 1, p, None)
    assert b"16777216" in L.sfci_last_error()

"""The linear (shift-invert) solver on the device through the C ABI, against the
lin_*.npz fixtures (the reference's own spmspvm_bucket_linear and
spmspvm_bucket_res_norm, and the linear driver restated over them) and the
oracle restatement over the port backend.

Tolerances: single products at the parity bar of tests/parity.py (Hij: the
device sums term by term where the reference dots merged sums, so 1e-12
relative); driver results within 1e-8 relative (the restart loop amplifies
last-bit differences about tenfold per restart)."""
import numpy as np
import pytest

import sfci_gb300 as sg
from parity import close, compare_vectors

pytestmark = pytest.mark.gpu
CUT = 1e-5
NAMES = ("c1", "u8")


def _ctx(golden_in, name, nd_key="Nd"):
    g, path = golden_in("lin_" + name)
    return g, path, sg.Context(path, 2 * int(g["M"]), int(g["ne"]), Nd=int(g[nd_key]))


@pytest.mark.parametrize("name", NAMES)
def test_linear_products_match_reference(golden_in, name):
    g, _, c = _ctx(golden_in, name)
    cap, lam = int(g["cap"]), float(g["lam"])
    v1 = c.vec_from(g["v1_keys"], g["v1_amps"])
    w = c.vec_from(g["w_keys"], g["w_amps"])
    n0 = c.launches()
    out = c.vec(cap)
    h = c.spmspvm_bucket_linear(v1, out, lam, [v1])
    k, a = out.download()
    compare_vectors(g["P0_keys"], g["P0_amps"], k, a, cut=CUT, capped=len(a) == cap)
    assert all(close(x, y) for x, y in zip(h, g["P0_hij"]))
    h = c.spmspvm_bucket_linear(w, out, lam, [v1, w])
    k, a = out.download()
    compare_vectors(g["P1_keys"], g["P1_amps"], k, a, cut=CUT, capped=len(a) == cap)
    assert all(close(x, y) for x, y in zip(h, g["P1_hij"]))
    r = c.vec(cap)
    rn = c.spmspvm_bucket_res_norm(w, r, v1, lam)
    k, a = r.download()
    compare_vectors(g["R_keys"], g["R_amps"], k, a, cut=CUT, capped=len(a) == cap)
    assert close(rn, float(g["R_norm"]))
    assert c.launches() > n0


@pytest.mark.parametrize("name", NAMES)
def test_linear_driver_matches_reference(golden_in, name):
    g, _, c = _ctx(golden_in, name, "D_Nd")
    b = c.vec_from(g["v1_keys"], g["v1_amps"])
    x = c.vec(int(g["D_Nd"]))
    res = c.sparse_krylov_solve_linear(b, x, float(g["D_lam"]), int(g["D_iter"]), int(g["D_restarts"]))
    assert np.allclose(res, g["D_res"], rtol=1e-8, atol=0)
    k, a = x.download()
    compare_vectors(g["D_keys"], g["D_amps"], k, a, capped=True, rtol=1e-8, atol=1e-11, edge_rtol=1e-6)


def test_shift_invert_step_matches_oracle(golden_in, port):
    """sparse_solve_SI: the normalised solution and its calc_energy."""
    g, path, c = _ctx(golden_in, "u8", "D_Nd")
    Nd = int(g["D_Nd"])
    b = c.vec_from(g["v1_keys"], g["v1_amps"], cap=Nd)
    e = c.sparse_solve_SI(b, float(g["D_lam"]), 5, 3)
    k, a = b.download()
    be = port.PortLib(words=1)
    be.setup(path, 2 * int(g["M"]), int(g["ne"]), Nd, nthread=8)
    xk, xa, _ = port.krylov_linear(be, (g["v1_keys"], g["v1_amps"]), float(g["D_lam"]), 5, 3, Nd)
    xa = xa / np.linalg.norm(xa)
    compare_vectors(xk, xa, k, a, capped=True, rtol=1e-8, atol=1e-11, edge_rtol=1e-6)
    assert abs(e - be.energy(xk, xa)) < 1e-8


def test_two_word_keys_match_oracle(tmp_path, port):
    """66 spin orbitals: the linear product and the residual norm with two-word keys."""
    from sfci_gb300 import fcidump as fd
    M, ne = 33, 6
    p = str(tmp_path / "w_IN")
    fd.rhf_to_in_file(p, M, ne, 11)
    c = sg.Context(p, 2 * M, ne, Nd=100000)
    hf = (1 << ne) - 1
    v0 = c.vec_from(sg.keys_from_ints([hf], 2), np.array([1.0]))
    t = c.vec(3000)
    c.SpMVMtply_bucket(v0, t, 0.0, 1.0)
    tk, ta = t.download()
    ta = ta / np.linalg.norm(ta)
    w = c.vec_from(tk, ta)
    be = port.PortLib(words=2)
    be.setup(p, 2 * M, ne, 100000, nthread=8)
    lam = -1.0
    out = c.vec(2000)
    h = c.spmspvm_bucket_linear(w, out, lam, [v0, w])
    k, a = out.download()
    rk, ra, rh = be.spmspv_linear([(sg.keys_from_ints([hf], 2), np.array([1.0])), (tk, ta)], 1, lam, 2000)
    compare_vectors(rk, ra, k, a, cut=CUT, capped=len(a) == 2000)
    assert all(close(x, y) for x, y in zip(h, rh))
    r = c.vec(2000)
    rn = c.spmspvm_bucket_res_norm(w, r, v0, lam)
    k, a = r.download()
    rk, ra, rr = be.res_norm(tk, ta, sg.keys_from_ints([hf], 2), np.array([1.0]), lam, 2000)
    compare_vectors(rk, ra, k, a, cut=CUT, capped=len(a) == 2000)
    assert close(rn, rr)


def test_edge_cases(golden_in):
    g, _, c = _ctx(golden_in, "c1")
    lam = float(g["lam"])
    v1 = c.vec_from(g["v1_keys"], g["v1_amps"])
    empty = c.vec(10)
    out = c.vec(100)
    import ctypes as C
    h = np.full(1, 7.0)
    arr = (C.c_void_p * 1)(empty.h)
    st = c.L.sfci_spmspv_linear(c.h, empty.h, out.h, lam, arr, 1, h.ctypes.data_as(C.c_void_p))
    assert st == 0 and len(out) == 0 and h[0] == 7.0  # empty input: Hij left as it was
    r = c.vec(5000)
    rn = c.spmspvm_bucket_res_norm(empty, r, v1, lam)  # A x = 0: r = -b, |r| = |b|
    assert close(rn, float(np.linalg.norm(g["v1_amps"])))
    k, a = r.download()
    keep = np.abs(g["v1_amps"]) > CUT
    assert np.array_equal(k, g["v1_keys"][keep]) and np.array_equal(a, -g["v1_amps"][keep])

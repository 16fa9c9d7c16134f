"""The linear solver's oracle (the port's spmspv_linear / res_norm and
oracle.krylov_linear over them) against the lin_*.npz fixtures, which the
reference's own spmspvm_bucket_linear and spmspvm_bucket_res_norm produced
(src/functions.cpp:858-1269) and oracle.krylov_linear restated over them.

Tolerances: the parity bar of tests/parity.py for single products; driver
results within 1e-8 relative: each restart feeds a truncated, least-squares
solution into the next, and last-bit differences of the products (summation
order) grow about tenfold per restart (1e-14, 1e-10, 1e-9 measured over three)."""
import numpy as np
import pytest

from parity import close, compare_vectors

CUT = 1e-5
NAMES = ("c1", "u8")


def _wide(keys):
    k = np.asarray(keys, np.uint64)
    return np.stack([k, np.zeros_like(k)], axis=1)


def _be(port, golden_in, name, words=1):
    g, path = golden_in("lin_" + name)
    be = port.PortLib(words=words)
    be.setup(path, 2 * int(g["M"]), int(g["ne"]), int(g["Nd"]), nthread=8)
    return g, be


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("words", (1, 2))
def test_port_linear_products_match_reference(port, golden_in, name, words):
    g, be = _be(port, golden_in, name, words)
    conv = _wide if words == 2 else (lambda k: k)
    v1 = (conv(g["v1_keys"]), g["v1_amps"])
    w = (conv(g["w_keys"]), g["w_amps"])
    cap, lam = int(g["cap"]), float(g["lam"])
    k, a, h = be.spmspv_linear([v1], 0, lam, cap)
    compare_vectors(conv(g["P0_keys"]), g["P0_amps"], k, a, cut=CUT, capped=len(a) == cap)
    assert all(close(x, y) for x, y in zip(h, g["P0_hij"]))
    k, a, h = be.spmspv_linear([v1, w], 1, lam, cap)
    compare_vectors(conv(g["P1_keys"]), g["P1_amps"], k, a, cut=CUT, capped=len(a) == cap)
    assert all(close(x, y) for x, y in zip(h, g["P1_hij"]))
    k, a, r = be.res_norm(w[0], w[1], v1[0], v1[1], lam, cap)
    compare_vectors(conv(g["R_keys"]), g["R_amps"], k, a, cut=CUT, capped=len(a) == cap)
    assert close(r, float(g["R_norm"]))


@pytest.mark.parametrize("name", NAMES)
def test_port_linear_driver_matches_reference(port, golden_in, name):
    g, be = _be(port, golden_in, name)
    be.setup(golden_in("lin_" + name)[1], 2 * int(g["M"]), int(g["ne"]), int(g["D_Nd"]), nthread=8)
    xk, xa, rh = port.krylov_linear(be, (g["v1_keys"], g["v1_amps"]), float(g["D_lam"]), int(g["D_iter"]),
                                    int(g["D_restarts"]), int(g["D_Nd"]))
    assert np.allclose(rh, g["D_res"], rtol=1e-8, atol=0)
    compare_vectors(g["D_keys"], g["D_amps"], xk, xa, capped=True, rtol=1e-8, atol=1e-11, edge_rtol=1e-6)


def test_linear_driver_reduces_the_residual():
    from conftest import load_golden
    for name in NAMES:
        r = load_golden("lin_" + name)["D_res"]
        assert r[-1] < r[0]


def test_port_linear_driver_two_word_keys(port, golden_in):
    """The restated driver over the port's 128-bit backend gives the one-word
    fixture's run on a 64-bit system."""
    g, path = golden_in("lin_u8")
    be = port.PortLib(words=2)
    be.setup(path, 2 * int(g["M"]), int(g["ne"]), int(g["D_Nd"]), nthread=8)
    xk, xa, rh = port.krylov_linear(be, (_wide(g["v1_keys"]), g["v1_amps"]), float(g["D_lam"]), int(g["D_iter"]),
                                    int(g["D_restarts"]), int(g["D_Nd"]))
    assert np.allclose(rh, g["D_res"], rtol=1e-8, atol=0)
    compare_vectors(_wide(g["D_keys"]), g["D_amps"], xk, xa, capped=True, rtol=1e-8, atol=1e-11, edge_rtol=1e-6)

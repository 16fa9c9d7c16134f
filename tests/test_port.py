"""The oracle restatement (oracle/sfci_port.cpp) pinned against the reference's
own outputs (tests/golden, produced by the compiled reference sources)."""
import numpy as np
import pytest

from conftest import SYSTEMS
from parity import close, compare_vectors

CUT = 1e-5


def _setup(port, path, g, Nd):
    be = port.PortLib(words=1)
    be.setup(path, 2 * int(g["M"]), int(g["ne"]), int(Nd), nthread=4)
    return be


@pytest.mark.parametrize("name", SYSTEMS)
def test_diag_and_offdiag(port, golden_in, name):
    g, path = golden_in(name)
    be = _setup(port, path, g, 200000)
    d = be.diag(g["diag_dets"])
    assert np.allclose(d, g["diag_vals"], rtol=1e-13, atol=1e-13)
    for t in range(3):
        k, a = be.offdiag(np.array([g["off%d_det" % t]], np.uint64))
        u, inv = np.unique(k, return_inverse=True)
        s = np.zeros(u.size)
        np.add.at(s, inv, a)
        assert np.array_equal(u, g["off%d_keys" % t])
        assert np.allclose(s, g["off%d_amps" % t], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("name", SYSTEMS)
def test_spmspv_cases(port, golden_in, name):
    g, path = golden_in(name)
    be = _setup(port, path, g, 200000)
    if "A_keys" in g:
        k, a, d = be.spmspv(g["A_in_keys"], g["A_in_amps"], 2000000, 0.0, 1.0)
        compare_vectors(g["A_keys"], g["A_amps"], k, a, cut=CUT)
        assert close(d, float(g["A_diag"]))
    k, a, d = be.spmspv(g["B_in_keys"], g["B_in_amps"], int(g["B_cap"]), 0.0, 1.0)
    compare_vectors(g["B_keys"], g["B_amps"], k, a, cut=CUT, capped=len(g["B_amps"]) == int(g["B_cap"]))
    assert close(d, float(g["B_diag"]))
    be = _setup(port, path, g, int(g["C_Nd"]))
    k, a, d = be.spmspv(g["B_in_keys"], g["B_in_amps"], int(g["C_cap"]), float(g["C_lambda"]), float(g["C_coeff"]))
    compare_vectors(g["C_keys"], g["C_amps"], k, a, cut=CUT, capped=len(g["C_amps"]) == int(g["C_cap"]))
    assert close(d, float(g["C_diag"]))


@pytest.mark.parametrize("name", SYSTEMS)
def test_vector_algebra_and_energy(port, golden_in, name):
    g, path = golden_in(name)
    be = _setup(port, path, g, 200000)
    assert close(be.energy(g["B_in_keys"], g["B_in_amps"]), float(g["E_v1"]), 1e-12)
    assert close(be.energy(g["w_keys"], g["w_amps"]), float(g["E_w"]), 1e-12)
    kB, aB = g["B_keys"], g["B_amps"]
    assert close(be.dot(g["B_in_keys"], g["B_in_amps"], kB, aB), float(g["dot_v1_B"]))
    assert close(be.dot(g["w_keys"], g["w_amps"], kB, aB), float(g["dot_w_B"]))
    assert close(be.norm(kB, aB), float(g["norm_B"]))
    for cap in (10 ** 7, 1000):
        k, a = be.add_two(kB, aB, cap, g["B_in_keys"], g["B_in_amps"], -0.37)
        ref_k, ref_a = g["add2_%d_keys" % cap], g["add2_%d_amps" % cap]
        compare_vectors(ref_k, ref_a, k, a, capped=len(ref_a) == cap)
    be = _setup(port, path, g, int(g["add3_Nd"]))
    k, a = be.add_three(g["w_keys"], g["w_amps"], g["B_in_keys"], g["B_in_amps"], kB, aB, 0.5, -1.25, 0.75)
    compare_vectors(g["add3_keys"], g["add3_amps"], k, a, capped=len(g["add3_amps"]) == int(g["add3_Nd"]))
    k, a = be.shrink_from(kB, aB, int(g["shrink_cap"]))
    compare_vectors(g["shrink_keys"], g["shrink_amps"], k, a, capped=True)


@pytest.mark.parametrize("name", ["u8", "r16", "c1"])
def test_lanczos_energies(port, golden_in, name):
    g, path = golden_in(name)
    if "L_energies" not in g:
        pytest.skip("no Lanczos case")
    be = _setup(port, path, g, int(g["L_Nd"]))
    hf = np.array([g["hf"]], np.uint64)
    en, fe, _ = port.lanczos(be, hf, np.array([1.0]), int(g["L_Nl"]), int(g["L_restarts"]), int(g["L_Nd"]),
                             hpsi_cap=int(g["L_hpsi_cap"]))
    ref = g["L_energies"]
    assert len(en) == len(ref)
    assert np.max(np.abs(en - ref)) < 1e-8
    assert abs(fe - float(g["L_final_e"])) < 1e-8
    if "fci_energy" in g:
        assert abs(fe - float(g["fci_energy"])) < 1e-6

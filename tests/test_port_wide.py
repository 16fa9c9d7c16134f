"""The oracle restatement's two-word (128-bit) key path pinned against the
reference's own outputs.

The reference stops at 64 spin orbitals (src/main.cpp:84-85), so the
restatement's 128-bit path is the only checker for the 128-spin-orbital system.
Here it runs the golden systems (at most 64 spin orbitals) with every key
widened to two words, high word zero, and must reproduce the reference's
diagonal elements, emitted terms, SpMSpV products, energies, vector algebra and
Lanczos energies to the same tolerances as the one-word path
(tests/test_port.py): the key width changes the representation, not the
arithmetic.  The Lanczos runs take the two smaller systems, which keep the CPU
suite short."""
import numpy as np
import pytest

from conftest import SYSTEMS
from parity import close, compare_vectors

CUT = 1e-5


def wide(k):
    k = np.asarray(k, np.uint64).reshape(-1)
    return np.stack([k, np.zeros_like(k)], axis=1)


def narrow(k2):
    k2 = np.asarray(k2, np.uint64).reshape(-1, 2)
    assert not k2[:, 1].any()
    return k2[:, 0].copy()


def _setup(port, path, g, Nd):
    be = port.PortLib(words=2)
    be.setup(path, 2 * int(g["M"]), int(g["ne"]), int(Nd), nthread=4)
    return be


@pytest.mark.parametrize("name", SYSTEMS)
def test_diag_and_offdiag_wide(port, golden_in, name):
    g, path = golden_in(name)
    be = _setup(port, path, g, 200000)
    d = be.diag(wide(g["diag_dets"]))
    assert np.allclose(d, g["diag_vals"], rtol=1e-13, atol=1e-13)
    for t in range(3):
        k2, a = be.offdiag(wide([g["off%d_det" % t]]))
        k = narrow(k2)
        u, inv = np.unique(k, return_inverse=True)
        s = np.zeros(u.size)
        np.add.at(s, inv, a)
        assert np.array_equal(u, g["off%d_keys" % t])
        assert np.allclose(s, g["off%d_amps" % t], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("name", SYSTEMS)
def test_spmspv_cases_wide(port, golden_in, name):
    g, path = golden_in(name)
    be = _setup(port, path, g, 200000)
    if "A_keys" in g:
        k, a, d = be.spmspv(wide(g["A_in_keys"]), g["A_in_amps"], 2000000, 0.0, 1.0)
        compare_vectors(g["A_keys"], g["A_amps"], narrow(k), a, cut=CUT)
        assert close(d, float(g["A_diag"]))
    k, a, d = be.spmspv(wide(g["B_in_keys"]), g["B_in_amps"], int(g["B_cap"]), 0.0, 1.0)
    compare_vectors(g["B_keys"], g["B_amps"], narrow(k), a, cut=CUT, capped=len(g["B_amps"]) == int(g["B_cap"]))
    assert close(d, float(g["B_diag"]))
    be = _setup(port, path, g, int(g["C_Nd"]))
    k, a, d = be.spmspv(wide(g["B_in_keys"]), g["B_in_amps"], int(g["C_cap"]), float(g["C_lambda"]),
                        float(g["C_coeff"]))
    compare_vectors(g["C_keys"], g["C_amps"], narrow(k), a, cut=CUT, capped=len(g["C_amps"]) == int(g["C_cap"]))
    assert close(d, float(g["C_diag"]))


@pytest.mark.parametrize("name", SYSTEMS)
def test_vector_algebra_and_energy_wide(port, golden_in, name):
    g, path = golden_in(name)
    be = _setup(port, path, g, 200000)
    v1k, wk, kB = wide(g["B_in_keys"]), wide(g["w_keys"]), wide(g["B_keys"])
    v1a, wa, aB = g["B_in_amps"], g["w_amps"], g["B_amps"]
    assert close(be.energy(v1k, v1a), float(g["E_v1"]), 1e-12)
    assert close(be.energy(wk, wa), float(g["E_w"]), 1e-12)
    assert close(be.dot(v1k, v1a, kB, aB), float(g["dot_v1_B"]))
    assert close(be.dot(wk, wa, kB, aB), float(g["dot_w_B"]))
    assert close(be.norm(kB, aB), float(g["norm_B"]))
    for cap in (10 ** 7, 1000):
        k, a = be.add_two(kB, aB, cap, v1k, v1a, -0.37)
        ref_k, ref_a = g["add2_%d_keys" % cap], g["add2_%d_amps" % cap]
        compare_vectors(ref_k, ref_a, narrow(k), a, capped=len(ref_a) == cap)
    be = _setup(port, path, g, int(g["add3_Nd"]))
    k, a = be.add_three(wk, wa, v1k, v1a, kB, aB, 0.5, -1.25, 0.75)
    compare_vectors(g["add3_keys"], g["add3_amps"], narrow(k), a, capped=len(g["add3_amps"]) == int(g["add3_Nd"]))
    k, a = be.shrink_from(kB, aB, int(g["shrink_cap"]))
    compare_vectors(g["shrink_keys"], g["shrink_amps"], narrow(k), a, capped=True)


@pytest.mark.parametrize("name", ["u8", "r16"])
def test_lanczos_energies_wide(port, golden_in, name):
    g, path = golden_in(name)
    if "L_energies" not in g:
        pytest.skip("no Lanczos case")
    be = _setup(port, path, g, int(g["L_Nd"]))
    en, fe, _ = port.lanczos(be, wide([g["hf"]]), np.array([1.0]), int(g["L_Nl"]), int(g["L_restarts"]),
                             int(g["L_Nd"]), hpsi_cap=int(g["L_hpsi_cap"]))
    ref = g["L_energies"]
    assert len(en) == len(ref)
    assert np.max(np.abs(en - ref)) < 1e-8
    assert abs(fe - float(g["L_final_e"])) < 1e-8

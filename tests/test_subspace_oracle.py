"""The restated calc_CISD / fci oracle (oracle.cisd, oracle.fci) over the port
backend, pinned to the sub_*.npz fixtures that the same restatement produced
over the reference's own DiagCal_bit and OffDiagGen_bit_e.

Tolerances: eigenvalues within 1e-10 Eh; eigenvector amplitudes within 1e-9
(unit vectors; the port's matrix elements differ from the reference's in the
last bits only, and the smallest gap among the compared states is 5e-3)."""
import numpy as np
import pytest

from conftest import load_golden

SUB = ("c1", "r16", "u8")
FCI = ("u8", "r8")


def _port(port, golden_in, name, words=1):
    g, path = golden_in("sub_" + name)
    be = port.PortLib(words=words)
    be.setup(path, 2 * int(g["M"]), int(g["ne"]), 200000, nthread=8)
    return g, be


def _wide(keys):
    k = np.asarray(keys, np.uint64)
    return np.stack([k, np.zeros_like(k)], axis=1)


@pytest.mark.parametrize("name", SUB)
def test_cisd_oracle_matches_reference(port, golden_in, name):
    g, be = _port(port, golden_in, name)
    hf = int(g["hf"])
    states = sorted(int(k[4:-5]) for k in g if k.startswith("cisd") and k.endswith("_amps"))
    for st in states:
        k, a, ev = port.cisd(be, hf, st, 10)
        assert np.array_equal(k, g["cisd_keys"])
        assert np.allclose(ev, g["cisd_evals"], rtol=0, atol=1e-10)
        assert np.allclose(a, g["cisd%d_amps" % st], rtol=0, atol=1e-9)


def test_cisd_block_is_singles_and_doubles():
    """The reference's block (distinct OffDiagGen_bit_e targets of the reference
    determinant, plus itself) has 1 + S + dSS + dOS members for these inputs."""
    c2 = lambda x: x * (x - 1) // 2
    for name in SUB:
        g = load_golden("sub_" + name)
        M, ne = int(g["M"]), int(g["ne"])
        na = nb = ne // 2
        size = 1 + na * (M - na) + nb * (M - nb) + c2(na) * c2(M - na) + c2(nb) * c2(M - nb) \
            + na * (M - na) * nb * (M - nb)
        assert g["cisd_keys"].size == size


@pytest.mark.parametrize("name", FCI)
def test_fci_oracle_matches_reference(port, golden_in, name):
    g, be = _port(port, golden_in, name)
    ev, k, a = port.fci(be, 2 * int(g["M"]), int(g["ne"]), 5)
    assert np.array_equal(k, g["fci_keys"])
    assert np.allclose(ev, g["fci_evals"], rtol=0, atol=1e-10)
    assert np.allclose(a, g["fci_amps"], rtol=0, atol=1e-9)


def test_fci_agrees_with_the_older_dense_fixture():
    """sub_u8's ground energy equals u8.npz's independently assembled dense FCI."""
    assert abs(float(load_golden("sub_u8")["fci_evals"][0]) - float(load_golden("u8")["fci_energy"])) < 1e-11


def test_two_word_oracle_path_matches_one_word(port, golden_in):
    """oracle.cisd / oracle.fci with 128-bit keys give the one-word results on a
    64-bit system."""
    g, be = _port(port, golden_in, "u8", words=2)
    hf = np.array([[int(g["hf"]), 0]], np.uint64)
    k, a, ev = port.cisd(be, hf, 0, 10)
    assert np.array_equal(k, _wide(g["cisd_keys"]))
    assert np.allclose(a, g["cisd0_amps"], rtol=0, atol=1e-9)
    ev2, k2, a2 = port.fci(be, 2 * int(g["M"]), int(g["ne"]), 5)
    assert np.array_equal(k2, _wide(g["fci_keys"]))
    assert np.allclose(ev2, g["fci_evals"], rtol=0, atol=1e-10)
    assert np.allclose(a2, g["fci_amps"], rtol=0, atol=1e-9)


def test_fix_sign_convention(port):
    x = np.array([0.1, -0.7, 0.7, 0.2])
    assert np.array_equal(port.fix_sign(x), -x)  # first of the tied largest is negative
    assert np.array_equal(port.fix_sign(-x), -x)

"""Subspace eigenproblems on the device (calc_CISD, fci) through the C ABI,
against the sub_*.npz fixtures (dense diagonalisation of the reference's own
matrix elements) and the oracle restatement over the port backend.

Tolerances: eigenvalues within 1e-9 Eh; unit eigenvectors within 1e-8 per
amplitude (Lanczos stops at Ritz residuals below 1e-11 relative; the smallest
gap among the compared states is 5e-3); residual norms below 1e-8."""
import numpy as np
import pytest

import sfci_gb300 as sg
from conftest import load_golden

pytestmark = pytest.mark.gpu

EV_TOL = 1e-9
VEC_TOL = 1e-8


def _ctx(golden_in, name):
    g, path = golden_in("sub_" + name)
    return g, path, sg.Context(path, 2 * int(g["M"]), int(g["ne"]), Nd=200000)


@pytest.mark.parametrize("name", ("c1", "r16", "u8"))
def test_cisd_matches_reference(golden_in, name):
    g, _, c = _ctx(golden_in, name)
    n0 = c.launches()
    states = sorted(int(k[4:-5]) for k in g if k.startswith("cisd") and k.endswith("_amps"))
    for st in states:
        v, ev, r = c.calc_CISD(int(g["hf"]), st, 10)
        k, a = v.download()
        assert np.array_equal(k, g["cisd_keys"])
        assert np.allclose(ev, g["cisd_evals"], rtol=0, atol=EV_TOL)
        assert np.allclose(a, g["cisd%d_amps" % st], rtol=0, atol=VEC_TOL)
        assert r < 1e-8
        assert abs(np.linalg.norm(a) - 1.0) < 1e-12
    assert c.launches() > n0


@pytest.mark.parametrize("name", ("u8", "r8"))
def test_fci_matches_reference(golden_in, name):
    g, _, c = _ctx(golden_in, name)
    ev, v, r = c.fci(5)
    k, a = v.download()
    assert np.array_equal(k, g["fci_keys"])
    assert np.allclose(ev, g["fci_evals"], rtol=0, atol=EV_TOL)
    assert np.allclose(a, g["fci_amps"], rtol=0, atol=VEC_TOL)
    assert r < 1e-8


def test_fci_full_space_of_the_20_orbital_case(golden_in):
    """63,504 determinants (no dense oracle fits): the ground state's Rayleigh
    quotient through calc_energy (hash-probe path) equals the eigenvalue, the
    energy lies below the CISD energy and the truncated SFCI energy (variational),
    and the residual is small."""
    g, _, c = _ctx(golden_in, "c1")
    ev, v, r = c.fci(3)
    assert len(v) == 63504
    assert r < 1e-8
    assert abs(c.calc_energy(v) - ev[0]) < 1e-9
    assert ev[0] < float(g["cisd_evals"][0])
    assert ev[0] <= float(load_golden("c1")["L_final_e"]) + 1e-9
    assert ev[0] < ev[1] < ev[2]


def test_two_word_keys_match_oracle(tmp_path, port):
    """66 spin orbitals (two-word keys): CISD with 4 electrons and FCI with 2,
    against the oracle restatement with the port's 128-bit backend."""
    from sfci_gb300 import fcidump as fd
    M = 33
    for ne in (4, 2):
        p = str(tmp_path / ("w%d_IN" % ne))
        fd.rhf_to_in_file(p, M, ne, 11)
        c = sg.Context(p, 2 * M, ne, Nd=200000)
        assert c.words == 2
        be = port.PortLib(words=2)
        be.setup(p, 2 * M, ne, 200000, nthread=8)
        hf = (1 << ne) - 1
        if ne == 4:
            v, ev, r = c.calc_CISD(hf, 1, 4)
            k, a = v.download()
            rk, ra, rev = port.cisd(be, sg.keys_from_ints([hf], 2), 1, 4)
        else:
            ev, v, r = c.fci(4)
            k, a = v.download()
            rev, rk, ra = port.fci(be, 2 * M, ne, 4)
        assert np.array_equal(k, rk)
        assert np.allclose(ev, rev, rtol=0, atol=EV_TOL)
        assert np.allclose(a, ra, rtol=0, atol=VEC_TOL)
        assert r < 1e-8


def test_argument_errors(golden_in):
    g, path, c = _ctx(golden_in, "c1")
    small = c.vec(10)
    ev = np.zeros(2)
    import ctypes as C
    key = sg.keys_from_ints([int(g["hf"])], 1)
    bs = C.c_uint64()
    st = c.L.sfci_cisd(c.h, key.ctypes.data_as(C.c_void_p), 0, 2, ev.ctypes.data_as(C.c_void_p), small.h, None,
                       C.byref(bs))
    assert st != 0 and bs.value == 876  # capacity error, block size reported first
    with pytest.raises(sg.SfciError):
        c.calc_CISD(int(g["hf"]) | (1 << 12), 0, 1)  # wrong electron count
    odd = sg.Context(path, 2 * int(g["M"]), 9, Nd=1000)
    with pytest.raises(sg.SfciError):
        odd.fci(1)  # the FCI block is Sz = 0: needs an even electron count

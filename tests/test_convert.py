"""FCIDUMP -> _IN converter and the synthetic generator, against the reference converter's output."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN, SYSTEMS, load_golden
from sfci_gb300 import fcidump as fd


@pytest.mark.parametrize("kind,M", [("rhf", 4), ("uhf", 4), ("rhf", 6)])
def test_converter_byte_identical(tmp_path, kind, M):
    p = str(tmp_path / "sys_fcidump")
    if kind == "rhf":
        h, q, v, e = fd.synthetic_rhf(M, 7)
        fd.write_fcidump_rhf(p, h, q, v, e, 4)
        groups = fd.convert_rhf(p)
    else:
        hs, aa, bb, ab, e = fd.synthetic_uhf(M, 8, 9)
        fd.write_fcidump_uhf(p, hs, aa, bb, ab, e, 4)
        groups = fd.convert_uhf(p)
    out = str(tmp_path / "mine_IN")
    fd.write_in(out, groups)
    ref = open(os.path.join(GOLDEN, "conv_%s_m%d_IN" % (kind, M))).read()
    assert open(out).read() == ref


@pytest.mark.parametrize("name", SYSTEMS)
def test_golden_systems_regenerate_identically(golden_in, name):
    g, path = golden_in(name)
    assert hashlib.sha256(open(path, "rb").read()).hexdigest() == str(g["in_sha256"])


def test_synthetic_distributions():
    h, (i, j, k, l), v, e = fd.synthetic_rhf(10, 0)
    assert np.allclose(np.diag(h), -3.0 + 0.25 * np.arange(10))
    assert np.allclose(h, h.T)
    coul = (i == j) & (k == l)
    assert np.all((v[coul] >= 0.3) & (v[coul] <= 0.8))
    exch = ~coul & (((i == k) & (j == l)) | ((i == l) & (j == k)))
    assert np.all((v[exch] >= 0.01) & (v[exch] <= 0.1))
    # canonical uniqueness: i>=j, k>=l, ij>=kl
    assert np.all(i >= j) and np.all(k >= l)
    assert e == 0.0


def test_namelist_terminator_required(tmp_path):
    p = tmp_path / "bad_fcidump"
    p.write_text(" &FCI NORB=2,NELEC=2,\n/\n 1.0 1 1 1 1\n")
    with pytest.raises(ValueError):
        fd.read_fcidump(str(p))

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SYSTEMS = ("c1", "u8", "r16", "r28")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


_IN_CACHE = {}


def in_file_for(g, tmpdir_factory):
    """Regenerate the _IN file of a golden system with this repo's converter."""
    from sfci_gb300 import fcidump as fd
    key = (str(g["kind"]), int(g["M"]), int(g["ne"]), tuple(int(s) for s in g["seeds"]))
    if key in _IN_CACHE:
        return _IN_CACHE[key]
    d = str(tmpdir_factory.mktemp("in"))
    p = os.path.join(d, "sys_IN")
    if key[0] == "rhf":
        fd.rhf_to_in_file(p, key[1], key[2], key[3][0], fcidump_path=os.path.join(d, "sys_fcidump"))
    else:
        fd.uhf_to_in_file(p, key[1], key[2], key[3][0], key[3][1], fcidump_path=os.path.join(d, "sys_fcidump"))
    _IN_CACHE[key] = p
    return p


@pytest.fixture(scope="session")
def golden_in(tmp_path_factory):
    def get(name):
        g = load_golden(name)
        return g, in_file_for(g, tmp_path_factory)
    return get


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as orc
    orc.build_port()
    return orc

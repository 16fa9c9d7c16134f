"""The drop-in `sfci` binary on a reference run directory (sfci.input + _IN file)
for the 20-spin-orbital, 10-electron system: its printed E_hf, per-restart "gsaes energy" and
"final e" lines against the reference driver's golden values (within 1e-8 Eh,
the Lanczos parity bar)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

@pytest.mark.gpu
def test_sfci_binary_reproduces_the_reference_run(golden_in, tmp_path):
    from sfci_gb300 import build as b
    b.build()
    g, path = golden_in("c1")
    shutil.copy(path, tmp_path / "c1_IN")
    (tmp_path / "sfci.input").write_text(
        "task=ground\nNd=%d\nNl=%d\nnum_restart=%d\nnum_orb=20\nnum_e=10\ninit_hf=1023\nbucket_unit=60000\n"
        "num_thread=16\nfilename=c1_IN\n" % (int(g["L_Nd"]), int(g["L_Nl"]), int(g["L_restarts"])))
    r = subprocess.run([b.EXE], cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    ehf = float(re.search(r"E_hf:(\S+)", out).group(1))
    hf_idx = [int(x) for x in g["diag_dets"]].index(1023)
    assert abs(ehf - float(g["diag_vals"][hf_idx])) < 1e-10
    energies = [float(x) for x in re.findall(r"gsaes energy:(\S+)", out)]
    ref = np.asarray(g["L_energies"], float)
    assert len(energies) == ref.size
    assert np.allclose(energies, ref, rtol=0, atol=1e-8)
    fe = float(re.search(r"final e:(\S+)", out).group(1))
    assert abs(fe - float(g["L_final_e"])) < 1e-8
    assert "SFCI time:" in out


def test_sfci_binary_reports_a_missing_integral_file(tmp_path):
    """Runs without a GPU: the integral file is read before any device call."""
    from sfci_gb300 import build as b
    b.build()
    (tmp_path / "sfci.input").write_text("task=ground\nNd=100\nNl=5\nnum_restart=1\nnum_orb=20\nnum_e=10\n"
                                         "init_hf=1023\nfilename=missing_IN\n")
    r = subprocess.run([b.EXE], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "sfci:" in r.stderr


@pytest.mark.parametrize("lines,msg", [
    ("Nd=abc\n", "bad value for Nd"),
    ("num_orb=twenty\n", "bad value for num_orb"),
    ("Nl=99999999999999999999\n", "bad value for Nl"),
    ("init_hf=10x23\n", "init_hf must be a decimal integer"),
    ("init_hf=340282366920938463463374607431768211456\n", "init_hf must be a decimal integer"),  # 2^128
    ("init_hf=1048576\n", "at or above num_orb=20"),  # bit 20 of a 20-spin-orbital system
])
def test_sfci_binary_rejects_bad_input_values(tmp_path, lines, msg):
    """Runs without a GPU: sfci.input is parsed and checked before any device call.
    A malformed number or an init_hf that does not fit num_orb spin orbitals is an
    error message and exit status 1, not an abort."""
    from sfci_gb300 import build as b
    b.build()
    base = {"task": "ground", "Nd": "100", "Nl": "5", "num_restart": "1", "num_orb": "20", "num_e": "10",
            "init_hf": "1023", "filename": "missing_IN"}
    k = lines.split("=", 1)[0]
    base[k] = lines.split("=", 1)[1].strip()
    (tmp_path / "sfci.input").write_text("".join("%s=%s\n" % kv for kv in base.items()))
    r = subprocess.run([b.EXE], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    assert r.returncode == 1, (r.returncode, r.stderr)
    assert msg in r.stderr, r.stderr

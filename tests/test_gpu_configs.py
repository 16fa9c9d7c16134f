"""Parity on the systems of the benchmark configurations, through the C ABI.

* The 56-spin-orbital, 14-electron RHF system of seed 1: the truncated Lanczos
  driver (sparse_krylov_solve_eigenval, src/sparse_solver.cpp:246-548) at a
  truncating Nd against the same driver over the compiled reference's own
  SpMSpV and vector algebra (tests/golden/lz_r28.npz), within 1e-8 Eh.
* The 128-spin-orbital, 20-electron UHF system of seeds 2 (alpha) and 3 (beta),
  two-word keys: one SpMSpV of a 1,000-determinant vector, calc_energy,
  DiagCal_bit, a short truncated Lanczos run, and one MINRES correction at
  lambda = that Lanczos energy with tol 1e-8 (minres_sp, src/minres.cpp:73-225),
  each against the oracle restatement's 128-bit path (the reference itself
  stops at 64 spin orbitals, src/main.cpp:84-85).

Tolerances are those of tests/parity.py: key sets bit-exact off the selection
edges, amplitudes within 1e-12 relative (MINRES vectors, whose coefficients
come from square roots and divisions of dots, within 1e-9), scalars within
1e-12, energies within 1e-8 Eh."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from parity import close, compare_vectors

import sfci_gb300 as sg

pytestmark = pytest.mark.gpu
CUT = 1e-5


def test_lanczos_56_orbital_system_truncating(golden_in):
    """The 56-spin-orbital system at Nd = 2e4, Nl = 30: the energies of every restart and
    the final calc_energy against the reference driver.  The reference's signed
    convergence test (previousE - E < dE with previousE = 0, :535) ends a run
    with a positive energy after its first restart, and so does this one.  The
    same driver over the oracle restatement, which breaks magnitude ties at the
    top-Nd edges by key where the reference's introsort breaks them arbitrarily,
    is recorded beside it: the spread between the two CPU runs is how far
    tie-breaking alone moves the energy on this RHF system, whose spin-mirror
    determinants tie exactly."""
    g = load_golden("lz_r28")
    _, path = golden_in("r28")
    c = sg.Context(path, 56, 14, Nd=int(g["L_Nd"]), hpsi_cap=int(g["L_hpsi_cap"]))
    v = c.vec(int(g["L_Nd"]))
    v.upload(np.array([g["hf"]], np.uint64), np.array([1.0]))
    en, fe = c.sparse_krylov_solve_eigenval(v, int(g["L_Nl"]), int(g["L_restarts"]))
    en = en[~np.isnan(en)]
    ref, alt = g["L_energies"], g["P_energies"]
    spread = float(np.max(np.abs(ref - alt))) if len(alt) == len(ref) else float("nan")
    print("56-spin-orbital Lanczos at Nd=%d: GPU %s (final %.12f), reference %s (final %.12f), "
          "max |GPU - reference| %.3e, tie-breaking spread of the CPU runs %.3e"
          % (int(g["L_Nd"]), en, fe, ref, float(g["L_final_e"]), np.max(np.abs(en - ref)), spread))
    assert len(en) == len(ref)
    assert np.max(np.abs(en - ref)) < 1e-8
    assert abs(fe - float(g["L_final_e"])) < 1e-8


@pytest.fixture(scope="module")
def sys128(tmp_path_factory):
    from sfci_gb300 import fcidump as fd
    p = str(tmp_path_factory.mktemp("u64") / "u64_IN")
    fd.uhf_to_in_file(p, 64, 20, 2, 3)
    return p


def _sample_vector(rng, N, ne, n):
    """|HF> and random Sz-preserving excitations of it (ranks 1..4), normalised
    amplitudes spread over several decades."""
    hf = (1 << ne) - 1
    occ = [b for b in range(N) if hf >> b & 1]
    out = {hf}
    while len(out) < n:
        d = hf
        for _ in range(int(rng.integers(1, 5))):
            i = int(rng.choice(occ))
            if not d >> i & 1:
                continue
            cand = [a for a in range(N) if (a & 1) == (i & 1) and not d >> a & 1]
            d ^= (1 << i) ^ (1 << int(rng.choice(cand)))
        out.add(d)
    ints = sorted(out)
    amps = rng.normal(size=len(ints)) * np.exp(-rng.uniform(0, 5, size=len(ints)))
    return ints, amps / np.linalg.norm(amps)


def test_128_orbital_system_products_lanczos_and_minres(sys128, port):
    N, ne = 128, 20
    rng = np.random.default_rng(23)
    ints, amps = _sample_vector(rng, N, ne, 1000)
    keys = sg.keys_from_ints(ints, 2)
    be = port.PortLib(words=2)
    be.setup(sys128, N, ne, 200000, nthread=os.cpu_count())
    c = sg.Context(sys128, N, ne, Nd=200000)
    assert c.words == 2
    # SpMSpV of the whole vector (SpMVMtply_bucket, src/functions.cpp:511-804)
    vin = c.vec_from(keys, amps)
    out = c.vec(4000000)
    d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    st = c.last_stats()
    assert st["terms"] == 1000 * (421470 + 1)
    k, a = out.download()
    rk, ra, rd = be.spmspv(keys, amps, 4000000, 0.0, 1.0)
    rep = compare_vectors(rk, ra, k, a, cut=CUT, capped=len(ra) == 4000000)
    assert close(d, rd)
    print("128-orbital SpMSpV: %d determinants, max rel diff %.2e" % (rep["common"], rep["max_rel"]))
    # the same product in class passes (a 3 GB budget: several passes, each
    # generating only the terms whose target alpha class it owns): bit for bit
    cc = sg.Context(sys128, N, ne, Nd=200000, mem_budget=3 << 30)
    cc.set_class_passes(1)
    out_c = cc.vec(4000000)
    d_c = cc.SpMVMtply_bucket(cc.vec_from(keys, amps), out_c, 0.0, 1.0)
    kc, ac = out_c.download()
    assert cc.last_stats()["passes"] > 1
    assert np.array_equal(kc, k) and np.array_equal(ac.view(np.uint64), a.view(np.uint64))
    assert close(d_c, d)
    del cc, out_c
    # top-Nd slice, shift and a negative coefficient, capped output
    c.set_Nd(400)
    be.set_nd(400)
    out2 = c.vec(5000)
    d2 = c.SpMVMtply_bucket(vin, out2, -3.25, -0.5)
    k2, a2 = out2.download()
    rk2, ra2, rd2 = be.spmspv(keys, amps, 5000, -3.25, -0.5)
    compare_vectors(rk2, ra2, k2, a2, cut=CUT, capped=True)
    assert close(d2, rd2)
    # calc_energy (src/functions.cpp:1272-1313) and DiagCal_bit (src/bitstr.cpp:433-476)
    assert close(c.calc_energy(vin), be.energy(keys, amps))
    assert np.allclose(c.DiagCal_bit(keys[:50]), be.diag(keys[:50]), rtol=1e-13, atol=1e-13)
    # a short truncated Lanczos run from |HF> (UHF: no spin-mirror ties at the edges)
    Nd, Nl = 300, 8
    c.set_Nd(Nd)
    be.set_nd(Nd)
    hf = sg.keys_from_ints([(1 << ne) - 1], 2)
    v = c.vec(Nd)
    v.upload(hf, np.array([1.0]))
    en, fe = c.sparse_krylov_solve_eigenval(v, Nl, 1)
    en = en[~np.isnan(en)]
    ren, rfe, _ = port.lanczos(be, hf, np.array([1.0]), Nl, 1, Nd)
    print("128-orbital Lanczos at Nd=%d, Nl=%d: GPU %s, oracle %s" % (Nd, Nl, en, ren))
    assert len(en) == len(ren) and np.max(np.abs(en - ren)) < 1e-8
    assert abs(fe - rfe) < 1e-8
    # one MINRES correction at lambda = the Lanczos energy, tol 1e-8 (the squared
    # residual is compared with tol, src/minres.cpp:211)
    lam = float(en[-1])
    Ndm = 500
    c.set_Nd(Ndm)
    be.set_nd(Ndm)
    top = np.sort(np.argsort(-np.abs(amps), kind="stable")[:Ndm])
    bk, ba = keys[top], amps[top] / np.linalg.norm(amps[top])
    rhs = c.vec_from(bk, ba, cap=Ndm)
    guess = c.vec(Ndm)
    res = c.vec(Ndm)
    it = c.minres_sp(rhs, guess, res, 6, 1e-8, lam)
    (xk, xa), it2 = port.minres(be, (bk, ba), (np.zeros((0, 2), np.uint64), np.zeros(0)), 6, 1e-8, lam, Ndm)
    assert it == it2
    k3, a3 = res.download()
    rep = compare_vectors(xk, xa, k3, a3, capped=len(xa) == Ndm, rtol=1e-9, atol=1e-12)
    print("128-orbital MINRES at lambda=%.10f: %d iterations, max rel diff %.2e" % (lam, it, rep["max_rel"]))

"""GPU hot path through the C ABI, against the reference's golden outputs and the
oracle restatement (same seeded inputs).

Tolerances (see tests/parity.py): key sets bit-exact except keys on a selection
edge (the 1e-5 cut or a top-cap tie); amplitudes within 1e-12 relative with a
1e-14 absolute floor; scalar products within 1e-12 relative; Lanczos energies
within 1e-8 Eh of the reference driver."""
import numpy as np
import pytest

from conftest import SYSTEMS
from parity import close, compare_vectors

import sfci_gb300 as sg

pytestmark = pytest.mark.gpu
CUT = 1e-5


def ctx_for(golden_in, name, Nd=200000, **kw):
    g, path = golden_in(name)
    return g, path, sg.Context(path, 2 * int(g["M"]), int(g["ne"]), Nd=Nd, **kw)


@pytest.mark.parametrize("name", SYSTEMS)
def test_diag_elements(golden_in, name):
    g, _, c = ctx_for(golden_in, name)
    d = c.DiagCal_bit(g["diag_dets"])
    assert np.allclose(d, g["diag_vals"], rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("name", SYSTEMS)
def test_spmspv_matches_reference(golden_in, name):
    g, path, c = ctx_for(golden_in, name)
    n0 = c.launches()
    if "A_keys" in g:
        vin = c.vec_from(g["A_in_keys"], g["A_in_amps"])
        out = c.vec(2000000)
        d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
        k, a = out.download()
        compare_vectors(g["A_keys"], g["A_amps"], k, a, cut=CUT)
        assert close(d, float(g["A_diag"]))
    vin = c.vec_from(g["B_in_keys"], g["B_in_amps"])
    out = c.vec(int(g["B_cap"]))
    d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    k, a = out.download()
    compare_vectors(g["B_keys"], g["B_amps"], k, a, cut=CUT, capped=len(g["B_amps"]) == int(g["B_cap"]))
    assert close(d, float(g["B_diag"]))
    # top-Nd of the input, energy shift, negative coefficient, capped output
    c.set_Nd(int(g["C_Nd"]))
    out = c.vec(int(g["C_cap"]))
    d = c.SpMVMtply_bucket(vin, out, float(g["C_lambda"]), float(g["C_coeff"]))
    k, a = out.download()
    compare_vectors(g["C_keys"], g["C_amps"], k, a, cut=CUT, capped=len(g["C_amps"]) == int(g["C_cap"]))
    assert close(d, float(g["C_diag"]))
    assert c.launches() > n0  # the CUDA path ran


@pytest.mark.parametrize("name", SYSTEMS)
def test_vector_algebra_and_energy(golden_in, name):
    g, path, c = ctx_for(golden_in, name)
    v1 = c.vec_from(g["B_in_keys"], g["B_in_amps"])
    w = c.vec_from(g["w_keys"], g["w_amps"])
    B = c.vec_from(g["B_keys"], g["B_amps"], cap=max(len(g["B_amps"]), 1))
    assert close(c.calc_energy(v1), float(g["E_v1"]))
    assert close(c.calc_energy(w), float(g["E_w"]))
    assert close(v1.dot(B), float(g["dot_v1_B"]))
    assert close(w.dot(B), float(g["dot_w_B"]))
    assert close(B.norm(), float(g["norm_B"]))
    for cap in (10 ** 7, 1000):
        # v.addTwo(w, a) keeps the top v.cap of the merge (src/all.h:456-478); a vector
        # cannot hold more than its capacity here, so the capped case merges into a
        # large vector and applies the same top-cap selection with shrinkFrom
        ref_k, ref_a = g["add2_%d_keys" % cap], g["add2_%d_amps" % cap]
        v = c.vec(len(g["B_amps"]) + len(g["B_in_amps"]))
        v.upload(g["B_keys"], g["B_amps"])
        v.addTwo(v1, -0.37)
        if cap < v.cap:
            r = c.vec(cap)
            r.shrinkFrom(v)
            v = r
        k, a = v.download()
        compare_vectors(ref_k, ref_a, k, a, capped=len(ref_a) == cap)
    c.set_Nd(int(g["add3_Nd"]))
    r = c.vec(int(g["add3_Nd"]))
    r.addThree(w, v1, B, 0.5, -1.25, 0.75)
    k, a = r.download()
    compare_vectors(g["add3_keys"], g["add3_amps"], k, a, capped=len(g["add3_amps"]) == int(g["add3_Nd"]))
    s = c.vec(int(g["shrink_cap"]))
    s.shrinkFrom(B)
    k, a = s.download()
    compare_vectors(g["shrink_keys"], g["shrink_amps"], k, a, capped=True)


@pytest.mark.parametrize("name", ["u8", "r16", "c1"])
def test_lanczos_energies(golden_in, name):
    g, path = golden_in(name)
    c = sg.Context(path, 2 * int(g["M"]), int(g["ne"]), Nd=int(g["L_Nd"]), hpsi_cap=int(g["L_hpsi_cap"]))
    v = c.vec(int(g["L_Nd"]))
    v.upload(np.array([g["hf"]], np.uint64), np.array([1.0]))
    en, fe = c.sparse_krylov_solve_eigenval(v, int(g["L_Nl"]), int(g["L_restarts"]))
    ref = g["L_energies"]
    en = en[~np.isnan(en)]
    assert len(en) == len(ref)
    assert np.max(np.abs(en - ref)) < 1e-8
    assert abs(fe - float(g["L_final_e"])) < 1e-8
    if "fci_energy" in g:
        assert abs(fe - float(g["fci_energy"])) < 1e-6


def test_minres_matches_oracle(golden_in, port):
    g, path = golden_in("u8")
    Nd = 2000
    c = sg.Context(path, 16, 6, Nd=Nd)
    be = port.PortLib(words=1)
    be.setup(path, 16, 6, Nd, nthread=8)
    rk, ra = g["B_in_keys"], g["B_in_amps"]
    lam = float(g["L_energies"][-1]) + 0.05
    rhs = c.vec_from(rk, ra, cap=Nd)
    guess = c.vec(Nd)
    res = c.vec(Nd)
    it = c.minres_sp(rhs, guess, res, 6, 1e-8, lam)
    (xk, xa), it2 = port.minres(be, (rk, ra), (np.zeros(0, np.uint64), np.zeros(0)), 6, 1e-8, lam, Nd)
    assert it == it2
    k, a = res.download()
    compare_vectors(xk, xa, k, a, capped=len(xa) == Nd, rtol=1e-9, atol=1e-12)


def test_vectors_of_another_context_are_rejected(golden_in):
    """Entry points taking a context check that its vectors belong to it (another
    context's keys may have another width) before any device work."""
    g, path, c = ctx_for(golden_in, "c1")
    c2 = sg.Context(path, 2 * int(g["M"]), int(g["ne"]), Nd=1000)
    v = c.vec_from(np.array([g["hf"]], np.uint64), np.array([1.0]))
    w = c2.vec_from(np.array([g["hf"]], np.uint64), np.array([1.0]))
    out2 = c2.vec(10)
    for call in (lambda: c2.SpMVMtply_bucket(v, out2, 0.0, 1.0), lambda: v.dot(w), lambda: v.addTwo(w, 1.0),
                 lambda: w.naiveCopy(v), lambda: c2.calc_energy(v)):
        with pytest.raises(sg.SfciError) as e:
            call()
        assert e.value.status == "SFCI_ERR_ARG"
    assert v.len == 1 and w.len == 1 and out2.len == 0
    assert close(v.dot(v), 1.0)


def test_empty_input_leaves_diag_untouched(golden_in):
    g, path, c = ctx_for(golden_in, "c1")
    vin = c.vec(10)
    out = c.vec(10)
    out.upload(np.array([g["hf"]], np.uint64), np.array([1.0]))
    d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0, diag=123.0)
    assert d == 123.0 and out.len == 0


def test_multipass_equals_single_pass(golden_in):
    """A small device-memory budget forces several generation passes and level-1
    groups; the result must not depend on the plan."""
    g, path = golden_in("r28")
    kw = dict(Nd=200000)
    c1 = sg.Context(path, 56, 14, **kw)
    c2 = sg.Context(path, 56, 14, mem_budget=64 << 20, **kw)
    outs = []
    for c in (c1, c2):
        vin = c.vec_from(g["B_in_keys"], g["B_in_amps"])
        out = c.vec(int(g["B_cap"]))
        d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
        outs.append((out.download(), d, c.last_stats()))
    assert outs[1][2]["passes"] > 1, outs[1][2]
    (k1, a1), d1, _ = outs[0]
    (k2, a2), d2, _ = outs[1]
    compare_vectors(k1, a1, k2, a2, cut=CUT, capped=True)
    assert close(d1, d2)
    compare_vectors(g["B_keys"], g["B_amps"], k2, a2, cut=CUT, capped=True)


def _sample_vector(rng, N, ne, n):
    hf = (1 << ne) - 1
    occ = [b for b in range(N) if hf >> b & 1]
    out = {hf}
    while len(out) < n:
        d = hf
        for _ in range(int(rng.integers(1, 4))):
            i = int(rng.choice(occ))
            if not d >> i & 1:
                continue
            cand = [a for a in range(N) if (a & 1) == (i & 1) and not d >> a & 1]
            d ^= (1 << i) ^ (1 << int(rng.choice(cand)))
        out.add(d)
    ints = sorted(out)
    amps = rng.normal(size=len(ints)) * np.exp(-rng.uniform(0, 6, size=len(ints)))
    return ints, amps / np.linalg.norm(amps)


def test_128bit_keys_match_oracle(tmp_path, port):
    """66 spin orbitals: two-word keys on the device against the oracle's 128-bit path."""
    from sfci_gb300 import fcidump as fd
    M, ne = 33, 6
    p = str(tmp_path / "w_IN")
    fd.rhf_to_in_file(p, M, ne, 11)
    rng = np.random.default_rng(5)
    ints, amps = _sample_vector(rng, 2 * M, ne, 300)
    keys = sg.keys_from_ints(ints, 2)
    c = sg.Context(p, 2 * M, ne, Nd=200000)
    assert c.words == 2
    vin = c.vec_from(keys, amps)
    out = c.vec(200000)
    d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    k, a = out.download()
    be = port.PortLib(words=2)
    be.setup(p, 2 * M, ne, 200000, nthread=8)
    rk, ra, rd = be.spmspv(keys, amps, 200000, 0.0, 1.0)
    compare_vectors(rk, ra, k, a, cut=CUT)
    assert close(d, rd)
    assert close(c.calc_energy(vin), be.energy(keys, amps))
    dd = c.DiagCal_bit(keys[:20])
    assert np.allclose(dd, be.diag(keys[:20]), rtol=1e-13, atol=1e-13)


def test_full_size_properties_56_orbital_system(golden_in, port):
    """The benchmark system (56 spin orbitals, 14 electrons) at a size where the
    two-level partition is active: parity with the oracle on the same input."""
    g, path = golden_in("r28")
    rng = np.random.default_rng(9)
    ints, amps = _sample_vector(rng, 56, 14, 20000)
    keys = np.array(ints, np.uint64)
    c = sg.Context(path, 56, 14, Nd=200000)
    vin = c.vec_from(keys, amps)
    out = c.vec(2000000)
    d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    st = c.last_stats()
    assert st["terms"] == 20000 * (30723 + 1)
    k, a = out.download()
    assert np.all(np.diff(k.astype(np.float64)) >= 0) and np.unique(k).size == k.size
    assert np.all(np.abs(a) > CUT)
    be = port.PortLib(words=1)
    be.setup(path, 56, 14, 200000, nthread=16)
    rk, ra, rd = be.spmspv(keys, amps, 2000000, 0.0, 1.0)
    compare_vectors(rk, ra, k, a, cut=CUT, capped=len(ra) == 2000000)
    assert close(d, rd)


def test_cut_levels_select_from_one_exact_merge(golden_in):
    """The merge sums each determinant's terms exactly (fixed point) and cuts once:
    a product at a larger coeff_cut must be exactly the entries of a product at a
    smaller one whose |amplitude| exceeds the larger cut, with identical bits."""
    g, path = golden_in("r28")
    rng = np.random.default_rng(21)
    ints, amps = _sample_vector(rng, 56, 14, 2000)
    keys = np.array(ints, np.uint64)
    base = None
    for cut in (1e-12, 1e-9, 1e-5, 1e-3, 0.02):
        c = sg.Context(path, 56, 14, Nd=200000, coeff_cut=cut)
        vin = c.vec_from(keys, amps)
        out = c.vec(60000000)
        d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
        k, a = out.download()
        assert np.all(np.abs(a) > cut)
        if base is None:
            base = (k, a, d)
            continue
        sel = np.abs(base[1]) > cut
        assert np.array_equal(k, base[0][sel])
        assert np.array_equal(a.view(np.uint64), base[1][sel].view(np.uint64))
        assert close(d, base[2])  # <v|Hv> sums leaves in launch order: equal to rounding


def test_restart_vector_file_round_trip(golden_in, tmp_path):
    """Device vector -> wf_self_as_guess.out text (src/minres.cpp:59-70) -> device
    vector: keys exact, amplitudes at the file's 12 significant digits."""
    g, path = golden_in("r28")
    c = sg.Context(path, 56, 14, Nd=200000)
    rng = np.random.default_rng(31)
    ints, amps = _sample_vector(rng, 56, 14, 500)
    v = c.vec_from(np.array(ints, np.uint64), amps)
    k0, a0 = v.download()
    p = tmp_path / "wf_self_as_guess.out"
    v.writePsi(str(p))
    kh, ah = sg.psi_read(str(p), 56)
    assert np.array_equal(kh, k0)
    w = c.vec(1000).readPsi(str(p))
    k1, a1 = w.download()
    assert np.array_equal(k1, k0)
    assert np.array_equal(a1, np.array([float("%.12g" % x) for x in a0]))
    with pytest.raises(sg.SfciError) as e:
        c.vec(10).readPsi(str(p))
    assert e.value.status == "SFCI_ERR_CAPACITY"


def test_pass_plans_give_identical_products(golden_in):
    """Device budgets that force 2 to 4 generation passes (planned passes with
    recorded pass ids) and more (passes planned from the counts) must give the
    single-pass product bit for bit: the merge sums are exact."""
    g, path = golden_in("r28")
    rng = np.random.default_rng(41)
    ints, amps = _sample_vector(rng, 56, 14, 3000)
    keys = np.array(ints, np.uint64)
    ref = None
    seen = []
    for budget in (0, 1536 << 20, 1 << 30, 640 << 20, 400 << 20):
        c = sg.Context(path, 56, 14, Nd=200000, mem_budget=budget)
        vin = c.vec_from(keys, amps)
        out = c.vec(2000000)
        d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
        k, a = out.download()
        seen.append(c.last_stats()["passes"])
        if ref is None:
            ref = (k, a, d)
            assert seen[0] == 1
            continue
        assert np.array_equal(k, ref[0])
        assert np.array_equal(a.view(np.uint64), ref[1].view(np.uint64))
        assert close(d, ref[2])
    assert any(2 <= p <= 4 for p in seen[1:]) and any(p > 4 for p in seen[1:]), seen


@pytest.mark.parametrize("nsrc,target", [(None, 5e-5), (1100, 1.2e-5)])
def test_hot_key_sum_rounds_to_nearest(golden_in, port, nsrc, target):
    """One determinant (|HF> of the 56-spin-orbital system) receives a term from
    every input determinant: all 30,723 it connects to (a leaf for the CTA tier's
    wide accumulators), or the 1,100 with the largest elements (a warp-table
    leaf, narrow accumulators).  The amplitudes are chosen so that every term has
    the same sign and the merged amplitude sits near the 1e-5 cut.  It must agree
    within 1e-12 relative with math.fsum of the oracle's raw terms
    (OffDiagGen_bit, src/bitstr.cpp:162-302, from the receiving side by the
    symmetry of H).  Terms truncated toward zero would drift by n * 2.7e-20
    (2.5e-12 to 1.7e-11 relative here); rounded to nearest they stay near
    sqrt(n) * 1.6e-20."""
    import math
    g, path = golden_in("r28")
    hf = (1 << 14) - 1
    be = port.PortLib(words=1)
    be.setup(path, 56, 14, 200000, nthread=8)
    rk, ra = be.offdiag(np.array([hf], np.uint64))
    keys, inv = np.unique(rk, return_inverse=True)
    H = np.zeros(len(keys))
    np.add.at(H, inv, ra)
    if nsrc is not None:
        keep = np.sort(np.argsort(-np.abs(H), kind="stable")[:nsrc])
        sel = np.zeros(len(keys), bool)
        sel[keep] = True
        keys, H = keys[keep], H[keep]
        raw = sel[inv]
        rk, ra, inv = rk[raw], ra[raw], np.searchsorted(keys, rk[raw])
    rng = np.random.default_rng(17)
    w = rng.uniform(0.5, 1.5, len(keys))
    amps = np.sign(H) * w
    amps *= target / float(np.sum(np.abs(H) * w))
    want = math.fsum(float(x) for x in amps[inv] * ra)
    c = sg.Context(path, 56, 14, Nd=200000)
    vin = c.vec_from(keys, amps)
    out = c.vec(2000000)
    c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    k, a = out.download()
    i = np.searchsorted(k, np.uint64(hf))
    assert i < len(k) and k[i] == hf
    assert abs(a[i] - want) <= 1e-12 * abs(want), (a[i], want, (a[i] - want) / want)


@pytest.mark.parametrize("budget", [640 << 20, 400 << 20, 200 << 20])
def test_class_passes_give_the_single_pass_product(golden_in, budget):
    """Generation passes that own ranges of the targets' alpha class (each pass
    generating only its own terms) must give the single-pass product bit for
    bit, whatever the budget and hence the number of passes."""
    g, path = golden_in("r28")
    rng = np.random.default_rng(43)
    ints, amps = _sample_vector(rng, 56, 14, 3000)
    keys = np.array(ints, np.uint64)
    c0 = sg.Context(path, 56, 14, Nd=200000)
    vin = c0.vec_from(keys, amps)
    out = c0.vec(2000000)
    d0 = c0.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    k0, a0 = out.download()
    t0 = c0.last_stats()["terms"]
    c = sg.Context(path, 56, 14, Nd=200000, mem_budget=budget)
    c.set_class_passes(1)
    vin = c.vec_from(keys, amps)
    out = c.vec(2000000)
    d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    st = c.last_stats()
    k, a = out.download()
    assert st["passes"] > 1 and st["terms"] == t0, st
    assert np.array_equal(k, k0)
    assert np.array_equal(a.view(np.uint64), a0.view(np.uint64))
    assert close(d, d0)

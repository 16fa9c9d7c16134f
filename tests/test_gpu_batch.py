"""Batched instances through the C ABI: several Hamiltonians in one context, one
product over all of them per Krylov step.

* One batched product of several instances' vectors must give, per instance,
  exactly the unbatched product (keys and amplitude bits: the merge is exact)
  and the same <v|H|v> within 1e-12 relative.
* The batched Lanczos driver (sparse_krylov_solve_eigenval,
  src/sparse_solver.cpp:246-548, on every instance) must give each instance's
  energies within 1e-10 Eh of an unbatched run of the same instance.
* The autotuner times product plans and keeps one; every plan gives the same
  product bit for bit.
* Host keys whose tag names no instance, or that set a bit beyond their
  instance's spin orbitals, are rejected before they reach the device.
"""
import numpy as np
import pytest

from parity import close

import sfci_gb300 as sg
from sfci_gb300 import fcidump as fd

pytestmark = pytest.mark.gpu

# (M spatial orbitals, electrons, t on the curve, Nd)
INSTANCES = [(10, 6, 0.0, 600), (12, 8, 0.35, 900), (11, 6, 0.7, 500), (14, 8, 1.0, 1200)]


@pytest.fixture(scope="module")
def curve(tmp_path_factory):
    d = tmp_path_factory.mktemp("curve")
    paths = []
    for k, (M, ne, t, nd) in enumerate(INSTANCES):
        p = str(d / ("i%d_IN" % k))
        fd.bond_stretch_to_in_file(p, M, ne, 4, t)
        paths.append(p)
    return paths


def hf_tagged(ne, inst):
    return sg.tag_keys(np.array([[(1 << ne) - 1, 0]], np.uint64), inst)


def test_batched_product_equals_unbatched_products(curve):
    orbs = [2 * M for M, _, _, _ in INSTANCES]
    nes = [ne for _, ne, _, _ in INSTANCES]
    bc = sg.Context.batch(curve, orbs, nes, Nd=10 ** 6)
    # a two-step Krylov vector of each instance, built unbatched
    vecs = []
    for k, (M, ne, t, nd) in enumerate(INSTANCES):
        c = sg.Context(curve[k], 2 * M, ne, Nd=10 ** 6)
        hf = c.vec(1)
        hf.upload(sg.keys_from_ints([(1 << ne) - 1], c.words), np.array([1.0]))
        w = c.vec(10 ** 6)
        c.SpMVMtply_bucket(hf, w, 0.0, 1.0)
        w.normalize()
        kk, aa = w.download()
        ints = [int(x) for x in (kk if kk.ndim == 1 else kk[:, 0])]
        vecs.append((ints, aa))
    # unbatched products, in each instance's own (single-Hamiltonian) context
    want = []
    for k, (M, ne, t, nd) in enumerate(INSTANCES):
        c = sg.Context(curve[k], 2 * M, ne, Nd=10 ** 6)
        v = c.vec_from(sg.keys_from_ints(vecs[k][0], c.words), vecs[k][1])
        o = c.vec(10 ** 7)
        d = c.SpMVMtply_bucket(v, o, 0.0, 1.0)
        kk, aa = o.download()
        want.append(([int(x) for x in (kk if kk.ndim == 1 else kk[:, 0])], aa, d))
    # one batched product of all instances
    allk = np.concatenate([sg.tag_keys(sg.keys_from_ints(vecs[k][0], 2), k) for k in range(len(INSTANCES))])
    alla = np.concatenate([vecs[k][1] for k in range(len(INSTANCES))])
    vin = bc.vec_from(allk, alla)
    out = bc.vec(10 ** 7)
    bc.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    kk, aa = out.download()
    inst = (kk[:, 1] >> np.uint64(sg.INST_SHIFT)).astype(int)
    assert np.all(np.diff(inst) >= 0)
    for k in range(len(INSTANCES)):
        sel = inst == k
        got_k = [int(x) for x in kk[sel, 0]]
        assert got_k == want[k][0], k
        assert np.array_equal(aa[sel].view(np.uint64), want[k][1].view(np.uint64)), k


def test_upload_rejects_keys_outside_the_batch(curve):
    """Uploads (and DiagCal_bit's host keys) are checked on the host before any
    copy: a tag naming no instance, or a bit at or above its instance's spin
    orbitals, is SFCI_ERR_ARG and the vector keeps its contents.  The batched
    driver rejects vectors passed out of instance order."""
    orbs = [2 * M for M, _, _, _ in INSTANCES]
    nes = [ne for _, ne, _, _ in INSTANCES]
    bc = sg.Context.batch(curve, orbs, nes, Nd=10 ** 4)
    v = bc.vec(4)
    good = hf_tagged(nes[0], 0)
    v.upload(good, np.array([1.0]))
    bad_tag = np.array([[1, np.uint64(len(INSTANCES)) << np.uint64(sg.INST_SHIFT)]], np.uint64)
    bad_bit = sg.tag_keys(sg.keys_from_ints([1 << orbs[1]], 2), 1)
    for bad in (bad_tag, bad_bit):
        with pytest.raises(sg.SfciError) as e:
            v.upload(np.concatenate([good, bad]), np.array([1.0, 1.0]))
        assert e.value.status == "SFCI_ERR_ARG"
        assert len(v) == 1
        with pytest.raises(sg.SfciError) as e:
            bc.DiagCal_bit(np.concatenate([good, bad]))
        assert e.value.status == "SFCI_ERR_ARG"
    # the batched driver takes instance k's vector in place k
    vs = []
    for k, (M, ne, t, nd) in enumerate(INSTANCES):
        w = bc.vec(nd)
        w.upload(hf_tagged(ne, k), np.array([1.0]))
        vs.append(w)
    with pytest.raises(sg.SfciError) as e:
        bc.batch_lanczos(vs[::-1], 4, 1)
    assert e.value.status == "SFCI_ERR_ARG"


@pytest.mark.parametrize("cap", [2000000, 3000])
def test_batched_lanczos_matches_unbatched_runs(curve, cap):
    """cap is every instance's hpsi_cap; at 3000 it cuts each instance's
    products, so the batched driver's per-instance cut (after a batch output
    that grew to hold every survivor) must pick what each unbatched run keeps."""
    Nl, restarts = 8, 2
    orbs = [2 * M for M, _, _, _ in INSTANCES]
    nes = [ne for _, ne, _, _ in INSTANCES]
    ref = []
    for k, (M, ne, t, nd) in enumerate(INSTANCES):
        c = sg.Context(curve[k], 2 * M, ne, Nd=nd, hpsi_cap=cap)
        v = c.vec(nd)
        v.upload(sg.keys_from_ints([(1 << ne) - 1], c.words), np.array([1.0]))
        en, fe = c.sparse_krylov_solve_eigenval(v, Nl, restarts)
        ref.append((en, fe))
    bc = sg.Context.batch(curve, orbs, nes, Nd=10 ** 6, hpsi_cap=cap)
    vs = []
    for k, (M, ne, t, nd) in enumerate(INSTANCES):
        v = bc.vec(nd)
        v.upload(hf_tagged(ne, k), np.array([1.0]))
        vs.append(v)
    en, fe = bc.batch_lanczos(vs, Nl, restarts)
    for k in range(len(INSTANCES)):
        r_en, r_fe = ref[k]
        m = ~np.isnan(r_en)
        assert np.array_equal(m, ~np.isnan(en[k])), (k, r_en, en[k])
        assert np.max(np.abs(en[k][m] - r_en[m])) < 1e-10, (k, en[k], r_en)
        assert abs(fe[k] - r_fe) < 1e-10, (k, fe[k], r_fe)


def test_autotune_keeps_results(curve):
    M, ne, t, nd = INSTANCES[-1]
    c = sg.Context(curve[-1], 2 * M, ne, Nd=10 ** 6)
    hf = c.vec(1)
    hf.upload(sg.keys_from_ints([(1 << ne) - 1], c.words), np.array([1.0]))
    w = c.vec(10 ** 6)
    c.SpMVMtply_bucket(hf, w, 0.0, 1.0)
    w.normalize()
    out = c.vec(10 ** 7)
    d0 = c.SpMVMtply_bucket(w, out, 0.0, 1.0)
    k0, a0 = out.download()
    plan, ms = c.autotune(w, out)
    assert ms > 0 and plan == c.tuning()
    for l1, dg, leaf, g in ((9, 9, 120, 2), (7, 8, 60, 1), (plan["l1_bits"], plan["digit_bits"], plan["leaf_keys"],
                                                              plan["gen_ctas_per_sm"])):
        c.set_tuning(l1, dg, leaf, g)
        d = c.SpMVMtply_bucket(w, out, 0.0, 1.0)
        k, a = out.download()
        assert np.array_equal(k, k0) and np.array_equal(a.view(np.uint64), a0.view(np.uint64))
        assert close(d, d0)

"""The learned excitation screen through the C ABI.

* Threshold 0 keeps every term group: the screened product must be the plain
  product bit for bit.
* A partial screen: the screened product must equal the merge of exactly the
  kept groups' terms, built on the CPU from the oracle restatement's raw terms
  (OffDiagGen_bit, src/bitstr.cpp:162-302) and the group of each term's
  excitation; tolerances of tests/parity.py (keys bit-exact off the 1e-5 cut
  edge, amplitudes 1e-12 relative).
* The MLP's forward pass (tensor cores, BF16 weights and activations, FP32
  accumulation) against a torch FP32 evaluation with the same BF16 roundings:
  probabilities within 5e-3 absolute.
* One training step's gradients (tensor-core backward and weight-gradient
  products) against torch autograd with the same roundings: every parameter
  block within 2e-2 of the reference in relative norm.
"""
import math

import numpy as np
import pytest

from parity import close, compare_vectors

import sfci_gb300 as sg

pytestmark = pytest.mark.gpu
CUT = 1e-5
FEAT_SCALE = 0.1
HID, KIN = 256, 576


def c2(n):
    return n * (n - 1) // 2


def unrank(k):
    y = int((1 + math.sqrt(1 + 8 * k)) / 2)
    while y * (y - 1) // 2 > k:
        y -= 1
    while (y + 1) * y // 2 <= k:
        y += 1
    return k - y * (y - 1) // 2, y


def det_groups(d, N):
    """Groups g >= 1 of determinant d in the screen's order: (cls, p, q, r, size)."""
    occ = [[b for b in range(s, N, 2) if d >> b & 1] for s in (0, 1)]
    vir = [[b for b in range(s, N, 2) if not d >> b & 1] for s in (0, 1)]
    out = []
    for s in (0, 1):
        for op in range(c2(len(occ[s]))):
            x, y = unrank(op)
            for v in range(1, len(vir[s])):
                out.append((1 + s, occ[s][x], occ[s][y], vir[s][v], v))
    for xs in range(len(occ[0]) * len(vir[0])):
        ii, aa = divmod(xs, len(vir[0]))
        for jj in range(len(occ[1])):
            out.append((3, occ[0][ii], occ[1][jj], vir[0][aa], len(vir[1])))
    return out


def group_of_target(d, k, N):
    """Screen group of the term of source d landing on k (0: diagonal or single)."""
    rem, add = d & ~k, k & ~d
    rb = [b for b in range(N) if rem >> b & 1]
    ab = [b for b in range(N) if add >> b & 1]
    if len(rb) < 2:
        return 0
    occ = [[b for b in range(s, N, 2) if d >> b & 1] for s in (0, 1)]
    vir = [[b for b in range(s, N, 2) if not d >> b & 1] for s in (0, 1)]
    na = [len(o) for o in occ]
    nv = [len(v) for v in vir]
    gss = [c2(na[s]) * (nv[s] - 1) if nv[s] else 0 for s in (0, 1)]
    if rb[0] % 2 == rb[1] % 2:  # same spin
        s = rb[0] % 2
        x, y = sorted(occ[s].index(b) for b in rb)
        v = max(vir[s].index(b) for b in ab)
        op = y * (y - 1) // 2 + x
        return 1 + (gss[0] if s else 0) + op * (nv[s] - 1) + (v - 1)
    i = [b for b in rb if b % 2 == 0][0]
    j = [b for b in rb if b % 2 == 1][0]
    a = [b for b in ab if b % 2 == 0][0]
    xs = occ[0].index(i) * nv[0] + vir[0].index(a)
    return 1 + gss[0] + gss[1] + xs * na[1] + occ[1].index(j)


def vmax_table(M, seed):
    from sfci_gb300 import fcidump as fd
    _, (i, j, k, l), v, _ = fd.synthetic_rhf(M, seed)
    P = M * (M + 1) // 2
    pid = lambda x, y: np.maximum(x, y) * (np.maximum(x, y) + 1) // 2 + np.minimum(x, y)
    t = np.zeros((P, P))
    t[pid(i, j), pid(k, l)] = v
    t[pid(k, l), pid(i, j)] = v
    vm = np.zeros((P, M))
    for o in range(M):
        cols = pid(np.full(M, o), np.arange(M))
        vm[:, o] = np.abs(t[:, cols]).max(axis=1)
    return np.stack([vm] * 4).astype(np.float32)  # RHF: the four spin blocks are equal


def features(keys, amps, N, M, vmax):
    rows = []
    P = M * (M + 1) // 2
    pid = lambda x, y: max(x, y) * (max(x, y) + 1) // 2 + min(x, y)
    for d, c in zip(keys, amps):
        d = int(d)
        occ = [b for b in range(N) if d >> b & 1]
        lc = np.float32(FEAT_SCALE) * np.float32(math.log10(max(abs(c), 1e-30)))
        for cls, p, q, r, size in det_groups(d, N):
            ps, qs, rs = p >> 1, q >> 1, r >> 1
            if cls < 3:
                blk = 3 * (cls - 1)
                vb = np.float32(vmax[blk, pid(qs, rs), ps]) + np.float32(vmax[blk, pid(ps, rs), qs])
            else:
                vb = max(vmax[1, pid(ps, rs), qs], vmax[2, pid(ps, rs), qs])
            lv = np.float32(FEAT_SCALE) * np.float32(math.log10(max(float(vb), 1e-30)))
            rows.append((occ, cls, p, q, r, float(lc), float(lv)))
    return rows


def bf16(t):
    import torch
    return t.to(torch.bfloat16).to(torch.float32)


def torch_forward(params, rows, torch):
    P = torch.tensor(params, dtype=torch.float32)
    W1 = bf16(P[: KIN * HID].reshape(KIN, HID))
    o = KIN * HID
    b1 = P[o:o + HID]; o += HID
    W2 = P[o:o + HID * HID].reshape(HID, HID); o += HID * HID
    b2 = P[o:o + HID]; o += HID
    w3 = P[o:o + HID]; o += HID
    b3 = P[o]
    X = torch.zeros(len(rows), KIN)
    for n, (occ, cls, p, q, r, lc, lv) in enumerate(rows):
        X[n, occ] = 1.0
        X[n, 128 + p] += 1.0
        X[n, 256 + q] += 1.0
        X[n, 384 + r] += 1.0
        X[n, 512 + cls] += 1.0
        X[n, 516] = lc
        X[n, 517] = lv
    return X, W1, b1, W2, b2, w3, b3


def _setup(golden_in, n=200, seed=3):
    g, path = golden_in("c1")
    c = sg.Context(path, 20, 10, Nd=200000)
    rng = np.random.default_rng(seed)
    hf = (1 << 10) - 1
    B = g["B_in_keys"]
    sel = np.sort(rng.choice(len(B), size=min(n, len(B)), replace=False))
    keys = np.array(B[sel], np.uint64)
    amps = rng.normal(size=len(keys)) * np.exp(-rng.uniform(0, 4, len(keys)))
    amps /= np.linalg.norm(amps)
    return g, path, c, keys, amps, hf


def test_threshold_zero_gives_the_plain_product(golden_in):
    g, path, c, keys, amps, _ = _setup(golden_in)
    vin = c.vec_from(keys, amps)
    out0 = c.vec(2000000)
    d0 = c.SpMVMtply_bucket(vin, out0, 0.0, 1.0)
    k0, a0 = out0.download()
    scr = sg.Screen(c, seed=7)
    c.set_screen(scr, 0.0)
    out1 = c.vec(2000000)
    d1 = c.SpMVMtply_bucket(vin, out1, 0.0, 1.0)
    k1, a1 = out1.download()
    st = c.screen_stats()
    assert st["products"] == 1 and st["kept_groups"] == st["groups"] > 0
    assert np.array_equal(k0, k1)
    assert np.array_equal(a0.view(np.uint64), a1.view(np.uint64))
    assert d0 == d1


def test_guard_keeps_groups_with_large_term_bounds(golden_in):
    """A threshold above every probability skips every double group; a guard
    below every group's term bound keeps them all again (the plain product bit
    for bit), and a guard in between keeps the groups it must."""
    g, path, c, keys, amps, _ = _setup(golden_in)
    vin = c.vec_from(keys, amps)
    out0 = c.vec(2000000)
    d0 = c.SpMVMtply_bucket(vin, out0, 0.0, 1.0)
    k0, a0 = out0.download()
    scr = sg.Screen(c, seed=7)
    c.set_screen(scr, 1.0, guard=1e-300)
    out1 = c.vec(2000000)
    d1 = c.SpMVMtply_bucket(vin, out1, 0.0, 1.0)
    k1, a1 = out1.download()
    st = c.screen_stats()
    assert st["kept_groups"] == st["groups"] > 0
    assert np.array_equal(k0, k1) and np.array_equal(a0.view(np.uint64), a1.view(np.uint64)) and d0 == d1
    # no guard: threshold 1 keeps no double group (a sigmoid output stays below 1 here)
    c.set_screen(scr, 1.0)
    s0 = c.screen_stats()
    c.SpMVMtply_bucket(vin, out1, 0.0, 1.0)
    s1 = c.screen_stats()
    none_kept = s1["kept_groups"] - s0["kept_groups"]
    # a lower guard keeps at least the groups a higher one keeps
    kept = [none_kept]
    for gd in (1e-2, 1e-4, 1e-6):
        c.set_screen(scr, 1.0, guard=gd)
        a_ = c.screen_stats()
        c.SpMVMtply_bucket(vin, out1, 0.0, 1.0)
        b_ = c.screen_stats()
        kept.append(b_["kept_groups"] - a_["kept_groups"])
    assert all(x <= y for x, y in zip(kept, kept[1:])), kept
    assert kept[-1] > kept[0], kept
    # a floor above every bound skips every double group without the network;
    # one below every bound changes nothing (threshold 0 keeps the rest)
    c.set_screen(scr, 0.0, floor=1e300)
    a_ = c.screen_stats()
    c.SpMVMtply_bucket(vin, out1, 0.0, 1.0)
    b_ = c.screen_stats()
    assert b_["kept_groups"] == a_["kept_groups"] and b_["groups"] > a_["groups"]
    c.set_screen(scr, 0.0, floor=1e-300)
    d2 = c.SpMVMtply_bucket(vin, out1, 0.0, 1.0)
    k2, a2 = out1.download()
    assert np.array_equal(k0, k2) and np.array_equal(a0.view(np.uint64), a2.view(np.uint64)) and d0 == d2
    with pytest.raises(sg.SfciError):
        c.set_screen(scr, 0.5, guard=-1.0)


def test_partial_screen_is_the_merge_of_the_kept_groups(golden_in, port):
    g, path, c, keys, amps, _ = _setup(golden_in, n=150, seed=5)
    N, M = 20, 10
    scr = sg.Screen(c, seed=11)
    # spread the untrained network's outputs: a wide output layer
    p = scr.params()
    o = KIN * HID + HID + HID * HID + HID
    p[o:o + HID] *= 40.0
    p[o + HID] = 0.0
    scr.set_params(p)
    vin = c.vec_from(keys, amps)
    prob = scr.predict(vin, 0.5, probs=True)["prob"]
    thr = np.float32(np.quantile(prob, 0.5))  # keep about half of the groups
    keepm = prob >= thr
    frac = float(np.mean(keepm))
    assert 0.1 < frac < 0.9, frac  # a real partial screen
    c.set_screen(scr, float(thr))
    out = c.vec(2000000)
    d = c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    k, a = out.download()
    # CPU: the oracle's raw terms of every source, kept when their group is
    be = port.PortLib(words=1)
    be.setup(path, N, 20 // 2, 200000, nthread=8)
    acc = {}
    e = 0
    for dj, cj in zip(keys, amps):
        dj = int(dj)
        groups = det_groups(dj, N)
        keep = keepm[e:e + len(groups)]
        e += len(groups)
        rk, ra = be.offdiag(np.array([dj], np.uint64))
        for kk, aa in zip(rk, ra):
            gi = group_of_target(dj, int(kk), N)
            if gi == 0 or keep[gi - 1]:
                acc.setdefault(int(kk), []).append(cj * aa)
        acc.setdefault(dj, []).append(cj * float(be.diag(np.array([dj], np.uint64))[0]))
    assert e == len(prob)
    merged = {kk: math.fsum(v) for kk, v in acc.items()}
    want_d = math.fsum(merged.get(int(dj), 0.0) * cj for dj, cj in zip(keys, amps))
    rk = np.array(sorted(kk for kk, v in merged.items() if abs(v) > CUT), np.uint64)
    ra = np.array([merged[int(x)] for x in rk])
    rep = compare_vectors(rk, ra, k, a, cut=CUT)
    assert close(d, want_d)
    assert rep["common"] > 100


def test_mlp_forward_matches_torch(golden_in):
    torch = pytest.importorskip("torch")
    g, path, c, keys, amps, _ = _setup(golden_in, n=40, seed=9)
    scr = sg.Screen(c, seed=13)
    p = scr.params()
    rng = np.random.default_rng(1)
    p[: KIN * HID] += rng.normal(0, 0.2, KIN * HID).astype(np.float32)
    o = KIN * HID + HID + HID * HID + HID
    p[o:o + HID] *= 8.0
    scr.set_params(p)
    vin = c.vec_from(keys, amps)
    got = scr.predict(vin, 0.5, probs=True)["prob"]
    rows = features(keys, amps, 20, 10, vmax_table(10, 0))
    assert len(rows) == len(got)
    X, W1, b1, W2, b2, w3, b3 = torch_forward(p, rows, torch)
    h1 = bf16(torch.relu(X @ W1 + b1))
    h2 = torch.relu(h1 @ bf16(W2).T + b2)
    ref = torch.sigmoid(h2 @ w3 + b3).numpy()
    assert np.std(ref) > 0.05  # a discriminating network, not a constant
    err = np.abs(ref - got)
    assert err.max() < 5e-3, (err.max(), int(np.argmax(err)))


def test_training_gradients_match_torch(golden_in):
    torch = pytest.importorskip("torch")
    g, path, c, keys, amps, _ = _setup(golden_in, n=60, seed=15)
    vin = c.vec_from(keys, amps)
    out = c.vec(2000000)
    c.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    scr = sg.Screen(c, seed=17)
    p = scr.params()
    rng = np.random.default_rng(2)
    p[: KIN * HID] += rng.normal(0, 0.1, KIN * HID).astype(np.float32)
    scr.set_params(p)
    ne, npos = scr.log(vin, out)
    assert ne > 512 and 0 < npos < ne
    pw = 3.0
    scr.train(1, batch_tiles=4, lr=0.0, pos_weight=pw, sequential=True)
    gg = scr.grads()
    # the same batch on the CPU: examples 0..511 in order, labels from the output's support
    ok, _ = out.download()
    support = set(int(x) for x in ok)
    rows, ys = [], []
    be_rows = features(keys, amps, 20, 10, vmax_table(10, 0))
    e = 0
    for dj in keys:
        dj = int(dj)
        occ = [b for b in range(20) if dj >> b & 1]
        for cls, pp, q, r, size in det_groups(dj, 20):
            if e >= 512:
                break
            # terms of the group: the free index runs over the holes of its spin
            vir = [[b for b in range(s, 20, 2) if not dj >> b & 1] for s in (0, 1)]
            if cls < 3:
                s = cls - 1
                v = vir[s].index(r)
                tg = [dj ^ (1 << pp) ^ (1 << q) ^ (1 << vir[s][u]) ^ (1 << r) for u in range(v)]
            else:
                tg = [dj ^ (1 << pp) ^ (1 << r) ^ (1 << q) ^ (1 << b) for b in vir[1]]
            ys.append(1.0 if any(t in support for t in tg) else 0.0)
            rows.append(be_rows[e])
            e += 1
    assert len(rows) == 512
    X, W1, b1, W2, b2, w3, b3 = torch_forward(p, rows, torch)
    for t_ in (W1, b1, W2, b2, w3):
        t_.requires_grad_(True)
    b3 = b3.clone().requires_grad_(True)
    z1 = X @ W1 + b1
    h1 = bf16(torch.relu(z1))
    W2b = bf16(W2)
    z2 = h1 @ W2b.T + b2
    logit = torch.relu(z2) @ w3 + b3
    y = torch.tensor(ys)
    wt = torch.where(y > 0, torch.tensor(pw), torch.tensor(1.0))
    loss = (wt * torch.nn.functional.binary_cross_entropy_with_logits(logit, y, reduction="none")).mean()
    loss.backward()
    o = 0
    blocks = [("W1", KIN * HID), ("b1", HID), ("W2", HID * HID), ("b2", HID), ("w3", HID)]
    refs = {"W1": W1.grad, "b1": b1.grad, "W2": W2.grad, "b2": b2.grad, "w3": w3.grad}
    for name, n in blocks:
        got = gg[o:o + n]
        ref = refs[name].numpy().reshape(-1)
        o += n
        rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert rel < 2e-2, (name, rel)
    assert abs(gg[o] - float(b3.grad)) <= 2e-2 * abs(float(b3.grad)) + 1e-7

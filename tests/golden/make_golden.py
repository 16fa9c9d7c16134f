"""Generate the golden fixtures of tests/golden from the reference itself.

Run in a checkout that has the reference tree (the x86 development container):

    python tests/golden/make_golden.py [REF_ROOT]
    python tests/golden/make_golden.py --subspace [REF_ROOT]
    python tests/golden/make_golden.py --linear [REF_ROOT]

It (1) runs the reference converter ``util/convert_fcidump.py`` on small
synthetic FCIDUMPs and stores the resulting ``_IN`` files, and (2) builds the
reference SpMSpV sources into ``oracle/_ref/libsfci_ref.so`` and records, for a
few synthetic systems, the outputs of DiagCal_bit, OffDiagGen_bit_e,
SpMVMtply_bucket, calc_energy, dynVec::dot/addTwo/addThree/shrinkFrom and a
restated Lanczos driver over those primitives.  With ``--subspace`` it writes
only the ``sub_*.npz`` fixtures: calc_CISD and fci (src/sparse_solver.cpp:15-114,
src/dense_algo.cpp:77-124) restated by oracle.cisd / oracle.fci over the
reference's own DiagCal_bit and OffDiagGen_bit_e.  With ``--linear`` it writes
the ``lin_*.npz`` fixtures: the reference's spmspvm_bucket_linear and
spmspvm_bucket_res_norm (src/functions.cpp:858-1269) on golden vectors, and the
linear Krylov driver (src/sparse_solver.cpp:561-730) restated by
oracle.krylov_linear over them.  The fixtures pin both the
oracle restatement (oracle/sfci_port.cpp) and the GPU path; neither needs the
reference tree afterwards.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from sfci_gb300 import fcidump as fd  # noqa: E402
from oracle import oracle as orc  # noqa: E402

BUNIT = 1000000
_ARGS = [a for a in sys.argv[1:] if not a.startswith("--")]
# the reference tree: the first argument, else $SFCI_REFERENCE_ROOT, else a
# checkout named "reference" beside this repository
REF = _ARGS[0] if _ARGS else os.environ.get("SFCI_REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")

# name, kind, M, ne, seeds, Nd for the Lanczos case (0 = no Lanczos)
SYSTEMS = [
    ("c1", "rhf", 10, 10, (0,), 20000, 20, 3),        # the 20-spin-orbital, 10-electron benchmark case
    ("u8", "uhf", 8, 6, (2, 3), 4000, 12, 3),         # small UHF, FCI dim 3136 < Nd
    ("r16", "rhf", 16, 8, (1,), 3000, 10, 2),         # wider virtual space
    ("r28", "rhf", 28, 14, (1,), 0, 0, 0),            # the 56-spin-orbital, 14-electron benchmark shape (SpMSpV level only)
]


def ref_convert(fcidump_path: str, flag: str) -> str:
    d = tempfile.mkdtemp()
    try:
        name = os.path.basename(fcidump_path)
        shutil.copy(fcidump_path, os.path.join(d, name))
        subprocess.run([sys.executable, os.path.join(REF, "util", "convert_fcidump.py"), flag, name], cwd=d,
                       check=True, capture_output=True)
        return open(os.path.join(d, name.split("_")[0] + "_IN")).read()
    finally:
        shutil.rmtree(d)


def merged(keys, amps):
    u, inv = np.unique(keys, return_inverse=True)
    s = np.zeros(u.size)
    np.add.at(s, inv, amps)
    return u, s


def sample_dets(hf: int, N: int, ne: int, rng, n: int):
    """HF plus random Sz-preserving excitations of it (ranks 1..4)."""
    occ = [b for b in range(N) if hf >> b & 1]
    vir = [b for b in range(N) if not hf >> b & 1]
    out = {hf}
    while len(out) < n:
        k = int(rng.integers(1, 5))
        d = hf
        for _ in range(k):
            i = int(rng.choice(occ))
            cand = [a for a in vir if (a & 1) == (i & 1) and not d >> a & 1]
            if not (d >> i & 1) or not cand:
                continue
            a = int(rng.choice(cand))
            d = d ^ (1 << i) ^ (1 << a)
        out.add(d)
    return np.array(sorted(out), dtype=np.uint64)


def main():
    so = orc.build_ref(REF)
    if not so:
        raise SystemExit("reference sources not available under %s" % REF)
    ref = orc.RefLib(so)
    # (1) converter fixtures: small RHF and UHF files
    for kind, M in (("rhf", 4), ("uhf", 4), ("rhf", 6)):
        tmp = tempfile.mkdtemp()
        try:
            p = os.path.join(tmp, "sys_fcidump")
            if kind == "rhf":
                h, q, v, e = fd.synthetic_rhf(M, 7)
                fd.write_fcidump_rhf(p, h, q, v, e, 4)
                txt = ref_convert(p, "-r")
            else:
                hs, aa, bb, ab, e = fd.synthetic_uhf(M, 8, 9)
                fd.write_fcidump_uhf(p, hs, aa, bb, ab, e, 4)
                txt = ref_convert(p, "-u")
            with open(os.path.join(HERE, "conv_%s_m%d_IN" % (kind, M)), "w") as f:
                f.write(txt)
        finally:
            shutil.rmtree(tmp)
    # (2) hot-path fixtures
    for name, kind, M, ne, seeds, lnd, nl, nres in SYSTEMS:
        N = 2 * M
        tmp = tempfile.mkdtemp()
        try:
            fpath = os.path.join(tmp, "sys_fcidump")
            if kind == "rhf":
                h, q, v, e = fd.synthetic_rhf(M, seeds[0])
                fd.write_fcidump_rhf(fpath, h, q, v, e, ne)
                txt = ref_convert(fpath, "-r")
            else:
                hs, aa, bb, ab, e = fd.synthetic_uhf(M, seeds[0], seeds[1])
                fd.write_fcidump_uhf(fpath, hs, aa, bb, ab, e, ne)
                txt = ref_convert(fpath, "-u")
            inp = os.path.join(tmp, "sys_IN")
            open(inp, "w").write(txt)
            Nd_big = 200000
            ref.setup(inp, N, ne, Nd_big, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            rng = np.random.default_rng(100 + M)
            hf = (1 << ne) - 1
            out = {"M": M, "ne": ne, "kind": kind, "seeds": np.array(seeds), "hf": np.uint64(hf),
                   "in_sha256": hashlib.sha256(txt.encode()).hexdigest()}
            dets = sample_dets(hf, N, ne, rng, 40)
            out["diag_dets"] = dets
            out["diag_vals"] = ref.diag(dets)
            for t, d in enumerate(dets[:3]):
                k, a = ref.offdiag(d)
                u, s = merged(k, a)
                out["off%d_det" % t] = np.uint64(d)
                out["off%d_keys" % t] = u
                out["off%d_amps" % t] = s
            # SpMSpV cases
            cap_big = 2000000
            k0 = np.array([hf], np.uint64)
            a0 = np.array([1.0])
            if N <= 40:
                kA, aA, dA = ref.spmspv(k0, a0, cap_big, 0.0, 1.0)
            else:
                # a 1-det input on this size overflows the reference's len*5000 buffer
                # (src/functions.cpp:566); start from a 2000-det vector instead
                kA, aA = None, None
            if kA is not None:
                out.update(A_in_keys=k0, A_in_amps=a0, A_keys=kA, A_amps=aA, A_diag=dA)
                order = np.argsort(-np.abs(aA), kind="stable")[: min(400, aA.size)]
                v1k = kA[np.sort(order)]
                v1a = aA[np.sort(order)]
            else:
                v1k = sample_dets(hf, N, ne, rng, 2000)
                v1a = rng.normal(size=v1k.size) * np.exp(-rng.uniform(0, 8, size=v1k.size))
            v1a = v1a / np.linalg.norm(v1a)
            out_cap_B = cap_big if N <= 40 else 20000
            kB, aB, dB = ref.spmspv(v1k, v1a, out_cap_B, 0.0, 1.0)
            out.update(B_in_keys=v1k, B_in_amps=v1a, B_keys=kB, B_amps=aB, B_diag=dB, B_cap=out_cap_B)
            # Nd smaller than the input + shift + negative coefficient + small output cap
            # an Nd whose boundary is not a magnitude tie (RHF spin-mirror determinants
            # have equal |amp|, and the reference breaks ties arbitrarily)
            mags = np.sort(np.abs(v1a))[::-1]
            nd_c = max(2, v1k.size // 3)
            while nd_c < v1k.size - 1 and not mags[nd_c - 1] > mags[nd_c] * (1 + 1e-9):
                nd_c += 1
            ref.setup(inp, N, ne, nd_c, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            eh = float(ref.diag(np.array([hf], np.uint64))[0])
            cap_c = 5000
            kC, aC, dC = ref.spmspv(v1k, v1a, cap_c, eh, -1.0)
            out.update(C_Nd=nd_c, C_cap=cap_c, C_lambda=eh, C_coeff=-1.0, C_keys=kC, C_amps=aC, C_diag=dC)
            ref.setup(inp, N, ne, Nd_big, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            # energies and vector algebra (vectors sorted by key, as dynVec keeps them)
            out["E_v1"] = ref.energy(v1k, v1a)
            bsel = np.argsort(-np.abs(aB), kind="stable")[: min(3000, aB.size)]
            wk, wa = kB[np.sort(bsel)], aB[np.sort(bsel)]
            wa = wa / np.linalg.norm(wa)
            out.update(w_keys=wk, w_amps=wa)
            out["E_w"] = ref.energy(wk, wa)
            out["dot_v1_B"] = ref.dot(v1k, v1a, kB, aB)
            out["dot_w_B"] = ref.dot(wk, wa, kB, aB)
            out["norm_B"] = ref.norm(kB, aB)
            for cap in (10 ** 7, 1000):
                k2, a2 = ref.add_two(kB, aB, cap, v1k, v1a, -0.37)
                out["add2_%d_keys" % cap] = k2
                out["add2_%d_amps" % cap] = a2
            ref.setup(inp, N, ne, 2000, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            k3, a3 = ref.add_three(wk, wa, v1k, v1a, kB, aB, 0.5, -1.25, 0.75)
            out.update(add3_keys=k3, add3_amps=a3, add3_Nd=2000)
            ref.setup(inp, N, ne, Nd_big, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            ks, as_ = ref.shrink_from(kB, aB, 777)
            out.update(shrink_keys=ks, shrink_amps=as_, shrink_cap=777)
            # Lanczos through the reference primitives
            if lnd:
                ref.setup(inp, N, ne, lnd, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
                en, fe, (vk, va) = orc.lanczos(ref, k0, a0, nl, nres, lnd, hpsi_cap=2000000)
                out.update(L_hpsi_cap=2000000)
                out.update(L_Nd=lnd, L_Nl=nl, L_restarts=nres, L_energies=en, L_final_e=fe)
                if kind == "uhf" or M <= 8:
                    out["fci_energy"] = exact_fci(ref, N, ne, hf)
            np.savez_compressed(os.path.join(HERE, "%s.npz" % name), **out)
            print(name, {k: (v.shape if hasattr(v, "shape") else v) for k, v in out.items() if "keys" not in k})
        finally:
            shutil.rmtree(tmp)


def exact_fci(ref, N, ne, hf):
    """Dense FCI over the Sz-sector of hf, from the reference's own elements."""
    import itertools
    import scipy.linalg as sl
    M = N // 2
    na = bin(hf & 0x5555555555555555).count("1")
    nb = bin(hf & 0xAAAAAAAAAAAAAAAA).count("1")
    alphas = [sum(1 << (2 * o) for o in c) for c in itertools.combinations(range(M), na)]
    betas = [sum(1 << (2 * o + 1) for o in c) for c in itertools.combinations(range(M), nb)]
    dets = np.array(sorted(a | b for a in alphas for b in betas), dtype=np.uint64)
    index = {int(d): i for i, d in enumerate(dets)}
    H = np.zeros((dets.size, dets.size))
    diag = ref.diag(dets)
    for j, d in enumerate(dets):
        H[j, j] += diag[j]
        k, a = ref.offdiag(d)
        for kk, aa in zip(k, a):
            H[index[int(kk)], j] += aa
    return float(sl.eigh(H, eigvals_only=True)[0])


# name, kind, M, ne, seeds, CISD states (empty: none), FCI (bool)
SUBSPACE = [
    ("c1", "rhf", 10, 10, (0,), (0, 2), False),
    ("r16", "rhf", 16, 8, (1,), (0,), False),
    ("u8", "uhf", 8, 6, (2, 3), (0,), True),
    ("r8", "rhf", 8, 8, (11,), (), True),
]


def subspace():
    so = orc.build_ref(REF)
    if not so:
        raise SystemExit("reference sources not available under %s" % REF)
    ref = orc.RefLib(so)
    for name, kind, M, ne, seeds, states, with_fci in SUBSPACE:
        N = 2 * M
        tmp = tempfile.mkdtemp()
        try:
            fpath = os.path.join(tmp, "sys_fcidump")
            if kind == "rhf":
                h, q, v, e = fd.synthetic_rhf(M, seeds[0])
                fd.write_fcidump_rhf(fpath, h, q, v, e, ne)
                txt = ref_convert(fpath, "-r")
            else:
                hs, aa, bb, ab, e = fd.synthetic_uhf(M, seeds[0], seeds[1])
                fd.write_fcidump_uhf(fpath, hs, aa, bb, ab, e, ne)
                txt = ref_convert(fpath, "-u")
            inp = os.path.join(tmp, "sys_IN")
            open(inp, "w").write(txt)
            ref.setup(inp, N, ne, 200000, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            hf = (1 << ne) - 1
            out = {"M": M, "ne": ne, "kind": kind, "seeds": np.array(seeds), "hf": np.uint64(hf),
                   "in_sha256": hashlib.sha256(txt.encode()).hexdigest()}
            for st in states:
                k, a, ev = orc.cisd(ref, hf, st, 10)
                out["cisd_keys"] = k
                out["cisd%d_amps" % st] = a
                out["cisd_evals"] = ev
            if with_fci:
                ev, k, a = orc.fci(ref, N, ne, 5)
                out.update(fci_evals=ev, fci_keys=k, fci_amps=a)
            np.savez_compressed(os.path.join(HERE, "sub_%s.npz" % name), **out)
            print(name, {k: (v.shape if hasattr(v, "shape") else v) for k, v in out.items() if "keys" not in k})
        finally:
            shutil.rmtree(tmp)


def linear():
    so = orc.build_ref(REF)
    if not so:
        raise SystemExit("reference sources not available under %s" % REF)
    ref = orc.RefLib(so)
    # (name, Nd of the products, output cap, Nd of the driver run): the RHF case's
    # driver runs untruncated (70000 > its 63504 determinants) because spin-mirror
    # determinants tie exactly in magnitude at a top-Nd edge and the reference
    # breaks such ties arbitrarily; the UHF case covers the truncating driver
    for name, Nd, cap, Nd_d in (("c1", 2000, 2000, 70000), ("u8", 1000, 600, 1000)):
        g = dict(np.load(os.path.join(HERE, name + ".npz")))
        M, ne, kind, seeds = int(g["M"]), int(g["ne"]), str(g["kind"]), tuple(int(x) for x in g["seeds"])
        N = 2 * M
        tmp = tempfile.mkdtemp()
        try:
            fpath = os.path.join(tmp, "sys_fcidump")
            if kind == "rhf":
                h, q, v, e = fd.synthetic_rhf(M, seeds[0])
                fd.write_fcidump_rhf(fpath, h, q, v, e, ne)
                txt = ref_convert(fpath, "-r")
            else:
                hs, aa, bb, ab, e = fd.synthetic_uhf(M, seeds[0], seeds[1])
                fd.write_fcidump_uhf(fpath, hs, aa, bb, ab, e, ne)
                txt = ref_convert(fpath, "-u")
            inp = os.path.join(tmp, "sys_IN")
            open(inp, "w").write(txt)
            ref.setup(inp, N, ne, Nd, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            v1 = (g["B_in_keys"], g["B_in_amps"])
            w = (g["w_keys"], g["w_amps"])
            e0 = float(g["L_final_e"])
            lam = e0 + 0.3
            out = {"M": M, "ne": ne, "kind": kind, "seeds": np.array(seeds),
                   "in_sha256": hashlib.sha256(txt.encode()).hexdigest(), "Nd": Nd, "cap": cap, "lam": lam,
                   "v1_keys": v1[0], "v1_amps": v1[1], "w_keys": w[0], "w_amps": w[1]}
            k, a, hh = ref.spmspv_linear([v1], 0, lam, cap)
            out.update(P0_keys=k, P0_amps=a, P0_hij=hh)
            k, a, hh = ref.spmspv_linear([v1, w], 1, lam, cap)
            out.update(P1_keys=k, P1_amps=a, P1_hij=hh)
            k, a, r = ref.res_norm(w[0], w[1], v1[0], v1[1], lam, cap)
            out.update(R_keys=k, R_amps=a, R_norm=r)
            lam_d = e0 - 0.5
            ref.setup(inp, N, ne, Nd_d, bucket_unit=BUNIT, nthread=os.cpu_count(), num_connected=2000000)
            xk, xa, rh = orc.krylov_linear(ref, v1, lam_d, 5, 3, Nd_d)
            out.update(D_Nd=Nd_d, D_lam=lam_d, D_iter=5, D_restarts=3, D_keys=xk, D_amps=xa, D_res=rh)
            np.savez_compressed(os.path.join(HERE, "lin_%s.npz" % name), **out)
            print(name, {k: (v.shape if hasattr(v, "shape") else v) for k, v in out.items() if "keys" not in k})
        finally:
            shutil.rmtree(tmp)


def krylov56(Nd=20000, Nl=30, restarts=2):
    """The truncated Lanczos driver on the 56-spin-orbital, 14-electron RHF system
    of seed 1 at a truncating Nd, over the compiled reference's SpMSpV and vector
    algebra (oracle.lanczos restates src/sparse_solver.cpp:246-548 around them),
    and the same driver over the oracle restatement.  The two CPU runs break
    magnitude ties at every top-Nd edge differently (the reference's introsort
    arbitrarily, the restatement by key): RHF spin-mirror determinants tie
    exactly, so their difference measures how far tie-breaking alone moves the
    energy.  Output: lz_r28.npz."""
    import time
    so = orc.build_ref(REF)
    if not so:
        raise SystemExit("reference sources not available under %s" % REF)
    ref = orc.RefLib(so)
    M, ne, seed = 28, 14, 1
    N = 2 * M
    tmp = tempfile.mkdtemp()
    try:
        fpath = os.path.join(tmp, "sys_fcidump")
        h, q, v, e = fd.synthetic_rhf(M, seed)
        fd.write_fcidump_rhf(fpath, h, q, v, e, ne)
        txt = ref_convert(fpath, "-r")
        inp = os.path.join(tmp, "sys_IN")
        open(inp, "w").write(txt)
        hf = np.array([(1 << ne) - 1], np.uint64)
        out = {"M": M, "ne": ne, "kind": "rhf", "seeds": np.array([seed]), "hf": np.uint64(hf[0]),
               "in_sha256": hashlib.sha256(txt.encode()).hexdigest(), "L_Nd": Nd, "L_Nl": Nl,
               "L_restarts": restarts, "L_hpsi_cap": 60000000}
        nt = os.cpu_count()
        ref.setup(inp, N, ne, Nd, bucket_unit=BUNIT, nthread=nt, num_connected=2000000)
        # The reference sizes its final buffer as len * 5000 for an input of len
        # determinants (src/functions.cpp:542,565): |HF> alone (len 1) has 12,770
        # survivors and overflows it.  Two zero-amplitude excitations of |HF> make
        # len 3; they add only zero terms, so every amplitude and energy is unchanged.
        h0 = int(hf[0])
        start = np.array(sorted([h0, h0 ^ (1 << 12) ^ (1 << 14), h0 ^ (1 << 13) ^ (1 << 15)]), np.uint64)
        start_a = np.where(start == h0, 1.0, 0.0)
        t = time.time()
        en, fe, vec = orc.lanczos(ref, start, start_a, Nl, restarts, Nd, log=print)
        out.update(L_energies=en, L_final_e=fe, L_vec_len=len(vec[1]), L_seconds=time.time() - t)
        print("reference driver:", en, fe, "%.0f s" % (time.time() - t))
        port = orc.PortLib(words=1)
        port.setup(inp, N, ne, Nd, nthread=nt)
        t = time.time()
        en2, fe2, vec2 = orc.lanczos(port, hf, np.array([1.0]), Nl, restarts, Nd)
        out.update(P_energies=en2, P_final_e=fe2, P_seconds=time.time() - t)
        ka, kb = set(int(x) for x in vec[0]), set(int(x) for x in vec2[0])
        out["P_vec_keys_differ"] = len(ka ^ kb)
        print("restated driver:", en2, fe2, "keys differing in the final vectors:", len(ka ^ kb))
        np.savez_compressed(os.path.join(HERE, "lz_r28.npz"), **out)
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    if "--krylov56" in sys.argv[1:]:
        krylov56()
    elif "--subspace" in sys.argv[1:]:
        subspace()
    elif "--linear" in sys.argv[1:]:
        linear()
    else:
        main()

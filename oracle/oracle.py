"""Oracle for the SFCI hot path — TEST INFRASTRUCTURE ONLY.

Nothing in the product imports this module; only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it, and only
as the oracle the GPU results are compared with, or as the timed CPU
reference.

Two CPU backends with one interface:

* ``RefLib`` — the reference's own SpMSpV sources (src/functions.cpp,
  src/bitstr.cpp, src/introsort.cpp) compiled unmodified into
  ``oracle/_ref/libsfci_ref.so`` by ``oracle/build_ref.sh`` (x86 container only:
  the reference tree is not present on the GPU host);
* ``PortLib`` — ``oracle/sfci_port.cpp``, a C++/OpenMP restatement of the same
  algorithm (64- and 128-bit keys), built by ``oracle/build_port.sh`` wherever it
  runs; pinned against ``RefLib`` through the golden fixtures in ``tests/golden``.

On top of either backend, ``lanczos`` restates sparse_krylov_solve_eigenval
(src/sparse_solver.cpp:246-548) and ``minres`` restates minres_sp
(src/minres.cpp:73-225) line by line; the generalised eigensolve is
scipy.linalg.eigh(K, S) (Eigen's GSAES at :450 in the reference).  ``cisd``
restates calc_CISD (src/sparse_solver.cpp:15-114) and ``fci`` restates fci over
generateBasis (src/dense_algo.cpp:14-124): dense blocks filled from the
backend's OffDiagGen_bit_e and DiagCal_bit, diagonalised by numpy.linalg.eigh
(Eigen's SelfAdjointEigenSolver in the reference; both read the lower triangle).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libsfci_ref.so")
PORT_SO = os.path.join(HERE, "_port", "libsfci_port.so")

_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ui = C.c_uint
_pu = C.POINTER(C.c_uint)
_pd = C.POINTER(C.c_double)


def build_ref(ref_root: str | None = None) -> str | None:
    """Build oracle/_ref (needs the reference tree); returns the path or None."""
    cmd = [os.path.join(HERE, "build_ref.sh")] + ([ref_root] if ref_root else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    return REF_SO if r.returncode == 0 and os.path.exists(REF_SO) else None


def build_port() -> str:
    r = subprocess.run([os.path.join(HERE, "build_port.sh")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle port build failed:\n" + r.stdout + r.stderr)
    return PORT_SO


class _Backend:
    """Common ctypes interface of the two backends (64-bit keys)."""

    prefix = ""
    words = 1

    def __init__(self, so: str):
        self.L = C.CDLL(so)
        p = self.prefix
        f = lambda n: getattr(self.L, p + n)
        f("setup").argtypes = [C.c_char_p, _ui, _ui, _ui, _ui, _ui, _ui]
        f("diag").restype = C.c_double
        f("spmspv").argtypes = [_u64p, _f64p, _ui, _ui, _ui, C.c_double, C.c_double, _u64p, _f64p, _pu, _pd]
        f("energy").restype = C.c_double
        f("energy").argtypes = [_u64p, _f64p, _ui]
        f("dot").restype = C.c_double
        f("dot").argtypes = [_u64p, _f64p, _ui, _u64p, _f64p, _ui]
        f("norm").restype = C.c_double
        f("norm").argtypes = [_u64p, _f64p, _ui]
        f("add_two").argtypes = [_u64p, _f64p, _ui, _ui, _u64p, _f64p, _ui, C.c_double, _u64p, _f64p, _pu]
        f("add_three").argtypes = [_u64p, _f64p, _ui, _u64p, _f64p, _ui, _u64p, _f64p, _ui,
                                   C.c_double, C.c_double, C.c_double, _u64p, _f64p, _pu]
        f("shrink_from").argtypes = [_u64p, _f64p, _ui, _ui, _u64p, _f64p, _pu]
        f("sort_merge").argtypes = [_u64p, _f64p, _ui]
        f("sort_merge").restype = _ui
        f("offdiag").restype = _ui
        f("spmspv_linear").argtypes = [_u64p, _f64p, np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS"), _ui,
                                       _ui, C.c_double, _ui, _u64p, _f64p, _pu, _f64p]
        f("res_norm").restype = C.c_double
        f("res_norm").argtypes = [_u64p, _f64p, _ui, _u64p, _f64p, _ui, C.c_double, _ui, _u64p, _f64p, _pu]
        self.f = f

    def _k(self, keys):
        return np.ascontiguousarray(keys, dtype=np.uint64).reshape(-1)

    def _n(self, keys):
        return np.asarray(keys).reshape(-1).size // self.words

    def setup(self, in_path, num_orb, num_e, Nd, bucket_unit=60000, nthread=0, num_connected=0):
        nthread = nthread or os.cpu_count() or 1
        self.Nd = Nd
        self.f("setup")(in_path.encode(), num_orb, num_e, Nd, bucket_unit, nthread, num_connected)

    def diag(self, dets):
        d = self._k(dets).reshape(-1, self.words)
        fn = self.f("diag")
        if self.words == 1:
            fn.argtypes = [C.c_uint64]
            return np.array([fn(int(x[0])) for x in d])
        fn.argtypes = [C.c_uint64, C.c_uint64]
        return np.array([fn(int(x[0]), int(x[1])) for x in d])

    def offdiag(self, det, cap=4000000):
        """Raw emitted terms of one determinant (unit coefficient), unmerged."""
        fn = self.f("offdiag")
        k = np.zeros(cap * self.words, np.uint64)
        a = np.zeros(cap)
        dw = self._k(det)
        if self.words == 1:
            fn.argtypes = [C.c_uint64, _u64p, _f64p, _ui]
            n = fn(int(dw[0]), k, a, cap)
        else:
            fn.argtypes = [C.c_uint64, C.c_uint64, _u64p, _f64p, _ui]
            n = fn(int(dw[0]), int(dw[1]), k, a, cap)
        n = min(n, cap)
        return k[: n * self.words].reshape(-1, self.words) if self.words > 1 else k[:n], a[:n]

    def spmspv(self, keys, amps, out_cap, lam, coeff, in_cap=None):
        keys = self._k(keys)
        amps = np.ascontiguousarray(amps, np.float64)
        n = amps.size
        ok = np.zeros(out_cap * self.words, np.uint64)
        oa = np.zeros(out_cap)
        ol = C.c_uint()
        d = C.c_double()
        self.f("spmspv")(keys, amps, n, in_cap or max(n, 1), out_cap, lam, coeff, ok, oa, C.byref(ol), C.byref(d))
        m = ol.value
        return self._shape(ok[: m * self.words]), oa[:m].copy(), d.value

    def _shape(self, k):
        return k.reshape(-1, self.words) if self.words > 1 else k.copy()

    def energy(self, keys, amps):
        return self.f("energy")(self._k(keys), np.ascontiguousarray(amps, np.float64), np.asarray(amps).size)

    def dot(self, k1, a1, k2, a2):
        return self.f("dot")(self._k(k1), np.ascontiguousarray(a1, np.float64), np.asarray(a1).size,
                             self._k(k2), np.ascontiguousarray(a2, np.float64), np.asarray(a2).size)

    def norm(self, k, a):
        return self.f("norm")(self._k(k), np.ascontiguousarray(a, np.float64), np.asarray(a).size)

    def add_two(self, vk, va, vcap, wk, wa, a):
        n = np.asarray(va).size + np.asarray(wa).size
        ok = np.zeros(max(n, 1) * self.words, np.uint64)
        oa = np.zeros(max(n, 1))
        ol = C.c_uint()
        self.f("add_two")(self._k(vk), np.ascontiguousarray(va, np.float64), np.asarray(va).size, vcap,
                          self._k(wk), np.ascontiguousarray(wa, np.float64), np.asarray(wa).size, a, ok, oa,
                          C.byref(ol))
        m = ol.value
        return self._shape(ok[: m * self.words]), oa[:m].copy()

    def add_three(self, xk, xa, yk, ya, zk, za, a, b, c):
        n = np.asarray(xa).size + np.asarray(ya).size + np.asarray(za).size
        ok = np.zeros(max(n, 1) * self.words, np.uint64)
        oa = np.zeros(max(n, 1))
        ol = C.c_uint()
        self.f("add_three")(self._k(xk), np.ascontiguousarray(xa, np.float64), np.asarray(xa).size,
                            self._k(yk), np.ascontiguousarray(ya, np.float64), np.asarray(ya).size,
                            self._k(zk), np.ascontiguousarray(za, np.float64), np.asarray(za).size,
                            a, b, c, ok, oa, C.byref(ol))
        m = ol.value
        return self._shape(ok[: m * self.words]), oa[:m].copy()

    def shrink_from(self, sk, sa, dcap):
        n = max(np.asarray(sa).size, 1)
        ok = np.zeros(n * self.words, np.uint64)
        oa = np.zeros(n)
        ol = C.c_uint()
        self.f("shrink_from")(self._k(sk), np.ascontiguousarray(sa, np.float64), np.asarray(sa).size, dcap, ok, oa,
                              C.byref(ol))
        m = ol.value
        return self._shape(ok[: m * self.words]), oa[:m].copy()

    def spmspv_linear(self, basis, cur, lam, out_cap):
        """spmspvm_bucket_linear with input basis[cur]; basis is a list of (keys, amps).
        Returns (keys, amps, Hij[0..len(basis)))."""
        bk = np.concatenate([self._k(k) for k, _ in basis]) if basis else np.zeros(0, np.uint64)
        ba = np.concatenate([np.asarray(a, np.float64) for _, a in basis])
        bl = np.array([np.asarray(a).size for _, a in basis], np.uint32)
        ok = np.zeros(max(out_cap, 1) * self.words, np.uint64)
        oa = np.zeros(max(out_cap, 1))
        ol = C.c_uint()
        h = np.zeros(len(basis))
        self.f("spmspv_linear")(np.ascontiguousarray(bk), np.ascontiguousarray(ba), bl, len(basis), cur, lam, out_cap,
                                ok, oa, C.byref(ol), h)
        m = ol.value
        return self._shape(ok[: m * self.words]), oa[:m].copy(), h

    def res_norm(self, xk, xa, bk, ba, lam, out_cap):
        """spmspvm_bucket_res_norm: (keys, amps) of the cut, top-capped A x - b and |A x - b|."""
        ok = np.zeros(max(out_cap, 1) * self.words, np.uint64)
        oa = np.zeros(max(out_cap, 1))
        ol = C.c_uint()
        r = self.f("res_norm")(self._k(xk), np.ascontiguousarray(xa, np.float64), np.asarray(xa).size, self._k(bk),
                               np.ascontiguousarray(ba, np.float64), np.asarray(ba).size, lam, out_cap, ok, oa,
                               C.byref(ol))
        m = ol.value
        return self._shape(ok[: m * self.words]), oa[:m].copy(), r

    def sort_merge(self, keys, amps):
        k = self._k(keys).copy()
        a = np.ascontiguousarray(amps, np.float64).copy()
        m = self.f("sort_merge")(k, a, a.size)
        return self._shape(k[: m * self.words]), a[:m].copy()


class RefLib(_Backend):
    prefix = "ref_"
    words = 1

    def __init__(self, so: str = REF_SO):
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        super().__init__(so)


class PortLib(_Backend):
    prefix = "port_"

    def __init__(self, so: str = PORT_SO, words: int = 1):
        if not os.path.exists(so):
            build_port()
        self.words = words
        self.prefix = "port%d_" % (64 * words)
        super().__init__(so)

    def set_nd(self, Nd):
        """Change the global Nd without re-reading the integral file."""
        self.f("set_nd").argtypes = [_ui]
        self.f("set_nd")(int(Nd))
        self.Nd = int(Nd)

    def set_cut(self, cut):
        """The post-merge cut |a| > cut of spmspv (1e-5 by default; negative keeps every term)."""
        self.f("set_cut").argtypes = [C.c_double]
        self.f("set_cut")(float(cut))


# ---------------------------------------------------------------------------
# drivers restated on top of a backend
# ---------------------------------------------------------------------------

def gsaes(K, S):
    import scipy.linalg as sl
    return sl.eigh(K, S)


def lanczos(be, v_keys, v_amps, Nl, num_restart, Nd, hpsi_cap=60000000, log=None):
    """sparse_krylov_solve_eigenval, restated (src/sparse_solver.cpp:246-548)."""
    deltaE = 0.00001
    previousE = 0.0
    nearestE = -1000000.0
    v = (np.asarray(v_keys), np.asarray(v_amps, np.float64))
    energies = []
    for res in range(num_restart):
        KB = [None] * Nl
        KB[0] = (v[0].copy(), v[1].copy())
        KM = np.zeros((Nl, Nl))
        S = np.zeros((Nl, Nl))
        uk, ua, alpha = be.spmspv(v[0], v[1], hpsi_cap, 0.0, 1.0)
        KM[0, 0] = alpha
        for i in range(1, Nl):
            tk, ta = be.add_two(uk, ua, hpsi_cap, v[0], v[1], -alpha)
            nk, na = be.shrink_from(tk, ta, Nd)
            gamma = be.norm(nk, na)
            beta = gamma
            na = na * (1.0 / gamma)
            tuk, tua, alpha = be.spmspv(nk, na, hpsi_cap, 0.0, 1.0)
            KM[i, i] = alpha
            for j in range(i):
                KM[j, i] = be.dot(KB[j][0], KB[j][1], tuk, tua)
                KM[i, j] = KM[j, i]
            uk, ua = be.add_two(tuk, tua, hpsi_cap, v[0], v[1], -beta)
            v = (nk, na)
            KB[i] = (nk.copy(), na.copy())
        for i in range(Nl):
            for j in range(i, Nl):
                S[i, j] = be.dot(KB[i][0], KB[i][1], KB[j][0], KB[j][1])
                S[j, i] = S[i, j]
        lam, vec = gsaes(KM, S)
        idx = 0
        gap = abs(nearestE - lam[0])
        for i in range(1, Nl):
            if abs(nearestE - lam[i]) < gap:
                gap = abs(nearestE - lam[i])
                idx = i
        nearestE = lam[idx]
        coeff = vec[:, idx]
        ck = np.concatenate([KB[i][0] for i in range(Nl)])
        ca = np.concatenate([KB[i][1] * coeff[i] for i in range(Nl)])
        vk, va = be.sort_merge(ck, ca)
        vk, va = be.shrink_from(vk, va, Nd)
        va = va * (1.0 / be.norm(vk, va))
        v = (vk, va)
        energies.append(lam[idx])
        if log:
            log("gsaes energy:%.12f" % lam[idx])
        if previousE - lam[idx] < deltaE:
            break
        previousE = lam[idx]
    final_e = be.energy(v[0], v[1])
    return np.array(energies), final_e, v


def minres(be, rhs, guess, iters, tol, lam, Nd):
    """minres_sp, restated (src/minres.cpp:73-225); vectors are (keys, amps)."""
    rk, ra = rhs
    x = (np.asarray(guess[0]).copy(), np.asarray(guess[1], np.float64).copy())
    vk, va, _ = be.spmspv(x[0], x[1], Nd, lam, -1.0)
    v_new = be.add_two(vk, va, Nd, rk, ra, 1.0)
    residualNorm2 = be.norm(*v_new) ** 2
    w_new = (v_new[0].copy(), v_new[1].copy())
    beta_new2 = be.dot(v_new[0], v_new[1], w_new[0], w_new[1])
    beta_new = np.sqrt(beta_new2)
    beta_one = beta_new
    v_new = (v_new[0], v_new[1] / beta_new)
    w_new = (w_new[0], w_new[1] / beta_new)
    c = 1.0; c_old = 1.0; s = 0.0; s_old = 0.0; eta = 1.0
    empty = (np.zeros((0, be.words) if be.words > 1 else 0, np.uint64), np.zeros(0))
    v = empty
    p_old = empty
    p = empty
    it = 0
    done = 0
    while it < iters:
        beta = beta_new
        v_old = v
        v = v_new
        w = w_new
        nk, na, _ = be.spmspv(w[0], w[1], Nd, lam, 1.0)
        v_new = be.add_two(nk, na, Nd, v_old[0], v_old[1], -beta)
        alpha = be.dot(v_new[0], v_new[1], w[0], w[1])
        v_new = be.add_two(v_new[0], v_new[1], Nd, v[0], v[1], -alpha)
        w_new = (v_new[0].copy(), v_new[1].copy())
        beta_new2 = be.dot(v_new[0], v_new[1], w_new[0], w_new[1])
        beta_new = np.sqrt(beta_new2)
        v_new = (v_new[0], v_new[1] / beta_new)
        w_new = (w_new[0], w_new[1] / beta_new)
        r2 = s * alpha + c * c_old * beta
        r3 = s_old * beta
        r1_hat = c * alpha - c_old * s * beta
        r1 = np.sqrt(r1_hat ** 2 + beta_new ** 2)
        c_old = c
        s_old = s
        c = r1_hat / r1
        s = beta_new / r1
        p_oold = p_old
        p_old = p
        p = be.add_three(w[0], w[1], p_old[0], p_old[1], p_oold[0], p_oold[1], 1.0 / r1, -r2 / r1, -r3 / r1)
        x = be.add_two(x[0], x[1], Nd, p[0], p[1], beta_one * c * eta)
        residualNorm2 *= s * s
        done += 1
        if residualNorm2 < tol:
            break
        eta = -s * eta
        it += 1
    return x, done


# ---------------------------------------------------------------------------
# dense subspace diagonalisations
# ---------------------------------------------------------------------------

def _rows(be, keys):
    """(n, words) uint64 rows of a key array."""
    return np.ascontiguousarray(keys, dtype=np.uint64).reshape(-1, be.words)


def _void(rows):
    """One opaque sortable scalar per key row (byte order; a consistent total order)."""
    r = np.ascontiguousarray(rows)
    return r.view(np.dtype((np.void, r.shape[1] * 8))).reshape(-1)


def _ints(rows):
    return [int(r[0]) | (int(r[1]) << 64) if r.size > 1 else int(r[0]) for r in rows]


def _sort_by_key(rows, amps):
    order = sorted(range(len(rows)), key=lambda i: _ints(rows[i:i + 1])[0])
    return rows[order], amps[order]


def fix_sign(x):
    """The device results' sign convention: the largest |x| (lowest index on ties) is positive."""
    x = np.asarray(x, np.float64)
    i = int(np.argmax(np.abs(x)))
    return -x if x[i] < 0 else x


def dense_block(be, basis):
    """H restricted to ``basis`` (rows of key words), filled row by row as
    calc_CISD does (src/sparse_solver.cpp:54-85): H[i, i] = DiagCal_bit, and
    H[i, p] = the summed OffDiagGen_bit_e amplitudes of basis[i] that land on
    basis[p] (summed in emission order, as its unordered_map accumulates)."""
    basis = _rows(be, basis)
    n = basis.shape[0]
    bv = _void(basis)
    order = np.argsort(bv, kind="stable")
    sorted_v = bv[order]
    H = np.zeros((n, n))
    diag = be.diag(basis)
    cap = 4000000
    for i in range(n):
        det = basis[i] if be.words > 1 else basis[i, 0]
        k, a = be.offdiag(det, cap)
        while a.size == cap:  # possibly truncated: retry wider
            cap *= 4
            k, a = be.offdiag(det, cap)
        cap = max(cap if i else 0, 2 * a.size + 1024)
        kv = _void(_rows(be, k))
        u, inv = np.unique(kv, return_inverse=True)
        sums = np.zeros(u.size)
        np.add.at(sums, inv, a)
        H[i, i] = diag[i]
        loc = np.searchsorted(sorted_v, u)
        ok = loc < n
        ok[ok] = sorted_v[loc[ok]] == u[ok]
        H[i, order[loc[ok]]] = sums[ok]
    return H


def cisd(be, ref_det, state_idx=0, n_evals=10):
    """calc_CISD, restated (src/sparse_solver.cpp:15-114).  Returns (keys ascending,
    eigenvector state_idx with fix_sign applied, the n_evals lowest eigenvalues)."""
    ref = _rows(be, ref_det)[:1]
    k, _ = be.offdiag(ref[0] if be.words > 1 else ref[0, 0])
    kr = _rows(be, k)
    # basis: ref_det, then the distinct targets in first-appearance order (:28-43)
    _, first = np.unique(_void(kr), return_index=True)
    basis = np.concatenate([ref, kr[np.sort(first)]])
    H = dense_block(be, basis)
    ev, X = np.linalg.eigh(H, UPLO="L")
    keys, amps = _sort_by_key(basis, X[:, state_idx])
    keys = keys if be.words > 1 else keys[:, 0]
    return keys, fix_sign(amps), ev[:n_evals]


def fci_basis(be, N, ne):
    """Every determinant with ne/2 alpha (even bits) and ne/2 beta (odd bits)
    electrons: the set comb_det keeps (src/dense_algo.cpp:14-52), keys ascending."""
    import itertools
    M = N // 2
    na = nb = ne // 2
    alphas = [sum(1 << (2 * o) for o in c) for c in itertools.combinations(range(M), na)]
    betas = [sum(1 << (2 * o + 1) for o in c) for c in itertools.combinations(range(M), nb)]
    dets = sorted(a | b for a in alphas for b in betas)
    m = (1 << 64) - 1
    rows = np.array([[d & m, d >> 64] if be.words > 1 else [d] for d in dets], dtype=np.uint64)
    return rows


def fci(be, N, ne, n_evals=1):
    """fci, restated (src/dense_algo.cpp:77-124).  Returns (the n_evals lowest
    eigenvalues, keys ascending, ground state with fix_sign applied)."""
    basis = fci_basis(be, N, ne)
    H = dense_block(be, basis)
    ev, X = np.linalg.eigh(H, UPLO="L")
    keys = basis if be.words > 1 else basis[:, 0]
    return ev[:n_evals], keys, fix_sign(X[:, 0])


# ---------------------------------------------------------------------------
# linear (shift-invert) solver
# ---------------------------------------------------------------------------

def krylov_linear(be, b, target_energy, num_iter, num_restart, Nd, log=None):
    """sparse_krylov_solve_linear, restated (src/sparse_solver.cpp:561-730), on a
    backend's spmspv_linear / res_norm / dot / norm / add_two primitives; the
    least-squares solve is numpy.linalg.lstsq (Eigen's colPivHouseholderQr at
    :692).  b = (keys, amps); returns (x keys, x amps, residual norms per restart)."""
    bk, ba = np.asarray(b[0]), np.asarray(b[1], np.float64)
    n1 = num_iter + 1
    x = (bk[:0].copy(), np.zeros(0))
    r0 = (bk.copy(), ba.copy())
    hess = np.zeros((n1, n1))
    S = np.zeros((n1, n1))
    res_hist = []
    for res in range(num_restart):
        beta = be.norm(*r0)
        V = [(r0[0].copy(), r0[1] / be.norm(*r0))]
        if log:
            log("initial residue: %.12g" % beta)
        for i in range(n1):
            wk, wa, h = be.spmspv_linear(V, i, target_energy, Nd)
            for j in range(i, -1, -1):
                hess[j, i] = h[j]
                hess[i, j] = hess[j, i]
                S[i, j] = be.dot(V[j][0], V[j][1], V[i][0], V[i][1])
                S[j, i] = S[i, j]
            wa = wa / be.norm(wk, wa)
            if i < num_iter:
                V.append((wk, wa))
        y = np.linalg.lstsq(S @ hess[:, :num_iter], S[:, 0] * beta, rcond=None)[0]
        # add_bucketed_vec (src/functions.cpp:807-856): sum_j y_j V_j, merged, no cut
        ck = np.concatenate([V[j][0] for j in range(num_iter)])
        ca = np.concatenate([V[j][1] * y[j] for j in range(num_iter)])
        rk, ra = be.sort_merge(ck, ca)
        x = be.add_two(x[0], x[1], Nd, rk, ra, 1.0)
        r0k, r0a, rn = be.res_norm(x[0], x[1], bk, ba, target_energy, Nd)
        r0 = (r0k, -r0a)
        res_hist.append(rn)
        if log:
            log("residue after truncation: %.12g" % rn)
    return x[0], x[1], np.array(res_hist)

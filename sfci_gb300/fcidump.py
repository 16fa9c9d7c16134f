"""FCIDUMP tools: a seeded synthetic-integral generator, an FCIDUMP writer/reader,
and the FCIDUMP -> ``_IN`` converter.

The ``_IN`` format is the reformatted integral file read by SFCI
(``util/convert_fcidump.py`` writes it, ``src/functions.cpp:297-395`` reads it):
seven groups ``uu, dd, ud, du, u, d, c``, each a count line followed by
``coeff m n p q`` lines.  Spin orbital ``2*i + s`` (``i`` the 1-based spatial
index, ``s = 1`` for "u" and ``0`` for "d") is written, and the reader subtracts 2,
so spin orbital ``b`` has spatial index ``b >> 1`` and spin ``b & 1``
(``util/convert_fcidump.py:100-108``).

The converter here restates ``conv_rhf`` (``util/convert_fcidump.py:31-151``)
and ``conv_uhf`` (``:154-276``) with numpy instead of per-line dict lookups:

* every two-body item ``(ij|kl)`` of a spin group ``(s1, s2)`` expands to the
  spin-orbital tuples ``m=2i+s1, n=2j+s1, p=2k+s2, q=2l+s2`` and up to eight
  permutations, the first four kept when ``m != p and n != q`` and the last four
  when ``n != p and m != q`` (``:110-122``);
* a tuple is written only the first time it is met, across all four two-body
  groups, in emission order (the shared ``isIn`` dict, ``:21-29,86``);
* one-body items write ``(m, n)`` and, when ``m != n``, ``(n, m)`` (``:131-143``);
* the coefficient token is copied from the FCIDUMP text unchanged (``:19``).

The UHF layout splits the data after the namelist at lines whose four indices
and value are all zero (``:180-183``) and reuses the third block (alpha-beta)
for both ``ud`` and ``du`` (``:194-197``).  Both readers start data after the
line that is exactly ``' /\\n'`` (``:77,190``).
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "synthetic_rhf", "synthetic_uhf", "write_fcidump_rhf", "write_fcidump_uhf",
    "read_fcidump", "convert_rhf", "convert_uhf", "write_in", "rhf_to_in_file",
    "uhf_to_in_file", "format_coeff", "hf_determinant",
]


def format_coeff(x: float) -> str:
    """FCIDUMP coefficient token: 17 significant digits, so it parses back exactly."""
    return "%.16E" % x


# --------------------------------------------------------------------------
# synthetic integrals
# --------------------------------------------------------------------------

def _unique_quads(M: int):
    """Canonical unique (ij|kl) index quadruples, 0-based: i>=j, k>=l, ij>=kl."""
    ii, jj = np.tril_indices(M)          # i >= j, row-major over i
    P = ii.size
    a, b = np.tril_indices(P)            # pair index a >= b
    return ii[a], jj[a], ii[b], jj[b]


def _two_body_values(rng, i, j, k, l):
    """Values of the synthetic two-electron distribution for canonical quads.

    (pp|qq) ~ U(0.3, 0.8); (pq|pq) ~ U(0.01, 0.1) for p != q; every other
    (pq|rs) ~ N(0, 0.01 * exp(-(|p-q| + |r-s|) / 4)).
    """
    n = i.size
    coulomb = (i == j) & (k == l)
    exchange = (~coulomb) & (((i == k) & (j == l)) | ((i == l) & (j == k)))
    other = ~(coulomb | exchange)
    v = np.empty(n)
    v[coulomb] = rng.uniform(0.3, 0.8, size=int(coulomb.sum()))
    v[exchange] = rng.uniform(0.01, 0.1, size=int(exchange.sum()))
    sig = 0.01 * np.exp(-(np.abs(i - j) + np.abs(k - l)) / 4.0)
    v[other] = rng.normal(0.0, 1.0, size=int(other.sum())) * sig[other]
    return v


def _one_body(rng, M: int):
    """h_pp = -3 + 0.25 p;  h_pq ~ N(0, 0.05 exp(-|p-q|/3)), symmetric."""
    h = np.diag(-3.0 + 0.25 * np.arange(M))
    p, q = np.tril_indices(M, -1)
    h[p, q] = rng.normal(0.0, 1.0, size=p.size) * 0.05 * np.exp(-np.abs(p - q) / 3.0)
    h[q, p] = h[p, q]
    return h


def synthetic_rhf(M: int, seed: int):
    """Seeded synthetic RHF integrals (8-fold symmetric, FP64, core energy 0).

    Returns ``(h, quads, values, ecore)``: ``h`` is the MxM one-body matrix,
    ``quads`` the canonical unique (i,j,k,l) 0-based index arrays and ``values``
    their (ij|kl).
    """
    rng = np.random.default_rng(seed)
    h = _one_body(rng, M)
    i, j, k, l = _unique_quads(M)
    v = _two_body_values(rng, i, j, k, l)
    return h, (i, j, k, l), v, 0.0


def bond_stretch_rhf(M: int, seed: int, t: float):
    """A point of the synthetic bond-stretch curve: the seeded RHF integrals with
    the off-diagonal one-body elements and the 'other' two-body values scaled by
    (1 + 3t), and the gap of the diagonal one-body elements, h_pp + 3 =
    0.25 p, scaled by (1 - 0.6t); Coulomb (pp|qq) and exchange (pq|pq) values
    are those of t = 0.  t runs over [0, 1]."""
    h, (i, j, k, l), v, e = synthetic_rhf(M, seed)
    off = ~np.eye(M, dtype=bool)
    h = h.copy()
    h[off] *= 1.0 + 3.0 * t
    h[np.diag_indices(M)] = -3.0 + 0.25 * np.arange(M) * (1.0 - 0.6 * t)
    coulomb = (i == j) & (k == l)
    exchange = (~coulomb) & (((i == k) & (j == l)) | ((i == l) & (j == k)))
    v = np.where(coulomb | exchange, v, v * (1.0 + 3.0 * t))
    return h, (i, j, k, l), v, e


def bond_stretch_to_in_file(out_path: str, M: int, ne: int, seed: int, t: float,
                            fcidump_path: str | None = None):
    """The bond-stretch point (M, seed, t) -> FCIDUMP -> ``_IN``.  Returns the _IN path."""
    h, q, v, e = bond_stretch_rhf(M, seed, t)
    fd = fcidump_path or (out_path + ".fcidump")
    write_fcidump_rhf(fd, h, q, v, e, ne)
    write_in(out_path, convert_rhf(fd))
    return out_path


def bond_stretch_curve(n: int = 32, seed: int = 4, scale: float = 1.0):
    """The n instances of the batched bond-stretch workload: t_i = i/(n-1);
    num_orb unevenly in [40, 80] spin orbitals (a quadratic ramp, even), num_e
    in {10, 12, 14, 16} by t, Nd geometric from 1e5 to 2e6 (times `scale`).
    Returns a list of dicts (t, num_orb, num_e, Nd, seed)."""
    out = []
    for i in range(n):
        t = i / max(n - 1, 1)
        M = 20 + int(round(20 * t * t))
        ne = 10 + 2 * min(3, int(4 * t))
        nd = int(round(1e5 * (20.0 ** t) * scale))
        out.append({"t": t, "num_orb": 2 * M, "num_e": ne, "Nd": max(nd, 16), "seed": seed})
    return out


def synthetic_uhf(M: int, seed_a: int, seed_b: int):
    """Seeded synthetic UHF integrals.

    alpha (h, (pq|rs)) come from ``seed_a``, beta from ``seed_b``, each with the
    RHF distributions.  The alpha-beta block is the mean of the two same-spin
    tensors, written over every i>=j, k>=l pair combination (not restricted to
    ij>=kl, since the block is not symmetric under pair exchange in general).
    """
    ha, (i, j, k, l), va, _ = synthetic_rhf(M, seed_a)
    hb, _, vb, _ = synthetic_rhf(M, seed_b)
    ii, jj = np.tril_indices(M)
    P = ii.size
    # full pair x pair table for the ab block: index by canonical pair ids
    pid = lambda x, y: np.maximum(x, y) * (np.maximum(x, y) + 1) // 2 + np.minimum(x, y)
    ta = np.zeros((P, P)); tb = np.zeros((P, P))
    a = pid(i, j); b = pid(k, l)
    ta[a, b] = va; ta[b, a] = va
    tb[a, b] = vb; tb[b, a] = vb
    tab = 0.5 * (ta + tb)
    A, B = np.meshgrid(np.arange(P), np.arange(P), indexing="ij")
    A = A.ravel(); B = B.ravel()
    ab = (ii[A], jj[A], ii[B], jj[B]), tab.ravel()
    return (ha, hb), ((i, j, k, l), va), ((i, j, k, l), vb), ab, 0.0


def hf_determinant(num_e: int) -> int:
    """Lowest ``num_e`` spin orbitals occupied (alpha/beta interleaved)."""
    return (1 << num_e) - 1


# --------------------------------------------------------------------------
# FCIDUMP text
# --------------------------------------------------------------------------

def _header(M: int, ne: int, uhf: bool) -> str:
    s = " &FCI NORB=%d,NELEC=%d,MS2=0,\n" % (M, ne)
    s += "  ORBSYM=" + ",".join(["1"] * M) + ",\n  ISYM=1,\n"
    if uhf:
        s += "  IUHF=1,\n"
    s += " /\n"
    return s


def _lines(vals, i, j, k, l):
    tok = [format_coeff(x) for x in np.asarray(vals, dtype=np.float64)]
    return ["%s %d %d %d %d\n" % (t, a, b, c, d)
            for t, a, b, c, d in zip(tok, i.tolist(), j.tolist(), k.tolist(), l.tolist())]


def _one_body_lines(h):
    M = h.shape[0]
    p, q = np.tril_indices(M)
    z = np.zeros_like(p)
    return _lines(h[p, q], p + 1, q + 1, z, z)


def write_fcidump_rhf(path: str, h, quads, values, ecore: float, ne: int):
    M = h.shape[0]
    i, j, k, l = quads
    with open(path, "w") as f:
        f.write(_header(M, ne, False))
        f.writelines(_lines(values, i + 1, j + 1, k + 1, l + 1))
        f.writelines(_one_body_lines(h))
        f.write("%s 0 0 0 0\n" % format_coeff(ecore))


def write_fcidump_uhf(path: str, hs, aa, bb, ab, ecore: float, ne: int):
    """UHF FCIDUMP in the block layout ``conv_uhf`` expects: aa, bb, ab, h_a,
    h_b, core, each block closed by an all-zero line."""
    ha, hb = hs
    M = ha.shape[0]
    zero = "%s 0 0 0 0\n" % format_coeff(0.0)
    with open(path, "w") as f:
        f.write(_header(M, ne, True))
        for (q, v) in (aa, bb, ab):
            i, j, k, l = q
            f.writelines(_lines(v, i + 1, j + 1, k + 1, l + 1))
            f.write(zero)
        for h in (ha, hb):
            f.writelines(_one_body_lines(h))
            f.write(zero)
        f.write("%s 0 0 0 0\n" % format_coeff(ecore))


def read_fcidump(path: str):
    """Parse an FCIDUMP: returns (header_text, tokens, idx[n,4]) for the data lines
    after the line that is exactly ``' /\\n'``."""
    head = []
    toks = []
    idx = []
    started = False
    with open(path) as f:
        for line in f:
            if started:
                t = line.split()
                if len(t) < 5:
                    continue
                toks.append(t[0])
                idx.append((int(t[1]), int(t[2]), int(t[3]), int(t[4])))
            else:
                head.append(line)
            if line == " /\n":
                started = True
    if not started:
        raise ValueError("FCIDUMP namelist terminator ' /' line not found: %s" % path)
    return "".join(head), np.array(toks, dtype=object), np.array(idx, dtype=np.int64).reshape(-1, 4)


# --------------------------------------------------------------------------
# FCIDUMP -> _IN
# --------------------------------------------------------------------------

_PERM_A = ((0, 1, 2, 3), (1, 0, 3, 2), (2, 3, 0, 1), (3, 2, 1, 0))   # m!=p and n!=q
_PERM_B = ((1, 0, 2, 3), (2, 3, 1, 0), (0, 1, 3, 2), (3, 2, 0, 1))   # n!=p and m!=q


def _expand_two_body(idx, s1, s2):
    """Candidate spin-orbital tuples of one two-body group in emission order.
    Returns (tuples[n*8,4], item_index[n*8]) restricted to the valid slots."""
    m = (idx[:, 0] << 1) + s1
    n = (idx[:, 1] << 1) + s1
    p = (idx[:, 2] << 1) + s2
    q = (idx[:, 3] << 1) + s2
    base = np.stack([m, n, p, q], axis=1)
    okA = (m != p) & (n != q)
    okB = (n != p) & (m != q)
    slots = []
    valid = []
    for perm in _PERM_A:
        slots.append(base[:, perm]); valid.append(okA)
    for perm in _PERM_B:
        slots.append(base[:, perm]); valid.append(okB)
    tup = np.stack(slots, axis=1).reshape(-1, 4)          # item-major, slot-minor
    val = np.stack(valid, axis=1).reshape(-1)
    item = np.repeat(np.arange(idx.shape[0]), 8)
    return tup[val], item[val]


def _convert(groups2, groups1, const_toks):
    """groups2: list of 4 (tokens, idx, s1, s2); groups1: list of 2 (tokens, idx, s)."""
    out = []
    cand = []
    for toks, idx, s1, s2 in groups2:
        t, it = _expand_two_body(idx, s1, s2)
        cand.append((toks, t, it))
    allkeys = np.concatenate([(c[1][:, 0] << 27) | (c[1][:, 1] << 18) | (c[1][:, 2] << 9) | c[1][:, 3]
                              for c in cand]) if cand else np.zeros(0, np.int64)
    _, first = np.unique(allkeys, return_index=True)
    keep = np.zeros(allkeys.size, dtype=bool)
    keep[first] = True
    off = 0
    for toks, t, it in cand:
        kk = keep[off:off + t.shape[0]]
        off += t.shape[0]
        out.append((toks[it[kk]], t[kk]))
    for toks, idx, s in groups1:
        m = (idx[:, 0] << 1) + s
        n = (idx[:, 1] << 1) + s
        z = np.zeros_like(m)
        a = np.stack([m, n, z, z], axis=1)
        b = np.stack([n, m, z, z], axis=1)
        both = np.stack([a, b], axis=1).reshape(-1, 4)
        ok = np.stack([np.ones(m.size, bool), m != n], axis=1).reshape(-1)
        it = np.repeat(np.arange(m.size), 2)[ok]
        out.append((toks[it], both[ok]))
    out.append((np.asarray(const_toks, dtype=object), np.zeros((len(const_toks), 4), np.int64)))
    return out


def convert_rhf(path: str):
    """FCIDUMP (RHF) -> list of 7 groups ``(tokens, tuples[n,4])`` as conv_rhf writes them."""
    _, toks, idx = read_fcidump(path)
    isconst = np.all(idx == 0, axis=1)
    isone = (~isconst) & (idx[:, 2] == 0) & (idx[:, 3] == 0)
    istwo = ~(isconst | isone)
    t2, i2 = toks[istwo], idx[istwo]
    t1, i1 = toks[isone], idx[isone][:, :2]
    groups2 = [(t2, i2, 1, 1), (t2, i2, 0, 0), (t2, i2, 1, 0), (t2, i2, 0, 1)]
    groups1 = [(t1, i1, 1), (t1, i1, 0)]
    return _convert(groups2, groups1, list(toks[isconst]))


def convert_uhf(path: str):
    """FCIDUMP (UHF block layout) -> list of 7 groups as conv_uhf writes them."""
    _, toks, idx = read_fcidump(path)
    vals = np.array([float(t) for t in toks]) if toks.size else np.zeros(0)
    sep = np.all(idx == 0, axis=1) & (vals == 0.0)
    blocks = []
    start = 0
    for s in np.nonzero(sep)[0].tolist() + [idx.shape[0]]:
        blocks.append((toks[start:s], idx[start:s]))
        start = s + 1
    blocks = blocks[:3] + [blocks[2]] + blocks[3:]
    while len(blocks) < 7:
        blocks.append((np.zeros(0, dtype=object), np.zeros((0, 4), np.int64)))
    groups2 = [(blocks[0][0], blocks[0][1], 1, 1), (blocks[1][0], blocks[1][1], 0, 0),
               (blocks[2][0], blocks[2][1], 1, 0), (blocks[3][0], blocks[3][1], 0, 1)]
    groups1 = [(blocks[4][0], blocks[4][1][:, :2], 1), (blocks[5][0], blocks[5][1][:, :2], 0)]
    return _convert(groups2, groups1, list(blocks[6][0]))


def write_in(path: str, groups):
    with open(path, "w") as f:
        for toks, t in groups:
            f.write("%d\n" % len(toks))
            f.writelines(["%s %d %d %d %d\n" % (a, m, n, p, q)
                          for a, (m, n, p, q) in zip(toks, t.tolist())])


def rhf_to_in_file(out_path: str, M: int, ne: int, seed: int, fcidump_path: str | None = None):
    """Synthetic RHF system (seed) -> FCIDUMP -> ``_IN``.  Returns the _IN path."""
    h, q, v, e = synthetic_rhf(M, seed)
    fd = fcidump_path or (out_path + ".fcidump")
    write_fcidump_rhf(fd, h, q, v, e, ne)
    write_in(out_path, convert_rhf(fd))
    return out_path


def uhf_to_in_file(out_path: str, M: int, ne: int, seed_a: int, seed_b: int,
                   fcidump_path: str | None = None):
    hs, aa, bb, ab, e = synthetic_uhf(M, seed_a, seed_b)
    fd = fcidump_path or (out_path + ".fcidump")
    write_fcidump_uhf(fd, hs, aa, bb, ab, e, ne)
    write_in(out_path, convert_uhf(fd))
    return out_path

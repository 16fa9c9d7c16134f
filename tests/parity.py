"""Comparison of sparse vectors produced by two implementations of the hot path.

Bit-exact key sets are required except for keys whose magnitude sits on a
selection boundary, which both implementations may decide either way:

* the post-merge cut |a| > cut (src/functions.cpp:750): amplitudes are sums whose
  order differs between implementations (the reference's introsort is unstable),
  so a key within ``edge_rtol`` of the cut is reported, not failed;
* a top-cap truncation: keys tied (within ``edge_rtol``) with the smallest kept
  magnitude are reported, not failed.

Amplitudes of common keys must agree within ``rtol`` relative, with an absolute
floor ``atol`` for sums that cancel to far below their summands (the reference's
own summation order is arbitrary, so no ordering is "the" exact answer).
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-12
ATOL = 1e-14
EDGE_RTOL = 1e-9


def _as_obj_keys(k):
    k = np.asarray(k, dtype=np.uint64)
    if k.ndim == 2:
        return [int(a) | (int(b) << 64) for a, b in k]
    return [int(x) for x in k]


def compare_vectors(ref_k, ref_a, got_k, got_a, cut=None, capped=False, rtol=RTOL, atol=ATOL,
                    edge_rtol=EDGE_RTOL):
    """Returns a report dict; raises AssertionError on a real mismatch."""
    rk = _as_obj_keys(ref_k)
    gk = _as_obj_keys(got_k)
    ra = np.asarray(ref_a, dtype=np.float64)
    ga = np.asarray(got_a, dtype=np.float64)
    assert len(set(gk)) == len(gk), "duplicate keys in result"
    assert all(gk[i] < gk[i + 1] for i in range(len(gk) - 1)), "result not in ascending key order"
    rmap = dict(zip(rk, ra))
    gmap = dict(zip(gk, ga))
    only_r = [k for k in rk if k not in gmap]
    only_g = [k for k in gk if k not in rmap]
    floor = None
    if capped and len(ra):
        floor = min(np.min(np.abs(ra)), np.min(np.abs(ga)) if len(ga) else np.inf)

    def on_edge(a):
        a = abs(a)
        if cut is not None and abs(a - cut) <= edge_rtol * cut:
            return True
        if floor is not None and a <= floor * (1 + edge_rtol) + atol:
            return True
        return False

    bad_r = [k for k in only_r if not on_edge(rmap[k])]
    bad_g = [k for k in only_g if not on_edge(gmap[k])]
    assert not bad_r and not bad_g, (
        "key sets differ beyond the selection edges: %d only in reference (e.g. %s), %d only in result (e.g. %s)"
        % (len(bad_r), [(hex(k), rmap[k]) for k in bad_r[:3]], len(bad_g), [(hex(k), gmap[k]) for k in bad_g[:3]]))
    common = [k for k in rk if k in gmap]
    a = np.array([rmap[k] for k in common])
    b = np.array([gmap[k] for k in common])
    err = np.abs(a - b)
    lim = rtol * np.maximum(np.abs(a), np.abs(b)) + atol
    worst = int(np.argmax(err - lim)) if len(err) else 0
    assert np.all(err <= lim), "amplitude mismatch at %s: %r vs %r" % (hex(common[worst]), a[worst], b[worst])
    rel = float(np.max(err / np.maximum(np.abs(a), 1e-300))) if len(err) else 0.0
    return {"common": len(common), "edge_only_ref": len(only_r), "edge_only_got": len(only_g), "max_rel": rel}


def close(a, b, rtol=1e-12, atol=1e-12):
    return abs(a - b) <= rtol * max(abs(a), abs(b)) + atol

// Term groups of the learned excitation screen.
//
// A source determinant's terms (the index space of gen.cuh) are split into
// groups that the screen keeps or skips as a whole:
//   group 0                the diagonal and every single excitation (always kept)
//   same-spin doubles      (occupied pair x < y of spin s, larger hole v): the
//                          v terms i_x i_y -> a_u a_v, u < v; contiguous in the
//                          term index space (colex pair ranks with a fixed larger
//                          element are consecutive)
//   opposite-spin doubles  (spin-0 single i -> a, spin-1 occupied j): the nv1
//                          terms i -> a, j -> b over the spin-1 holes b
// A group is named by its excitation prefix (p, q, r) = (i, j, a_v) or
// (i, j, a) in spin orbitals and a class (1, 2: same-spin of spin 0, 1;
// 3: opposite spin); the one index left free is what the group spans.
//
// The screen's features per group are the source's occupancy bits, one-hot
// p, q, r and class, log10 |c_j| and log10 of a bound on the group's largest
// two-body element, max over the free index of |(pq|rs)|-type integrals,
// read from a table of row maxima built once per Hamiltonian.
#pragma once

#include "gen.cuh"

namespace sfci {

// groups of a determinant with na[s] electrons and nv[s] holes, group 0 included
SFCI_HD u64 det_groups(unsigned na0, unsigned nv0, unsigned na1, unsigned nv1) {
  const u64 g0 = nv0 ? (u64)c2(na0) * (nv0 - 1) : 0, g1 = nv1 ? (u64)c2(na1) * (nv1 - 1) : 0;
  return 1ull + g0 + g1 + (u64)na0 * nv0 * na1;
}

struct GroupCounts {
  unsigned na[2], nv[2];
  unsigned gss[2];  // same-spin groups per spin
  unsigned gos;     // opposite-spin groups
};
SFCI_HD GroupCounts group_counts(unsigned na0, unsigned nv0, unsigned na1, unsigned nv1) {
  GroupCounts g;
  g.na[0] = na0;
  g.na[1] = na1;
  g.nv[0] = nv0;
  g.nv[1] = nv1;
  g.gss[0] = nv0 ? c2(na0) * (nv0 - 1) : 0;
  g.gss[1] = nv1 ? c2(na1) * (nv1 - 1) : 0;
  g.gos = na0 * nv0 * na1;
  return g;
}

// A group g >= 1 as (class, list positions) and its term range in the full
// term index space of the determinant (class boundaries c[2], c[3], c[4]).
struct GroupDesc {
  int cls;                 // 1, 2: same-spin of spin cls-1; 3: opposite spin
  unsigned x, y, v;        // same-spin: occupied positions x < y, larger hole v; opposite: single x, beta occ y
  unsigned start, size;    // full term index range [start, start + size)
};

SFCI_HD void unrank_pair(unsigned k, unsigned& x, unsigned& y) {
  // colex: k = y(y-1)/2 + x, x < y
  unsigned yy = (unsigned)((1.0f + sqrtf(1.0f + 8.0f * (float)k)) * 0.5f);
  while (yy * (yy - 1) / 2 > k) --yy;
  while ((yy + 1) * yy / 2 <= k) ++yy;
  y = yy;
  x = k - yy * (yy - 1) / 2;
}

SFCI_HD GroupDesc group_desc(const GroupCounts& gc, const unsigned c[6], unsigned g) {
  GroupDesc d;
  unsigned r = g - 1;
  for (int s = 0; s < 2; ++s) {
    if (r < gc.gss[s]) {
      const unsigned nv = gc.nv[s], op = r / (nv - 1), v = 1 + r % (nv - 1);
      d.cls = 1 + s;
      unrank_pair(op, d.x, d.y);
      d.v = v;
      d.start = c[2 + s] + op * c2(nv) + v * (v - 1) / 2;
      d.size = v;
      return d;
    }
    r -= gc.gss[s];
  }
  d.cls = 3;
  d.x = r / gc.na[1];
  d.y = r - d.x * gc.na[1];
  d.v = 0;
  d.start = c[4] + d.x * (gc.na[1] * gc.nv[1]) + d.y * gc.nv[1];
  d.size = gc.nv[1];
  return d;
}

// group of full term index l (0 for the diagonal and singles)
SFCI_HD unsigned group_of_term(const GroupCounts& gc, const unsigned c[6], unsigned l) {
  if (l < c[2]) return 0;
  if (l < c[4]) {
    const int s = l < c[3] ? 0 : 1;
    const unsigned nv = gc.nv[s], nvp = c2(nv);
    const unsigned r = l - c[2 + s], op = r / nvp, rem = r - op * nvp;
    unsigned u, v;
    unrank_pair(rem, u, v);
    return 1 + (s ? gc.gss[0] : 0) + op * (nv - 1) + (v - 1);
  }
  const unsigned r = l - c[4], nsb = gc.na[1] * gc.nv[1];
  const unsigned x = r / nsb, jj = (r - x * nsb) / gc.nv[1];
  return 1 + gc.gss[0] + gc.gss[1] + x * gc.na[1] + jj;
}

// index of the k-th set bit (k from 0) of a 64-bit word
SFCI_HD int select64(u64 w, unsigned k) {
  int base = 0;
  for (; base < 64; base += 8) {  // skip whole bytes by their counts
    const unsigned n = (unsigned)popc64((w >> base) & 0xffull);
    if (k < n) break;
    k -= n;
  }
  for (int b = base; b < base + 8 && b < 64; ++b) {
    if ((w >> b) & 1ull) {
      if (k == 0) return b;
      --k;
    }
  }
  return -1;
}

// the k-th occupied (occ = true) or empty spin orbital of spin s among N
template <class KT>
SFCI_HD int nth_orbital(const KT& key, int N, int s, bool occ, unsigned k) {
  for (int w = 0; w < (N + 63) / 64; ++w) {
    u64 word = kword(key, w);
    if (!occ) word = ~word;
    const int lo = 64 * w, hi = (lo + 64 < N) ? lo + 64 : N;
    u64 m = (hi - lo >= 64 ? ~0ull : ((1ull << (hi - lo)) - 1ull)) & (s ? 0xaaaaaaaaaaaaaaaaull : 0x5555555555555555ull);
    const u64 sel = word & m;
    const unsigned n = (unsigned)popc64(sel);
    if (k < n) return lo + select64(sel, k);
    k -= n;
  }
  return -1;
}

// spin orbitals (p, q, r) of a group
template <class KT>
SFCI_HD void group_orbitals(const KT& key, int N, const GroupCounts& gc, const GroupDesc& d, int& p, int& q,
                            int& r) {
  if (d.cls < 3) {
    const int s = d.cls - 1;
    p = nth_orbital(key, N, s, true, d.x);
    q = nth_orbital(key, N, s, true, d.y);
    r = nth_orbital(key, N, s, false, d.v);
  } else {
    const unsigned ii = d.x / gc.nv[0], aa = d.x - ii * gc.nv[0];
    p = nth_orbital(key, N, 0, true, ii);
    r = nth_orbital(key, N, 0, false, aa);
    q = nth_orbital(key, N, 1, true, d.y);
  }
}

// bound on the group's two-body elements from the row-maxima table
// vmax[blk][pair][o] = max over spatial o' of |V[blk][pair][pair(o, o')]| and
// |V[blk][pair(o, o')][pair]| (both orientations)
SFCI_HD float group_vbound(const float* vmax, int M, int P, int cls, int p, int q, int r) {
  const int ps = p >> 1, qs = q >> 1, rs = r >> 1;
  if (cls < 3) {
    const int blk = 3 * (cls - 1);
    // (p u | q r) - (p r | q u), u free
    return vmax[((size_t)blk * P + spatial_pair(qs, rs)) * M + ps] + vmax[((size_t)blk * P + spatial_pair(ps, rs)) * M + qs];
  }
  // (r p | b q) over b, block 1 or 2 by orientation
  const float a = vmax[((size_t)1 * P + spatial_pair(ps, rs)) * M + qs];
  const float b = vmax[((size_t)2 * P + spatial_pair(ps, rs)) * M + qs];
  return a > b ? a : b;
}

}  // namespace sfci

// Excitation generation over bitstring determinants (device side).
//
// Reference: OffDiagGen_bit (src/bitstr.cpp:162-302) walks, for one source
// determinant, every occupied pair and every two-body list entry stored for
// that pair, rejects entries whose creation orbitals are occupied, and emits
// each surviving entry as a separate term; one-body entries follow (:269-300);
// the caller adds the diagonal term (src/functions.cpp:636-638).
//
// Here the same matrix elements are enumerated directly: the term index space
// of a determinant is split into classes
//   [0]              diagonal
//   [1, c1)          singles, spin 0   (i -> a)
//   [c1, c2)         singles, spin 1
//   [c2, c3)         same-spin doubles, spin 0   (i<j -> a<b)
//   [c3, c4)         same-spin doubles, spin 1
//   [c4, c5)         opposite-spin doubles       (i -> a, j -> b)
// and every index decodes in O(1) to its excitation, so any thread can build
// any term without scanning lists.  Each connected determinant appears once:
// the reference's direct and exchange entries for the same target (and the
// one- and two-body pieces of a single) are summed into one element.  Phases
// follow signCal_bit exactly: for an entry (m,n,p,q) the reference moves
// q -> p first and then n -> m on the updated string (src/bitstr.cpp:212-216),
// and it keeps all-distinct entries only with n < q (src/functions.cpp:364).
#pragma once

#include "common.cuh"

namespace sfci {

struct HamView {
  int N, M, P;
  const double* __restrict__ h1;  // [2][M][M]
  const double* __restrict__ V;   // [4][P][P]
  double ecore;
};

template <class KT>
struct DetInfo {
  KT key;
  double cc;     // coeff * amp
  double dterm;  // (D - lambda) * cc
  unsigned c[6]; // class boundaries; c[5] = total terms
  unsigned na[2], nv[2];
  unsigned nvp[2];  // C(nv, 2)
  unsigned nsb;     // na[1] * nv[1]
  float inv_nv[2], inv_nvp[2], inv_nsb;
  unsigned char occ[2][64];
  unsigned char vir[2][64];
  u64 hd;        // key_hash(key)
  // single excitations of spin s, entry ii * nv[s] + aa (na * nv <= 32 * 32 for
  // 64 orbitals of a spin): the orbitals occ[s][ii] | vir[s][aa] << 8, and the
  // change of key_hash the move causes
  unsigned short ia[2][1024];
  u64 hs[2][1024];
};

// fill the single-excitation tables; thread k0 of `step` threads
template <class KT>
SFCI_HD void det_fill_singles(DetInfo<KT>& d, unsigned k0, unsigned step) {
  for (int s = 0; s < 2; ++s) {
    const unsigned nv = d.nv[s], n = d.na[s] * nv;
    for (unsigned k = k0; k < n; k += step) {
      const unsigned ii = k / nv, aa = k - ii * nv;
      d.ia[s][k] = (unsigned short)(d.occ[s][ii] | (d.vir[s][aa] << 8));
      d.hs[s][k] = hash_move(d.occ[s][ii], d.vir[s][aa]);
    }
  }
}

SFCI_HD unsigned c2(unsigned n) { return n * (n - 1) / 2; }

// number of terms (incl. diagonal) of a determinant with na[s] electrons and
// nv[s] holes per spin
SFCI_HD u64 det_terms(unsigned na0, unsigned nv0, unsigned na1, unsigned nv1) {
  return 1ull + (u64)na0 * nv0 + (u64)na1 * nv1 + (u64)c2(na0) * c2(nv0) + (u64)c2(na1) * c2(nv1) +
         (u64)na0 * nv0 * na1 * nv1;
}

#ifdef __CUDA_ARCH__
#define SFCI_LDG(p) __ldg(p)
#else
#define SFCI_LDG(p) (*(p))
#endif

SFCI_HD unsigned fdiv(unsigned r, unsigned d, float inv) {
  unsigned q = (unsigned)((float)r * inv);
  if (q * d > r) --q;
  else if ((q + 1) * d <= r) ++q;
  return q;
}

#ifdef __CUDACC__
// spin counts of a key restricted to N spin orbitals
__device__ __forceinline__ void spin_counts(const u64& k, int N, unsigned& a0, unsigned& a1) {
  const u64 ev = 0x5555555555555555ull;
  u64 m = mask_below(N);
  a0 = __popcll(k & ev & m);
  a1 = __popcll(k & ~ev & m);
}
__device__ __forceinline__ void spin_counts(const K128& k, int N, unsigned& a0, unsigned& a1) {
  const u64 ev = 0x5555555555555555ull;
  u64 m0 = mask_below(N < 64 ? N : 64), m1 = mask_below(N > 64 ? N - 64 : 0);
  a0 = __popcll(k.lo & ev & m0) + __popcll(k.hi & ev & m1);
  a1 = __popcll(k.lo & ~ev & m0) + __popcll(k.hi & ~ev & m1);
}

// Warp 0 fills the determinant's orbital lists and class boundaries.
template <class KT>
__device__ void det_setup_warp(DetInfo<KT>& d, const KT& key, double cc, double D, double lambda, int M) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    d.key = key;
    d.hd = key_hash(key);
    d.cc = cc;
    d.dterm = (D - lambda) * cc;
  }
  unsigned cnt_o[2] = {0, 0}, cnt_v[2] = {0, 0};
  for (int base = 0; base < M; base += 32) {
    int o = base + lane;
    bool in = o < M;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      int b = 2 * o + s;
      bool occ = in && key_test(key, b);
      bool vir = in && !occ;
      unsigned bo = __ballot_sync(0xffffffffu, occ), bv = __ballot_sync(0xffffffffu, vir);
      unsigned lt = (1u << lane) - 1u;
      if (occ) d.occ[s][cnt_o[s] + __popc(bo & lt)] = (unsigned char)b;
      if (vir) d.vir[s][cnt_v[s] + __popc(bv & lt)] = (unsigned char)b;
      cnt_o[s] += __popc(bo);
      cnt_v[s] += __popc(bv);
    }
  }
  if (lane == 0) {
    for (int s = 0; s < 2; ++s) {
      d.na[s] = cnt_o[s];
      d.nv[s] = cnt_v[s];
      d.nvp[s] = c2(cnt_v[s]);
      d.inv_nv[s] = cnt_v[s] ? 1.0f / (float)cnt_v[s] : 0.f;
      d.inv_nvp[s] = d.nvp[s] ? 1.0f / (float)d.nvp[s] : 0.f;
    }
    d.nsb = cnt_o[1] * cnt_v[1];
    d.inv_nsb = d.nsb ? 1.0f / (float)d.nsb : 0.f;
    d.c[0] = 1;
    d.c[1] = d.c[0] + cnt_o[0] * cnt_v[0];
    d.c[2] = d.c[1] + cnt_o[1] * cnt_v[1];
    d.c[3] = d.c[2] + c2(cnt_o[0]) * d.nvp[0];
    d.c[4] = d.c[3] + c2(cnt_o[1]) * d.nvp[1];
    d.c[5] = d.c[4] + cnt_o[0] * cnt_v[0] * d.nsb;
  }
}

#endif  // __CUDACC__

// decoded excitation
struct Exc {
  int cls;  // 0 diag, 1 single, 2 same-spin double, 3 opposite-spin double
  int s;    // spin of single / same-spin double
  int i, j, a, b;
};

// 31-bit packed form (orbitals < 128)
SFCI_HD unsigned exc_pack(const Exc& e) {
  return (unsigned)e.cls | ((unsigned)e.s << 2) | ((unsigned)e.i << 3) | ((unsigned)e.j << 10) |
         ((unsigned)e.a << 17) | ((unsigned)e.b << 24);
}
SFCI_HD Exc exc_unpack(unsigned p) {
  Exc e;
  e.cls = (int)(p & 3u);
  e.s = (int)((p >> 2) & 1u);
  e.i = (int)((p >> 3) & 127u);
  e.j = (int)((p >> 10) & 127u);
  e.a = (int)((p >> 17) & 127u);
  e.b = (int)((p >> 24) & 127u);
  return e;
}

// colex pair unranking table: k = y(y-1)/2 + x, x < y < 64
SFCI_HD void pair_of(const unsigned short* pt, unsigned k, int& x, int& y) {
  unsigned short v = pt[k];
  x = v & 0xff;
  y = v >> 8;
}

#ifdef __CUDACC__
__device__ __forceinline__ void fill_pair_table(unsigned short* pt) {
  for (int k = threadIdx.x; k < 2016; k += blockDim.x) {
    int y = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)k)) * 0.5f);
    while (y * (y - 1) / 2 > k) --y;
    while ((y + 1) * y / 2 <= k) ++y;
    int x = k - y * (y - 1) / 2;
    pt[k] = (unsigned short)(x | (y << 8));
  }
}
#endif  // __CUDACC__

template <class KT>
SFCI_HD Exc decode(const DetInfo<KT>& d, const unsigned short* pt, unsigned l) {
  Exc e;
  e.i = e.j = e.a = e.b = 0;
  e.s = 0;
  if (l == 0) {
    e.cls = 0;
    return e;
  }
  if (l < d.c[2]) {
    e.cls = 1;
    int s = l < d.c[1] ? 0 : 1;
    const unsigned short t = d.ia[s][l - d.c[s]];
    e.s = s;
    e.i = t & 0xff;
    e.a = t >> 8;
    return e;
  }
  if (l < d.c[4]) {
    e.cls = 2;
    int s = l < d.c[3] ? 0 : 1;
    unsigned r = l - d.c[2 + s];
    unsigned op = fdiv(r, d.nvp[s], d.inv_nvp[s]);
    unsigned vp = r - op * d.nvp[s];
    int x, y, u, v;
    pair_of(pt, op, x, y);
    pair_of(pt, vp, u, v);
    e.s = s;
    e.i = d.occ[s][x];
    e.j = d.occ[s][y];
    e.a = d.vir[s][u];
    e.b = d.vir[s][v];
    return e;
  }
  e.cls = 3;
  unsigned r = l - d.c[4];
  const unsigned sa = fdiv(r, d.nsb, d.inv_nsb);
  const unsigned short t0 = d.ia[0][sa], t1 = d.ia[1][r - sa * d.nsb];
  e.i = t0 & 0xff;
  e.a = t0 >> 8;
  e.j = t1 & 0xff;
  e.b = t1 >> 8;
  return e;
}

// key_hash of the target of term l, from the source's hash and the per-move
// deltas (equals key_hash(target_key(d, decode(d, pt, l))))
template <class KT>
SFCI_HD u64 term_hash(const DetInfo<KT>& d, const unsigned short* pt, unsigned l) {
  if (l == 0) return d.hd;
  if (l < d.c[2]) {
    const int s = l < d.c[1] ? 0 : 1;
    return d.hd + d.hs[s][l - d.c[s]];
  }
  if (l < d.c[4]) {
    const int s = l < d.c[3] ? 0 : 1;
    const unsigned r = l - d.c[2 + s];
    const unsigned op = fdiv(r, d.nvp[s], d.inv_nvp[s]);
    const unsigned vp = r - op * d.nvp[s];
    int x, y, u, v;
    pair_of(pt, op, x, y);
    pair_of(pt, vp, u, v);
    const unsigned nv = d.nv[s];
    return d.hd + d.hs[s][x * nv + u] + d.hs[s][y * nv + v];
  }
  const unsigned r = l - d.c[4];
  const unsigned sa = fdiv(r, d.nsb, d.inv_nsb);
  return d.hd + d.hs[0][sa] + d.hs[1][r - sa * d.nsb];
}

template <class KT>
SFCI_HD KT target_key(const DetInfo<KT>& d, const Exc& e) {
  KT k = d.key;
  if (e.cls == 0) return k;
  key_flip(k, e.i);
  key_flip(k, e.a);
  if (e.cls >= 2) {
    key_flip(k, e.j);
    key_flip(k, e.b);
  }
  return k;
}

SFCI_HD double vget(const HamView& h, int blk, int m, int n, int p, int q) {
  int pa = spatial_pair(m >> 1, n >> 1), pb = spatial_pair(p >> 1, q >> 1);
  return SFCI_LDG(h.V + ((size_t)blk * h.P + pa) * h.P + pb);
}

// Matrix element <target|H|source> times cc (diagonal: (D - lambda) * cc).
template <class KT>
SFCI_HD double term_amp(const DetInfo<KT>& d, const Exc& e, const HamView& h) {
  const KT& D = d.key;
  if (e.cls == 0) return d.dterm;
  if (e.cls == 1) {
    // one-body h(a,i) + sum_k (ai|kk) - sum_{k same spin} (ak|ki), src/bitstr.cpp:230-262,269-300
    const int s = e.s, a = e.a, i = e.i;
    double v = SFCI_LDG(h.h1 + ((size_t)s * h.M + (a >> 1)) * h.M + (i >> 1));
    const int pai = spatial_pair(a >> 1, i >> 1);
    for (int t = 0; t < 2; ++t) {
      const double* row = h.V + ((size_t)(2 * s + t) * h.P + pai) * h.P;
      for (unsigned kk = 0; kk < d.na[t]; ++kk) {
        int k = d.occ[t][kk];
        if (k == i) continue;
        int kp = k >> 1;
        v += SFCI_LDG(row + kp * (kp + 1) / 2 + kp);
        if (t == s) v -= vget(h, 3 * s, a, k, k, i);
      }
    }
    return between_parity(D, a, i) ? -d.cc * v : d.cc * v;
  }
  if (e.cls == 2) {
    // entries (a,i,b,j) and (b,i,a,j) of pair (i<j); the second has the opposite phase
    const int i = e.i, j = e.j, a = e.a, b = e.b;
    double v1 = vget(h, 3 * e.s, a, i, b, j);
    double v2 = vget(h, 3 * e.s, b, i, a, j);
    int par = between_parity2(D, b, j, a, i) ^ (int)strictly_between(j, a, i) ^ (int)strictly_between(b, a, i);
    double v = v1 - v2;
    return par ? -d.cc * v : d.cc * v;
  }
  // opposite spin: the single entry of pair (min(i,j), max(i,j))
  const int i = e.i, j = e.j, a = e.a, b = e.b;
  double v;
  int par;
  if (i < j) {
    v = vget(h, 1, a, i, b, j);
    par = between_parity2(D, b, j, a, i) ^ (int)strictly_between(j, a, i) ^ (int)strictly_between(b, a, i);
  } else {
    v = vget(h, 2, b, j, a, i);
    par = between_parity2(D, a, i, b, j) ^ (int)strictly_between(i, b, j) ^ (int)strictly_between(a, b, j);
  }
  return par ? -d.cc * v : d.cc * v;
}

#ifdef __CUDACC__
// <D|H|D>: E_core + sum_occ h(i,i) + sum_{i<j} [J_ij - delta_spin K_ij], with
// J and K symmetrised over the two stored orientations as DiagCal_bit's
// half-weighted scan of both entries does (src/bitstr.cpp:433-476).
template <class KT>
__device__ double diag_element_warp(const KT& key, const HamView& h) {
  const int lane = threadIdx.x & 31;
  int nocc = 0;
  unsigned char list[128];  // occupied spin orbitals, ascending
  for (int b = 0; b < h.N; ++b)
    if (key_test(key, b)) list[nocc++] = (unsigned char)b;
  double s = 0.0;
  int npairs = nocc * (nocc - 1) / 2;
  for (int k = lane; k < npairs; k += 32) {
    int y = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)k)) * 0.5f);
    while (y * (y - 1) / 2 > k) --y;
    while ((y + 1) * y / 2 <= k) ++y;
    int x = k - y * (y - 1) / 2;
    int i = list[x], j = list[y];
    int si = i & 1, sj = j & 1;
    double J = 0.5 * (vget(h, 2 * si + sj, i, i, j, j) + vget(h, 2 * sj + si, j, j, i, i));
    double K = (si == sj) ? vget(h, 3 * si, i, j, j, i) : 0.0;
    s += J - K;
  }
  for (int k = lane; k < nocc; k += 32) {
    int i = list[k];
    s += SFCI_LDG(h.h1 + ((size_t)(i & 1) * h.M + (i >> 1)) * h.M + (i >> 1));
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s + h.ecore;
}

#endif  // __CUDACC__

}  // namespace sfci

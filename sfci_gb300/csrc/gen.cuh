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
  // Batched contexts: one view per instance, selected by the instance id that
  // two-word keys carry in their top INST_BITS bits (nullptr: one Hamiltonian)
  const HamView* inst;
};

// Instance tag of a batched context's keys: bits 123..127 of a two-word key
// (instances need at most 120 spin orbitals, so the tag never meets an orbital
// bit).  Keys of different instances never compare equal, so one product
// merges every instance's terms separately.
constexpr int INST_BITS = 5;
constexpr int INST_SHIFT = 64 - INST_BITS;  // within the high word
constexpr int INST_MAX = 1 << INST_BITS;
constexpr int INST_MAX_ORB = 120;
SFCI_HD unsigned inst_of(const u64&) { return 0u; }
SFCI_HD unsigned inst_of(const K128& k) { return (unsigned)(k.hi >> INST_SHIFT); }
template <class KT>
SFCI_HD HamView ham_for(const HamView& h, const KT& k) {
  return h.inst ? h.inst[inst_of(k)] : h;
}

// Host check of two-word keys (lo, hi word pairs) entering a batched context,
// whose kernels index the per-instance tables by the tag: the index of the
// first key whose tag names no instance (tag >= ninst) or that sets a bit at
// or above its instance's spin-orbital count inst_N[tag]; n when all are valid.
inline u64 first_bad_batched_key(const u64* kw, u64 n, const int* inst_N, int ninst) {
  const u64 body = (1ull << INST_SHIFT) - 1ull;
  for (u64 i = 0; i < n; ++i) {
    const u64 lo = kw[2 * i], hi = kw[2 * i + 1];
    const u64 t = hi >> INST_SHIFT;
    if (t >= (u64)ninst) return i;
    const int N = inst_N[t];
    const bool over = N >= 64 ? ((hi & body) >> (N - 64)) != 0ull : ((hi & body) != 0ull || (lo >> N) != 0ull);
    if (over) return i;
  }
  return n;
}

// Single-excitation descriptor of spin orbitals i (occupied) -> a (empty):
// i | a << 7 | spatial_pair(i>>1, a>>1) << 14 | phase << 26, where the phase
// bit is the parity of the occupied orbitals strictly between i and a.
SFCI_HD unsigned sd_i(unsigned t) { return t & 127u; }
SFCI_HD unsigned sd_a(unsigned t) { return (t >> 7) & 127u; }
SFCI_HD unsigned sd_pair(unsigned t) { return (t >> 14) & 4095u; }
SFCI_HD unsigned sd_par(unsigned t) { return t >> 26; }

// per-determinant scalars (kernels copy them to registers once per determinant)
template <class KT>
struct DetHead {
  KT key;
  double cc;     // coeff * amp
  double dterm;  // (D - lambda) * cc
  unsigned c[6]; // class boundaries; c[5] = total terms
  unsigned na[2], nv[2];
  unsigned nvp[2];  // C(nv, 2)
  unsigned nsb;     // na[1] * nv[1]
  float inv_nvp[2], inv_nsb;
  unsigned acls;    // alpha class of the determinant (see alpha_class_of_orb)
};

// Alpha class: an 8-bit XOR-linear hash of a determinant's spin-0 (alpha)
// occupation, the XOR of a fixed pseudo-random byte per spin-0 orbital.  A
// move i -> a changes it by the XOR of the two orbitals' bytes, so every term
// that keeps the alpha string (the diagonal, spin-1 singles and spin-1 doubles)
// has its source's class, and an opposite-spin double has the class of its
// spin-0 move, whatever its spin-1 move.  Generation passes own ranges of
// classes, so a pass skips whole blocks of terms without building their keys.
SFCI_HD unsigned alpha_class_of_orb(int o) { return (unsigned)(mix64(0x5bd1e995ull + (u64)o) >> 56); }

template <class KT>
struct DetInfo {
  DetHead<KT> h;
  unsigned char occ[2][64];
  unsigned char vir[2][64];
  // single excitations of spin s, entry ii * nv[s] + aa (na * nv <= 32 * 32
  // for 64 orbitals of a spin): descriptor of occ[s][ii] -> vir[s][aa] and
  // the two key bits it flips
  unsigned sd[2][1024];
  KT kx[2][1024];
  unsigned char hx[1024];  // alpha-class change of each spin-0 single
};

// fill the single-excitation tables; thread k0 of `step` threads
template <class KT>
SFCI_HD void det_fill_singles(DetInfo<KT>& d, unsigned k0, unsigned step) {
  for (int s = 0; s < 2; ++s) {
    const unsigned nv = d.h.nv[s], n = d.h.na[s] * nv;
    for (unsigned k = k0; k < n; k += step) {
      const unsigned ii = k / nv, aa = k - ii * nv;
      const int i = d.occ[s][ii], a = d.vir[s][aa];
      d.sd[s][k] = (unsigned)i | ((unsigned)a << 7) | ((unsigned)spatial_pair(i >> 1, a >> 1) << 14) |
                   ((unsigned)between_parity(d.h.key, i, a) << 26);
      KT m = key_zero<KT>();
      key_flip(m, i);
      key_flip(m, a);
      d.kx[s][k] = m;
      if (s == 0) d.hx[k] = (unsigned char)(alpha_class_of_orb(i) ^ alpha_class_of_orb(a));
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
    d.h.key = key;
    d.h.cc = cc;
    d.h.dterm = (D - lambda) * cc;
  }
  unsigned cnt_o[2] = {0, 0}, cnt_v[2] = {0, 0};
  unsigned acls = 0;
  for (int base = 0; base < M; base += 32) {
    int o = base + lane;
    bool in = o < M;
    if (in && key_test(key, 2 * o)) acls ^= alpha_class_of_orb(2 * o);
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
  acls = __reduce_xor_sync(0xffffffffu, acls);
  if (lane == 0) {
    d.h.acls = acls;
    for (int s = 0; s < 2; ++s) {
      d.h.na[s] = cnt_o[s];
      d.h.nv[s] = cnt_v[s];
      d.h.nvp[s] = c2(cnt_v[s]);
      d.h.inv_nvp[s] = d.h.nvp[s] ? 1.0f / (float)d.h.nvp[s] : 0.f;
    }
    d.h.nsb = cnt_o[1] * cnt_v[1];
    d.h.inv_nsb = d.h.nsb ? 1.0f / (float)d.h.nsb : 0.f;
    d.h.c[0] = 1;
    d.h.c[1] = d.h.c[0] + cnt_o[0] * cnt_v[0];
    d.h.c[2] = d.h.c[1] + cnt_o[1] * cnt_v[1];
    d.h.c[3] = d.h.c[2] + c2(cnt_o[0]) * d.h.nvp[0];
    d.h.c[4] = d.h.c[3] + c2(cnt_o[1]) * d.h.nvp[1];
    d.h.c[5] = d.h.c[4] + cnt_o[0] * cnt_v[0] * d.h.nsb;
  }
}

#endif  // __CUDACC__

// decoded excitation, as indices into the determinant's single-excitation
// tables of spin s
struct Exc {
  int cls;  // 0 diag, 1 single, 2 same-spin double, 3 opposite-spin double
  int s;    // spin of single / same-spin double
  // cls 1: x = single; cls 2: occupied pair x < y and empty pair u < v (list
  // positions); cls 3: x = spin-0 single, y = spin-1 single
  unsigned x, y, u, v;
};

// colex pair unranking table: k = y(y-1)/2 + x, x < y < 64
SFCI_HD void pair_of(const unsigned short* pt, unsigned k, unsigned& x, unsigned& y) {
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

// (fields are selected, not indexed by spin, so that a register copy of the
// head stays in registers)
template <class KT>
SFCI_HD Exc decode(const DetHead<KT>& d, const unsigned short* pt, unsigned l) {
  Exc e;
  e.s = 0;
  e.x = e.y = e.u = e.v = 0;
  if (l == 0) {
    e.cls = 0;
    return e;
  }
  if (l < d.c[2]) {
    e.cls = 1;
    e.s = l < d.c[1] ? 0 : 1;
    e.x = l - (e.s ? d.c[1] : d.c[0]);
    return e;
  }
  if (l < d.c[4]) {
    e.cls = 2;
    const int s = l < d.c[3] ? 0 : 1;
    const unsigned r = l - (s ? d.c[3] : d.c[2]);
    const unsigned nvp = s ? d.nvp[1] : d.nvp[0];
    const unsigned op = fdiv(r, nvp, s ? d.inv_nvp[1] : d.inv_nvp[0]);
    e.s = s;
    pair_of(pt, op, e.x, e.y);
    pair_of(pt, r - op * nvp, e.u, e.v);
    return e;
  }
  e.cls = 3;
  const unsigned r = l - d.c[4];
  e.x = fdiv(r, d.nsb, d.inv_nsb);
  e.y = r - e.x * d.nsb;
  return e;
}

template <class KT>
SFCI_HD KT target_key(const DetHead<KT>& h, const DetInfo<KT>& d, const Exc& e) {
  KT k = h.key;
  if (e.cls == 1) {
    key_xor(k, d.kx[e.s][e.x]);
  } else if (e.cls == 2) {
    const unsigned nv = e.s ? h.nv[1] : h.nv[0];
    key_xor(k, d.kx[e.s][e.x * nv + e.u]);
    key_xor(k, d.kx[e.s][e.y * nv + e.v]);
  } else if (e.cls == 3) {
    key_xor(k, d.kx[0][e.x]);
    key_xor(k, d.kx[1][e.y]);
  }
  return k;
}

// Alpha class of the target of full term index l (see alpha_class_of_orb)
template <class KT>
SFCI_HD unsigned term_class(const DetHead<KT>& dh, const DetInfo<KT>& d, const unsigned short* pt, unsigned l) {
  if (l < dh.c[1]) return l == 0 ? dh.acls : dh.acls ^ d.hx[l - dh.c[0]];  // diagonal, spin-0 singles
  if (l < dh.c[2]) return dh.acls;                                          // spin-1 singles
  if (l < dh.c[3]) {                                                        // spin-0 doubles
    const unsigned r = l - dh.c[2], op = fdiv(r, dh.nvp[0], dh.inv_nvp[0]);
    unsigned x, y, u, v;
    pair_of(pt, op, x, y);
    pair_of(pt, r - op * dh.nvp[0], u, v);
    return dh.acls ^ d.hx[x * dh.nv[0] + u] ^ d.hx[y * dh.nv[0] + v];
  }
  if (l < dh.c[4]) return dh.acls;                                          // spin-1 doubles
  return dh.acls ^ d.hx[fdiv(l - dh.c[4], dh.nsb, dh.inv_nsb)];             // opposite spin
}

// V[blk][pa][pb]
SFCI_HD double vat(const HamView& h, int blk, unsigned pa, unsigned pb) {
  return SFCI_LDG(h.V + ((size_t)blk * h.P + pa) * h.P + pb);
}
SFCI_HD double vget(const HamView& h, int blk, int m, int n, int p, int q) {
  return vat(h, blk, (unsigned)spatial_pair(m >> 1, n >> 1), (unsigned)spatial_pair(p >> 1, q >> 1));
}
SFCI_HD double signed_by(unsigned par, double x) { return par ? -x : x; }

// Matrix element <target|H|source> times cc (diagonal: (D - lambda) * cc).
// Phases follow signCal_bit: for the move pair (i->a, j->b) the parity of the
// occupied orbitals strictly between each pair's ends, corrected where one
// move's ends fall between the other's (the second move acts on the string the
// first one left).
template <class KT>
SFCI_HD double term_amp(const DetHead<KT>& dh, const DetInfo<KT>& d, const Exc& e, const HamView& h) {
  if (e.cls == 0) return dh.dterm;
  if (e.cls == 1) {
    // one-body h(a,i) + sum_k (ai|kk) - sum_{k same spin} (ak|ki), src/bitstr.cpp:230-262,269-300
    const int s = e.s;
    const unsigned t = d.sd[s][e.x];
    const int i = (int)sd_i(t), a = (int)sd_a(t);
    double v = SFCI_LDG(h.h1 + ((size_t)s * h.M + (a >> 1)) * h.M + (i >> 1));
    const unsigned pai = sd_pair(t);
    for (int u = 0; u < 2; ++u) {
      const double* row = h.V + ((size_t)(2 * s + u) * h.P + pai) * h.P;
      const unsigned nau = u ? dh.na[1] : dh.na[0];
      for (unsigned kk = 0; kk < nau; ++kk) {
        int k = d.occ[u][kk];
        if (k == i) continue;
        int kp = k >> 1;
        v += SFCI_LDG(row + kp * (kp + 1) / 2 + kp);
        if (u == s) v -= vget(h, 3 * s, a, k, k, i);
      }
    }
    return signed_by(sd_par(t), dh.cc * v);
  }
  if (e.cls == 2) {
    // entries (a,i,b,j) and (b,i,a,j) of pair (i<j); the second has the opposite phase
    const unsigned nv = e.s ? dh.nv[1] : dh.nv[0];
    const unsigned* sd = d.sd[e.s];
    const unsigned t1 = sd[e.x * nv + e.u], t2 = sd[e.y * nv + e.v];  // i->a, j->b
    const unsigned t3 = sd[e.x * nv + e.v], t4 = sd[e.y * nv + e.u];  // i->b, j->a
    const int i = (int)sd_i(t1), a = (int)sd_a(t1), j = (int)sd_i(t2), b = (int)sd_a(t2);
    const double v = vat(h, 3 * e.s, sd_pair(t1), sd_pair(t2)) - vat(h, 3 * e.s, sd_pair(t3), sd_pair(t4));
    const unsigned par =
        sd_par(t1) ^ sd_par(t2) ^ (unsigned)strictly_between(j, a, i) ^ (unsigned)strictly_between(b, a, i);
    return signed_by(par, dh.cc * v);
  }
  // opposite spin: the single entry of pair (min(i,j), max(i,j))
  const unsigned t0 = d.sd[0][e.x], t1 = d.sd[1][e.y];  // i->a (spin 0), j->b (spin 1)
  const int i = (int)sd_i(t0), a = (int)sd_a(t0), j = (int)sd_i(t1), b = (int)sd_a(t1);
  const bool ij = i < j;
  const double v = ij ? vat(h, 1, sd_pair(t0), sd_pair(t1)) : vat(h, 2, sd_pair(t1), sd_pair(t0));
  const unsigned cross = ij ? ((unsigned)strictly_between(j, a, i) ^ (unsigned)strictly_between(b, a, i))
                            : ((unsigned)strictly_between(i, b, j) ^ (unsigned)strictly_between(a, b, j));
  return signed_by(sd_par(t0) ^ sd_par(t1) ^ cross, dh.cc * v);
}

// Key and element of a term that is not a single (diagonal, same-spin or
// opposite-spin double), computed on one straight-line path: the two classes
// of doubles differ only in which table rows, divisor and integral block they
// use, so a warp holding both kinds does not run two branches.  Gives the same
// key and element as target_key and term_amp.
template <class KT>
SFCI_HD double double_term(const DetHead<KT>& dh, const DetInfo<KT>& d, const unsigned short* pt, const HamView& h,
                           unsigned l, KT& key) {
  const bool opp = l >= dh.c[4];                      // opposite-spin double
  const int s = (!opp && l >= dh.c[3]) ? 1 : 0;        // spin of a same-spin double
  const unsigned r = l - (opp ? dh.c[4] : (s ? dh.c[3] : dh.c[2]));
  const unsigned dv = opp ? dh.nsb : (s ? dh.nvp[1] : dh.nvp[0]);
  const float inv = opp ? dh.inv_nsb : (s ? dh.inv_nvp[1] : dh.inv_nvp[0]);
  const unsigned q = fdiv(r, dv, inv), rem = r - q * dv;
  unsigned k1, k2, k3 = 0, k4 = 0;  // single-table entries: i->a, j->b (and i->b, j->a for same spin)
  if (opp) {
    k1 = q;
    k2 = rem;
  } else {
    unsigned x, y, u, v;
    pair_of(pt, q, x, y);
    pair_of(pt, rem, u, v);
    const unsigned nv = s ? dh.nv[1] : dh.nv[0];
    k1 = x * nv + u;
    k2 = y * nv + v;
    k3 = x * nv + v;
    k4 = y * nv + u;
  }
  const int r1 = opp ? 0 : s, r2 = opp ? 1 : s;
  const unsigned t1 = d.sd[r1][k1], t2 = d.sd[r2][k2];
  key = dh.key;
  key_xor(key, d.kx[r1][k1]);
  key_xor(key, d.kx[r2][k2]);
  const int i = (int)sd_i(t1), a = (int)sd_a(t1), j = (int)sd_i(t2), b = (int)sd_a(t2);
  // opposite spin: the entry of pair (min(i,j), max(i,j)); same spin: (a,i,b,j) - (b,i,a,j)
  const bool fwd = !opp || i < j;
  const int blk = opp ? (fwd ? 1 : 2) : 3 * s;
  double v = vat(h, blk, fwd ? sd_pair(t1) : sd_pair(t2), fwd ? sd_pair(t2) : sd_pair(t1));
  if (!opp) {
    const unsigned t3 = d.sd[s][k3], t4 = d.sd[s][k4];
    v -= vat(h, blk, sd_pair(t3), sd_pair(t4));
  }
  const unsigned cross = fwd ? ((unsigned)strictly_between(j, a, i) ^ (unsigned)strictly_between(b, a, i))
                             : ((unsigned)strictly_between(i, b, j) ^ (unsigned)strictly_between(a, b, j));
  return signed_by(sd_par(t1) ^ sd_par(t2) ^ cross, dh.cc * v);
}

#ifdef __CUDACC__
// lane `sub` of 16: its share of a single's sum over occupied orbitals
template <class KT>
__device__ double single_amp_sum(const DetHead<KT>& dh, const DetInfo<KT>& d, const Exc& e, const HamView& h,
                                 int sub) {
  const int s = e.s;
  const unsigned t = d.sd[s][e.x];
  const int i = (int)sd_i(t), a = (int)sd_a(t);
  const unsigned pai = sd_pair(t);
  double v = 0.0;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const double* row = h.V + ((size_t)(2 * s + u) * h.P + pai) * h.P;
    const unsigned nau = u ? dh.na[1] : dh.na[0];
    for (unsigned kk = sub; kk < nau; kk += 16) {
      const int k = d.occ[u][kk];
      if (k == i) continue;
      const int kp = k >> 1;
      v += SFCI_LDG(row + kp * (kp + 1) / 2 + kp);
      if (u == s) v -= vget(h, 3 * s, a, k, k, i);
    }
  }
  return v;
}

// term_amp of a single excitation evaluated by a half-warp: its 16 lanes split
// the sum over occupied orbitals (one integral load each, all in flight
// together) and combine it with a shuffle reduction within the half.  All 32
// lanes must call it (each half with its own excitation; `active` false adds
// nothing); every lane of a half returns that half's element.
template <class KT>
__device__ double single_amp_half(const DetHead<KT>& dh, const DetInfo<KT>& d, const Exc& e, const HamView& h,
                                  bool active) {
  const int sub = threadIdx.x & 15;
  double v = 0.0;
  if (active) v = single_amp_sum(dh, d, e, h, sub);
#pragma unroll
  for (int o = 8; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (!active) return 0.0;
  const unsigned t = d.sd[e.s][e.x];
  const int i = (int)sd_i(t), a = (int)sd_a(t);
  v += SFCI_LDG(h.h1 + ((size_t)e.s * h.M + (a >> 1)) * h.M + (i >> 1));
  return signed_by(sd_par(t), dh.cc * v);
}

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

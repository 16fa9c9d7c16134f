// Test-only harness: the device excitation decoder (sfci_gb300/csrc/gen.cuh)
// and the screen's term groups (sfci_gb300/csrc/screen.cuh), compiled for the
// host so that their enumeration, phases and matrix elements can be checked on a
// CPU-only machine against the reference's emitted terms.  Built by
// tests/test_gen_host.py and tests/test_screen_host.py; not part of the library.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gen.cuh"
#include "screen.cuh"
#include "internal.h"

using namespace sfci;

static HamHost g_h;

template <class KT>
static void setup_host(DetInfo<KT>& d, const KT& key, int M, double cc, double D) {
  d.h.key = key;
  d.h.cc = cc;
  d.h.dterm = D * cc;
  for (int s = 0; s < 2; ++s) {
    unsigned no = 0, nv = 0;
    for (int o = 0; o < M; ++o) {
      int b = 2 * o + s;
      if (key_test(key, b)) d.occ[s][no++] = (unsigned char)b;
      else d.vir[s][nv++] = (unsigned char)b;
    }
    d.h.na[s] = no;
    d.h.nv[s] = nv;
    d.h.nvp[s] = c2(nv);
    d.h.inv_nvp[s] = d.h.nvp[s] ? 1.0f / (float)d.h.nvp[s] : 0.f;
  }
  d.h.nsb = d.h.na[1] * d.h.nv[1];
  d.h.inv_nsb = d.h.nsb ? 1.0f / (float)d.h.nsb : 0.f;
  d.h.c[0] = 1;
  d.h.c[1] = d.h.c[0] + d.h.na[0] * d.h.nv[0];
  d.h.c[2] = d.h.c[1] + d.h.na[1] * d.h.nv[1];
  d.h.c[3] = d.h.c[2] + c2(d.h.na[0]) * d.h.nvp[0];
  d.h.c[4] = d.h.c[3] + c2(d.h.na[1]) * d.h.nvp[1];
  d.h.c[5] = d.h.c[4] + d.h.na[0] * d.h.nv[0] * d.h.nsb;
  det_fill_singles(d, 0, 1);
}

static void pair_table(unsigned short* pt) {
  for (int y = 1; y < 64; ++y)
    for (int x = 0; x < y; ++x) pt[y * (y - 1) / 2 + x] = (unsigned short)(x | (y << 8));
}

template <class KT>
static double diag_host(const KT& key, const HamView& h) {
  std::vector<int> occ;
  for (int b = 0; b < h.N; ++b)
    if (key_test(key, b)) occ.push_back(b);
  double s = 0;
  for (size_t x = 0; x < occ.size(); ++x)
    for (size_t y = x + 1; y < occ.size(); ++y) {
      int i = occ[x], j = occ[y], si = i & 1, sj = j & 1;
      double J = 0.5 * (vget(h, 2 * si + sj, i, i, j, j) + vget(h, 2 * sj + si, j, j, i, i));
      double K = si == sj ? vget(h, 3 * si, i, j, j, i) : 0.0;
      s += J - K;
    }
  for (int i : occ) s += h.h1[((size_t)(i & 1) * h.M + (i >> 1)) * h.M + (i >> 1)];
  return s + h.ecore;
}

extern "C" int gh_load(const char* path, int N) {
  std::string err;
  return load_in_file(path, N, g_h, err);
}

// All terms of one determinant with unit amplitude: returns the count, writes
// up to cap (key words, element) pairs; term 0 is the diagonal.
extern "C" long gh_terms(const uint64_t* kw, uint64_t* out_k, double* out_a, long cap) {
  HamView h{g_h.N, g_h.M, g_h.P, g_h.h1.data(), g_h.V.data(), g_h.ecore};
  static unsigned short pt[2016];
  pair_table(pt);
  long n = 0;
  if (g_h.N <= 64) {
    DetInfo<u64> d;
    u64 key = kw[0];
    setup_host(d, key, g_h.M, 1.0, diag_host(key, h));
    for (unsigned l = 0; l < d.h.c[5]; ++l, ++n) {
      Exc e = decode(d.h, pt, l);
      if (n < cap) {
        out_k[n] = target_key(d.h, d, e);
        out_a[n] = term_amp(d.h, d, e, h);
      }
    }
  } else {
    DetInfo<K128> d;
    K128 key{kw[0], kw[1]};
    setup_host(d, key, g_h.M, 1.0, diag_host(key, h));
    for (unsigned l = 0; l < d.h.c[5]; ++l, ++n) {
      Exc e = decode(d.h, pt, l);
      if (n < cap) {
        K128 t = target_key(d.h, d, e);
        out_k[2 * n] = t.lo;
        out_k[2 * n + 1] = t.hi;
        out_a[n] = term_amp(d.h, d, e, h);
      }
    }
  }
  return n;
}

// The merge's split fixed-point accumulator (common.cuh) on the host: adds the
// two addends of n terms into the two words as the device reductions do, and
// converts the sum back.
extern "C" double gh_fx_sum(const double* a, long n, int* bad) {
  u64 acc_lo = 0, acc_hi = 0;
  unsigned b = 0;
  for (long i = 0; i < n; ++i) {
    u64 xl, xh;
    fx_addends(a[i], xl, xh, b);
    acc_lo += xl;
    acc_hi += xh;
  }
  *bad = (int)b;
  return fx_acc_double(acc_lo, acc_hi);
}

// one term converted in and straight back (truncation to the 2^-64 grid)
extern "C" double gh_fx_roundtrip(double x, int* bad) { return gh_fx_sum(&x, 1, bad); }

// The narrow digit form: sums n terms as the warp tables do (four 32-bit words
// of signed base-2^21 digits) and converts back.  *big reports an out-of-range
// term.
extern "C" double gh_fx32_sum(const double* a, long n, int* big) {
  int w[4] = {0, 0, 0, 0};
  unsigned b = 0;
  for (long i = 0; i < n; ++i) {
    int dg[4];
    fx32_digits(a[i], dg, b);
    for (int k = 0; k < 4; ++k) w[k] = (int)((unsigned)w[k] + (unsigned)dg[k]);
  }
  *big = (int)b;
  u64 L, H;
  fx32_value(w, L, H);
  return fx_to_double(L, H);
}

// Doubles of one source whose branch-free key and element (double_term) differ
// in any bit from target_key / term_amp; 0 when the paths agree.
extern "C" long gh_double_term_mismatches(const uint64_t* kw, int words) {
  static unsigned short pt[2016];
  pair_table(pt);
  HamView h{g_h.N, g_h.M, g_h.P, g_h.h1.data(), g_h.V.data(), g_h.ecore};
  long bad = 0;
  auto run = [&](auto& d) {
    for (unsigned l = d.h.c[2]; l < d.h.c[5]; ++l) {
      const Exc e = decode(d.h, pt, l);
      auto k0 = target_key(d.h, d, e);
      const double a0 = term_amp(d.h, d, e, h);
      decltype(k0) k1;
      const double a1 = double_term(d.h, d, pt, h, l, k1);
      if (!key_eq(k0, k1) || dbl_bits(a0) != dbl_bits(a1)) ++bad;
    }
  };
  if (words == 1) {
    DetInfo<u64> d;
    setup_host(d, (u64)kw[0], g_h.M, 0.37, 0.0);
    run(d);
  } else {
    DetInfo<K128> d;
    setup_host(d, K128{kw[0], kw[1]}, g_h.M, 0.37, 0.0);
    run(d);
  }
  return bad;
}

// The screen's term groups of one determinant.  Writes per group g >= 1 the row
// (cls, p, q, r, start, size) into rows (6 ints a group, at most cap groups) and
// per double-excitation term l in [c[2], c[5]) its target key words and
// group_of_term(l) (at most tcap terms); returns the number of groups and sets
// *bad to the number of failed checks: the groups tile [c[2], c[5]) in index
// order, group_of_term maps each of their terms back to g, and each term's
// excitation removes p and q and adds r (the larger added orbital of a
// same-spin pair, the spin-0 one of an opposite-spin pair).
template <class KT>
static long groups_of(const KT& key, int N, int* rows, long cap, uint64_t* tk, unsigned* tg, long tcap,
                      long* nterms, long* bad) {
  static unsigned short pt[2016];
  pair_table(pt);
  DetInfo<KT> d;
  setup_host(d, key, N / 2, 1.0, 0.0);
  const GroupCounts gc = group_counts(d.h.na[0], d.h.nv[0], d.h.na[1], d.h.nv[1]);
  const u64 ng = det_groups(d.h.na[0], d.h.nv[0], d.h.na[1], d.h.nv[1]);
  const int W = (int)(sizeof(KT) / 8);
  long nb = 0;
  unsigned next = d.h.c[2];
  for (unsigned g = 1; g < ng; ++g) {
    const GroupDesc gd = group_desc(gc, d.h.c, g);
    int p, q, r;
    group_orbitals(key, N, gc, gd, p, q, r);
    if ((long)g <= cap) {
      int* o = rows + 6 * (g - 1);
      o[0] = gd.cls, o[1] = p, o[2] = q, o[3] = r, o[4] = (int)gd.start, o[5] = (int)gd.size;
    }
    if (gd.start != next || gd.size == 0) ++nb;
    next = gd.start + gd.size;
    for (unsigned l = gd.start; l < gd.start + gd.size; ++l) {
      if (group_of_term(gc, d.h.c, l) != g) ++nb;
      const KT t = target_key(d.h, d, decode(d.h, pt, l));
      int rem[4], add[4], nr = 0, na = 0;
      for (int b = 0; b < N; ++b) {
        const bool was = key_test(key, b), is = key_test(t, b);
        if (was && !is && nr < 4) rem[nr++] = b;
        if (is && !was && na < 4) add[na++] = b;
      }
      if (nr != 2 || na != 2) {
        ++nb;
        continue;
      }
      const bool pq = (rem[0] == p && rem[1] == q) || (rem[0] == q && rem[1] == p);
      const int rr = gd.cls < 3 ? add[1] : ((add[0] & 1) ? add[1] : add[0]);
      if (!pq || rr != r) ++nb;
    }
  }
  if (next != d.h.c[5]) ++nb;
  long nt = 0;
  for (unsigned l = d.h.c[2]; l < d.h.c[5]; ++l, ++nt)
    if (nt < tcap) {
      const KT t = target_key(d.h, d, decode(d.h, pt, l));
      for (int w = 0; w < W; ++w) tk[W * nt + w] = kword(t, w);
      tg[nt] = group_of_term(gc, d.h.c, l);
    }
  *nterms = nt;
  *bad = nb;
  return (long)ng - 1;
}

extern "C" long gh_groups(const uint64_t* kw, int N, int* rows, long cap, uint64_t* tk, unsigned* tg, long tcap,
                          long* nterms, long* bad) {
  if (N <= 64) return groups_of<u64>(kw[0], N, rows, cap, tk, tg, tcap, nterms, bad);
  return groups_of<K128>(K128{kw[0], kw[1]}, N, rows, cap, tk, tg, tcap, nterms, bad);
}

// unrank_pair for every k < n against the colex definition; select64 and
// nth_orbital against a scan of the bits of random words.  Returns the failures.
extern "C" long gh_screen_index_checks(unsigned n, uint64_t seed) {
  long bad = 0;
  for (unsigned k = 0; k < n; ++k) {
    unsigned x, y;
    unrank_pair(k, x, y);
    if (!(x < y) || y * (y - 1) / 2 + x != k) ++bad;
  }
  uint64_t st = seed | 1;
  auto rnd = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return st;
  };
  for (int it = 0; it < 20000; ++it) {
    const u64 w = rnd() & rnd();
    unsigned k = 0;
    for (int b = 0; b < 64; ++b)
      if ((w >> b) & 1ull) {
        if (select64(w, k) != b) ++bad;
        ++k;
      }
    if (select64(w, k) != -1) ++bad;
    const K128 key{rnd(), rnd()};
    for (int s = 0; s < 2; ++s)
      for (int occ = 0; occ < 2; ++occ) {
        unsigned kk = 0;
        for (int b = s; b < 128; b += 2)
          if (key_test(key, b) == (occ != 0)) {
            if (nth_orbital(key, 128, s, occ != 0, kk) != b) ++bad;
            ++kk;
          }
        if (nth_orbital(key, 128, s, occ != 0, kk) != -1) ++bad;
      }
  }
  return bad;
}

// The integer magnitude cut of the compactions (common.cuh: cut_key, above_cut)
// for n values against one cut: out[i] = above_cut(x[i], cut_key(cut)).
extern "C" void gh_above_cut(const double* x, long n, double cut, unsigned char* out) {
  const long long ck = cut_key(cut);
  for (long i = 0; i < n; ++i) out[i] = above_cut(x[i], ck) ? 1 : 0;
}

// The batched-key check of uploads (gen.cuh: first_bad_batched_key).
extern "C" unsigned long long gh_first_bad_batched_key(const uint64_t* kw, unsigned long long n, const int* inst_N,
                                                       int ninst) {
  return first_bad_batched_key((const u64*)kw, n, inst_N, ninst);
}

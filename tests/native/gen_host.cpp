// Test-only harness: the device excitation decoder (sfci_gb300/csrc/gen.cuh),
// compiled for the host so that its enumeration, phases and matrix elements can
// be checked on a CPU-only machine against the reference's emitted terms.
// Built by tests/test_gen_host.py; not part of the library.
#include <cstring>
#include <string>
#include <vector>

#include "gen.cuh"
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

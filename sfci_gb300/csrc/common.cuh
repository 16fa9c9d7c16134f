// Shared device/host helpers: determinant keys, bit arithmetic, hashing, status.
//
// A determinant is an occupation bitstring over N spin orbitals (src/all.h:90-91
// uses one uint64, so N <= 64).  Here a key is W 64-bit words (W = 1 for N <= 64,
// W = 2 for N <= 128).  Spin orbital b has spatial index b >> 1 and spin b & 1,
// the layout the _IN converter writes (util/convert_fcidump.py:100-108).
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#include "../../include/sfci_gb300.h"

#define SFCI_HD __host__ __device__ __forceinline__

namespace sfci {

typedef unsigned long long u64;

struct K128 {
  u64 lo, hi;
};

template <int W> struct KeyOf;
template <> struct KeyOf<1> { typedef u64 T; };
template <> struct KeyOf<2> { typedef K128 T; };

// ---- key primitives -------------------------------------------------------

SFCI_HD u64 kword(const u64& k, int) { return k; }
SFCI_HD u64 kword(const K128& k, int w) { return w ? k.hi : k.lo; }

SFCI_HD bool key_eq(const u64& a, const u64& b) { return a == b; }
SFCI_HD bool key_eq(const K128& a, const K128& b) { return a.lo == b.lo && a.hi == b.hi; }
SFCI_HD bool key_lt(const u64& a, const u64& b) { return a < b; }
SFCI_HD bool key_lt(const K128& a, const K128& b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
SFCI_HD bool key_le(const u64& a, const u64& b) { return a <= b; }
SFCI_HD bool key_le(const K128& a, const K128& b) { return !key_lt(b, a); }

// An all-ones key would need every spin orbital occupied; contexts reject
// num_e == num_orb, so it never names a determinant and marks empty slots.
template <class KT> SFCI_HD KT key_empty();
template <> SFCI_HD u64 key_empty<u64>() { return ~0ull; }
template <> SFCI_HD K128 key_empty<K128>() { K128 k; k.lo = ~0ull; k.hi = ~0ull; return k; }

template <class KT> SFCI_HD KT key_zero();
template <> SFCI_HD u64 key_zero<u64>() { return 0ull; }
template <> SFCI_HD K128 key_zero<K128>() { K128 k; k.lo = 0ull; k.hi = 0ull; return k; }
SFCI_HD void key_xor(u64& k, const u64& m) { k ^= m; }
SFCI_HD void key_xor(K128& k, const K128& m) { k.lo ^= m.lo; k.hi ^= m.hi; }

SFCI_HD void key_flip(u64& k, int b) { k ^= (1ull << b); }
SFCI_HD void key_flip(K128& k, int b) {
  if (b < 64) k.lo ^= (1ull << b); else k.hi ^= (1ull << (b - 64));
}
SFCI_HD bool key_test(const u64& k, int b) { return (k >> b) & 1ull; }
SFCI_HD bool key_test(const K128& k, int b) {
  return b < 64 ? ((k.lo >> b) & 1ull) : ((k.hi >> (b - 64)) & 1ull);
}

// radix digit of the key: bits [shift, shift+8)
SFCI_HD unsigned key_digit(const u64& k, int shift) { return (unsigned)(k >> shift) & 0xffu; }
SFCI_HD unsigned key_digit(const K128& k, int shift) {
  return shift < 64 ? (unsigned)(k.lo >> shift) & 0xffu : (unsigned)(k.hi >> (shift - 64)) & 0xffu;
}

// ---- bit helpers ----------------------------------------------------------

// bits strictly below b of a 64-bit word, b in [0, 64]
SFCI_HD u64 mask_below(int b) { return b >= 64 ? ~0ull : ((1ull << b) - 1ull); }

SFCI_HD int popc64(u64 x) {
#ifdef __CUDA_ARCH__
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}

// Parity of the occupied spin orbitals strictly between p and q (either order):
// the fermionic phase of moving one electron between p and q, as
// signCal_bit computes it (src/bitstr.cpp:133-160).
SFCI_HD int between_parity(const u64& d, int p, int q) {
  int lo = p < q ? p : q, hi = p < q ? q : p;
  u64 m = mask_below(hi) & ~mask_below(lo + 1);
  return popc64(d & m) & 1;
}
SFCI_HD void between_mask(int p, int q, u64& m0, u64& m1) {
  int lo = p < q ? p : q, hi = p < q ? q : p;
  int a = lo + 1;
  m0 = mask_below(hi < 64 ? hi : 64) & ~mask_below(a < 64 ? a : 64);
  int h1 = hi - 64, a1 = a - 64;
  m1 = mask_below(h1 > 0 ? h1 : 0) & ~mask_below(a1 > 0 ? a1 : 0);
}
SFCI_HD int between_parity(const K128& d, int p, int q) {
  u64 m0, m1;
  between_mask(p, q, m0, m1);
  return (popc64(d.lo & m0) + popc64(d.hi & m1)) & 1;
}
// parity of popc(d & (btw(p,q) ^ btw(r,s))) in one go
SFCI_HD int between_parity2(const u64& d, int p, int q, int r, int s) {
  int lo = p < q ? p : q, hi = p < q ? q : p;
  int lo2 = r < s ? r : s, hi2 = r < s ? s : r;
  u64 m = (mask_below(hi) & ~mask_below(lo + 1)) ^ (mask_below(hi2) & ~mask_below(lo2 + 1));
  return popc64(d & m) & 1;
}
SFCI_HD int between_parity2(const K128& d, int p, int q, int r, int s) {
  u64 a0, a1, b0, b1;
  between_mask(p, q, a0, a1);
  between_mask(r, s, b0, b1);
  return (popc64(d.lo & (a0 ^ b0)) + popc64(d.hi & (a1 ^ b1))) & 1;
}
SFCI_HD bool strictly_between(int x, int p, int q) {
  int lo = p < q ? p : q, hi = p < q ? q : p;
  return x > lo && x < hi;
}

// ---- hashing ---------------------------------------------------------------

SFCI_HD u64 mix64(u64 z) {
  z ^= z >> 30; z *= 0xbf58476d1ce4e5b9ull;
  z ^= z >> 27; z *= 0x94d049bb133111ebull;
  z ^= z >> 31;
  return z;
}
// Partition hash: a multiplication by an odd constant (per word), whose top
// bits spread determinants over bins, digits and leaves about as evenly as a
// full mixing hash does, for one or two multiplies.  Its low bits are weak;
// tables index by the top bits or use slot_hash.
constexpr u64 HMUL0 = 0x9e3779b97f4a7c15ull, HMUL1 = 0xc2b2ae3d27d4eb4full;
SFCI_HD u64 key_hash(const u64& k) { return k * HMUL0; }
SFCI_HD u64 key_hash(const K128& k) { return k.lo * HMUL0 + k.hi * HMUL1; }

// Mixing hash for tables indexed by their low bits.
SFCI_HD u64 slot_hash(const u64& k) { return mix64(k + 0x9e3779b97f4a7c15ull); }
SFCI_HD u64 slot_hash(const K128& k) {
  return mix64(k.lo + 0x9e3779b97f4a7c15ull) ^ mix64(k.hi ^ 0x632be59bd9b4e019ull) * 0x9e3779b97f4a7c15ull;
}

// order-preserving integer image of |x| (positive doubles compare as integers)
SFCI_HD u64 abs_bits(double x) {
#ifdef __CUDA_ARCH__
  return (u64)__double_as_longlong(x) & 0x7fffffffffffffffull;
#else
  u64 u; __builtin_memcpy(&u, &x, 8); return u & 0x7fffffffffffffffull;
#endif
}

// ---- exact amplitude accumulation -------------------------------------------
// GB300 issues FP64 arithmetic at a small fraction of its integer rate, and a
// double atomicAdd to shared memory is a compare-and-swap loop around an FP64
// add.  The merge therefore sums amplitudes as integers in units of
// 2^-FX_FRAC, with integer reductions only, so a merged amplitude does not
// depend on the order in which its terms arrive: each term is rounded once to
// the 2^-FX_FRAC grid, the sum of the rounded terms is exact, and the sum is
// rounded once back to double (round to nearest, ties to even).
//
// A term x becomes F = x * 2^FX_FRAC rounded to the nearest integer, ties to
// even (an error of at most 2^-(FX_FRAC+1) = 2.7e-20 per term, unbiased, so k
// terms of one key drift by about sqrt(k) * 1.6e-20, not k * 5.4e-20 as a
// truncation toward zero would; |x| must stay below 2^FX_MAX_EXP), split into
// two addends: lo = F mod 2^FX_SPLIT (unsigned) and hi = F >> FX_SPLIT
// (signed).  An accumulator is two 64-bit words that add the lo and hi addends
// independently, without carries between them, so each add is a plain
// fire-and-forget reduction.  Neither word can overflow while one accumulator
// receives at most FX_MAX_TERMS terms; the value is hi * 2^FX_SPLIT + lo.
constexpr int FX_FRAC = 64;
constexpr int FX_MAX_EXP = 24;
constexpr int FX_SPLIT = 44;
constexpr unsigned FX_MAX_TERMS = 1u << 19;  // (2^(FX_MAX_EXP+FX_FRAC-FX_SPLIT) and 2^FX_SPLIT headroom)

SFCI_HD u64 dbl_bits(double x) {
#ifdef __CUDA_ARCH__
  return (u64)__double_as_longlong(x);
#else
  u64 u; __builtin_memcpy(&u, &x, 8); return u;
#endif
}
SFCI_HD double bits_dbl(u64 u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x; __builtin_memcpy(&x, &u, 8); return x;
#endif
}
SFCI_HD int clz64(u64 x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// m * 2^-k rounded to the nearest integer, ties to even (m < 2^53, 1 <= k <= 53)
SFCI_HD u64 shr_round(u64 m, int k) {
  const u64 q = m >> k, r = m & ((1ull << k) - 1ull), half = 1ull << (k - 1);
  return q + ((r > half || (r == half && (q & 1ull))) ? 1ull : 0ull);
}

// the two addends of x; sets *bad for |x| >= 2^FX_MAX_EXP, infinities and NaNs
// (which then add nothing)
SFCI_HD void fx_addends(double x, u64& lo, u64& hi, unsigned& bad) {
  const u64 b = dbl_bits(x);
  const int e = (int)((b >> 52) & 0x7ff);
  const u64 m = (b & 0xfffffffffffffull) | (1ull << 52);
  const int s = e - (1075 - FX_FRAC);  // F = m * 2^s
  lo = 0;
  hi = 0;
  if (e >= 1023 + FX_MAX_EXP) {
    bad = 1u;
    return;
  }
  if (e == 0 || s < -53) return;  // zero, subnormal, or |F| < 1/2 (rounds to 0)
  u64 l, h;                       // F as a 128-bit two's-complement (h:l), |F| < 2^(FX_MAX_EXP+FX_FRAC)
  if (s < 0) {
    l = shr_round(m, -s);
    h = 0;
  } else {
    l = m << s;
    h = s ? (m >> (64 - s)) : 0ull;
  }
  if (b >> 63) {
    h = ~h + (l == 0 ? 1ull : 0ull);
    l = 0ull - l;
  }
  lo = l & ((1ull << FX_SPLIT) - 1ull);
  hi = (l >> FX_SPLIT) | (h << (64 - FX_SPLIT));  // F >> FX_SPLIT (fits 64 bits)
}

// the 128-bit sum (H:L) an accumulator holds
SFCI_HD void fx_value(u64 acc_lo, u64 acc_hi, u64& L, u64& H) {
  const u64 l0 = acc_hi << FX_SPLIT;
  L = l0 + acc_lo;
  H = (u64)((long long)acc_hi >> (64 - FX_SPLIT)) + (L < l0 ? 1ull : 0ull);
}

// Narrow form for merge tables whose slots receive at most FX32_MAX_TERMS terms:
// F (same units) as four signed base-2^21 digits, each summed in its own 32-bit
// word (11 bits of headroom) with native 32-bit reductions.  A term below 2^-44
// touches one word, a typical one three; |x| must stay below 2^FX32_MAX_EXP.
constexpr int FX32_DIG = 21;
constexpr int FX32_MAX_EXP = 18;
constexpr unsigned FX32_MAX_TERMS = 1u << 11;

// the four digits of x; sets *big for |x| >= 2^FX32_MAX_EXP or not finite
SFCI_HD void fx32_digits(double x, int dg[4], unsigned& big) {
  const u64 b = dbl_bits(x);
  const int e = (int)((b >> 52) & 0x7ff);
  dg[0] = dg[1] = dg[2] = dg[3] = 0;
  if (e >= 1023 + FX32_MAX_EXP) {
    big = 1u;
    return;
  }
  const u64 m = (b & 0xfffffffffffffull) | (1ull << 52);
  const int s = e - (1075 - FX_FRAC);  // |F| = m * 2^s < 2^(FX_FRAC + FX32_MAX_EXP), rounded as in fx_addends
  if (e == 0 || s < -53) return;
  __int128 f = s < 0 ? (__int128)shr_round(m, -s) : ((__int128)m << s);
  if (b >> 63) f = -f;
  for (int k = 0; k < 3; ++k) {
    const long long d = (long long)(((unsigned long long)f + (1ull << (FX32_DIG - 1))) & ((1ull << FX32_DIG) - 1)) -
                        (1ll << (FX32_DIG - 1));
    dg[k] = (int)d;
    f = (f - d) >> FX32_DIG;  // exact: the low FX32_DIG bits of f - d are zero
  }
  dg[3] = (int)f;  // |f| <= 2^(FX_FRAC + FX32_MAX_EXP - 3 * FX32_DIG) = 2^19: 2^11 of them fit a word
}

// the 128-bit sum (H:L) of four digit-word sums
SFCI_HD void fx32_value(const int w[4], u64& L, u64& H) {
  __int128 f = (__int128)w[3];
  for (int k = 2; k >= 0; --k) f = f * (__int128)(1ll << FX32_DIG) + (__int128)w[k];
  L = (u64)f;
  H = (u64)(f >> 64);
}

// (H:L) * 2^-FX_FRAC rounded to the nearest double, ties to even
SFCI_HD double fx_to_double(u64 lo, u64 hi) {
  const u64 neg = hi >> 63;
  if (neg) {
    hi = ~hi + (lo == 0 ? 1ull : 0ull);
    lo = 0ull - lo;
  }
  if ((hi | lo) == 0) return 0.0;
  int top = hi ? 127 - clz64(hi) : 63 - clz64(lo);  // leading bit
  u64 mant;
  if (top <= 52) {
    mant = lo << (52 - top);
  } else {
    const int sh = top - 52;  // bits dropped, 1..75
    u64 rb, st;               // round bit, sticky bits
    if (sh < 64) {
      mant = (lo >> sh) | (hi << (64 - sh));
      rb = (lo >> (sh - 1)) & 1ull;
      st = lo & ((1ull << (sh - 1)) - 1ull);
    } else {
      mant = hi >> (sh - 64);
      if (sh == 64) {
        rb = lo >> 63;
        st = lo & 0x7fffffffffffffffull;
      } else {
        rb = (hi >> (sh - 65)) & 1ull;
        st = lo | (hi & ((1ull << (sh - 65)) - 1ull));
      }
    }
    if (rb && (st || (mant & 1ull))) {
      ++mant;
      if (mant >> 53) {
        mant >>= 1;
        ++top;
      }
    }
  }
  return bits_dbl((neg << 63) | ((u64)(top - FX_FRAC + 1023) << 52) | (mant & 0xfffffffffffffull));
}

// x * 2^FX_FRAC rounded to the nearest integer (ties to even), as a 128-bit
// two's-complement (h:l); sets *bad for |x| >= 2^62 or not finite (then 0).
// The wide form for sums with more terms than the split accumulators take.
SFCI_HD void fx128_of(double x, u64& l, u64& h, unsigned& bad) {
  const u64 b = dbl_bits(x);
  const int e = (int)((b >> 52) & 0x7ff);
  const u64 m = (b & 0xfffffffffffffull) | (1ull << 52);
  const int s = e - (1075 - FX_FRAC);  // F = m * 2^s
  l = 0;
  h = 0;
  if (e >= 1023 + 62) {
    bad = 1u;
    return;
  }
  if (e == 0 || s < -53) return;
  if (s < 0) {
    l = shr_round(m, -s);
  } else if (s < 64) {
    l = m << s;
    h = s ? (m >> (64 - s)) : 0ull;
  } else {
    h = m << (s - 64);
  }
  if (b >> 63) {
    h = ~h + (l == 0 ? 1ull : 0ull);
    l = 0ull - l;
  }
}

// an accumulator's value as a double
SFCI_HD double fx_acc_double(u64 acc_lo, u64 acc_hi) {
  u64 L, H;
  fx_value(acc_lo, acc_hi, L, H);
  return fx_to_double(L, H);
}

// |x| > cut for a cut given as cut_key(cut): an integer compare of the bits
SFCI_HD long long cut_key(double cut) { return cut < 0.0 ? -1ll : (long long)abs_bits(cut); }
SFCI_HD bool above_cut(double x, long long ck) { return (long long)abs_bits(x) > ck; }

SFCI_HD int spatial_pair(int i, int j) {  // packed (i,j) ~ (j,i) index, spatial
  return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
}

}  // namespace sfci

// SpMSpV over bitstring determinants: the GB300 replacement of SpMVMtply_bucket
// (src/functions.cpp:511-804) and calc_energy (src/functions.cpp:1272-1313).
//
// Pipeline (all on one stream; sizes come from prefix sums, so nothing can
// overflow — the reference's bucket_unit / len*5000 / numConnected buffers are
// gone):
//   1. top-Nd of the input by |amp| (radix select, stable) — :535-550
//   2. per-determinant term counts -> exclusive scan -> term offsets; diagonal
//      elements D_j (DiagCal_bit, src/bitstr.cpp:433)
//   3. COUNT sweep: every CTA generates the target keys of a fixed contiguous
//      slice of the term space and histograms hash(key) into 2^b1 level-1 bins
//      (one row of a [bin x CTA] count matrix, no global atomics)
//   4. the scanned matrix gives every CTA its own write cursor per bin; bins are
//      grouped into passes that fit the device-memory budget
//   5. per pass, SCATTER sweep: regenerate, keep terms of the pass's bins, write
//      (key, c*H_kj) to the level-1 buffer through shared-memory cursors
//   6. per group of bins, level-2 partition into 2^b2 leaves per bin (count
//      matrix + cursors again), then one CTA per leaf merges duplicates in a
//      shared-memory hash table (segmented FP64 sums, :646-731), adds the
//      leaf's share of <v|H|v> (:674-677) and emits survivors |a| > cut (:750)
//   7. top-cap of the survivors (radix select) and LSD radix sort by key (:777-793)
// The oversized-leaf fallback merges in a global-memory table instead.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gen.cuh"
#include "prims.cuh"
#include "spmspv.h"

namespace sfci {

constexpr int GEN_THREADS = 512;
constexpr int GEN_IPT = 4;
constexpr int GEN_ROUND = GEN_THREADS * GEN_IPT;
constexpr int P2_THREADS = 512;
constexpr int P2_IPT = 4;
constexpr int P2_ROUND = P2_THREADS * P2_IPT;
constexpr int LEAF_THREADS = 256;
constexpr int TBL_BITS = 12;
constexpr int TBL = 1 << TBL_BITS;
constexpr int LEAF_LIMIT = (TBL * 3) / 4;
constexpr double LEAF_AVG = 1024.0;
constexpr int B2_MAX = 12;
constexpr int B1_MAX = 14;

enum { M_COUNT = 0, M_SCATTER = 1, M_ENERGY = 2 };

SFCI_HD size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// ---------------------------------------------------------------------------
// 128-bit compare-and-swap (generic address, sm_90+)
// ---------------------------------------------------------------------------
__device__ __forceinline__ K128 cas_key(K128* addr, K128 cmp, K128 val) {
  K128 out;
  asm volatile(
      "{\n\t.reg .b128 d, c, v;\n\t"
      "mov.b128 c, {%2, %3};\n\t"
      "mov.b128 v, {%4, %5};\n\t"
      "atom.cas.b128 d, [%6], c, v;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(out.lo), "=l"(out.hi)
      : "l"(cmp.lo), "l"(cmp.hi), "l"(val.lo), "l"(val.hi), "l"(addr)
      : "memory");
  return out;
}
__device__ __forceinline__ u64 cas_key(u64* addr, u64 cmp, u64 val) { return atomicCAS(addr, cmp, val); }

__device__ __forceinline__ u64 vload(const volatile u64* p) { return *p; }
__device__ __forceinline__ K128 vload(const volatile K128* p) {
  K128 k;
  k.lo = p->lo;
  k.hi = p->hi;
  return k;
}

// Insert-or-accumulate into an open-addressing table; returns false when the
// table claimed more than `limit` distinct keys (caller falls back).
// 64-bit keys are read with one plain load (single-copy atomic); a 128-bit key
// is read through the CAS itself so that a concurrent claim is never seen torn.
template <class KT>
__device__ __forceinline__ bool table_add(KT* tk, double* ta, unsigned mask, const KT& key, double amp,
                                          unsigned* nuniq, unsigned limit) {
  unsigned slot = (unsigned)key_hash(key) & mask;
  const KT empty = key_empty<KT>();
  for (unsigned probe = 0; probe <= mask; ++probe) {
    KT prev;
    if (sizeof(KT) == 8) {
      KT cur = vload((volatile KT*)&tk[slot]);
      if (key_eq(cur, key)) {
        atomicAdd(&ta[slot], amp);
        return true;
      }
      prev = key_eq(cur, empty) ? cas_key(&tk[slot], empty, key) : cur;
    } else {
      prev = cas_key(&tk[slot], empty, key);
    }
    if (key_eq(prev, empty)) {
      atomicAdd(&ta[slot], amp);
      unsigned u = atomicAdd(nuniq, 1u);
      return u < limit;
    }
    if (key_eq(prev, key)) {
      atomicAdd(&ta[slot], amp);
      return true;
    }
    slot = (slot + 1) & mask;
  }
  return false;
}

template <class KT>
__device__ __forceinline__ int table_find(const KT* tk, unsigned mask, const KT& key) {
  unsigned slot = (unsigned)key_hash(key) & mask;
  const KT empty = key_empty<KT>();
  for (unsigned probe = 0; probe <= mask; ++probe) {
    KT cur = tk[slot];
    if (key_eq(cur, key)) return (int)slot;
    if (key_eq(cur, empty)) return -1;
    slot = (slot + 1) & mask;
  }
  return -1;
}

// Global-memory variant for tables built with atomics by an earlier kernel: the
// reads go to L2 (ld.global.cg).  Letting the compiler route them through the
// non-coherent read-only path returned stale slots in practice.
__device__ __forceinline__ u64 ldcg_key(const u64* p) { return __ldcg((const unsigned long long*)p); }
__device__ __forceinline__ K128 ldcg_key(const K128* p) {
  K128 k;
  k.lo = __ldcg((const unsigned long long*)p);
  k.hi = __ldcg((const unsigned long long*)p + 1);
  return k;
}

template <class KT>
__device__ __forceinline__ int table_find_global(const KT* tk, unsigned mask, const KT& key) {
  unsigned slot = (unsigned)key_hash(key) & mask;
  const KT empty = key_empty<KT>();
  for (unsigned probe = 0; probe <= mask; ++probe) {
    KT cur = ldcg_key(tk + slot);
    if (key_eq(cur, key)) return (int)slot;
    if (key_eq(cur, empty)) return -1;
    slot = (slot + 1) & mask;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// per-determinant preparation: term counts and diagonal elements
// ---------------------------------------------------------------------------
template <class KT>
__global__ void k_det_prep(const KT* __restrict__ keys, u64 n, HamView h, u64* __restrict__ cnt,
                           double* __restrict__ diagE) {
  const int lane = threadIdx.x & 31;
  u64 w = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  u64 nw = ((u64)gridDim.x * blockDim.x) >> 5;
  for (; w < n; w += nw) {
    KT k = keys[w];
    double D = diag_element_warp(k, h);
    if (lane == 0) {
      unsigned a0, a1;
      spin_counts(k, h.N, a0, a1);
      unsigned v0 = h.M - a0, v1 = h.M - a1;
      cnt[w] = det_terms(a0, v0, a1, v1);
      diagE[w] = D;
    }
  }
}

// ---------------------------------------------------------------------------
// generation sweep
// ---------------------------------------------------------------------------
template <class KT>
struct GenArgs {
  const KT* keys;
  const double* amps;
  u64 ndet;
  const u64* doff;
  const double* diagE;
  double coeff, lambda;
  HamView h;
  u64 T;
  int b1;
  unsigned bin_lo, bin_hi;  // bins of this pass (SCATTER)
  u64* cntm;                // COUNT: [bin * G + cta]
  const u64* basem;         // SCATTER: scanned cntm
  u64 pass_base;            // SCATTER: basem[bin_lo * G]
  KT* okeys;
  double* oamps;
  const KT* tkeys;          // ENERGY: support table
  const double* tvals;
  unsigned tmask;
  double* epart;            // ENERGY: per-CTA partial
};

template <class KT, int MODE>
__global__ void __launch_bounds__(GEN_THREADS, 2) k_gen(GenArgs<KT> g) {
  extern __shared__ __align__(16) unsigned char smem[];
  DetInfo<KT>& d = *reinterpret_cast<DetInfo<KT>*>(smem);
  size_t off = al16(sizeof(DetInfo<KT>));
  unsigned short* pt = reinterpret_cast<unsigned short*>(smem + off);
  off += al16(2016 * sizeof(unsigned short));
  const unsigned nbp = (MODE == M_COUNT) ? (1u << g.b1) : (g.bin_hi - g.bin_lo);
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem + off);
  off += al16(sizeof(uint32_t) * (MODE == M_ENERGY ? 0 : nbp));
  u64* cur = reinterpret_cast<u64*>(smem + off);
  __shared__ u64 s_det;
  __shared__ double s_red[GEN_THREADS / 32];

  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned G = gridDim.x;
  fill_pair_table(pt);
  if (MODE != M_ENERGY)
    for (unsigned b = tid; b < nbp; b += GEN_THREADS) hist[b] = 0;
  if (MODE == M_SCATTER)
    for (unsigned b = tid; b < nbp; b += GEN_THREADS)
      cur[b] = g.basem[(u64)(g.bin_lo + b) * G + blockIdx.x] - g.pass_base;
  u64 t0 = (u64)((unsigned __int128)g.T * blockIdx.x / G);
  u64 t1 = (u64)((unsigned __int128)g.T * (blockIdx.x + 1) / G);
  if (tid == 0 && t0 < t1) {
    u64 lo = 0, hi = g.ndet;  // largest i with doff[i] <= t0
    while (hi - lo > 1) {
      u64 mid = (lo + hi) >> 1;
      if (g.doff[mid] <= t0) lo = mid; else hi = mid;
    }
    s_det = lo;
  }
  __syncthreads();
  double eacc = 0.0;
  const int shift1 = 64 - g.b1;
  u64 det = (t0 < t1) ? s_det : 0;
  while (t0 < t1) {
    const u64 dbeg = g.doff[det], dend = g.doff[det + 1];
    if (tid < 32) det_setup_warp(d, g.keys[det], g.coeff * g.amps[det], g.diagE[det], g.lambda, g.h.M);
    __syncthreads();
    const unsigned l0 = (unsigned)(t0 - dbeg);
    const unsigned l1 = (unsigned)((t1 < dend ? t1 : dend) - dbeg);
    for (unsigned rb = l0; rb < l1; rb += GEN_ROUND) {
      if (MODE == M_SCATTER) {
        KT kk[GEN_IPT];
        double aa[GEN_IPT];
        unsigned br[GEN_IPT];  // (rank << 16) | bin, or ~0u
#pragma unroll
        for (int it = 0; it < GEN_IPT; ++it) {
          unsigned l = rb + it * GEN_THREADS + tid;
          br[it] = ~0u;
          if (l < l1) {
            Exc e = decode(d, pt, l);
            KT key = target_key(d, e);
            unsigned bin = (unsigned)(key_hash(key) >> shift1);
            if (bin >= g.bin_lo && bin < g.bin_hi) {
              kk[it] = key;
              aa[it] = term_amp(d, e, g.h);
              unsigned lb = bin - g.bin_lo;
              unsigned r = atomicAdd(&hist[lb], 1u);
              br[it] = (r << 16) | lb;
            }
          }
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < GEN_IPT; ++it) {
          if (br[it] != ~0u) {
            unsigned lb = br[it] & 0xffffu, r = br[it] >> 16;
            u64 pos = cur[lb] + r;
            g.okeys[pos] = kk[it];
            g.oamps[pos] = aa[it];
          }
        }
        __syncthreads();
        // the holder of rank 0 advances its bin's cursor
#pragma unroll
        for (int it = 0; it < GEN_IPT; ++it) {
          if (br[it] != ~0u && (br[it] >> 16) == 0) {
            unsigned lb = br[it] & 0xffffu;
            cur[lb] += hist[lb];
            hist[lb] = 0;
          }
        }
        __syncthreads();
      } else {
#pragma unroll 2
        for (int it = 0; it < GEN_IPT; ++it) {
          unsigned l = rb + it * GEN_THREADS + tid;
          if (l < l1) {
            Exc e = decode(d, pt, l);
            KT key = target_key(d, e);
            if (MODE == M_COUNT) {
              atomicAdd(&hist[(unsigned)(key_hash(key) >> shift1)], 1u);
            } else {
              int s = table_find_global(g.tkeys, g.tmask, key);
              if (s >= 0) eacc += term_amp(d, e, g.h) * __ldcg(g.tvals + s);
            }
          }
        }
      }
    }
    t0 = t1 < dend ? t1 : dend;
    ++det;
    __syncthreads();
  }
  if (MODE == M_COUNT) {
    __syncthreads();
    for (unsigned b = tid; b < nbp; b += GEN_THREADS) g.cntm[(u64)b * G + blockIdx.x] = hist[b];
  }
  if (MODE == M_ENERGY) {
    double v = warp_sum(eacc);
    if (lane == 0) s_red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < GEN_THREADS / 32; ++w) s += s_red[w];
      g.epart[blockIdx.x] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// level-2 partition of level-1 bins into leaves
// ---------------------------------------------------------------------------
template <class KT>
struct P2Args {
  const KT* ikeys;
  const double* iamps;
  const u64* bin_off;  // nbg+1 item offsets of the group's bins in the level-1 buffer
  unsigned nbg;        // bins in group
  unsigned S;          // CTAs per bin
  int b, b2;
  u64* cntm;           // COUNT: [(lb << b2 | l2) * S + sub]
  const u64* basem;    // SCATTER: scanned cntm (positions in the level-2 buffer)
  KT* okeys;
  double* oamps;
};

template <class KT, int MODE>
__global__ void __launch_bounds__(P2_THREADS, 2) k_part2(P2Args<KT> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const unsigned nl = 1u << a.b2;
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem);
  u64* cur = reinterpret_cast<u64*>(smem + al16(sizeof(uint32_t) * nl));
  const int tid = threadIdx.x;
  const unsigned lmask = nl - 1;
  const int shift = 64 - a.b;
  for (unsigned unit = blockIdx.x; unit < a.nbg * a.S; unit += gridDim.x) {
    const unsigned lb = unit / a.S, sub = unit - lb * a.S;
    const u64 bb = a.bin_off[lb], be = a.bin_off[lb + 1], n = be - bb;
    const u64 s0 = bb + n * sub / a.S, s1 = bb + n * (sub + 1) / a.S;
    for (unsigned l = tid; l < nl; l += P2_THREADS) {
      hist[l] = 0;
      if (MODE == M_SCATTER) cur[l] = a.basem[((u64)lb * nl + l) * a.S + sub];
    }
    __syncthreads();
    for (u64 rb = s0; rb < s1; rb += P2_ROUND) {
      if (MODE == M_COUNT) {
#pragma unroll
        for (int it = 0; it < P2_IPT; ++it) {
          u64 i = rb + (u64)it * P2_THREADS + tid;
          if (i < s1) atomicAdd(&hist[(unsigned)(key_hash(a.ikeys[i]) >> shift) & lmask], 1u);
        }
      } else {
        KT kk[P2_IPT];
        double aa[P2_IPT];
        unsigned br[P2_IPT];
#pragma unroll
        for (int it = 0; it < P2_IPT; ++it) {
          u64 i = rb + (u64)it * P2_THREADS + tid;
          br[it] = ~0u;
          if (i < s1) {
            kk[it] = a.ikeys[i];
            aa[it] = a.iamps[i];
            unsigned l2 = (unsigned)(key_hash(kk[it]) >> shift) & lmask;
            unsigned r = atomicAdd(&hist[l2], 1u);
            br[it] = (r << 16) | l2;
          }
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < P2_IPT; ++it) {
          if (br[it] != ~0u) {
            u64 pos = cur[br[it] & 0xffffu] + (br[it] >> 16);
            a.okeys[pos] = kk[it];
            a.oamps[pos] = aa[it];
          }
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < P2_IPT; ++it) {
          if (br[it] != ~0u && (br[it] >> 16) == 0) {
            unsigned l2 = br[it] & 0xffffu;
            cur[l2] += hist[l2];
            hist[l2] = 0;
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (MODE == M_COUNT)
      for (unsigned l = tid; l < nl; l += P2_THREADS) a.cntm[((u64)lb * nl + l) * a.S + sub] = hist[l];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// leaf merge
// ---------------------------------------------------------------------------
template <class KT>
struct LeafArgs {
  const KT* keys;
  const double* amps;
  const u64* loff;     // leaf l spans [loff[l*lstride] - lbase, loff[(l+1)*lstride] - lbase)
  unsigned lstride;
  u64 lbase;
  u64 nleaves;
  u64 gleaf0;          // global leaf id of local leaf 0
  const KT* in_keys;   // input dets sorted by global leaf
  const double* in_amps;
  const u64* in_off;   // [2^b + 1]
  double cut;
  KT* skeys;
  double* samps;
  u64* scount;
  double* dpart;       // per-CTA <v|Hv> partials (accumulated across launches)
  unsigned* ovf;       // [0] = count, then leaf ids (global)
  unsigned ovf_cap;
  u64* uniq;           // merged distinct determinants (statistics)
};

template <class KT>
__global__ void __launch_bounds__(LEAF_THREADS) k_leaf(LeafArgs<KT> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  KT* tk = reinterpret_cast<KT*>(smem);
  double* ta = reinterpret_cast<double*>(smem + sizeof(KT) * TBL);
  __shared__ unsigned s_nuniq, s_ovf;
  __shared__ u64 s_sum[LEAF_THREADS / 32 + 1];
  __shared__ double s_red[LEAF_THREADS / 32];
  __shared__ u64 s_base;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const KT empty = key_empty<KT>();
  double dacc = 0.0;
  for (u64 leaf = blockIdx.x; leaf < a.nleaves; leaf += gridDim.x) {
    const u64 beg = a.loff[leaf * a.lstride] - a.lbase, end = a.loff[(leaf + 1) * a.lstride] - a.lbase;
    // table sized to the leaf: >= 2x its terms (so it cannot fill), 512..TBL slots
    const u64 n = end - beg;
    unsigned tb = 512;
    while (tb < TBL && (u64)tb < 2 * n) tb <<= 1;
    const unsigned limit = tb == TBL ? LEAF_LIMIT : tb;
    for (unsigned s = tid; s < tb; s += LEAF_THREADS) {
      tk[s] = empty;
      ta[s] = 0.0;
    }
    if (tid == 0) {
      s_nuniq = 0;
      s_ovf = 0;
    }
    __syncthreads();
    for (u64 e = beg + tid; e < end; e += LEAF_THREADS) {
      if (*(volatile unsigned*)&s_ovf) break;
      if (!table_add(tk, ta, tb - 1, a.keys[e], a.amps[e], &s_nuniq, limit)) s_ovf = 1;
    }
    __syncthreads();
    if (s_ovf) {
      if (tid == 0) {
        unsigned k = atomicAdd(&a.ovf[0], 1u);
        if (k < a.ovf_cap) a.ovf[1 + k] = (unsigned)(a.gleaf0 + leaf);
      }
      __syncthreads();
      continue;
    }
    // <v| (H - lambda) |v> share of this leaf
    const u64 gl = a.gleaf0 + leaf;
    for (u64 e = a.in_off[gl] + tid; e < a.in_off[gl + 1]; e += LEAF_THREADS) {
      int s = table_find(tk, tb - 1, a.in_keys[e]);
      if (s >= 0) dacc += ta[s] * a.in_amps[e];
    }
    // survivors |a| > cut: each thread owns tb/THREADS consecutive slots
    const unsigned per = tb / LEAF_THREADS;
    unsigned c = 0;
    for (unsigned q = 0; q < per; ++q) {
      unsigned s = tid * per + q;
      if (!key_eq(tk[s], empty) && fabs(ta[s]) > a.cut) ++c;
    }
    u64 tot;
    u64 ex = block_excl_scan<u64, LEAF_THREADS>((u64)c, &tot, s_sum);
    if (tid == 0) {
      s_base = tot ? atomicAdd(a.scount, tot) : 0;
      atomicAdd(a.uniq, (u64)s_nuniq);
    }
    __syncthreads();
    u64 pos = s_base + ex;
    for (unsigned q = 0; q < per; ++q) {
      unsigned s = tid * per + q;
      if (!key_eq(tk[s], empty) && fabs(ta[s]) > a.cut) {
        a.skeys[pos] = tk[s];
        a.samps[pos] = ta[s];
        ++pos;
      }
    }
    __syncthreads();
  }
  double v = warp_sum(dacc);
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < LEAF_THREADS / 32; ++w) s += s_red[w];
    atomicAdd(a.dpart + blockIdx.x, s);  // one adder per slot and launch: order stays fixed
  }
}

// oversized leaf: global-memory table
template <class KT>
__global__ void k_big_insert(const KT* __restrict__ keys, const double* __restrict__ amps, u64 beg, u64 end, KT* tk,
                             double* ta, unsigned mask, unsigned* nuniq) {
  for (u64 e = beg + (u64)blockIdx.x * blockDim.x + threadIdx.x; e < end; e += (u64)gridDim.x * blockDim.x)
    table_add(tk, ta, mask, keys[e], amps[e], nuniq, 0xffffffffu);
}

template <class KT>
__global__ void k_big_finish(const KT* tk, const double* ta, unsigned mask, const KT* in_keys, const double* in_amps,
                             u64 ib, u64 ie, double cut, KT* skeys, double* samps, u64* scount, double* dsum,
                             u64* uniq) {
  const KT empty = key_empty<KT>();
  u64 gt = (u64)blockIdx.x * blockDim.x + threadIdx.x, gs = (u64)gridDim.x * blockDim.x;
  double acc = 0.0;
  for (u64 e = ib + gt; e < ie; e += gs) {
    int s = table_find_global(tk, mask, in_keys[e]);
    if (s >= 0) acc += __ldcg(ta + s) * in_amps[e];
  }
  if (acc != 0.0) atomicAdd(dsum, acc);
  for (u64 s = gt; s <= mask; s += gs) {
    KT k = ldcg_key(tk + s);
    if (key_eq(k, empty)) continue;
    atomicAdd(uniq, 1ull);
    double v = __ldcg(ta + s);
    if (fabs(v) > cut) {
      u64 p = atomicAdd(scount, 1ull);
      skeys[p] = k;
      samps[p] = v;
    }
  }
}

template <class KT>
__global__ void k_fill_empty(KT* tk, double* ta, u64 n) {
  const KT empty = key_empty<KT>();
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    tk[i] = empty;
    if (ta) ta[i] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// input determinants grouped by global leaf (for the <v|Hv> lookups)
// ---------------------------------------------------------------------------
template <class KT>
__global__ void k_in_count(const KT* __restrict__ keys, u64 n, int b, u64* __restrict__ cnt) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
    atomicAdd(&cnt[key_hash(keys[i]) >> (64 - b)], 1ull);
}
template <class KT>
__global__ void k_in_scatter(const KT* __restrict__ keys, const double* __restrict__ amps, u64 n, int b,
                             u64* __restrict__ cur, KT* __restrict__ ok, double* __restrict__ oa) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    u64 p = atomicAdd(&cur[key_hash(keys[i]) >> (64 - b)], 1ull);
    ok[p] = keys[i];
    oa[p] = amps[i];
  }
}

// ENERGY support table
template <class KT>
__global__ void k_table_build(const KT* __restrict__ keys, const double* __restrict__ amps, u64 n, KT* tk, double* ta,
                              unsigned mask) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    unsigned slot = (unsigned)key_hash(keys[i]) & mask;
    const KT empty = key_empty<KT>();
    for (;;) {
      KT prev = cas_key(&tk[slot], empty, keys[i]);
      if (key_eq(prev, empty) || key_eq(prev, keys[i])) {
        ta[slot] = amps[i];  // duplicate keys keep one amplitude (support is a set)
        break;
      }
      slot = (slot + 1) & mask;
    }
  }
}

__global__ void k_sum_parts(const double* __restrict__ p, int n, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += __ldcg(p + i);
    *out = s;
  }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------

static HamView ham_view(Ctx& c) {
  HamView h;
  h.N = c.N;
  h.M = c.M;
  h.P = c.P;
  h.h1 = c.d_h1;
  h.V = c.d_V;
  h.ecore = c.ham.ecore;
  return h;
}

template <int W>
static size_t gen_smem(int mode, unsigned nbp) {
  typedef typename KeyOf<W>::T KT;
  size_t s = al16(sizeof(DetInfo<KT>)) + al16(2016 * sizeof(unsigned short));
  if (mode != M_ENERGY) s += al16(sizeof(uint32_t) * nbp);
  if (mode == M_SCATTER) s += al16(sizeof(u64) * nbp);
  return s;
}

template <int W, int MODE>
static int launch_gen(Ctx& c, const GenArgs<typename KeyOf<W>::T>& g, unsigned grid, unsigned nbp) {
  typedef typename KeyOf<W>::T KT;
  size_t sm = gen_smem<W>(MODE, nbp);
  static size_t configured = 0;
  if (sm > 48 * 1024 && sm > configured) {
    SFCI_CUDA(cudaFuncSetAttribute(k_gen<KT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    configured = sm;
  }
  SFCI_LAUNCH(c, (k_gen<KT, MODE>), grid, GEN_THREADS, sm, g);
  return SFCI_OK;
}

template <int W>
static int prep_dets(Ctx& c, const typename KeyOf<W>::T* keys, u64 n, u64** doff, double** diagE, u64* T) {
  u64* off = (u64*)scratch_get(c, "sp_doff", (n + 1) * sizeof(u64));
  double* dg = (double*)scratch_get(c, "sp_diag", (n ? n : 1) * sizeof(double));
  if (!off || !dg) return SFCI_ERR_NOMEM;
  unsigned grid = (unsigned)std::min<u64>((n * 32 + 255) / 256, (u64)c.sm_count * 16);
  if (grid == 0) grid = 1;
  if (n) SFCI_LAUNCH(c, k_det_prep<typename KeyOf<W>::T>, grid, 256, 0, keys, n, ham_view(c), off, dg);
  int st = scan_excl(c, off, off, n);
  if (st) return st;
  if ((st = read_words(c, off + n, sizeof(u64), T))) return st;
  *doff = off;
  *diagE = dg;
  return SFCI_OK;
}

static unsigned gen_grid(Ctx& c, u64 T) {
  u64 g = (u64)c.sm_count * 2;
  u64 need = (T + GEN_ROUND - 1) / GEN_ROUND;
  if (need < g) g = need;
  return (unsigned)(g ? g : 1);
}

template <int W>
int spmspv_impl(Ctx& c, const Vec& in, Vec& out, double lambda, double coeff, double* diag) {
  typedef typename KeyOf<W>::T KT;
  for (auto& s : c.stats) s = 0;
  if (in.len == 0) {
    out.len = 0;
    return SFCI_OK;
  }
  const double cut = c.opts.coeff_cut;
  const u64 Nd = c.opts.Nd;
  int st;
  int tok = phase_begin(c, PH_OTHER);
  // 1. top-Nd of the input by |amp|
  const KT* src_k = (const KT*)in.keys;
  const double* src_a = in.amps;
  u64 ns = in.len;
  if (in.len > Nd) {
    KT* tk = (KT*)scratch_get(c, "sp_src_k", in.len * sizeof(KT));
    double* ta = (double*)scratch_get(c, "sp_src_a", in.len * sizeof(double));
    if (!tk || !ta) return SFCI_ERR_NOMEM;
    size_t m = 0;
    if ((st = top_k_stable<W>(c, (KT*)in.keys, in.amps, in.len, Nd, -1.0, tk, ta, &m))) return st;
    src_k = tk;
    src_a = ta;
    ns = m;
  }
  c.stats[0] = ns;
  // 2. term offsets + diagonal elements
  u64 *doff = nullptr, T = 0;
  double* diagE = nullptr;
  if ((st = prep_dets<W>(c, src_k, ns, &doff, &diagE, &T))) return st;
  c.stats[1] = T;
  // hash-partition geometry
  int b = (int)std::ceil(std::log2(std::max(2.0, (double)T / LEAF_AVG)));
  if (b < 1) b = 1;
  int b2 = std::min(std::max(b - 11, 0), B2_MAX);
  int b1 = b - b2;
  if (b1 > B1_MAX) return set_error(SFCI_ERR_UNSUPPORTED, "SpMSpV term count beyond 2^26 leaves");
  const unsigned NB1 = 1u << b1;
  const unsigned G = gen_grid(c, T);
  phase_end(c, tok);

  // 3. COUNT sweep -> [bin x CTA] matrix
  tok = phase_begin(c, PH_COUNT);
  u64* cntm = (u64*)scratch_get(c, "sp_cntm", ((u64)NB1 * G + 1) * sizeof(u64));
  if (!cntm) return SFCI_ERR_NOMEM;
  GenArgs<KT> g{};
  g.keys = src_k;
  g.amps = src_a;
  g.ndet = ns;
  g.doff = doff;
  g.diagE = diagE;
  g.coeff = coeff;
  g.lambda = lambda;
  g.h = ham_view(c);
  g.T = T;
  g.b1 = b1;
  g.cntm = cntm;
  if ((st = launch_gen<W, M_COUNT>(c, g, G, NB1))) return st;
  if ((st = scan_excl(c, cntm, cntm, (u64)NB1 * G))) return st;
  std::vector<u64> binoff(NB1 + 1);
  {
    // bin start offsets: cntm[bin * G] for every bin, plus the total
    u64* bo = (u64*)scratch_get(c, "sp_binoff", (NB1 + 1) * sizeof(u64));
    if (!bo) return SFCI_ERR_NOMEM;
    SFCI_CUDA(cudaMemcpy2DAsync(bo, sizeof(u64), cntm, G * sizeof(u64), sizeof(u64), NB1, cudaMemcpyDeviceToDevice,
                                c.stream));
    SFCI_CUDA(cudaMemcpyAsync(bo + NB1, cntm + (u64)NB1 * G, sizeof(u64), cudaMemcpyDeviceToDevice, c.stream));
    if ((st = read_words(c, bo, (NB1 + 1) * sizeof(u64), binoff.data()))) return st;
  }
  phase_end(c, tok);
  if (binoff[NB1] != T) return set_error(SFCI_ERR_NUMERIC, "SpMSpV count sweep disagrees with term offsets");

  // 4. memory plan
  tok = phase_begin(c, PH_OTHER);
  const size_t tb = sizeof(KT) + sizeof(double);
  u64 maxbin = 0;
  for (unsigned i = 0; i < NB1; ++i) maxbin = std::max(maxbin, binoff[i + 1] - binoff[i]);
  size_t freeb = 0, totb = 0;
  SFCI_CUDA(cudaMemGetInfo(&freeb, &totb));
  // buffers this call may grow into: what it already holds plus what is free
  size_t held = 0;
  for (const char* nm : {"sp_l1k", "sp_l1a", "sp_l2k", "sp_l2a", "sp_sk", "sp_sa"}) {
    auto it = c.scratch.find(nm);
    if (it != c.scratch.end()) held += it->second.bytes;
  }
  size_t budget = c.opts.mem_budget ? (size_t)c.opts.mem_budget : (size_t)((freeb + held) * 0.80);
  u64 avail = budget / tb;
  const u64 cap = out.cap;
  // level-2 group capacity, survivor capacity (x2: a reduction of the survivors
  // stages through a second buffer of the same size), level-1 capacity
  u64 C2 = std::max<u64>(maxbin, std::min<u64>(T, std::max<u64>(avail / 16, 1u << 20)));
  if (b2 == 0) C2 = std::max<u64>(maxbin, std::min<u64>(T, avail / 6));
  u64 SC = std::min<u64>(cap, T) + std::min<u64>(C2, T);
  u64 C1 = T;
  u64 l2need = (b2 > 0) ? C2 : 0;
  if (C1 + l2need + 2 * SC > avail) {
    if (avail < l2need + 2 * SC + maxbin) return set_error(SFCI_ERR_NOMEM, "SpMSpV device-memory budget too small");
    C1 = avail - l2need - 2 * SC;
  }
  if (C1 < maxbin || C2 < maxbin) return set_error(SFCI_ERR_NOMEM, "SpMSpV level-1 bin exceeds its buffer");
  KT* l1k = (KT*)scratch_get(c, "sp_l1k", C1 * sizeof(KT));
  double* l1a = (double*)scratch_get(c, "sp_l1a", C1 * sizeof(double));
  KT* l2k = b2 ? (KT*)scratch_get(c, "sp_l2k", C2 * sizeof(KT)) : nullptr;
  double* l2a = b2 ? (double*)scratch_get(c, "sp_l2a", C2 * sizeof(double)) : nullptr;
  KT* sk = (KT*)scratch_get(c, "sp_sk", SC * sizeof(KT));
  double* sa = (double*)scratch_get(c, "sp_sa", SC * sizeof(double));
  if (!l1k || !l1a || !sk || !sa || (b2 && (!l2k || !l2a))) return SFCI_ERR_NOMEM;
  u64* scount = (u64*)scratch_get(c, "sp_scount", 4 * sizeof(u64));  // [0] survivors, [1] distinct
  unsigned leafgrid = (unsigned)c.sm_count * 6;
  double* dpart = (double*)scratch_get(c, "sp_dpart", (leafgrid + 1) * sizeof(double));
  const unsigned OVF_CAP = 1u << 16;
  unsigned* ovf = (unsigned*)scratch_get(c, "sp_ovf", (OVF_CAP + 1) * sizeof(unsigned));
  if (!scount || !dpart || !ovf) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemsetAsync(scount, 0, 4 * sizeof(u64), c.stream));
  SFCI_CUDA(cudaMemsetAsync(dpart, 0, (leafgrid + 1) * sizeof(double), c.stream));

  // input dets grouped by global leaf
  const u64 NL = 1ull << b;
  u64* inoff = (u64*)scratch_get(c, "sp_inoff", (NL + 1) * sizeof(u64));
  u64* incur = (u64*)scratch_get(c, "sp_incur", (NL + 1) * sizeof(u64));
  KT* ink = (KT*)scratch_get(c, "sp_ink", ns * sizeof(KT));
  double* ina = (double*)scratch_get(c, "sp_ina", ns * sizeof(double));
  if (!inoff || !incur || !ink || !ina) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemsetAsync(inoff, 0, (NL + 1) * sizeof(u64), c.stream));
  {
    unsigned gr = (unsigned)std::min<u64>((ns + 255) / 256, (u64)c.sm_count * 8);
    SFCI_LAUNCH(c, k_in_count<KT>, gr, 256, 0, src_k, ns, b, inoff);
    if ((st = scan_excl(c, inoff, inoff, NL))) return st;
    SFCI_CUDA(cudaMemcpyAsync(incur, inoff, NL * sizeof(u64), cudaMemcpyDeviceToDevice, c.stream));
    SFCI_LAUNCH(c, k_in_scatter<KT>, gr, 256, 0, src_k, src_a, ns, b, incur, ink, ina);
  }
  phase_end(c, tok);

  // pass plan over level-1 bins
  std::vector<std::pair<unsigned, unsigned>> passes;
  {
    unsigned lo = 0;
    while (lo < NB1) {
      unsigned hi = lo + 1;
      while (hi < NB1 && binoff[hi + 1] - binoff[lo] <= C1) ++hi;
      passes.push_back({lo, hi});
      lo = hi;
    }
  }
  c.stats[5] = passes.size();
  c.stats[6] = NL;
  const size_t lsm = (sizeof(KT) + sizeof(double)) * TBL;
  {
    static size_t cfg = 0;
    if (lsm > cfg) {
      SFCI_CUDA(cudaFuncSetAttribute(k_leaf<KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsm));
      cfg = lsm;
    }
  }
  u64 scount_h = 0, merged = 0, big_leaves = 0;
  double dbig_h = 0.0;
  double* dbig = (double*)scratch_get(c, "sp_dbig", sizeof(double));
  if (!dbig) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemsetAsync(dbig, 0, sizeof(double), c.stream));
  std::vector<u64> gbo;
  for (auto& ps : passes) {
    const unsigned lo = ps.first, hi = ps.second;
    // 5. SCATTER sweep for this pass
    tok = phase_begin(c, PH_SCATTER);
    g.bin_lo = lo;
    g.bin_hi = hi;
    g.basem = cntm;
    g.pass_base = binoff[lo];
    g.okeys = l1k;
    g.oamps = l1a;
    if ((st = launch_gen<W, M_SCATTER>(c, g, G, hi - lo))) return st;
    phase_end(c, tok);
    // groups of bins
    unsigned glo = lo;
    while (glo < hi) {
      unsigned ghi = glo + 1;
      while (ghi < hi && binoff[ghi + 1] - binoff[glo] <= C2) ++ghi;
      const u64 gterms = binoff[ghi] - binoff[glo];
      // survivors buffer headroom
      if (scount_h + gterms > SC && scount_h > cap) {
        int t2 = phase_begin(c, PH_SELECT);
        size_t m = 0;
        if ((st = top_k_stable<W>(c, sk, sa, scount_h, cap, -1.0, sk, sa, &m))) return st;
        scount_h = m;
        SFCI_CUDA(cudaMemcpyAsync(scount, &scount_h, sizeof(u64), cudaMemcpyHostToDevice, c.stream));
        phase_end(c, t2);
      }
      const unsigned nbg = ghi - glo;
      LeafArgs<KT> la{};
      la.in_keys = ink;
      la.in_amps = ina;
      la.in_off = inoff;
      la.cut = cut;
      la.skeys = sk;
      la.samps = sa;
      la.scount = scount;
      la.dpart = dpart;
      la.ovf = ovf;
      la.ovf_cap = OVF_CAP;
      la.uniq = scount + 1;
      const KT* lkeys;
      const double* lamps;
      if (b2 > 0) {
        // 6a. level-2 partition of the group's bins
        tok = phase_begin(c, PH_PARTITION);
        gbo.assign(nbg + 1, 0);
        for (unsigned i = 0; i <= nbg; ++i) gbo[i] = binoff[glo + i] - binoff[lo];
        u64* dgbo = (u64*)scratch_get(c, "sp_gbo", (nbg + 1) * sizeof(u64));
        if (!dgbo) return SFCI_ERR_NOMEM;
        SFCI_CUDA(cudaMemcpyAsync(dgbo, gbo.data(), (nbg + 1) * sizeof(u64), cudaMemcpyHostToDevice, c.stream));
        const unsigned nl = 1u << b2;
        unsigned S = (unsigned)std::min<u64>(16, std::max<u64>(1, ((u64)c.sm_count * 4 + nbg - 1) / nbg));
        u64 mlen = (u64)nbg * nl * S;
        u64* cm2 = (u64*)scratch_get(c, "sp_cm2", (mlen + 1) * sizeof(u64));
        if (!cm2) return SFCI_ERR_NOMEM;
        P2Args<KT> pa{};
        pa.ikeys = l1k;
        pa.iamps = l1a;
        pa.bin_off = dgbo;
        pa.nbg = nbg;
        pa.S = S;
        pa.b = b;
        pa.b2 = b2;
        pa.cntm = cm2;
        pa.basem = cm2;
        pa.okeys = l2k;
        pa.oamps = l2a;
        size_t psm = al16(sizeof(uint32_t) * nl) + al16(sizeof(u64) * nl);
        unsigned pgrid = (unsigned)std::min<u64>((u64)nbg * S, (u64)c.sm_count * 4);
        {
          static size_t cfg2 = 0;
          if (psm > 48 * 1024 && psm > cfg2) {
            SFCI_CUDA(cudaFuncSetAttribute(k_part2<KT, M_COUNT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm));
            SFCI_CUDA(cudaFuncSetAttribute(k_part2<KT, M_SCATTER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm));
            cfg2 = psm;
          }
        }
        SFCI_LAUNCH(c, (k_part2<KT, M_COUNT>), pgrid, P2_THREADS, psm, pa);
        if ((st = scan_excl(c, cm2, cm2, mlen))) return st;
        SFCI_LAUNCH(c, (k_part2<KT, M_SCATTER>), pgrid, P2_THREADS, psm, pa);
        phase_end(c, tok);
        lkeys = l2k;
        lamps = l2a;
        la.loff = cm2;
        la.lstride = S;
        la.lbase = 0;
        la.nleaves = (u64)nbg * nl;
        la.gleaf0 = (u64)glo << b2;
      } else {
        lkeys = l1k;
        lamps = l1a;
        la.loff = cntm + (u64)glo * G;
        la.lstride = G;
        la.lbase = binoff[lo];
        la.nleaves = nbg;
        la.gleaf0 = glo;
        if (ghi == NB1) {
          // loff[(nleaves) * G] must be the total: cntm has NB1*G+1 entries with the total last
        }
      }
      // 6b. leaf merge
      tok = phase_begin(c, PH_MERGE);
      la.keys = lkeys;
      la.amps = lamps;
      SFCI_CUDA(cudaMemsetAsync(ovf, 0, sizeof(unsigned), c.stream));
      unsigned lg = (unsigned)std::min<u64>(la.nleaves, leafgrid);
      SFCI_LAUNCH(c, k_leaf<KT>, lg, LEAF_THREADS, lsm, la);
      unsigned novf = 0;
      if ((st = read_words(c, ovf, sizeof(unsigned), &novf))) return st;
      if (novf > OVF_CAP) return set_error(SFCI_ERR_NOMEM, "too many oversized SpMSpV leaves");
      if (novf) {
        std::vector<unsigned> ids(novf);
        if ((st = read_words(c, ovf + 1, novf * sizeof(unsigned), ids.data()))) return st;
        big_leaves += novf;
        for (unsigned id : ids) {
          u64 lid = id - la.gleaf0;
          u64 lb2[2];
          if ((st = read_words(c, la.loff + lid * la.lstride, sizeof(u64), &lb2[0]))) return st;
          if ((st = read_words(c, la.loff + (lid + 1) * la.lstride, sizeof(u64), &lb2[1]))) return st;
          u64 beg = lb2[0] - la.lbase, end = lb2[1] - la.lbase, n = end - beg;
          u64 tsz = 1;
          while (tsz < 2 * n) tsz <<= 1;
          KT* bk = (KT*)scratch_get(c, "sp_bigk", tsz * sizeof(KT));
          double* ba = (double*)scratch_get(c, "sp_biga", tsz * sizeof(double));
          unsigned* bu = (unsigned*)scratch_get(c, "sp_bigu", sizeof(unsigned));
          if (!bk || !ba || !bu) return SFCI_ERR_NOMEM;
          unsigned gr = (unsigned)std::min<u64>((tsz + 255) / 256, (u64)c.sm_count * 8);
          SFCI_LAUNCH(c, k_fill_empty<KT>, gr, 256, 0, bk, ba, tsz);
          SFCI_CUDA(cudaMemsetAsync(bu, 0, sizeof(unsigned), c.stream));
          gr = (unsigned)std::min<u64>((n + 255) / 256, (u64)c.sm_count * 8);
          if (gr == 0) gr = 1;
          SFCI_LAUNCH(c, k_big_insert<KT>, gr, 256, 0, lkeys, lamps, beg, end, bk, ba, (unsigned)(tsz - 1), bu);
          u64 ib_ie[2];
          if ((st = read_words(c, inoff + id, 2 * sizeof(u64), ib_ie))) return st;
          gr = (unsigned)std::min<u64>((tsz + 255) / 256, (u64)c.sm_count * 8);
          SFCI_LAUNCH(c, k_big_finish<KT>, gr, 256, 0, (const KT*)bk, (const double*)ba, (unsigned)(tsz - 1),
                      (const KT*)ink, (const double*)ina, ib_ie[0], ib_ie[1], cut, sk, sa, scount, dbig,
                      scount + 1);
        }
      }
      if ((st = read_words(c, scount, sizeof(u64), &scount_h))) return st;
      phase_end(c, tok);
      merged += gterms;
      glo = ghi;
    }
  }
  c.stats[7] = big_leaves;
  // 7. <v|Hv> and final selection + key sort
  tok = phase_begin(c, PH_OTHER);
  SFCI_LAUNCH(c, k_sum_parts, 1, 32, 0, (const double*)dpart, (int)leafgrid, dpart + leafgrid);
  double dl = 0.0;
  if ((st = read_words(c, dpart + leafgrid, sizeof(double), &dl))) return st;
  if ((st = read_words(c, dbig, sizeof(double), &dbig_h))) return st;
  phase_end(c, tok);
  c.stats[3] = scount_h;
  u64 nout = scount_h;
  if (nout > cap) {
    tok = phase_begin(c, PH_SELECT);
    size_t m = 0;
    if ((st = top_k_stable<W>(c, sk, sa, nout, cap, -1.0, sk, sa, &m))) return st;
    nout = m;
    phase_end(c, tok);
  }
  tok = phase_begin(c, PH_SORT);
  if ((st = radix_sort_pairs<W>(c, sk, sa, nout, c.N))) return st;
  SFCI_CUDA(cudaMemcpyAsync(out.keys, sk, nout * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
  SFCI_CUDA(cudaMemcpyAsync(out.amps, sa, nout * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  out.len = nout;
  phase_end(c, tok);
  c.stats[4] = nout;
  {
    u64 uq = 0;
    if ((st = read_words(c, scount + 1, sizeof(u64), &uq))) return st;
    c.stats[2] = uq;
  }
  (void)merged;
  *diag = dl + dbig_h;
  return SFCI_OK;
}

template <int W>
int energy_impl(Ctx& c, const Vec& psi, double* E) {
  typedef typename KeyOf<W>::T KT;
  if (psi.len == 0) {
    *E = 0.0;
    return SFCI_OK;
  }
  int st;
  u64 *doff = nullptr, T = 0;
  double* diagE = nullptr;
  if ((st = prep_dets<W>(c, (const KT*)psi.keys, psi.len, &doff, &diagE, &T))) return st;
  for (auto& s : c.stats) s = 0;
  c.stats[0] = psi.len;
  c.stats[1] = T;
  u64 tsz = 1;
  while (tsz < 2 * psi.len) tsz <<= 1;
  if (tsz > (1ull << 31)) return set_error(SFCI_ERR_UNSUPPORTED, "energy support table too large");
  KT* tk = (KT*)scratch_get(c, "en_tk", tsz * sizeof(KT));
  double* ta = (double*)scratch_get(c, "en_ta", tsz * sizeof(double));
  const unsigned G = gen_grid(c, T);
  double* part = (double*)scratch_get(c, "en_part", (G + 1) * sizeof(double));
  if (!tk || !ta || !part) return SFCI_ERR_NOMEM;
  unsigned gr = (unsigned)std::min<u64>((tsz + 255) / 256, (u64)c.sm_count * 8);
  SFCI_LAUNCH(c, k_fill_empty<KT>, gr, 256, 0, tk, ta, tsz);
  gr = (unsigned)std::min<u64>((psi.len + 255) / 256, (u64)c.sm_count * 8);
  SFCI_LAUNCH(c, k_table_build<KT>, gr, 256, 0, (const KT*)psi.keys, psi.amps, psi.len, tk, ta, (unsigned)(tsz - 1));
  GenArgs<KT> g{};
  g.keys = (const KT*)psi.keys;
  g.amps = psi.amps;
  g.ndet = psi.len;
  g.doff = doff;
  g.diagE = diagE;
  g.coeff = 1.0;
  g.lambda = 0.0;
  g.h = ham_view(c);
  g.T = T;
  g.b1 = 1;
  g.tkeys = tk;
  g.tvals = ta;
  g.tmask = (unsigned)(tsz - 1);
  g.epart = part;
  if ((st = launch_gen<W, M_ENERGY>(c, g, G, 0))) return st;
  SFCI_LAUNCH(c, k_sum_parts, 1, 32, 0, (const double*)part, (int)G, part + G);
  return read_words(c, part + G, sizeof(double), E);
}

template <int W>
int diag_elements_impl(Ctx& c, const typename KeyOf<W>::T* dkeys, u64 n, double* out_host) {
  u64* doff = nullptr;
  double* diagE = nullptr;
  u64 T = 0;
  int st = prep_dets<W>(c, dkeys, n, &doff, &diagE, &T);
  if (st) return st;
  return read_words(c, diagE, n * sizeof(double), out_host);
}

template int spmspv_impl<1>(Ctx&, const Vec&, Vec&, double, double, double*);
template int spmspv_impl<2>(Ctx&, const Vec&, Vec&, double, double, double*);
template int energy_impl<1>(Ctx&, const Vec&, double*);
template int energy_impl<2>(Ctx&, const Vec&, double*);
template int diag_elements_impl<1>(Ctx&, const u64*, u64, double*);
template int diag_elements_impl<2>(Ctx&, const K128*, u64, double*);

}  // namespace sfci

// SpMSpV over bitstring determinants: the GB300 replacement of SpMVMtply_bucket
// (src/functions.cpp:511-804) and calc_energy (src/functions.cpp:1272-1313).
//
// Pipeline (one stream; every buffer is sized by an exclusive scan of counts, so
// nothing can overflow — the reference's bucket_unit / len*5000 / numConnected
// buffers are gone):
//   1. top-Nd of the input by |amp| (radix select, stable) — :535-550
//   2. per-determinant term counts -> exclusive scan -> term offsets; diagonal
//      elements D_j (DiagCal_bit, src/bitstr.cpp:433)
//   3. COUNT sweep: every CTA generates the target keys of a fixed contiguous
//      slice of the term space and histograms the top d0 <= 9 bits of
//      hash(key) (one row of a [bin x CTA] count matrix, no global atomics)
//   4. the scanned matrix gives every CTA a private write cursor per bin; bins
//      are grouped into passes that fit the device-memory budget
//   5. per pass, SCATTER sweep: regenerate, keep the pass's bins, stage a round
//      of terms in shared memory sorted by bin, and write coalesced runs
//   6. per group of bins, MSD radix partition on further hash digits (levels
//      of <= 9 bits, segment-aligned units, count matrix + staged coalesced
//      writes) down to 2^b leaves, b chosen so that a leaf's expected distinct
//      keys fit a warp table; then one warp per leaf merges duplicates in a
//      private shared-memory hash table with exact fixed-point sums (the FP64
//      sums of :646-731, made order-independent), adds the leaf's share of
//      <v|H|v> (:674-677) and emits survivors |a| > cut (:750)
//   7. top-cap of the survivors (radix select) and LSD radix sort by key (:777-793)
// A leaf that overflows a warp table is merged by one CTA in a 4096-slot
// shared-memory table; one that overflows that, in a global-memory table.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gen.cuh"
#include "prims.cuh"
#include "plan.h"
#include "screen.cuh"
#include "spmspv.h"
#include "table.cuh"

namespace sfci {

constexpr int GEN_THREADS = 512;
constexpr int GEN_IPT = 8;
constexpr int GEN_ROUND = GEN_THREADS * GEN_IPT;  // terms staged per round
constexpr int L1_BITS = 9;                        // level-1 bins of the generation sweep
constexpr int PT_THREADS = 512;
constexpr int DIGIT_MAX = 9;                      // bits per partition level
constexpr unsigned long long UNIT_ITEMS = 1ull << 16;  // partition work unit
constexpr int LW_WARPS = 8;                       // warps per leaf-merge CTA
constexpr int TW_MAX = 256;                       // hash slots per warp (fast tier)
constexpr int TW_UNIQ = 120;                      // distinct keys a leaf is sized for (at most)
constexpr int LW_BATCH = 4;                       // leaf items per lane loaded ahead
constexpr int LC_THREADS = 256;                   // second tier: one CTA per leaf
constexpr int LC_SLOTS = 4096;
constexpr unsigned LW_PROBE = 32;                 // probes before a warp table counts as overflowed
constexpr unsigned LC_PROBE = 128;                // same for the second tier
constexpr int B_MAX = 30;
constexpr int CP_MAX = 2016;   // pairs of 64 orbitals of a spin: C(64, 2)
constexpr int RUN_CAP = 2048;  // class passes: (occupied pair, class block) runs of spin-0 doubles per determinant
constexpr double LEAF_TERMS = 1024.0;                 // terms a leaf is sized for (at most, on average)

enum { M_COUNT = 0, M_SCATTER = 1, M_ENERGY = 2, M_PROJECT = 3, M_LABEL = 4 };
constexpr int PROJ_MAX = 64;  // vectors of one projection sweep

template <int W> struct PartIPT;
template <> struct PartIPT<1> { static constexpr int v = 8; };
template <> struct PartIPT<2> { static constexpr int v = 4; };

SFCI_HD size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

__device__ __forceinline__ u64 vload(const volatile u64* p) { return *p; }
__device__ __forceinline__ K128 vload(const volatile K128* p) {
  K128 k;
  k.lo = p->lo;
  k.hi = p->hi;
  return k;
}

// Find or claim the slot of `key` in an open-addressing table, probing at most
// `max_probe` slots from `slot`; -1 when none is free within that many (the
// table is too full for this leaf: the caller falls back to a larger tier).
// 64-bit keys are read with one plain load (single-copy atomic); a 128-bit key
// is read through the CAS itself so that a concurrent claim is never seen torn.
template <class KT>
__device__ __forceinline__ int table_slot(KT* tk, unsigned mask, const KT& key, unsigned slot, unsigned max_probe) {
  const KT empty = key_empty<KT>();
  for (unsigned probe = 0; probe < max_probe; ++probe) {
    KT prev;
    if (sizeof(KT) == 8) {
      KT cur = vload((volatile KT*)&tk[slot]);
      if (key_eq(cur, key)) return (int)slot;
      prev = key_eq(cur, empty) ? cas_key(&tk[slot], empty, key) : cur;
    } else {
      prev = cas_key(&tk[slot], empty, key);
    }
    if (key_eq(prev, empty) || key_eq(prev, key)) return (int)slot;
    slot = (slot + 1) & mask;
  }
  return -1;
}

// Start slot inside a leaf's warp table of 2^tbits slots: the top bits of a
// second multiplicative hash.  The leaf already fixed the top bits of
// key_hash, so the slot uses other multipliers; within a leaf its collisions
// match uniform hashing.
__device__ __forceinline__ unsigned leaf_slot(const u64& k, int tbits) {
  return (unsigned)((k * 0xd6e8feb86659fd93ull) >> (64 - tbits));
}
__device__ __forceinline__ unsigned leaf_slot(const K128& k, int tbits) {
  return (unsigned)(((k.lo * 0xd6e8feb86659fd93ull) ^ (k.hi * 0x94d049bb133111ebull)) >> (64 - tbits));
}

// The post-merge cut |a| > cut as an integer test on the accumulated sum: sums
// whose magnitude is at most `below` (cut * 2^FX_FRAC * (1 - 2^-40), rounded
// down) cannot survive and are dropped without converting them; the rest are
// converted and compared exactly.  A negative cut keeps everything.
struct FxCut {
  u64 below_lo, below_hi;
  long long cutk;  // cut_key(cut)
  int all;
};
// the cut on a 128-bit sum (hi:lo) in units of 2^-FX_FRAC
__device__ __forceinline__ bool fx_survives_value(u64 lo, u64 hi, const FxCut& c, double& v) {
  if (!c.all) {
    u64 mlo = lo, mhi = hi;
    if ((long long)hi < 0) {
      mhi = ~hi + (lo == 0 ? 1ull : 0ull);
      mlo = 0ull - lo;
    }
    if (mhi < c.below_hi || (mhi == c.below_hi && mlo <= c.below_lo)) return false;
  }
  v = fx_to_double(lo, hi);
  return above_cut(v, c.cutk);
}
// the cut on a split accumulator (acc_hi * 2^FX_SPLIT + acc_lo)
__device__ __forceinline__ bool fx_survives(u64 acc_lo, u64 acc_hi, const FxCut& c, double& v) {
  u64 lo, hi;
  fx_value(acc_lo, acc_hi, lo, hi);
  return fx_survives_value(lo, hi, c, v);
}
static FxCut fx_cut(double cut) {
  FxCut c{};
  c.cutk = cut_key(cut);
  c.all = cut < 0.0 ? 1 : 0;
  if (!c.all) {
    // cut * 2^FX_FRAC is exact in double; the 2^-40 margin covers the rounding
    // of the product below and of the final conversion
    const double y = std::ldexp(cut, FX_FRAC) * (1.0 - std::ldexp(1.0, -40));
    const unsigned __int128 t = y >= std::ldexp(1.0, 127) ? ~(unsigned __int128)0 >> 1 : (unsigned __int128)y;
    c.below_lo = (u64)t;
    c.below_hi = (u64)(t >> 64);
  }
  return c;
}

// add x exactly to a 128-bit fixed-point accumulator acc[0..1] (low, high):
// the carry of each low-word addition is known from its returned old value, so
// the total is the exact sum whatever the order of the additions
__device__ __forceinline__ void fx_atomic_add128(u64* acc, double x, unsigned& bad) {
  u64 l, h;
  fx128_of(x, l, h, bad);
  if ((l | h) == 0) return;
  const u64 old = atomicAdd((unsigned long long*)acc, (unsigned long long)l);
  const u64 hh = h + ((old + l < old) ? 1ull : 0ull);
  if (hh) atomicAdd((unsigned long long*)(acc + 1), (unsigned long long)hh);
}

// add a term's two addends to an accumulator (results unused: reductions)
__device__ __forceinline__ void fx_red(u64* lo_p, u64* hi_p, u64 lo, u64 hi) {
  if (lo) atomicAdd((unsigned long long*)lo_p, (unsigned long long)lo);
  if (hi) atomicAdd((unsigned long long*)hi_p, (unsigned long long)hi);
}

template <class KT>
__device__ __forceinline__ int table_find(const KT* tk, unsigned mask, const KT& key, unsigned slot) {
  const KT empty = key_empty<KT>();
  for (unsigned probe = 0; probe <= mask; ++probe) {
    KT cur = tk[slot];
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
    const HamView hk = ham_for(h, k);
    double D = diag_element_warp(k, hk);
    if (lane == 0) {
      unsigned a0, a1;
      spin_counts(k, hk.N, a0, a1);
      unsigned v0 = hk.M - a0, v1 = hk.M - a1;
      cnt[w] = det_terms(a0, v0, a1, v1);
      diagE[w] = D;
    }
  }
}

// ---------------------------------------------------------------------------
// generation sweep
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
  const KT* tkeys;          // ENERGY / PROJECT: support table
  const double* tvals;
  unsigned tmask;
  double* epart;            // ENERGY: per-CTA partial
  u64 nmain = ~0ull;        // determinants from nmain on contribute one term, amplitude amps[det]
  u64* plo;                 // PROJECT: exact merged amplitude of each table slot (wide
  u64* phi;                 //   fixed point, low and high addends)
  unsigned* pbad;           // PROJECT: a term outside the fixed-point range
  // learned screen (COUNT / SCATTER): the term index space of determinant j is
  // the screened one, group 0 ([0, c[2])) followed by the kept groups listed at
  // kl_off[j] .. kl_off[j+1] (first full index, first screened index)
  const uint32_t* kl_start = nullptr;
  const uint32_t* kl_pre = nullptr;
  const u64* kl_off = nullptr;
  unsigned kl_cap = 0;      // shared-memory entries (the longest list)
  const u64* goff = nullptr;  // LABEL: first example of each source
  uint32_t* labels = nullptr; // LABEL: one bit per (source, group >= 1)
  double label_min = 0.0;     // LABEL: a term counts when |term| > label_min
  // class pass (COUNT / SCATTER): only targets whose alpha class is in
  // [cls_lo, cls_hi).  A determinant's index space is then [0, c[3]) (diagonal,
  // singles, spin-0 doubles: filtered term by term), its spin-1 doubles when its
  // own class is in the pass, and the opposite-spin blocks (one spin-0 single
  // each) whose class is in the pass
  int cls_on = 0;
  unsigned cls_lo = 0, cls_hi = 0;
  int cls_k = 0;  // the pass is (cls_hi - cls_lo) >> cls_k aligned blocks of 2^cls_k classes
};

// class-pass tables of a determinant: run starts, K >> k of each occupied
// spin-0 pair, the empty spin-0 pairs sorted by class bucket, each pair's
// bucket, and the bucket starts
__host__ __device__ inline size_t cls_smem_bytes() {
  return al16(sizeof(uint32_t) * (RUN_CAP + 1)) + al16(CP_MAX) + al16(sizeof(unsigned short) * CP_MAX) + al16(CP_MAX) +
         2 * al16(sizeof(uint32_t) * 257);
}

template <class KT>
__host__ __device__ inline size_t gen_smem_bytes(int mode, unsigned nbp, unsigned kl_cap = 0, bool cls = false) {
  size_t s = al16(sizeof(DetInfo<KT>)) + al16(2016 * sizeof(unsigned short));
  if (mode == M_COUNT || mode == M_SCATTER) s += al16(sizeof(uint32_t) * nbp);
  if (mode == M_SCATTER)
    s += al16(sizeof(uint32_t) * nbp) + 2 * al16(sizeof(u64) * nbp) + 3 * al16(sizeof(unsigned short) * GEN_ROUND);
  s += 2 * al16(sizeof(uint32_t) * kl_cap);
  if (cls) s += cls_smem_bytes();
  return s;
}

template <class KT, int MODE>
__global__ void __launch_bounds__(GEN_THREADS, 2) k_gen(GenArgs<KT> g) {
  extern __shared__ __align__(16) unsigned char smem[];
  DetInfo<KT>& d = *reinterpret_cast<DetInfo<KT>*>(smem);
  size_t off = al16(sizeof(DetInfo<KT>));
  unsigned short* pt = reinterpret_cast<unsigned short*>(smem + off);
  off += al16(2016 * sizeof(unsigned short));
  const unsigned nbp = (MODE == M_COUNT) ? (1u << g.b1) : (g.bin_hi - g.bin_lo);
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem + off);
  off += al16(sizeof(uint32_t) * ((MODE == M_COUNT || MODE == M_SCATTER) ? nbp : 0));
  uint32_t* bst = reinterpret_cast<uint32_t*>(smem + off);
  u64* cur = nullptr;            // next output position of each bin
  u64* rbase = nullptr;          // this round: output position of staged item 0's bin run, per bin
  unsigned short* sx = nullptr;  // staged: term index within the round
  unsigned short* sb = nullptr;  // staged: local bin
  unsigned short* sq = nullptr;  // staged positions of the round's single excitations
  if (MODE == M_SCATTER) {
    off += al16(sizeof(uint32_t) * nbp);
    cur = reinterpret_cast<u64*>(smem + off);
    off += al16(sizeof(u64) * nbp);
    rbase = reinterpret_cast<u64*>(smem + off);
    off += al16(sizeof(u64) * nbp);
    sx = reinterpret_cast<unsigned short*>(smem + off);
    off += al16(sizeof(unsigned short) * GEN_ROUND);
    sb = reinterpret_cast<unsigned short*>(smem + off);
    off += al16(sizeof(unsigned short) * GEN_ROUND);
    sq = reinterpret_cast<unsigned short*>(smem + off);
    off += al16(sizeof(unsigned short) * GEN_ROUND);
  }
  uint32_t* kst = reinterpret_cast<uint32_t*>(smem + off);  // kept groups of the current determinant
  uint32_t* kpr = kst + (al16(sizeof(uint32_t) * g.kl_cap) / sizeof(uint32_t));
  off += 2 * al16(sizeof(uint32_t) * g.kl_cap);
  // class passes (see the class-pass set-up below)
  uint32_t* rpre = reinterpret_cast<uint32_t*>(smem + off);
  unsigned char* kop = smem + off + al16(sizeof(uint32_t) * (RUN_CAP + 1));
  unsigned short* cperm = reinterpret_cast<unsigned short*>(kop + al16(CP_MAX));
  unsigned char* cbq = reinterpret_cast<unsigned char*>(cperm) + al16(sizeof(unsigned short) * CP_MAX);
  uint32_t* cbcnt = reinterpret_cast<uint32_t*>(cbq + al16(CP_MAX));  // bucket sizes
  uint32_t* cboff = cbcnt + al16(sizeof(uint32_t) * 257) / sizeof(uint32_t);  // bucket starts
  __shared__ unsigned s_nk, s_n2;
  __shared__ u64 s_det;
  __shared__ unsigned s_nsq;
  __shared__ double s_red[GEN_THREADS / 32];
  __shared__ uint32_t s_scan[GEN_THREADS / 32 + 1];

  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned G = gridDim.x;
  fill_pair_table(pt);
  if (MODE == M_COUNT || MODE == M_SCATTER)
    for (unsigned b = tid; b < nbp; b += GEN_THREADS) hist[b] = 0;
  if (MODE == M_SCATTER)
    for (unsigned b = tid; b < nbp; b += GEN_THREADS)
      cur[b] = g.basem[(u64)(g.bin_lo + b) * G + blockIdx.x] - g.pass_base;
  // Each CTA owns a slice of the term index space: an even share of it, or, in
  // a class pass, whole determinants (an even share of them), so that the order
  // of a determinant's terms never decides which CTA counts and writes them.
  u64 t0, t1;
  if (g.cls_on) {
    const u64 d0 = (u64)((unsigned __int128)g.nmain * blockIdx.x / G);
    const u64 d1 = (u64)((unsigned __int128)g.nmain * (blockIdx.x + 1) / G);
    t0 = g.doff[d0];
    t1 = g.doff[d1];
    if (tid == 0) s_det = d0;
  } else {
    t0 = (u64)((unsigned __int128)g.T * blockIdx.x / G);
    t1 = (u64)((unsigned __int128)g.T * (blockIdx.x + 1) / G);
    if (tid == 0 && t0 < t1) {
      u64 lo = 0, hi = g.ndet;  // largest i with doff[i] <= t0
      while (hi - lo > 1) {
        u64 mid = (lo + hi) >> 1;
        if (g.doff[mid] <= t0) lo = mid; else hi = mid;
      }
      s_det = lo;
    }
  }
  __syncthreads();
  double eacc = 0.0;
  unsigned pbad = 0;
  const int shift1 = 64 - g.b1;
  u64 det = (t0 < t1) ? s_det : 0;
  while (t0 < t1) {
    if ((MODE == M_COUNT || MODE == M_SCATTER) && det >= g.nmain) {
      // The rest of the slice belongs to single-term extra sources (they follow
      // the input determinants): term t is source nmain + (t - doff[nmain]).
      // Whole rounds of them, with no per-source set-up, so that a slice holding
      // many of them costs what a slice of ordinary terms does.
      const u64 Tm = g.doff[g.nmain];
      for (u64 rb = t0; rb < t1; rb += GEN_ROUND) {
        if (MODE == M_SCATTER) {
          unsigned br[GEN_IPT];
#pragma unroll
          for (int it = 0; it < GEN_IPT; ++it) {
            const u64 t = rb + (u64)it * GEN_THREADS + tid;
            br[it] = ~0u;
            if (t < t1) {
              const unsigned bin = (unsigned)(key_hash(g.keys[g.nmain + (t - Tm)]) >> shift1);
              if (bin >= g.bin_lo && bin < g.bin_hi) {
                const unsigned lb = bin - g.bin_lo;
                br[it] = (atomicAdd(&hist[lb], 1u) << 16) | lb;
              }
            }
          }
          __syncthreads();
          uint32_t cnt = 0;
          if (tid < (int)nbp) {
            cnt = hist[tid];
            hist[tid] = 0;
          }
          uint32_t tot;
          const uint32_t ex = block_excl_scan<uint32_t, GEN_THREADS>(cnt, &tot, s_scan);
          if (tid < (int)nbp) {
            bst[tid] = ex;
            rbase[tid] = cur[tid] - ex;
            cur[tid] += cnt;
          }
          __syncthreads();
#pragma unroll
          for (int it = 0; it < GEN_IPT; ++it) {
            if (br[it] != ~0u) {
              const unsigned lb = br[it] & 0xffffu, p = bst[lb] + (br[it] >> 16);
              sx[p] = (unsigned short)(it * GEN_THREADS + tid);
              sb[p] = (unsigned short)lb;
            }
          }
          __syncthreads();
          // (the next round writes rbase, sx and sb only after its first barrier)
          for (unsigned i = tid; i < tot; i += GEN_THREADS) {
            const u64 src = g.nmain + (rb + sx[i] - Tm);
            const u64 pos = rbase[sb[i]] + i;
            g.okeys[pos] = g.keys[src];
            g.oamps[pos] = g.amps[src];
          }
        } else {
#pragma unroll
          for (int it = 0; it < GEN_IPT; ++it) {
            const u64 t = rb + (u64)it * GEN_THREADS + tid;
            if (t < t1) atomicAdd(&hist[(unsigned)(key_hash(g.keys[g.nmain + (t - Tm)]) >> shift1)], 1u);
          }
        }
      }
      break;
    }
    const u64 dbeg = g.doff[det], dend = g.doff[det + 1];
    const HamView hv = ham_for(g.h, g.keys[det]);  // this determinant's Hamiltonian
    if (tid < 32) det_setup_warp(d, g.keys[det], g.coeff * g.amps[det], g.diagE[det], g.lambda, hv.M);
    if (tid == 0 && det >= g.nmain) d.h.dterm = g.amps[det];  // a single term, as given
    const bool cls_pass = (MODE == M_COUNT || MODE == M_SCATTER) && g.cls_on && det < g.nmain;
    const bool screened = (MODE == M_COUNT || MODE == M_SCATTER) && (g.kl_start || g.cls_on) && det < g.nmain;
    if (screened && !cls_pass) {
      const u64 k0 = g.kl_off[det], nk = g.kl_off[det + 1] - k0;
      for (unsigned i = tid; i < nk; i += GEN_THREADS) {
        kst[i] = g.kl_start[k0 + i];
        kpr[i] = g.kl_pre[k0 + i];
      }
      if (tid == 0) s_nk = (unsigned)nk;
    }
    __syncthreads();
    if (det < g.nmain) det_fill_singles(d, tid, GEN_THREADS);  // (term 0 needs no tables)
    if (cls_pass)
      for (unsigned bk = tid; bk <= (256u >> g.cls_k); bk += GEN_THREADS) cbcnt[bk] = 0;
    __syncthreads();
    if (cls_pass) {
      // The pass owns the aligned class blocks P0 .. P0 + nblk - 1 (of 2^kb
      // classes each).  Its index space for this determinant, in order:
      //   [0, c[2])  the diagonal and the singles, filtered term by term;
      //   runs       the spin-0 doubles whose target class is in the pass: for
      //              the occupied pair op the target class is K_op ^ g(u, v)
      //              (K_op = class ^ bytes of the pair, g = bytes of the empty
      //              pair), so it lies in block P0 + j exactly when g >> kb is
      //              bucket (P0 + j) ^ (K_op >> kb); with the empty pairs sorted
      //              by bucket, run (op, j) is one contiguous stretch;
      //   the spin-1 doubles when the determinant's own class is in the pass;
      //   the opposite-spin blocks of the spin-0 singles whose class is.
      const unsigned kb = (unsigned)g.cls_k, nb = 256u >> kb, P0 = g.cls_lo >> kb;
      const unsigned nblk = (g.cls_hi - g.cls_lo) >> kb;
      const bool own = d.h.acls >= g.cls_lo && d.h.acls < g.cls_hi;
      const unsigned nv0 = d.h.nv[0], nvp0 = d.h.nvp[0], nop = c2(d.h.na[0]);
      const unsigned nx = d.h.na[0] * nv0, nsb = d.h.nsb;
      const unsigned lt = (1u << lane) - 1u, warp = tid >> 5;
      const unsigned nrun = nop * nblk;  // <= RUN_CAP (the plan bounds nblk by the occupied pairs)
      // Three barriers: (1) bucket sizes and K_op >> kb (all threads), the tail
      // block list (the last warp); (2) bucket starts (warp 0) and run starts
      // (warp 1), both warp scans; (3) the empty pairs by bucket (all threads).
      for (unsigned q = tid; q < nvp0; q += GEN_THREADS) {
        unsigned u, v;
        pair_of(pt, q, u, v);
        const unsigned bk = (unsigned)(d.hx[u] ^ d.hx[v]) >> kb;  // row 0 of hx: the occupied byte cancels
        cbq[q] = (unsigned char)bk;
        atomicAdd(&cbcnt[bk], 1u);
      }
      for (unsigned op = tid; op < nop; op += GEN_THREADS) {
        unsigned x, y;
        pair_of(pt, op, x, y);
        kop[op] = (unsigned char)((d.h.acls ^ d.hx[x * nv0] ^ d.hx[y * nv0]) >> kb);  // the empty byte cancels
      }
      if (warp == GEN_THREADS / 32 - 1) {
        // the tail's blocks, screened starts relative to the tail: the spin-1
        // doubles when the determinant's own class is in the pass, then the
        // opposite-spin blocks of the spin-0 singles whose class is
        const unsigned e0 = own ? 1u : 0u, r1 = own ? d.h.c[4] - d.h.c[3] : 0u;
        if (lane == 0 && own) {
          kst[0] = d.h.c[3];
          kpr[0] = 0;
        }
        unsigned runk = 0;
        for (unsigned xb = 0; xb < nx; xb += 32) {
          const unsigned x = xb + lane;
          const unsigned cx = x < nx ? (d.h.acls ^ d.hx[x]) : 0u;
          const bool keep = x < nx && cx >= g.cls_lo && cx < g.cls_hi && nsb > 0;
          const unsigned bal = __ballot_sync(0xffffffffu, keep);
          if (keep) {
            const unsigned r = runk + __popc(bal & lt);
            kst[e0 + r] = d.h.c[4] + x * nsb;
            kpr[e0 + r] = r1 + r * nsb;
          }
          runk += __popc(bal);
        }
        if (lane == 0) s_nk = e0 + runk;
      }
      __syncthreads();
      if (warp == 0) {
        // bucket starts
        unsigned carry = 0;
        for (unsigned b0 = 0; b0 < nb; b0 += 32) {
          const unsigned bk = b0 + lane;
          const unsigned v = bk < nb ? cbcnt[bk] : 0u;
          unsigned x = v;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
          }
          if (bk < nb) cboff[bk] = carry + x - v;
          carry += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) cboff[nb] = carry;
      } else if (warp == 1) {
        // run starts, op-major: run (op, j) holds the empty pairs of bucket (P0 + j) ^ kop[op]
        unsigned carry = 0;
        for (unsigned r0 = 0; r0 < nrun; r0 += 32) {
          const unsigned r = r0 + lane;
          unsigned v = 0;
          if (r < nrun) {
            const unsigned op = r / nblk, j = r - op * nblk;
            v = cbcnt[(P0 + j) ^ kop[op]];
          }
          unsigned x = v;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
          }
          if (r < nrun) rpre[r] = carry + x - v;
          carry += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) {
          rpre[nrun] = carry;
          s_n2 = carry;
        }
      }
      __syncthreads();
      // the empty pairs by bucket, in any order within a bucket: a CTA owns
      // whole determinants in a class pass, so the order decides nothing that
      // the count sweep and the generation pass could disagree on (the bucket
      // sizes count down to zero, ready for the next determinant)
      for (unsigned q = tid; q < nvp0; q += GEN_THREADS) {
        const unsigned bk = cbq[q];
        cperm[cboff[bk] + atomicSub(&cbcnt[bk], 1u) - 1u] = (unsigned short)q;
      }
      __syncthreads();
    }
    const DetHead<KT> dh = d.h;
    const unsigned nk = screened ? s_nk : 0u;
    const unsigned n2 = cls_pass ? s_n2 : 0u;
    const unsigned c_nblk = cls_pass ? (g.cls_hi - g.cls_lo) >> g.cls_k : 1u, c_P0 = g.cls_lo >> g.cls_k;
    const unsigned c_nrun = cls_pass ? c2(dh.na[0]) * c_nblk : 0u;
    // screened term index -> full term index: group 0 (the diagonal and the
    // singles) maps to itself; in a class pass the spin-0 double runs come
    // next; then a binary search over the kept blocks' screened starts
    auto remap = [&](unsigned l) -> unsigned {
      if (!screened || l < dh.c[2]) return l;
      if (cls_pass) {
        const unsigned r = l - dh.c[2];
        if (r < n2) {
          unsigned lo = 0, hi = c_nrun;  // the last run starting at or before r
          while (hi - lo > 1) {
            const unsigned mid = (lo + hi) >> 1;
            if (rpre[mid] <= r) lo = mid; else hi = mid;
          }
          const unsigned op = lo / c_nblk, bk = (c_P0 + (lo - op * c_nblk)) ^ kop[op];
          return dh.c[2] + op * dh.nvp[0] + cperm[cboff[bk] + (r - rpre[lo])];
        }
        l = r - n2;  // the tail's blocks have screened starts relative to the tail
      }
      unsigned lo = 0, hi = nk;
      while (hi - lo > 1) {
        const unsigned mid = (lo + hi) >> 1;
        if (kpr[mid] <= l) lo = mid; else hi = mid;
      }
      return kst[lo] + (l - kpr[lo]);
    };
    // class pass: is the target of (full) term index lf in the pass?  Only the
    // diagonal and the singles are filtered; everything after was chosen whole
    auto in_pass = [&](unsigned lf) -> bool {
      if (!cls_pass || lf >= dh.c[2]) return true;
      const unsigned cl = term_class(dh, d, pt, lf);
      return cl >= g.cls_lo && cl < g.cls_hi;
    };
    const unsigned l0 = (unsigned)(t0 - dbeg);
    const unsigned l1 = (unsigned)((t1 < dend ? t1 : dend) - dbeg);
    for (unsigned rb = l0; rb < l1; rb += GEN_ROUND) {
      if (MODE == M_SCATTER) {
        // (1) bin every term of the round by its hash alone and rank the ones
        // in this pass; (2) stage their round indices sorted by bin; (3) decode,
        // build the keys and amplitudes of the staged terms only, with full
        // warps, and write each bin's run contiguously
        unsigned br[GEN_IPT];  // (rank << 16) | local bin, or ~0u
#pragma unroll
        for (int it = 0; it < GEN_IPT; ++it) {
          unsigned l = rb + it * GEN_THREADS + tid;
          br[it] = ~0u;
          const unsigned lf = l < l1 ? remap(l) : 0u;
          if (l < l1 && in_pass(lf)) {
            const unsigned bin = (unsigned)(key_hash(target_key(dh, d, decode(dh, pt, lf))) >> shift1);
            if (bin >= g.bin_lo && bin < g.bin_hi) {
              unsigned lb = bin - g.bin_lo;
              unsigned r = atomicAdd(&hist[lb], 1u);
              br[it] = (r << 16) | lb;
            }
          }
        }
        __syncthreads();
        // the owner of each bin takes its count (clearing it for the next
        // round), scans, and advances the bin's output position
        uint32_t cnt = 0;
        if (tid < (int)nbp) {
          cnt = hist[tid];
          hist[tid] = 0;
        }
        if (tid == 0) s_nsq = 0;
        uint32_t tot;
        uint32_t ex = block_excl_scan<uint32_t, GEN_THREADS>(cnt, &tot, s_scan);
        if (tid < (int)nbp) {
          bst[tid] = ex;
          rbase[tid] = cur[tid] - ex;
          cur[tid] += cnt;
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < GEN_IPT; ++it) {
          if (br[it] != ~0u) {
            unsigned lb = br[it] & 0xffffu, p = bst[lb] + (br[it] >> 16);
            sx[p] = (unsigned short)(it * GEN_THREADS + tid);
            sb[p] = (unsigned short)lb;
          }
        }
        __syncthreads();
        // the next round touches rbase, sx and sb only after its own first
        // barrier, which every thread reaches after finishing this loop
        // Singles (term indices 1 .. c[2]-1, so only in a determinant's first
        // rounds) are deferred to a half-warp each: their element sums over all
        // occupied orbitals, a chain of loads that would stall a whole warp.
        // Doubles (most terms) take one branch-free path whatever their kind.
        const bool with_singles = rb < dh.c[2];
        for (unsigned i = tid; i < tot; i += GEN_THREADS) {
          const unsigned l = rb + sx[i];
          if (with_singles && l != 0 && l < dh.c[2]) {
            sq[atomicAdd(&s_nsq, 1u)] = (unsigned short)i;
            continue;
          }
          const u64 pos = rbase[sb[i]] + i;
          KT key;
          double amp;
          if (l == 0) {
            key = dh.key;
            amp = dh.dterm;
          } else {
            amp = double_term(dh, d, pt, hv, remap(l), key);
          }
          g.okeys[pos] = key;
          g.oamps[pos] = amp;
        }
        if (with_singles) {
          __syncthreads();
          const unsigned nsq = s_nsq;
          for (unsigned q0 = (tid >> 5) * 2; q0 < nsq; q0 += GEN_THREADS / 16) {
            const unsigned q = q0 + ((tid >> 4) & 1u);
            const bool act = q < nsq;
            const unsigned i = act ? sq[q] : 0u;
            const Exc e = decode(dh, pt, rb + sx[i]);
            const double v = single_amp_half(dh, d, e, hv, act && e.cls == 1);
            if (act && (tid & 15) == 0) {
              const u64 pos = rbase[sb[i]] + i;
              g.okeys[pos] = target_key(dh, d, e);
              g.oamps[pos] = v;
            }
          }
        }
      } else {
#pragma unroll 2
        for (int it = 0; it < GEN_IPT; ++it) {
          unsigned l = rb + it * GEN_THREADS + tid;
          if (l < l1) {
            if (MODE == M_COUNT) {
              const unsigned lf = remap(l);
              if (in_pass(lf))
                atomicAdd(&hist[(unsigned)(key_hash(target_key(dh, d, decode(dh, pt, lf))) >> shift1)], 1u);
            } else if (MODE == M_LABEL) {
              // a group is alive when one of its terms lands on the product's output
              const Exc e = decode(dh, pt, l);
              if (table_find_global(g.tkeys, g.tmask, target_key(dh, d, e)) >= 0 &&
                  (g.label_min <= 0.0 || fabs(term_amp(dh, d, e, hv)) > g.label_min)) {
                const GroupCounts gc = group_counts(dh.na[0], dh.nv[0], dh.na[1], dh.nv[1]);
                const unsigned gi = group_of_term(gc, dh.c, l);
                if (gi) {
                  const u64 ex = g.goff[det] + gi - 1;
                  atomicOr(g.labels + (ex >> 5), 1u << (ex & 31));
                }
              }
            } else if (MODE == M_ENERGY) {
              const Exc e = decode(dh, pt, l);
              const KT key = target_key(dh, d, e);
              int s = table_find_global(g.tkeys, g.tmask, key);
              if (s >= 0) eacc += term_amp(dh, d, e, hv) * __ldcg(g.tvals + s);
            }
          }
          if (MODE == M_PROJECT && l < l1) {
            // a term landing on the projected vectors' support joins that key's
            // exact merged amplitude
            const Exc e = decode(dh, pt, l);
            const int s = table_find_global(g.tkeys, g.tmask, target_key(dh, d, e));
            if (s >= 0) {
              u64 xl, xh;
              fx_addends(term_amp(dh, d, e, hv), xl, xh, pbad);
              fx_red(g.plo + s, g.phi + s, xl, xh);
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
  if (MODE == M_PROJECT && pbad) atomicOr(g.pbad, 1u);
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
// MSD radix partition of segments on a further hash digit
// ---------------------------------------------------------------------------
// A unit is a contiguous piece (<= UNIT_ITEMS) of one segment.  Its count for
// digit dg lives at cbase + dg * stride of the level's count matrix, laid out
// so that one exclusive scan orders positions by (segment, digit, unit).
struct Unit {
  u64 start, end, cbase;
  unsigned stride, pad;
};

template <class KT>
struct PartArgs {
  const KT* ikeys;
  const double* iamps;
  const Unit* units;
  unsigned nunits;
  int shift;      // digit = (hash >> shift) & (nd - 1)
  unsigned nd;
  u64* cm;        // COUNT: counts out; SCATTER: scanned counts in
  u64 dst_base;   // added to scanned positions
  KT* okeys;
  double* oamps;
};

template <class KT, int IPT>
__host__ __device__ inline size_t part_smem_bytes(int mode, unsigned nd) {
  size_t s = al16(sizeof(uint32_t) * nd);
  if (mode == M_SCATTER) {
    const int R = PT_THREADS * IPT;
    s += al16(sizeof(uint32_t) * nd) + al16(sizeof(u64) * nd) + al16(sizeof(KT) * R) + al16(sizeof(double) * R) +
         al16(sizeof(unsigned short) * R);
  }
  return s;
}

template <class KT, int MODE, int IPT>
__global__ void __launch_bounds__(PT_THREADS, 2) k_part(PartArgs<KT> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int R = PT_THREADS * IPT;
  const unsigned nd = a.nd;
  size_t off = 0;
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem + off);
  off += al16(sizeof(uint32_t) * nd);
  uint32_t* bst = reinterpret_cast<uint32_t*>(smem + off);
  u64* cur = nullptr;
  KT* sk = nullptr;
  double* sa = nullptr;
  unsigned short* sb = nullptr;
  if (MODE == M_SCATTER) {
    off += al16(sizeof(uint32_t) * nd);
    cur = reinterpret_cast<u64*>(smem + off);
    off += al16(sizeof(u64) * nd);
    sk = reinterpret_cast<KT*>(smem + off);
    off += al16(sizeof(KT) * R);
    sa = reinterpret_cast<double*>(smem + off);
    off += al16(sizeof(double) * R);
    sb = reinterpret_cast<unsigned short*>(smem + off);
  }
  __shared__ uint32_t s_scan[PT_THREADS / 32 + 1];
  const int tid = threadIdx.x;
  const unsigned dmask = nd - 1;
  for (unsigned u = blockIdx.x; u < a.nunits; u += gridDim.x) {
    const Unit un = a.units[u];
    for (unsigned dg = tid; dg < nd; dg += PT_THREADS) {
      hist[dg] = 0;
      if (MODE == M_SCATTER) cur[dg] = __ldcg(a.cm + un.cbase + (u64)dg * un.stride) + a.dst_base;
    }
    __syncthreads();
    for (u64 rb = un.start; rb < un.end; rb += R) {
      if (MODE == M_COUNT) {
        KT kk[IPT];
#pragma unroll
        for (int it = 0; it < IPT; ++it) {  // all loads first, then the atomics
          u64 i = rb + (u64)it * PT_THREADS + tid;
          if (i < un.end) kk[it] = a.ikeys[i];
        }
#pragma unroll
        for (int it = 0; it < IPT; ++it) {
          u64 i = rb + (u64)it * PT_THREADS + tid;
          if (i < un.end) atomicAdd(&hist[(unsigned)(key_hash(kk[it]) >> a.shift) & dmask], 1u);
        }
      } else {
        KT kk[IPT];
        double aa[IPT];
        unsigned br[IPT];
#pragma unroll
        for (int it = 0; it < IPT; ++it) {
          u64 i = rb + (u64)it * PT_THREADS + tid;
          if (i < un.end) {
            kk[it] = a.ikeys[i];
            aa[it] = a.iamps[i];
          }
        }
#pragma unroll
        for (int it = 0; it < IPT; ++it) {
          u64 i = rb + (u64)it * PT_THREADS + tid;
          br[it] = ~0u;
          if (i < un.end) {
            unsigned dg = (unsigned)(key_hash(kk[it]) >> a.shift) & dmask;
            unsigned r = atomicAdd(&hist[dg], 1u);
            br[it] = (r << 16) | dg;
          }
        }
        __syncthreads();
        // exclusive scan of the digit histogram (nd <= 512 = PT_THREADS)
        uint32_t tot;
        uint32_t ex = block_excl_scan<uint32_t, PT_THREADS>(tid < (int)nd ? hist[tid] : 0u, &tot, s_scan);
        if (tid < (int)nd) bst[tid] = ex;
        __syncthreads();
#pragma unroll
        for (int it = 0; it < IPT; ++it) {
          if (br[it] != ~0u) {
            unsigned dg = br[it] & 0xffffu, p = bst[dg] + (br[it] >> 16);
            sk[p] = kk[it];
            sa[p] = aa[it];
            sb[p] = (unsigned short)dg;
          }
        }
        __syncthreads();
        for (unsigned i = tid; i < tot; i += PT_THREADS) {
          unsigned dg = sb[i];
          u64 pos = cur[dg] + (i - bst[dg]);
          a.okeys[pos] = sk[i];
          a.oamps[pos] = sa[i];
        }
        __syncthreads();
        if (tid < (int)nd) {
          cur[tid] += hist[tid];
          hist[tid] = 0;
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (MODE == M_COUNT)
      for (unsigned dg = tid; dg < nd; dg += PT_THREADS) a.cm[un.cbase + (u64)dg * un.stride] = hist[dg];
    __syncthreads();
  }
}

// next level's segment boundaries: out[s*nd + dg] = scanned[segbase[s] + dg*segnu[s]] + base
__global__ void k_seg_gather(const u64* __restrict__ cm, const u64* __restrict__ segbase,
                             const unsigned* __restrict__ segnu, u64 nseg, unsigned nd, u64 total_idx, u64 base,
                             u64* __restrict__ out) {
  const u64 n = nseg * nd;
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (u64)gridDim.x * blockDim.x) {
    if (i == n) {
      out[n] = __ldcg(cm + total_idx) + base;
    } else {
      u64 s = i / nd;
      unsigned dg = (unsigned)(i - s * nd);
      out[i] = __ldcg(cm + segbase[s] + (u64)dg * segnu[s]) + base;
    }
  }
}

// ---------------------------------------------------------------------------
// leaf merge: one warp per leaf, private shared-memory hash table
// ---------------------------------------------------------------------------
template <class KT>
struct LeafArgs {
  const KT* keys;
  const double* amps;
  const u64* loff;     // nleaves + 1 boundaries in keys/amps
  u64 nleaves;
  u64 gleaf0;          // global leaf id of local leaf 0
  const KT* in_keys;   // input dets sorted by global leaf
  const double* in_amps;
  const uint32_t* in_off;  // [2^b + 1]
  FxCut cut;           // the post-merge cut
  KT* skeys;
  double* samps;
  u64* scount;
  u64* dexact;         // <v|Hv>: exact 128-bit fixed-point sum (low, high)
  double* qpart;       // nullable: per-CTA sums of squared merged amplitudes (before the cut)
  unsigned* ovf;       // [0] = count, then leaf ids (global)
  unsigned ovf_cap;
  u64* uniq;           // merged distinct determinants (statistics)
  unsigned* bad;       // set when a term is outside the fixed-point range
  u64* dinst;          // nullable: <v|Hv> per instance of a batched context, exact, 2 words each
};

// Shared-memory layout of a merge table with `n` slots: keys, then the low and
// high words of the fixed-point accumulators.
template <class KT>
struct STable {
  KT* k;
  u64* lo;
  u64* hi;
  __device__ __forceinline__ STable(unsigned char* base, unsigned n)
      : k(reinterpret_cast<KT*>(base)),
        lo(reinterpret_cast<u64*>(base + sizeof(KT) * n)),
        hi(reinterpret_cast<u64*>(base + (sizeof(KT) + sizeof(u64)) * n)) {}
  __device__ __forceinline__ double amp(unsigned s) const { return fx_acc_double(lo[s], hi[s]); }
};
constexpr size_t SLOT_BYTES_EXTRA = 2 * sizeof(u64);

// Warp-table layout with `n` slots: keys, then the four 32-bit digit-sum words
// of the narrow accumulator (word k of slot s at w[k * n + s]).
template <class KT>
struct WTable {
  KT* k;
  unsigned* w;
  unsigned n;
  __device__ __forceinline__ WTable(unsigned char* base, unsigned n_)
      : k(reinterpret_cast<KT*>(base)), w(reinterpret_cast<unsigned*>(base + sizeof(KT) * n_)), n(n_) {}
  __device__ __forceinline__ void value(unsigned s, u64& L, u64& H) const {
    const int v[4] = {(int)w[s], (int)w[n + s], (int)w[2 * n + s], (int)w[3 * n + s]};
    fx32_value(v, L, H);
  }
  __device__ __forceinline__ double amp(unsigned s) const {
    u64 L, H;
    value(s, L, H);
    return fx_to_double(L, H);
  }
};
constexpr size_t WSLOT_BYTES_EXTRA = 4 * sizeof(unsigned);

template <class KT>
__global__ void __launch_bounds__(LW_WARPS * 32, sizeof(KT) == 8 ? 4 : 3) k_leafw(LeafArgs<KT> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  WTable<KT> t(smem + (sizeof(KT) + WSLOT_BYTES_EXTRA) * TW_MAX * warp, TW_MAX);
  __shared__ double s_rq[LW_WARPS];
  __shared__ u64 s_uq[LW_WARPS];
  const KT empty = key_empty<KT>();
  const unsigned lt = (1u << lane) - 1u;
  double qacc = 0.0;
  unsigned dbad = 0;
  u64 uq = 0;
  for (u64 leaf = (u64)blockIdx.x * LW_WARPS + warp; leaf < a.nleaves; leaf += (u64)gridDim.x * LW_WARPS) {
    const u64 beg = a.loff[leaf], end = a.loff[leaf + 1], n = end - beg;
    unsigned tb = 32;
    int tbits = 5;
    while (tb < (unsigned)TW_MAX && (u64)tb < 2 * n) {
      tb <<= 1;
      ++tbits;
    }
    for (unsigned s = lane; s < tb; s += 32) {
      t.k[s] = empty;
#pragma unroll
      for (int w = 0; w < 4; ++w) t.w[w * TW_MAX + s] = 0u;
    }
    __syncwarp();
    // a leaf too long for the narrow accumulators goes straight to the next tier
    bool ovf = n > FX32_MAX_TERMS;
    // batches of LW_BATCH items per lane: the loads of a batch are issued before
    // any shared-memory atomic, so their latencies overlap
    for (u64 e0 = beg; e0 < end && !ovf; e0 += 32 * LW_BATCH) {
      KT kb[LW_BATCH];
      double ab[LW_BATCH];
#pragma unroll
      for (int q = 0; q < LW_BATCH; ++q) {
        const u64 e = e0 + (u64)q * 32 + lane;
        if (e < end) {
          kb[q] = a.keys[e];
          ab[q] = a.amps[e];
        }
      }
#pragma unroll
      for (int q = 0; q < LW_BATCH; ++q) {
        const u64 e = e0 + (u64)q * 32 + lane;
        if (e < end && !ovf) {
          int dg[4];
          unsigned big = 0;
          fx32_digits(ab[q], dg, big);  // out of the narrow range: the next tier takes the leaf
          const int s = big ? -1 : table_slot(t.k, tb - 1, kb[q], leaf_slot(kb[q], tbits), LW_PROBE);
          if (s < 0) {
            ovf = true;
          } else {
#pragma unroll
            for (int w = 0; w < 4; ++w)
              if (dg[w]) atomicAdd(t.w + w * TW_MAX + s, (unsigned)dg[w]);
          }
        }
      }
    }
    ovf = __any_sync(0xffffffffu, ovf);
    __syncwarp();
    if (ovf) {
      if (lane == 0) {
        unsigned k = atomicAdd(&a.ovf[0], 1u);
        if (k < a.ovf_cap) a.ovf[1 + k] = (unsigned)(a.gleaf0 + leaf);
      }
      __syncwarp();
      continue;
    }
    const u64 gl = a.gleaf0 + leaf;
    for (u64 e = a.in_off[gl] + lane; e < a.in_off[gl + 1]; e += 32) {
      const KT k = a.in_keys[e];
      int s = table_find(t.k, tb - 1, k, leaf_slot(k, tbits));
      if (s >= 0) {
        const double x = t.amp(s) * a.in_amps[e];
        fx_atomic_add128(a.dexact, x, dbad);
        if (a.dinst) fx_atomic_add128(a.dinst + 2 * inst_of(k), x, dbad);
      }
    }
    for (unsigned base = 0; base < tb; base += 32) {
      const unsigned s = base + lane;
      const KT k = t.k[s];
      double v = 0.0;
      const bool used = !key_eq(k, empty);
      u64 L = 0, H = 0;
      if (used) t.value(s, L, H);
      if (a.qpart && used) {
        const double x = fx_to_double(L, H);
        qacc += x * x;
      }
      const bool keep = used && fx_survives_value(L, H, a.cut, v);
      uq += __popc(__ballot_sync(0xffffffffu, used));
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (m) {
        u64 b0 = 0;
        if (lane == 0) b0 = atomicAdd(a.scount, (u64)__popc(m));
        b0 = __shfl_sync(0xffffffffu, b0, 0);
        if (keep) {
          const u64 p = b0 + __popc(m & lt);
          a.skeys[p] = k;
          a.samps[p] = v;
        }
      }
    }
    __syncwarp();
  }
  if (dbad) atomicOr(a.bad, 1u);
  const double vq = warp_sum(qacc);
  if (lane == 0) {
    s_rq[warp] = vq;
    s_uq[warp] = uq;
  }
  __syncthreads();
  if (tid == 0) {
    double sq = 0.0;
    u64 q = 0;
    for (int w = 0; w < LW_WARPS; ++w) {
      sq += s_rq[w];
      q += s_uq[w];
    }
    if (a.qpart) atomicAdd(a.qpart + blockIdx.x, sq);
    if (q) atomicAdd(a.uniq, q);
  }
}

// Second tier: leaves that a warp table could not take (too many distinct keys,
// more than FX32_MAX_TERMS terms, or a term outside the narrow range), one CTA
// per leaf with a 4096-slot shared-memory table and wide accumulators; leaves
// that overflow this too go to the global-memory table below.
template <class KT>
__global__ void __launch_bounds__(LC_THREADS) k_leafc(LeafArgs<KT> a, const unsigned* __restrict__ ids, unsigned nids,
                                                      unsigned* __restrict__ ovf2) {
  extern __shared__ __align__(16) unsigned char smem[];
  STable<KT> t(smem, LC_SLOTS);
  __shared__ unsigned s_nuniq, s_ovf;  // s_nuniq: claimed slots, counted after the inserts
  __shared__ u64 s_sum[LC_THREADS / 32 + 1];
  __shared__ double s_rq[LC_THREADS / 32];
  __shared__ u64 s_base;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const KT empty = key_empty<KT>();
  double qacc = 0.0;
  u64 uq = 0;
  unsigned bad = 0;
  for (unsigned q = blockIdx.x; q < nids; q += gridDim.x) {
    const u64 leaf = ids[q] - a.gleaf0;
    const u64 beg = a.loff[leaf], end = a.loff[leaf + 1];
    for (int s = tid; s < LC_SLOTS; s += LC_THREADS) {
      t.k[s] = empty;
      t.lo[s] = 0;
      t.hi[s] = 0;
    }
    if (tid == 0) {
      s_nuniq = 0;
      s_ovf = 0;
    }
    __syncthreads();
    // Leaves reach this tier mostly because one hot determinant (receiving up
    // to tens of thousands of terms) makes them long, so lanes of a warp that
    // hit the same slot first combine their addends with shuffles and one lane
    // adds the sum: the slot sees one atomic per warp batch, not one per term.
    // The loop is warp-uniform (its body holds warp collectives).
    for (u64 e0 = beg + (tid & ~31); e0 < end; e0 += LC_THREADS) {
      if (__any_sync(0xffffffffu, *(volatile unsigned*)&s_ovf != 0u)) break;
      const u64 e = e0 + lane;
      u64 xl = 0, xh = 0;
      int s = -1;
      if (e < end) {
        fx_addends(a.amps[e], xl, xh, bad);
        const KT k = a.keys[e];
        s = table_slot(t.k, LC_SLOTS - 1, k, (unsigned)slot_hash(k) & (LC_SLOTS - 1), LC_PROBE);
        if (s < 0) s_ovf = 1;
      }
      const unsigned grp = __match_any_sync(0xffffffffu, s >= 0 ? s : -1 - lane);
      const bool lead = s >= 0 && lane == __ffs(grp) - 1;
      unsigned rest = lead ? (grp & (grp - 1u)) : 0u;  // the other members, for the leader
      while (__any_sync(0xffffffffu, rest != 0u)) {
        const int src = rest ? __ffs(rest) - 1 : lane;
        const u64 ol = __shfl_sync(0xffffffffu, xl, src), oh = __shfl_sync(0xffffffffu, xh, src);
        if (rest) {
          xl += ol;  // lo addends are below 2^44: 32 of them cannot overflow
          xh += oh;
          rest &= rest - 1u;
        }
      }
      if (lead) fx_red(t.lo + s, t.hi + s, xl, xh);
    }
    __syncthreads();
    if (s_ovf) {
      if (tid == 0) {
        unsigned k = atomicAdd(&ovf2[0], 1u);
        if (k < a.ovf_cap) ovf2[1 + k] = ids[q];
      }
      __syncthreads();
      continue;
    }
    const u64 gl = ids[q];
    for (u64 e = a.in_off[gl] + tid; e < a.in_off[gl + 1]; e += LC_THREADS) {
      const KT k = a.in_keys[e];
      int s = table_find(t.k, LC_SLOTS - 1, k, (unsigned)slot_hash(k) & (LC_SLOTS - 1));
      if (s >= 0) {
        const double x = t.amp(s) * a.in_amps[e];
        fx_atomic_add128(a.dexact, x, bad);
        if (a.dinst) fx_atomic_add128(a.dinst + 2 * inst_of(k), x, bad);
      }
    }
    constexpr int PER = LC_SLOTS / LC_THREADS;
    unsigned c = 0, cu = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      int s = tid * PER + k;
      double v;
      if (!key_eq(t.k[s], empty)) {
        ++cu;
        if (a.qpart) {
          const double x = t.amp(s);
          qacc += x * x;
        }
        if (fx_survives(t.lo[s], t.hi[s], a.cut, v)) ++c;
      }
    }
    if (cu) atomicAdd(&s_nuniq, cu);  // read by thread 0 after the scan's barriers
    u64 tot;
    u64 ex = block_excl_scan<u64, LC_THREADS>((u64)c, &tot, s_sum);
    if (tid == 0) {
      s_base = tot ? atomicAdd(a.scount, tot) : 0;
      uq += s_nuniq;
    }
    __syncthreads();
    u64 pos = s_base + ex;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      int s = tid * PER + k;
      double v = 0.0;
      if (!key_eq(t.k[s], empty) && fx_survives(t.lo[s], t.hi[s], a.cut, v)) {
        a.skeys[pos] = t.k[s];
        a.samps[pos] = v;
        ++pos;
      }
    }
    __syncthreads();
  }
  if (bad) atomicOr(a.bad, 1u);
  const double vq = warp_sum(qacc);
  if (lane == 0) s_rq[warp] = vq;
  __syncthreads();
  if (tid == 0) {
    double sq = 0.0;
    for (int w = 0; w < LC_THREADS / 32; ++w) sq += s_rq[w];
    if (a.qpart) atomicAdd(a.qpart + blockIdx.x, sq);
    if (uq) atomicAdd(a.uniq, uq);
  }
}

// oversized leaf: global-memory table (keys tk, accumulators tl/th zeroed)
template <class KT>
__global__ void k_big_insert(const KT* __restrict__ keys, const double* __restrict__ amps, u64 beg, u64 end, KT* tk,
                             u64* tl, u64* th, unsigned mask, unsigned* bad) {
  unsigned b = 0;
  for (u64 e = beg + (u64)blockIdx.x * blockDim.x + threadIdx.x; e < end; e += (u64)gridDim.x * blockDim.x) {
    u64 xl, xh;
    fx_addends(amps[e], xl, xh, b);
    const KT k = keys[e];
    const int s = table_slot(tk, mask, k, (unsigned)slot_hash(k) & mask, mask + 1u);
    if (s >= 0) fx_red(tl + s, th + s, xl, xh);
  }
  if (b) atomicOr(bad, 1u);
}

template <class KT>
__global__ void k_big_finish(const KT* tk, const u64* tl, const u64* th, unsigned mask, const KT* in_keys,
                             const double* in_amps, u64 ib, u64 ie, FxCut cut, KT* skeys, double* samps,
                             u64* scount, u64* dexact, u64* uniq, double* qsum, u64* dinst, unsigned* bad) {
  const KT empty = key_empty<KT>();
  u64 gt = (u64)blockIdx.x * blockDim.x + threadIdx.x, gs = (u64)gridDim.x * blockDim.x;
  double qacc = 0.0;
  unsigned dbad = 0;
  for (u64 e = ib + gt; e < ie; e += gs) {
    int s = table_find_global(tk, mask, in_keys[e]);
    if (s >= 0) {
      const double x = fx_acc_double(__ldcg(tl + s), __ldcg(th + s)) * in_amps[e];
      fx_atomic_add128(dexact, x, dbad);
      if (dinst) fx_atomic_add128(dinst + 2 * inst_of(in_keys[e]), x, dbad);
    }
  }
  if (dbad) atomicOr(bad, 1u);
  for (u64 s = gt; s <= mask; s += gs) {
    KT k = ldcg_key(tk + s);
    if (key_eq(k, empty)) continue;
    atomicAdd(uniq, 1ull);
    if (qsum) {
      const double x = fx_acc_double(__ldcg(tl + s), __ldcg(th + s));
      qacc += x * x;
    }
    double v = 0.0;
    if (fx_survives(__ldcg(tl + s), __ldcg(th + s), cut, v)) {
      u64 p = atomicAdd(scount, 1ull);
      skeys[p] = k;
      samps[p] = v;
    }
  }
  if (qsum && qacc != 0.0) atomicAdd(qsum, qacc);
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
__global__ void k_in_count(const KT* __restrict__ keys, u64 n, int b, uint32_t* __restrict__ cnt) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
    atomicAdd(&cnt[key_hash(keys[i]) >> (64 - b)], 1u);
}
template <class KT>
__global__ void k_in_scatter(const KT* __restrict__ keys, const double* __restrict__ amps, u64 n, int b,
                             uint32_t* __restrict__ cur, KT* __restrict__ ok, double* __restrict__ oa) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    u64 p = atomicAdd(&cur[key_hash(keys[i]) >> (64 - b)], 1u);
    ok[p] = keys[i];
    oa[p] = amps[i];
  }
}

// ENERGY support table
template <class KT>
__global__ void k_table_build(const KT* __restrict__ keys, const double* __restrict__ amps, u64 n, KT* tk, double* ta,
                              unsigned mask) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    unsigned slot = (unsigned)slot_hash(keys[i]) & mask;
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
  h.inst = (const HamView*)c.d_insts;
  return h;
}

template <int W, int MODE>
static int launch_gen(Ctx& c, const GenArgs<typename KeyOf<W>::T>& g, unsigned grid, unsigned nbp) {
  typedef typename KeyOf<W>::T KT;
  size_t sm = gen_smem_bytes<KT>(MODE, nbp, g.kl_cap, g.cls_on != 0);
  static size_t configured = 0;
  // opt in whenever the size grows: static shared memory (the projection's
  // per-warp sums) counts against the same 48 KB default
  if (sm > configured) {
    SFCI_CUDA(cudaFuncSetAttribute(k_gen<KT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    configured = sm;
  }
  SFCI_LAUNCH(c, (k_gen<KT, MODE>), grid, GEN_THREADS, sm, g);
  return SFCI_OK;
}

__global__ void k_fill_u64(u64* p, u64 n, u64 v) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) p[i] = v;
}

// ---------------------------------------------------------------------------
// class passes: term counts per alpha class, and per determinant within a pass
// ---------------------------------------------------------------------------
// One warp per determinant: its spin-0 occupied / empty orbitals' class bytes
// in shared memory; returns the determinant's class and its spin counts.
template <class KT>
__device__ __forceinline__ unsigned class_lists(const KT& k, int N, int M, unsigned char* oc, unsigned char* vc,
                                                unsigned* na, unsigned* nv) {
  const int lane = threadIdx.x & 31;
  unsigned cls = 0, no = 0, nvv = 0, nb1 = 0;
  for (int base = 0; base < M; base += 32) {
    const int o = base + lane;
    const bool in = o < M;
    const bool occ = in && key_test(k, 2 * o), vir = in && !occ;
    const unsigned bo = __ballot_sync(0xffffffffu, occ), bv = __ballot_sync(0xffffffffu, vir);
    const unsigned lt = (1u << lane) - 1u;
    const unsigned b = in ? alpha_class_of_orb(2 * o) : 0u;
    if (occ) {
      oc[no + __popc(bo & lt)] = (unsigned char)b;
      cls ^= b;
    }
    if (vir) vc[nvv + __popc(bv & lt)] = (unsigned char)b;
    no += __popc(bo);
    nvv += __popc(bv);
    nb1 += __popc(__ballot_sync(0xffffffffu, in && key_test(k, 2 * o + 1)));
  }
  __syncwarp();
  na[0] = no;
  nv[0] = nvv;
  na[1] = nb1;
  nv[1] = M - nb1;
  return __reduce_xor_sync(0xffffffffu, cls);
}

constexpr int CLS_N = 256;

// terms of every target class over all determinants (the plan of the class passes)
template <class KT>
__global__ void __launch_bounds__(256) k_class_hist(const KT* __restrict__ keys, u64 n, int N, int M,
                                                    u64* __restrict__ hist) {
  __shared__ unsigned long long sh[CLS_N];
  __shared__ unsigned char s_oc[8][64], s_vc[8][64];
  __shared__ unsigned s_hv[8][CLS_N];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < CLS_N; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  unsigned char* oc = s_oc[warp];
  unsigned char* vc = s_vc[warp];
  unsigned* hv = s_hv[warp];
  for (u64 j = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += ((u64)gridDim.x * blockDim.x) >> 5) {
    unsigned na[2], nv[2];
    const unsigned ac = class_lists(keys[j], N, M, oc, vc, na, nv);
    const u64 nsb = (u64)na[1] * nv[1];
    if (lane == 0) atomicAdd(&sh[ac], 1ull + nsb + (u64)c2(na[1]) * c2(nv[1]));  // keeps the alpha string
    // spin-0 singles (one term each) and opposite-spin blocks (nsb terms each)
    for (unsigned x = lane; x < na[0] * nv[0]; x += 32) {
      const unsigned ii = x / nv[0], aa = x - ii * nv[0];
      atomicAdd(&sh[ac ^ oc[ii] ^ vc[aa]], 1ull + nsb);
    }
    // spin-0 doubles: the class histogram of the empty pairs, shifted per occupied pair
    for (int i = lane; i < CLS_N; i += 32) hv[i] = 0;
    __syncwarp();
    const unsigned nvp = c2(nv[0]);
    for (unsigned q = lane; q < nvp; q += 32) {
      unsigned u, v;
      unrank_pair(q, u, v);
      atomicAdd(&hv[vc[u] ^ vc[v]], 1u);
    }
    __syncwarp();
    for (unsigned op = 0; op < c2(na[0]); ++op) {
      unsigned x, y;
      unrank_pair(op, x, y);
      const unsigned sh_c = ac ^ oc[x] ^ oc[y];
      for (int c = lane; c < CLS_N; c += 32)
        if (hv[c]) atomicAdd(&sh[sh_c ^ c], (unsigned long long)hv[c]);
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < CLS_N; i += blockDim.x)
    if (sh[i]) atomicAdd(hist + i, sh[i]);
}

// index-space size of every determinant in the class pass [lo, hi) of aligned
// blocks of 2^kb classes (the generator's class-pass index space): [0, c[2]),
// the spin-0 doubles whose target class is in the pass, the spin-1 doubles
// when its own class is, and nsb per spin-0 single whose class is
template <class KT>
__global__ void __launch_bounds__(256) k_pass_counts(const KT* __restrict__ keys, u64 n, int N, int M, unsigned lo,
                                                     unsigned hi, int kb, u64* __restrict__ cnt) {
  __shared__ unsigned char s_oc[8][64], s_vc[8][64];
  __shared__ unsigned s_bc[8][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned nb = 256u >> kb, P0 = lo >> kb, nblk = (hi - lo) >> kb;
  unsigned* bc = s_bc[warp];
  for (u64 j = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += ((u64)gridDim.x * blockDim.x) >> 5) {
    unsigned na[2], nv[2];
    const unsigned char* oc = s_oc[warp];
    const unsigned char* vc = s_vc[warp];
    const unsigned ac = class_lists(keys[j], N, M, s_oc[warp], s_vc[warp], na, nv);
    const u64 nsb = (u64)na[1] * nv[1];
    unsigned kept = 0;
    for (unsigned x = lane; x < na[0] * nv[0]; x += 32) {
      const unsigned ii = x / nv[0], aa = x - ii * nv[0];
      const unsigned cx = ac ^ oc[ii] ^ vc[aa];
      kept += (cx >= lo && cx < hi) ? 1u : 0u;
    }
    kept = warp_sum(kept);
    // spin-0 doubles: buckets of the empty pairs, then per occupied pair the
    // buckets its target classes in the pass need
    for (unsigned bk = lane; bk < nb; bk += 32) bc[bk] = 0;
    __syncwarp();
    const unsigned nvp = c2(nv[0]), nop = c2(na[0]);
    for (unsigned q = lane; q < nvp; q += 32) {
      unsigned u, v;
      unrank_pair(q, u, v);
      atomicAdd(&bc[(unsigned)(vc[u] ^ vc[v]) >> kb], 1u);
    }
    __syncwarp();
    u64 n2 = 0;
    for (unsigned op = lane; op < nop; op += 32) {
      unsigned x, y;
      unrank_pair(op, x, y);
      const unsigned K = (unsigned)(ac ^ oc[x] ^ oc[y]) >> kb;
      for (unsigned jb = 0; jb < nblk; ++jb) n2 += bc[(P0 + jb) ^ K];
    }
    n2 = warp_sum(n2);
    if (lane == 0) {
      const u64 cs2 = 1ull + (u64)na[0] * nv[0] + nsb;
      const bool own = ac >= lo && ac < hi;
      cnt[j] = cs2 + n2 + (own ? (u64)c2(na[1]) * c2(nv[1]) : 0ull) + (u64)kept * nsb;
    }
    __syncwarp();
  }
}

// screened term count of a source: group 0 (diagonal and singles) plus its kept groups' terms
template <class KT>
__global__ void k_screen_counts(const KT* __restrict__ keys, u64 n, int N, int M, const u64* __restrict__ kept,
                                u64* __restrict__ cnt) {
  for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (u64)gridDim.x * blockDim.x) {
    unsigned a0, a1;
    spin_counts(keys[j], N, a0, a1);
    cnt[j] = 1ull + (u64)a0 * (M - a0) + (u64)a1 * (M - a1) + kept[j];
  }
}

// term counts (one term for determinants from nmain on) -> offsets, and diagonal elements;
// with `kept` (the screen's kept terms per source) the counts are the screened ones
template <int W>
static int prep_dets(Ctx& c, const typename KeyOf<W>::T* keys, u64 n, u64** doff, double** diagE, u64* T,
                     u64 nmain = ~0ull, const u64* kept = nullptr) {
  u64* off = (u64*)scratch_get(c, "sp_doff", (n + 1) * sizeof(u64));
  double* dg = (double*)scratch_get(c, "sp_diag", (n ? n : 1) * sizeof(double));
  if (!off || !dg) return SFCI_ERR_NOMEM;
  unsigned grid = (unsigned)std::min<u64>((n * 32 + 255) / 256, (u64)c.sm_count * 16);
  if (grid == 0) grid = 1;
  if (n) SFCI_LAUNCH(c, k_det_prep<typename KeyOf<W>::T>, grid, 256, 0, keys, n, ham_view(c), off, dg);
  if (n && kept)
    SFCI_LAUNCH(c, k_screen_counts<typename KeyOf<W>::T>, std::min<unsigned>((unsigned)((n + 255) / 256), c.sm_count * 8),
                256, 0, keys, std::min<u64>(n, nmain), c.N, c.M, kept, off);
  if (nmain < n)
    SFCI_LAUNCH(c, k_fill_u64, std::min<unsigned>((unsigned)((n - nmain + 255) / 256), c.sm_count * 8), 256, 0,
                off + nmain, n - nmain, (u64)1);
  int st = scan_excl(c, off, off, n);
  if (st) return st;
  if ((st = read_words(c, off + n, sizeof(u64), T))) return st;
  *doff = off;
  *diagE = dg;
  return SFCI_OK;
}

static unsigned gen_grid(Ctx& c, u64 T) {
  u64 g = (u64)c.sm_count * std::max(1, std::min(2, c.tune_gen_ctas));
  u64 need = (T + GEN_ROUND - 1) / GEN_ROUND;
  if (need < g) g = need;
  return (unsigned)(g ? g : 1);
}

template <int W>
static int leaf_smem_config() {
  typedef typename KeyOf<W>::T KT;
  static bool done = false;
  if (!done) {
    const int sm = (int)((sizeof(KT) + WSLOT_BYTES_EXTRA) * TW_MAX * LW_WARPS);
    SFCI_CUDA(cudaFuncSetAttribute(k_leafw<KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    SFCI_CUDA(cudaFuncSetAttribute(k_leafc<KT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)((sizeof(KT) + SLOT_BYTES_EXTRA) * LC_SLOTS)));
    constexpr int IPT = PartIPT<W>::v;
    const int ps = (int)part_smem_bytes<KT, IPT>(M_SCATTER, 1u << DIGIT_MAX);
    SFCI_CUDA(cudaFuncSetAttribute(k_part<KT, M_SCATTER, IPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps));
    done = true;
  }
  return SFCI_OK;
}

__global__ void k_scaled_copy(double* __restrict__ dst, const double* __restrict__ src, double a, u64 n) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
    dst[i] = a * src[i];
}

template <int W>
int spmspv_impl(Ctx& c, const Vec& in, Vec& out, double lambda, double coeff, double* diag, const SpExtra* ex) {
  typedef typename KeyOf<W>::T KT;
  constexpr int IPT = PartIPT<W>::v;
  for (auto& s : c.stats) s = 0;
  if (in.len == 0) {
    out.len = 0;
    return SFCI_OK;
  }
  const double cut = c.opts.coeff_cut;
  const u64 Nd = c.opts.Nd;
  int st;
  if ((st = leaf_smem_config<W>())) return st;
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
  c.last_pruned = false;
  // extra single terms (coef * vector entries) join the generation sources
  // after the input determinants; the <v|Hv> share still covers the input only
  const KT* gen_k = src_k;
  const double* gen_a = src_a;
  u64 ng = ns;
  if (ex && ex->n > 0) {
    u64 nx = 0;
    for (int j = 0; j < ex->n; ++j) nx += ex->vecs[j]->len;
    if (nx) {
      KT* xk = (KT*)scratch_get(c, "sp_gen_k", (ns + nx) * sizeof(KT));
      double* xa = (double*)scratch_get(c, "sp_gen_a", (ns + nx) * sizeof(double));
      if (!xk || !xa) return SFCI_ERR_NOMEM;
      SFCI_CUDA(cudaMemcpyAsync(xk, src_k, ns * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
      SFCI_CUDA(cudaMemcpyAsync(xa, src_a, ns * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
      u64 o = ns;
      for (int j = 0; j < ex->n; ++j) {
        const Vec& v = *ex->vecs[j];
        if (!v.len) continue;
        SFCI_CUDA(cudaMemcpyAsync(xk + o, v.keys, v.len * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
        SFCI_LAUNCH(c, k_scaled_copy, std::min<unsigned>((unsigned)((v.len + 255) / 256), c.sm_count * 8), 256, 0,
                    xa + o, (const double*)v.amps, ex->coef[j], v.len);
        o += v.len;
      }
      gen_k = xk;
      gen_a = xa;
      ng = ns + nx;
    }
  }
  {
    // a merged determinant receives at most one term per input determinant
    // connected to it, i.e. at most the term count of a determinant with its
    // spin occupations; the merge accumulators are exact up to FX_MAX_TERMS
    u64 conn = 0;
    for (int a0 = 0; a0 <= c.ne; ++a0) {
      const int a1 = c.ne - a0;
      if (a0 > c.M || a1 > c.M) continue;
      conn = std::max<u64>(conn, det_terms(a0, c.M - a0, a1, c.M - a1));
    }
    if (std::min<u64>(conn, ns) > FX_MAX_TERMS)
      return set_error(SFCI_ERR_UNSUPPORTED, "SpMSpV: determinants connect to more than 2^19 others");
  }
  // learned screen: the kept term groups of each source.  Products with extra
  // single-term sources (the linear solver's) stay unscreened.
  ScreenList sl;
  const u64* kept = nullptr;
  if (c.screen && ng == ns) {
    tok = phase_begin(c, PH_OTHER);
    if ((st = screen_select(c, src_k, src_a, ns, &sl))) return st;
    kept = sl.kept_terms;
    phase_end(c, tok);
  }
  // 2. term offsets + diagonal elements
  u64 *doff = nullptr, T = 0;
  double* diagE = nullptr;
  if ((st = prep_dets<W>(c, gen_k, ng, &doff, &diagE, &T, ns, kept))) return st;
  c.stats[1] = T;
  // ---- generation plan.  One outer pass over every term; or, when the terms
  // need several generation passes, class passes: each outer pass owns a range
  // of alpha classes of the targets (alpha_class_of_orb), generates only its
  // own terms (whole blocks skipped by class, the rest filtered term by term)
  // and merges them completely, so the work is proportional to the terms and
  // not to terms x passes.  Ordinary multi-pass plans regenerate and bin every
  // term in every pass.
  tok = phase_begin(c, PH_OTHER);
  const size_t tb = sizeof(KT) + sizeof(double);
  const u64 cap = out.cap;
  const double dup = c.dup_est > 0.0 ? c.dup_est : 8.0;
  const int leaf_uniq = std::max(16, std::min(TW_UNIQ, c.tune_leaf_uniq));
  const int l1_bits = std::max(4, std::min(L1_BITS, c.tune_l1_bits));
  const int digit_bits = std::max(6, std::min(DIGIT_MAX, c.tune_digit_bits));
  // 2^b leaves for `terms` generated terms: the fewest (so the fewest partition
  // levels, each a full read and write of the terms, and the best amortised
  // per-leaf table set-up) whose expected distinct keys stay within the leaf
  // size, so that a warp table takes a leaf.  The distinct count is estimated
  // from the duplication (terms per distinct key) of the previous product on
  // this context (default 8).  At most LEAF_TERMS terms a leaf as well: with
  // many terms per key (hot determinants) a leaf sized by distinct keys alone
  // outgrows the warp tier's FX32_MAX_TERMS.
  auto leaf_bits = [&](u64 terms) -> int {
    const double uniq_est = std::max(1.0, (double)terms / std::max(1.0, dup));
    const int b_terms = (int)std::ceil(std::log2(std::max(2.0, (double)terms / LEAF_TERMS)));
    const int b_uniq = (int)std::ceil(std::log2(std::max(2.0, uniq_est / leaf_uniq)));
    return std::max(1, std::min(B_MAX, std::max(b_terms, b_uniq)));
  };
  size_t budget = 0;
  {
    size_t freeb = 0, totb = 0;
    SFCI_CUDA(cudaMemGetInfo(&freeb, &totb));
    // the plan's buffers (replaced in place when they grow): the two term
    // levels and the survivors; the plan also leaves room for the sort scratch
    // the survivors go through (not counted here: whatever it holds stays held)
    size_t held = 0;
    for (const char* nm : {"sp_l1k", "sp_l1a", "sp_l2k", "sp_l2a", "sp_sk", "sp_sa"}) {
      auto it = c.scratch.find(nm);
      if (it != c.scratch.end()) held += it->second.bytes;
    }
    // allocations made after the plan, kept out of it: per leaf the input
    // offsets and cursors, boundaries and overflow lists (24 B), the input
    // grouped by leaf, and a margin for the small tables
    const size_t reserve = ((size_t)24 << leaf_bits(T)) + (size_t)ns * tb + ((size_t)256 << 20);
    // a batched context's driver keeps growing per-instance vectors between
    // products, so its products leave it a larger margin
    const size_t pool = (size_t)((freeb + held) * (c.ninst ? 0.85 : 0.90));
    budget = c.opts.mem_budget ? (size_t)c.opts.mem_budget : (pool > reserve ? pool - reserve : 0);
  }
  const u64 avail = budget / tb;
  struct OuterPass {
    unsigned lo, hi;  // class range (class passes): aligned blocks of 2^k classes
    u64 terms;        // terms this outer pass generates
    int k;
  };
  std::vector<OuterPass> outer;
  bool cls_mode = false;
  MemPlan cmp;  // fixed buffers of the class passes
  if (!kept && ng == ns && c.tune_class_passes >= 0 && ns > 0) {
    cmp.C2 = std::max<u64>(avail / 16, 1ull << 20);
    cmp.SC = std::min<u64>(cap, T) + cmp.C2;
    if (avail > cmp.C2 + 2 * cmp.SC) cmp.C1 = avail - cmp.C2 - 2 * cmp.SC;
    const bool many = c.tune_class_passes > 0 ? true : T > 3 * cmp.C1;  // several passes: worth the split
    if (cmp.C1 > 0 && many) {
      u64* hist = (u64*)scratch_get(c, "sp_clshist", CLS_N * sizeof(u64));
      if (!hist) return SFCI_ERR_NOMEM;
      SFCI_CUDA(cudaMemsetAsync(hist, 0, CLS_N * sizeof(u64), c.stream));
      const unsigned gr = (unsigned)std::min<u64>((ns * 32 + 255) / 256, (u64)c.sm_count * 16);
      SFCI_LAUNCH(c, k_class_hist<KT>, gr, 256, 0, src_k, ns, c.N, c.M, hist);
      std::vector<u64> hh(CLS_N);
      if ((st = read_words(c, hist, CLS_N * sizeof(u64), hh.data()))) return st;
      u64 tot = 0, big = 0;
      for (u64 v : hh) {
        tot += v;
        big = std::max(big, v);
      }
      if (tot != T) return set_error(SFCI_ERR_NUMERIC, "SpMSpV class histogram disagrees with term offsets");
      (void)big;
      // runs of aligned class blocks (plan_class_passes, plan.h)
      cls_mode = true;
      const unsigned nop_max = std::max(1u, c2((unsigned)std::min(c.ne, c.M)));
      for (const ClassPass& cp : plan_class_passes(hh, cmp.C1, nop_max, (unsigned)RUN_CAP))
        outer.push_back({cp.lo, cp.hi, cp.terms, cp.k});
      cmp.passes = (int)outer.size();
    }
  }
  if (!cls_mode) outer.push_back({0u, 0u, T, 0});
  phase_end(c, tok);
  // [0] survivors, [1] distinct, [2] fixed-point range flag
  u64* scount = (u64*)scratch_get(c, "sp_scount", 4 * sizeof(u64));
  const unsigned leafgrid = (unsigned)c.sm_count * 8;
  unsigned leaf_resident = leafgrid;
  {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_leafw<KT>, LW_WARPS * 32,
                                                      (sizeof(KT) + WSLOT_BYTES_EXTRA) * TW_MAX * LW_WARPS) ==
            cudaSuccess &&
        per_sm > 0)
      leaf_resident = std::min<unsigned>(leafgrid, (unsigned)per_sm * c.sm_count);
    cudaGetLastError();
  }
  // <v|Hv>: exact 128-bit fixed-point sums, the total and one per instance, so
  // its value does not depend on the plan, the launch order or the batching
  u64* dexact = (u64*)scratch_get(c, "sp_dexact", (2 + 2 * INST_MAX) * sizeof(u64));
  if (!scount || !dexact) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemsetAsync(scount, 0, 4 * sizeof(u64), c.stream));
  SFCI_CUDA(cudaMemsetAsync(dexact, 0, (2 + 2 * INST_MAX) * sizeof(u64), c.stream));
  // optional sum of squared merged amplitudes: per-CTA partials, then the global tier's sum
  double* qpart = nullptr;
  if (ex && ex->sumsq) {
    qpart = (double*)scratch_get(c, "sp_qpart", (leafgrid + 2) * sizeof(double));
    if (!qpart) return SFCI_ERR_NOMEM;
    SFCI_CUDA(cudaMemsetAsync(qpart, 0, (leafgrid + 2) * sizeof(double), c.stream));
  }

  u64 scount_h = 0, big_leaves = 0, T_gen = 0;
  KT* sk = nullptr;    // survivors of every outer pass (kept across them: the buffers do not
  double* sa = nullptr;  // change size between class passes)
  u64* dinst = c.ninst ? dexact + 2 : nullptr;  // batched contexts: <v|Hv> per instance
  const size_t lsm = (sizeof(KT) + WSLOT_BYTES_EXTRA) * TW_MAX * LW_WARPS;
  std::vector<u64> segs, nsegs_h;
  std::vector<Unit> units;
  std::vector<u64> segbase;
  std::vector<unsigned> segnu;
  for (const OuterPass& opass : outer) {
    // the outer pass's index space: every term, or the class pass's blocks
    u64* doffp = doff;
    u64 Tp = T;
    if (cls_mode) {
      tok = phase_begin(c, PH_OTHER);
      doffp = (u64*)scratch_get(c, "sp_pdoff", (ns + 1) * sizeof(u64));
      if (!doffp) return SFCI_ERR_NOMEM;
      const unsigned gr = (unsigned)std::min<u64>((ns * 32 + 255) / 256, (u64)c.sm_count * 16);
      SFCI_LAUNCH(c, k_pass_counts<KT>, gr, 256, 0, src_k, ns, c.N, c.M, opass.lo, opass.hi, opass.k, doffp);
      if ((st = scan_excl(c, doffp, doffp, ns))) return st;
      if ((st = read_words(c, doffp + ns, sizeof(u64), &Tp))) return st;
      phase_end(c, tok);
    }
    // hash digits: level 1 (generation) d0 bits, then nlev partition levels
    const int b = leaf_bits(opass.terms);
    const int d0 = std::min(b, l1_bits);
    const int rem = b - d0;
    const int nlev = rem ? (rem + digit_bits - 1) / digit_bits : 0;
    std::vector<int> dig(nlev);
    for (int k = 0; k < nlev; ++k) dig[k] = rem / nlev + (k < rem % nlev ? 1 : 0);
    const unsigned NB1 = 1u << d0;
    const unsigned G = gen_grid(c, Tp);

    // 3. COUNT sweep -> [bin x CTA] matrix
    tok = phase_begin(c, PH_COUNT);
    u64* cntm = (u64*)scratch_get(c, "sp_cntm", ((u64)NB1 * G + 1) * sizeof(u64));
    if (!cntm) return SFCI_ERR_NOMEM;
    GenArgs<KT> g{};
    g.keys = gen_k;
    g.amps = gen_a;
    g.ndet = ng;
    g.nmain = ns;
    g.doff = doffp;
    g.diagE = diagE;
    g.coeff = coeff;
    g.lambda = lambda;
    g.h = ham_view(c);
    g.T = Tp;
    g.b1 = d0;
    g.cntm = cntm;
    if (kept) {
      g.kl_start = sl.start;
      g.kl_pre = sl.pre;
      g.kl_off = sl.off;
      g.kl_cap = std::max(sl.gmax, 1u);
    }
    if (cls_mode) {
      g.cls_on = 1;
      g.cls_lo = opass.lo;
      g.cls_hi = opass.hi;
      g.cls_k = opass.k;
      g.kl_cap = 3 + (unsigned)(c.M * c.M / 4);  // [0, c3), spin-1 doubles, na0 * nv0 <= M^2 / 4 blocks
    }
    if ((st = launch_gen<W, M_COUNT>(c, g, G, NB1))) return st;
    if ((st = scan_excl(c, cntm, cntm, (u64)NB1 * G))) return st;
    std::vector<u64> binoff(NB1 + 1);
    {
      u64* bo = (u64*)scratch_get(c, "sp_binoff", (NB1 + 1) * sizeof(u64));
      if (!bo) return SFCI_ERR_NOMEM;
      SFCI_CUDA(cudaMemcpy2DAsync(bo, sizeof(u64), cntm, G * sizeof(u64), sizeof(u64), NB1, cudaMemcpyDeviceToDevice,
                                  c.stream));
      SFCI_CUDA(cudaMemcpyAsync(bo + NB1, cntm + (u64)NB1 * G, sizeof(u64), cudaMemcpyDeviceToDevice, c.stream));
      if ((st = read_words(c, bo, (NB1 + 1) * sizeof(u64), binoff.data()))) return st;
    }
    phase_end(c, tok);
    if (binoff[NB1] != opass.terms)
      return set_error(SFCI_ERR_NUMERIC, "SpMSpV count sweep disagrees with term offsets");
    T_gen += binoff[NB1];

    // 4. memory plan
    tok = phase_begin(c, PH_OTHER);
    u64 maxbin = 0;
    for (unsigned i = 0; i < NB1; ++i) maxbin = std::max(maxbin, binoff[i + 1] - binoff[i]);
    MemPlan mp = cmp;
    if (!cls_mode && !plan_memory(binoff, NB1, T, avail, std::min<u64>(cap, T), maxbin, nlev > 0, mp))
      return set_error(SFCI_ERR_NOMEM, "SpMSpV device-memory budget too small");
    if (cls_mode && (maxbin > mp.C1 || maxbin > mp.C2))
      return set_error(SFCI_ERR_NOMEM, "SpMSpV class pass: a level-1 bin above the buffer capacity");
    const u64 C2 = mp.C2, C1 = mp.C1, SC = mp.SC;
    KT* l1k = (KT*)scratch_get(c, "sp_l1k", C1 * sizeof(KT));
    double* l1a = (double*)scratch_get(c, "sp_l1a", C1 * sizeof(double));
    KT* l2k = nlev ? (KT*)scratch_get(c, "sp_l2k", C2 * sizeof(KT)) : nullptr;
    double* l2a = nlev ? (double*)scratch_get(c, "sp_l2a", C2 * sizeof(double)) : nullptr;
    sk = (KT*)scratch_get(c, "sp_sk", SC * sizeof(KT));
    sa = (double*)scratch_get(c, "sp_sa", SC * sizeof(double));
    if (!l1k || !l1a || !sk || !sa || (nlev && (!l2k || !l2a))) return SFCI_ERR_NOMEM;
    // input dets grouped by global leaf (top b bits of the hash)
    const u64 NL = 1ull << b;
    uint32_t* inoff = (uint32_t*)scratch_get(c, "sp_inoff", (NL + 1) * sizeof(uint32_t));
    uint32_t* incur = (uint32_t*)scratch_get(c, "sp_incur", (NL + 1) * sizeof(uint32_t));
    KT* ink = (KT*)scratch_get(c, "sp_ink", ns * sizeof(KT));
    double* ina = (double*)scratch_get(c, "sp_ina", ns * sizeof(double));
    if (!inoff || !incur || !ink || !ina) return SFCI_ERR_NOMEM;
    SFCI_CUDA(cudaMemsetAsync(inoff, 0, (NL + 1) * sizeof(uint32_t), c.stream));
    {
      unsigned gr = (unsigned)std::min<u64>((ns + 255) / 256, (u64)c.sm_count * 8);
      SFCI_LAUNCH(c, k_in_count<KT>, gr, 256, 0, src_k, ns, b, inoff);
      if ((st = scan_excl_u32(c, inoff, inoff, NL))) return st;
      SFCI_CUDA(cudaMemcpyAsync(incur, inoff, NL * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.stream));
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
    c.stats[5] += passes.size();
    c.stats[6] = NL;
    for (auto& ps : passes) {
      const unsigned lo = ps.first, hi = ps.second;
      // 5. SCATTER sweep for this pass (level-1 buffer holds bins [lo, hi))
      tok = phase_begin(c, PH_SCATTER);
      g.bin_lo = lo;
      g.bin_hi = hi;
      g.basem = cntm;
      g.pass_base = binoff[lo];
      g.okeys = l1k;
      g.oamps = l1a;
      if ((st = launch_gen<W, M_SCATTER>(c, g, G, hi - lo))) return st;
      phase_end(c, tok);
      unsigned glo = lo;
      while (glo < hi) {
        unsigned ghi = glo + 1;
        while (ghi < hi && binoff[ghi + 1] - binoff[glo] <= C2) ++ghi;
        const u64 gterms = binoff[ghi] - binoff[glo];
        if (scount_h + gterms > SC && scount_h > cap) {
          int t2 = phase_begin(c, PH_SELECT);
          size_t m = 0;
          // key order first: exact ties at the cut keep the highest keys, whatever
          // order the leaves wrote their survivors in
          if ((st = select_sorted<W>(c, sk, sa, scount_h, cap, &m))) return st;
          scount_h = m;
          c.last_pruned = true;
          SFCI_CUDA(cudaMemcpyAsync(scount, &scount_h, sizeof(u64), cudaMemcpyHostToDevice, c.stream));
          phase_end(c, t2);
        }
        const unsigned nbg = ghi - glo;
        // segments of this group: its level-1 bins, positions in the level-1 buffer
        segs.assign(nbg + 1, 0);
        for (unsigned i = 0; i <= nbg; ++i) segs[i] = binoff[glo + i] - binoff[lo];
        const u64 gbase = segs[0];
        KT* srck = l1k;
        double* srca = l1a;
        KT* dstk = l2k;
        double* dsta = l2a;
        bool dst_is_l1 = false;
        u64* loff_dev = nullptr;
        // 6a. partition levels
        tok = phase_begin(c, PH_PARTITION);
        int consumed = d0;
        for (int k = 0; k < nlev; ++k) {
          const unsigned nd = 1u << dig[k];
          const u64 nseg = segs.size() - 1;
          units.clear();
          segbase.assign(nseg, 0);
          segnu.assign(nseg, 0);
          u64 cbase = 0;
          for (u64 s = 0; s < nseg; ++s) {
            const u64 a0 = segs[s], a1 = segs[s + 1], n = a1 - a0;
            const unsigned nu = (unsigned)std::max<u64>(1, (n + UNIT_ITEMS - 1) / UNIT_ITEMS);
            segbase[s] = cbase;
            segnu[s] = nu;
            for (unsigned j = 0; j < nu; ++j) {
              Unit un;
              un.start = a0 + (u64)j * UNIT_ITEMS;
              un.end = std::min<u64>(a1, un.start + UNIT_ITEMS);
              if (un.start > un.end) un.start = un.end;
              un.cbase = cbase + j;
              un.stride = nu;
              un.pad = 0;
              units.push_back(un);
            }
            cbase += (u64)nu * nd;
          }
          const u64 mlen = cbase;
          Unit* du = (Unit*)scratch_get(c, "sp_units", units.size() * sizeof(Unit));
          u64* cm = (u64*)scratch_get(c, "sp_cm", (mlen + 1) * sizeof(u64));
          u64* dsb = (u64*)scratch_get(c, "sp_segbase", nseg * sizeof(u64));
          unsigned* dsn = (unsigned*)scratch_get(c, "sp_segnu", nseg * sizeof(unsigned));
          u64* nextoff = (u64*)scratch_get(c, k == nlev - 1 ? "sp_loff" : "sp_segoff", (nseg * nd + 1) * sizeof(u64));
          if (!du || !cm || !dsb || !dsn || !nextoff) return SFCI_ERR_NOMEM;
          SFCI_CUDA(cudaMemcpyAsync(du, units.data(), units.size() * sizeof(Unit), cudaMemcpyHostToDevice, c.stream));
          SFCI_CUDA(cudaMemcpyAsync(dsb, segbase.data(), nseg * sizeof(u64), cudaMemcpyHostToDevice, c.stream));
          SFCI_CUDA(cudaMemcpyAsync(dsn, segnu.data(), nseg * sizeof(unsigned), cudaMemcpyHostToDevice, c.stream));
          PartArgs<KT> pa{};
          pa.ikeys = srck;
          pa.iamps = srca;
          pa.units = du;
          pa.nunits = (unsigned)units.size();
          pa.shift = 64 - consumed - dig[k];
          pa.nd = nd;
          pa.cm = cm;
          pa.dst_base = dst_is_l1 ? gbase : 0;
          pa.okeys = dstk;
          pa.oamps = dsta;
          const unsigned pgrid = (unsigned)std::min<u64>(units.size(), (u64)c.sm_count * 4);
          const size_t smc = part_smem_bytes<KT, IPT>(M_COUNT, nd);
          const size_t sms = part_smem_bytes<KT, IPT>(M_SCATTER, nd);
          SFCI_LAUNCH(c, (k_part<KT, M_COUNT, IPT>), pgrid, PT_THREADS, smc, pa);
          if ((st = scan_excl(c, cm, cm, mlen))) return st;
          SFCI_LAUNCH(c, (k_part<KT, M_SCATTER, IPT>), pgrid, PT_THREADS, sms, pa);
          {
            const u64 nn = nseg * nd + 1;
            unsigned gr = (unsigned)std::min<u64>((nn + 255) / 256, (u64)c.sm_count * 8);
            SFCI_LAUNCH(c, k_seg_gather, gr, 256, 0, (const u64*)cm, (const u64*)dsb, (const unsigned*)dsn, nseg, nd,
                        mlen, pa.dst_base, nextoff);
          }
          consumed += dig[k];
          if (k == nlev - 1) {
            loff_dev = nextoff;
            segs.resize(nseg * nd + 1);  // sizes only needed for the leaf count below
          } else {
            nsegs_h.resize(nseg * nd + 1);
            if ((st = read_words(c, nextoff, (nseg * nd + 1) * sizeof(u64), nsegs_h.data()))) return st;
            segs.swap(nsegs_h);
          }
          std::swap(srck, dstk);
          std::swap(srca, dsta);
          dst_is_l1 = !dst_is_l1;
        }
        phase_end(c, tok);
        const u64 nleaves = segs.size() - 1;
        if (nlev == 0) {
          loff_dev = (u64*)scratch_get(c, "sp_loff", (nleaves + 1) * sizeof(u64));
          if (!loff_dev) return SFCI_ERR_NOMEM;
          SFCI_CUDA(cudaMemcpyAsync(loff_dev, segs.data(), (nleaves + 1) * sizeof(u64), cudaMemcpyHostToDevice,
                                    c.stream));
        }
        // 6b. leaf merge (one warp per leaf)
        tok = phase_begin(c, PH_MERGE);
        LeafArgs<KT> la{};
        la.keys = srck;
        la.amps = srca;
        la.loff = loff_dev;
        la.nleaves = nleaves;
        la.gleaf0 = (u64)glo << (b - d0);
        la.in_keys = ink;
        la.in_amps = ina;
        la.in_off = inoff;
        la.cut = fx_cut(cut);
        la.skeys = sk;
        la.samps = sa;
        la.scount = scount;
        la.dexact = dexact;
        la.qpart = qpart;
        // overflow lists of the two table tiers: every leaf of the group can
        // overflow a tier at most once (the leaf count comes from the previous
        // product's duplication, which can be off by several times)
        unsigned* ovf = (unsigned*)scratch_get(c, "sp_ovf", (nleaves + 1) * sizeof(unsigned));
        unsigned* ovf2 = (unsigned*)scratch_get(c, "sp_ovf2", (nleaves + 1) * sizeof(unsigned));
        if (!ovf || !ovf2) return SFCI_ERR_NOMEM;
        const unsigned OVF_CAP = (unsigned)nleaves;
        la.ovf = ovf;
        la.ovf_cap = OVF_CAP;
        la.uniq = scount + 1;
        la.bad = (unsigned*)(scount + 2);
        la.dinst = dinst;
        SFCI_CUDA(cudaMemsetAsync(ovf, 0, sizeof(unsigned), c.stream));
        const unsigned lg = (unsigned)std::min<u64>((nleaves + LW_WARPS - 1) / LW_WARPS, leaf_resident);
        SFCI_LAUNCH(c, k_leafw<KT>, lg, LW_WARPS * 32, lsm, la);
        unsigned novf = 0;
        if ((st = read_words(c, ovf, sizeof(unsigned), &novf))) return st;
        if (novf > OVF_CAP) return set_error(SFCI_ERR_NOMEM, "too many oversized SpMSpV leaves");
        if (novf) {
          // second tier: one CTA per overflowed leaf, all in one launch
          SFCI_CUDA(cudaMemsetAsync(ovf2, 0, sizeof(unsigned), c.stream));
          const unsigned cg = std::min<unsigned>(novf, leafgrid);
          SFCI_LAUNCH(c, k_leafc<KT>, cg, LC_THREADS, (sizeof(KT) + SLOT_BYTES_EXTRA) * LC_SLOTS, la,
                      (const unsigned*)(ovf + 1), novf, ovf2);
          if ((st = read_words(c, ovf2, sizeof(unsigned), &novf))) return st;
          if (novf > OVF_CAP) return set_error(SFCI_ERR_NOMEM, "too many oversized SpMSpV leaves");
        }
        if (novf) {
          std::vector<unsigned> ids(novf);
          if ((st = read_words(c, ovf2 + 1, novf * sizeof(unsigned), ids.data()))) return st;
          big_leaves += novf;
          for (unsigned id : ids) {
            const u64 lid = id - la.gleaf0;
            u64 lb2[2];
            if ((st = read_words(c, loff_dev + lid, 2 * sizeof(u64), lb2))) return st;
            const u64 beg = lb2[0], end = lb2[1], n = end - beg;
            u64 tsz = 1;
            while (tsz < 2 * n) tsz <<= 1;
            KT* bk = (KT*)scratch_get(c, "sp_bigk", tsz * sizeof(KT));
            u64* ba = (u64*)scratch_get(c, "sp_biga", 2 * tsz * sizeof(u64));
            if (!bk || !ba) return SFCI_ERR_NOMEM;
            unsigned gr = (unsigned)std::min<u64>((tsz + 255) / 256, (u64)c.sm_count * 8);
            SFCI_LAUNCH(c, k_fill_empty<KT>, gr, 256, 0, bk, (double*)nullptr, tsz);
            SFCI_CUDA(cudaMemsetAsync(ba, 0, 2 * tsz * sizeof(u64), c.stream));
            gr = (unsigned)std::min<u64>((n + 255) / 256, (u64)c.sm_count * 8);
            if (gr == 0) gr = 1;
            SFCI_LAUNCH(c, k_big_insert<KT>, gr, 256, 0, (const KT*)srck, (const double*)srca, beg, end, bk, ba,
                        ba + tsz, (unsigned)(tsz - 1), la.bad);
            uint32_t ib_ie[2];
            if ((st = read_words(c, inoff + id, 2 * sizeof(uint32_t), ib_ie))) return st;
            gr = (unsigned)std::min<u64>((tsz + 255) / 256, (u64)c.sm_count * 8);
            SFCI_LAUNCH(c, k_big_finish<KT>, gr, 256, 0, (const KT*)bk, (const u64*)ba, (const u64*)(ba + tsz),
                        (unsigned)(tsz - 1), (const KT*)ink, (const double*)ina, (u64)ib_ie[0], (u64)ib_ie[1],
                        la.cut, sk, sa, scount, dexact, scount + 1, qpart ? qpart + leafgrid + 1 : nullptr, la.dinst,
                        la.bad);
          }
        }
        if ((st = read_words(c, scount, sizeof(u64), &scount_h))) return st;
        phase_end(c, tok);
        glo = ghi;
      }
    }
  }
  c.stats[7] = big_leaves;
  c.stats[1] = T_gen;
  // 7. <v|Hv> and final selection + key sort
  tok = phase_begin(c, PH_OTHER);
  std::vector<u64> dx(2 + 2 * INST_MAX);
  if ((st = read_words(c, dexact, dx.size() * sizeof(u64), dx.data()))) return st;
  const double dl = fx_to_double(dx[0], dx[1]);
  u64 fxbad = 0;
  if ((st = read_words(c, scount + 2, sizeof(u64), &fxbad))) return st;
  phase_end(c, tok);
  if (fxbad)
    return set_error(SFCI_ERR_NUMERIC,
                     "SpMSpV term with |amplitude| >= 2^24 or not finite: outside the merge accumulator's range");
  c.stats[3] = scount_h;
  u64 nout = scount_h;
  {
    tok = phase_begin(c, nout > cap ? PH_SELECT : PH_SORT);
    size_t m = 0;
    if ((st = select_sorted<W>(c, sk, sa, nout, cap, &m))) return st;
    nout = m;
    phase_end(c, tok);
  }
  tok = phase_begin(c, PH_SORT);
  SFCI_CUDA(cudaMemcpyAsync(out.keys, sk, nout * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
  SFCI_CUDA(cudaMemcpyAsync(out.amps, sa, nout * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  out.len = nout;
  phase_end(c, tok);
  c.stats[4] = nout;
  {
    u64 uq = 0;
    if ((st = read_words(c, scount + 1, sizeof(u64), &uq))) return st;
    c.stats[2] = uq;
    if (uq) c.dup_est = (double)T_gen / (double)uq;
  }
  *diag = dl;
  if (dinst) {
    c.inst_diag.assign(INST_MAX, 0.0);
    for (int i = 0; i < INST_MAX; ++i) c.inst_diag[i] = fx_to_double(dx[2 + 2 * i], dx[3 + 2 * i]);
  }
  if (qpart) {
    SFCI_LAUNCH(c, k_sum_parts, 1, 32, 0, (const double*)qpart, (int)leafgrid, qpart + leafgrid);
    double q2[2] = {0.0, 0.0};
    if ((st = read_words(c, qpart + leafgrid, 2 * sizeof(double), q2))) return st;
    *ex->sumsq = q2[0] + q2[1];
  }
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

// ---------------------------------------------------------------------------
// projection and the linear solver's products
// ---------------------------------------------------------------------------
// table of the union of several vectors' keys
template <class KT>
__global__ void k_key_insert(const KT* __restrict__ keys, u64 n, KT* tk, unsigned mask) {
  const KT empty = key_empty<KT>();
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    unsigned slot = (unsigned)slot_hash(keys[i]) & mask;
    for (unsigned probe = 0; probe <= mask; ++probe) {
      const KT prev = cas_key(&tk[slot], empty, keys[i]);
      if (key_eq(prev, empty) || key_eq(prev, keys[i])) break;
      slot = (slot + 1) & mask;
    }
  }
}

// per-CTA partial of sum_k v[k] * w[k], w the exact merged amplitudes in the table
template <class KT>
__global__ void __launch_bounds__(256) k_proj_dot(const KT* __restrict__ keys, const double* __restrict__ amps, u64 n,
                                                  const KT* tk, unsigned mask, const u64* plo, const u64* phi,
                                                  double* __restrict__ part) {
  __shared__ double s_red[8];
  double acc = 0.0;
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    const int s = table_find_global(tk, mask, keys[i]);
    if (s >= 0) acc += amps[i] * fx_acc_double(__ldcg(plo + s), __ldcg(phi + s));
  }
  acc = block_sum<256>(acc, s_red);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

__global__ void k_proj_sum(const double* __restrict__ part, int G, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < G; ++b) s += __ldcg(part + b);
    *out = s;
  }
}

// out[j] = <basis_j | merge((H - lambda) src)> for j < nv (src coefficient 1):
// one generation sweep over src merges, exactly, every term that lands on the
// union of the basis vectors' keys into that key's accumulator (the rest of
// the product is never stored); then each dot is one pass over its vector.
// These are the dots of the merged product with the basis vectors that
// src/functions.cpp:971-978 takes, up to the dots' summation order.
template <int W>
int project_impl(Ctx& c, const Vec& src, double lambda, const Vec* const* basis, int nv, double* out) {
  typedef typename KeyOf<W>::T KT;
  if (nv < 1 || nv > PROJ_MAX) return set_error(SFCI_ERR_ARG, "projection onto 1 to 64 vectors");
  for (int j = 0; j < nv; ++j) out[j] = 0.0;
  u64 nt = 0;
  for (int j = 0; j < nv; ++j) nt += basis[j]->len;
  if (src.len == 0 || nt == 0) return SFCI_OK;
  u64 tsz = 64;
  while (tsz < 2 * nt) tsz <<= 1;
  if (tsz > (1ull << 31)) return set_error(SFCI_ERR_UNSUPPORTED, "projection table above 2^31 slots");
  KT* tk = (KT*)scratch_get(c, "pj_tk", tsz * sizeof(KT));
  u64* acc = (u64*)scratch_get(c, "pj_acc", (2 * tsz + 1) * sizeof(u64));
  if (!tk || !acc) return SFCI_ERR_NOMEM;
  u64 *plo = acc, *phi = acc + tsz;
  unsigned* bad = (unsigned*)(acc + 2 * tsz);
  unsigned gr = (unsigned)std::min<u64>((tsz + 255) / 256, (u64)c.sm_count * 8);
  SFCI_LAUNCH(c, k_fill_empty<KT>, gr, 256, 0, tk, (double*)nullptr, tsz);
  SFCI_CUDA(cudaMemsetAsync(acc, 0, (2 * tsz + 1) * sizeof(u64), c.stream));
  for (int j = 0; j < nv; ++j) {
    const u64 l = basis[j]->len;
    if (!l) continue;
    gr = (unsigned)std::min<u64>((l + 255) / 256, (u64)c.sm_count * 8);
    SFCI_LAUNCH(c, k_key_insert<KT>, gr, 256, 0, (const KT*)basis[j]->keys, l, tk, (unsigned)(tsz - 1));
  }
  int st;
  u64 *doff = nullptr, T = 0;
  double* diagE = nullptr;
  if ((st = prep_dets<W>(c, (const KT*)src.keys, src.len, &doff, &diagE, &T))) return st;
  const unsigned G = gen_grid(c, T);
  GenArgs<KT> g{};
  g.keys = (const KT*)src.keys;
  g.amps = src.amps;
  g.ndet = src.len;
  g.doff = doff;
  g.diagE = diagE;
  g.coeff = 1.0;
  g.lambda = lambda;
  g.h = ham_view(c);
  g.T = T;
  g.b1 = 1;
  g.tkeys = tk;
  g.tmask = (unsigned)(tsz - 1);
  g.plo = plo;
  g.phi = phi;
  g.pbad = bad;
  if ((st = launch_gen<W, M_PROJECT>(c, g, G, 0))) return st;
  unsigned hbad = 0;
  if ((st = read_words(c, bad, sizeof(unsigned), &hbad))) return st;
  if (hbad)
    return set_error(SFCI_ERR_NUMERIC,
                     "projection term with |amplitude| >= 2^24 or not finite: outside the accumulator's range");
  const unsigned DG = (unsigned)c.sm_count * 2;
  double* part = (double*)scratch_get(c, "pj_part", ((u64)DG + 1) * nv * sizeof(double));
  if (!part) return SFCI_ERR_NOMEM;
  for (int j = 0; j < nv; ++j) {
    const u64 l = basis[j]->len;
    double* pj = part + (u64)j * (DG + 1);
    if (!l) {
      SFCI_CUDA(cudaMemsetAsync(pj + DG, 0, sizeof(double), c.stream));
      continue;
    }
    const unsigned dg = (unsigned)std::min<u64>((l + 255) / 256, DG);
    SFCI_LAUNCH(c, k_proj_dot<KT>, dg, 256, 0, (const KT*)basis[j]->keys, (const double*)basis[j]->amps, l,
                (const KT*)tk, (unsigned)(tsz - 1), (const u64*)plo, (const u64*)phi, pj);
    SFCI_LAUNCH(c, k_proj_sum, 1, 32, 0, (const double*)pj, (int)dg, pj + DG);
  }
  std::vector<double> all((u64)nv * (DG + 1));
  if ((st = read_words(c, part, all.size() * sizeof(double), all.data()))) return st;
  for (int j = 0; j < nv; ++j) out[j] = all[(u64)j * (DG + 1) + DG];
  return SFCI_OK;
}

// the whole input enters the product (the linear solver's products take no top-Nd slice)
template <int W>
static int product_all(Ctx& c, const Vec& in, Vec& out, double lambda, const SpExtra& ex) {
  const u64 nd = c.opts.Nd;
  c.opts.Nd = std::max<u64>(nd, in.len);
  double dg = 0.0;
  const int st = spmspv_impl<W>(c, in, out, lambda, 1.0, &dg, &ex);
  c.opts.Nd = nd;
  return st;
}

// spmspvm_bucket_linear (src/functions.cpp:858-1094) with current_idx = nb - 1
template <int W>
int spmspv_linear_impl(Ctx& c, const Vec& in, Vec& out, double lambda, const Vec* const* basis, int nb, double* hij) {
  if (in.len == 0) {  // :880-884: empty result, Hij left as it was
    out.len = 0;
    return SFCI_OK;
  }
  int st = project_impl<W>(c, in, lambda, basis, nb, hij);
  if (st) return st;
  SpExtra ex;
  ex.vecs[0] = basis[nb - 1];
  ex.coef[0] = -hij[nb - 1];
  ex.n = 1;
  if (nb > 1) {
    ex.vecs[1] = basis[nb - 2];
    ex.coef[1] = -hij[nb - 2];
    ex.n = 2;
  }
  return product_all<W>(c, in, out, lambda, ex);
}

// spmspvm_bucket_res_norm (src/functions.cpp:1096-1269)
template <int W>
int res_norm_impl(Ctx& c, const Vec& x, Vec& r, const Vec& b, double lambda, double* res) {
  typedef typename KeyOf<W>::T KT;
  int st;
  if (x.len == 0) {
    // A x = 0: r = -b through the cut and the top-cap, |A x - b| = |b|
    if ((st = norm_impl(c, b, res))) return st;
    const u64 n = b.len;
    KT* tk = (KT*)scratch_get(c, "rn_k", (n ? n : 1) * sizeof(KT));
    double* na = (double*)scratch_get(c, "rn_n", (n ? n : 1) * sizeof(double));
    double* ta = (double*)scratch_get(c, "rn_a", (n ? n : 1) * sizeof(double));
    if (!tk || !na || !ta) return SFCI_ERR_NOMEM;
    if (n) {
      SFCI_LAUNCH(c, k_scaled_copy, std::min<unsigned>((unsigned)((n + 255) / 256), c.sm_count * 8), 256, 0, na,
                  (const double*)b.amps, -1.0, n);
    }
    size_t m = 0;
    if ((st = compact_cut<W>(c, (const KT*)b.keys, na, n, c.opts.coeff_cut, tk, ta, &m))) return st;
    if (m > r.cap) {
      size_t m2 = 0;
      if ((st = top_k_stable<W>(c, tk, ta, m, r.cap, -1.0, tk, ta, &m2))) return st;
      m = m2;
    }
    SFCI_CUDA(cudaMemcpyAsync(r.keys, tk, m * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
    SFCI_CUDA(cudaMemcpyAsync(r.amps, ta, m * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    r.len = m;
    return SFCI_OK;
  }
  double q = 0.0;
  SpExtra ex;
  ex.vecs[0] = &b;
  ex.coef[0] = -1.0;
  ex.n = 1;
  ex.sumsq = &q;
  if ((st = product_all<W>(c, x, r, lambda, ex))) return st;
  *res = std::sqrt(q);
  return SFCI_OK;
}

// ---------------------------------------------------------------------------
// learned screen: group offsets and label logging
// ---------------------------------------------------------------------------
template <class KT>
__global__ void k_group_count(const KT* __restrict__ keys, u64 n, int N, int M, u64* __restrict__ cnt) {
  for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (u64)gridDim.x * blockDim.x) {
    unsigned a0, a1;
    spin_counts(keys[j], N, a0, a1);
    cnt[j] = det_groups(a0, M - a0, a1, M - a1) - 1;
  }
}

template <int W>
int group_offsets_impl(Ctx& c, const typename KeyOf<W>::T* keys, u64 n, u64* goff) {
  typedef typename KeyOf<W>::T KT;
  if (n)
    SFCI_LAUNCH(c, k_group_count<KT>, std::min<unsigned>((unsigned)((n + 255) / 256), c.sm_count * 8), 256, 0, keys, n,
                c.N, c.M, goff);
  return scan_excl(c, goff, goff, n);
}

template <int W>
int label_impl(Ctx& c, const typename KeyOf<W>::T* keys, const double* amps, u64 n, const u64* goff, const Vec& out,
               uint32_t* labels, double min_term) {
  typedef typename KeyOf<W>::T KT;
  if (n == 0 || out.len == 0) return SFCI_OK;
  int st;
  u64 *doff = nullptr, T = 0;
  double* diagE = nullptr;
  if ((st = prep_dets<W>(c, keys, n, &doff, &diagE, &T))) return st;
  u64 tsz = 1;
  while (tsz < 2 * out.len) tsz <<= 1;
  if (tsz > (1ull << 31)) return set_error(SFCI_ERR_UNSUPPORTED, "label table too large");
  KT* tk = (KT*)scratch_get(c, "lb_tk", tsz * sizeof(KT));
  double* ta = (double*)scratch_get(c, "lb_ta", tsz * sizeof(double));
  if (!tk || !ta) return SFCI_ERR_NOMEM;
  unsigned gr = (unsigned)std::min<u64>((tsz + 255) / 256, (u64)c.sm_count * 8);
  SFCI_LAUNCH(c, k_fill_empty<KT>, gr, 256, 0, tk, ta, tsz);
  gr = (unsigned)std::min<u64>((out.len + 255) / 256, (u64)c.sm_count * 8);
  SFCI_LAUNCH(c, k_table_build<KT>, gr, 256, 0, (const KT*)out.keys, out.amps, out.len, tk, ta, (unsigned)(tsz - 1));
  GenArgs<KT> g{};
  g.keys = keys;
  g.amps = amps;
  g.ndet = n;
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
  g.goff = goff;
  g.labels = labels;
  g.label_min = min_term;
  return launch_gen<W, M_LABEL>(c, g, gen_grid(c, T), 0);
}

template int group_offsets_impl<1>(Ctx&, const u64*, u64, u64*);
template int group_offsets_impl<2>(Ctx&, const K128*, u64, u64*);
template int label_impl<1>(Ctx&, const u64*, const double*, u64, const u64*, const Vec&, uint32_t*, double);
template int label_impl<2>(Ctx&, const K128*, const double*, u64, const u64*, const Vec&, uint32_t*, double);

template int spmspv_impl<1>(Ctx&, const Vec&, Vec&, double, double, double*, const SpExtra*);
template int spmspv_impl<2>(Ctx&, const Vec&, Vec&, double, double, double*, const SpExtra*);
template int project_impl<1>(Ctx&, const Vec&, double, const Vec* const*, int, double*);
template int project_impl<2>(Ctx&, const Vec&, double, const Vec* const*, int, double*);
template int spmspv_linear_impl<1>(Ctx&, const Vec&, Vec&, double, const Vec* const*, int, double*);
template int spmspv_linear_impl<2>(Ctx&, const Vec&, Vec&, double, const Vec* const*, int, double*);
template int res_norm_impl<1>(Ctx&, const Vec&, Vec&, const Vec&, double, double*);
template int res_norm_impl<2>(Ctx&, const Vec&, Vec&, const Vec&, double, double*);
template int energy_impl<1>(Ctx&, const Vec&, double*);
template int energy_impl<2>(Ctx&, const Vec&, double*);
template int diag_elements_impl<1>(Ctx&, const u64*, u64, double*);
template int diag_elements_impl<2>(Ctx&, const K128*, u64, double*);

}  // namespace sfci

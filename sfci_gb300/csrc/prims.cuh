// Device primitives: block scans, exclusive scans, LSD radix sort of
// (key, FP64) pairs, radix-select of the k largest |amp| and stable compaction.
// These replace the reference's hand-written introsort (src/introsort.cpp) and
// the serial top-k copies in src/all.h:281-299,456-478 and
// src/functions.cpp:777-793.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace sfci {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096

#ifdef __CUDACC__
// Exclusive block scan of one value per thread (blockDim.x == NT, multiple of 32).
template <typename T, int NT>
__device__ __forceinline__ T block_excl_scan(T v, T* total, T* sh /* >= NT/32 + 1 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < NT / 32 ? sh[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NT / 32) sh[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  T warp_off = warp ? sh[warp - 1] : T(0);
  if (total) *total = sh[NT / 32 - 1];
  T r = warp_off + x - v;
  __syncthreads();
  return r;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < NT / 32; ++w) r += sh[w];
  __syncthreads();
  return r;  // valid in thread 0
}
#endif

// out[i] = sum_{j<i} in[j] for i <= n (out has n+1 entries; out[n] = total).
// in may alias out only if in == out.
int scan_excl(Ctx& c, const u64* in, u64* out, size_t n);
int scan_excl_u32(Ctx& c, const uint32_t* in, uint32_t* out, size_t n);

// Stable LSD radix sort of (keys, vals) over key bits [0, nbits), in place.
template <int W>
int radix_sort_pairs(Ctx& c, typename KeyOf<W>::T* keys, double* vals, size_t n, int nbits);

// Radix-select on |amp| bit patterns: finds tau such that #(|a|>tau) < k <= #(|a|>=tau).
// Returns count_gt (number strictly above tau) through *gt.  Requires k < n.
int select_threshold(Ctx& c, const double* amps, size_t n, size_t k, u64* tau, size_t* gt);

// Stable compaction: keep entries with |a| > tau, plus the first need_eq entries
// (in index order) with |a| == tau; then, if tiny >= 0, also drop |a| <= tiny.
// Writes to (ok, oa) and returns the count via *m.
template <int W>
int compact_top(Ctx& c, const typename KeyOf<W>::T* ik, const double* ia, size_t n, u64 tau,
                size_t need_eq, double tiny, typename KeyOf<W>::T* ok, double* oa, size_t* m);

// Stable compaction of entries with |a| > cut.
template <int W>
int compact_cut(Ctx& c, const typename KeyOf<W>::T* ik, const double* ia, size_t n, double cut,
                typename KeyOf<W>::T* ok, double* oa, size_t* m);

// Keep the k largest |a| of (ik, ia), stably (key order preserved); in place allowed
// when ok==ik, oa==ia.  *m receives the new length.  tiny >= 0 adds a |a| > tiny filter
// after the selection.
template <int W>
int top_k_stable(Ctx& c, typename KeyOf<W>::T* ik, double* ia, size_t n, size_t k, double tiny,
                 typename KeyOf<W>::T* ok, double* oa, size_t* m);

// Sort (keys, vals) by key in place, then keep the k largest |a| in key order
// (all of them when n <= k): exact ties at the threshold keep the highest keys,
// whatever order the pairs came in.  The compaction writes into the sort's
// scratch and copies back, so no third n-sized buffer is needed.
template <int W>
int select_sorted(Ctx& c, typename KeyOf<W>::T* keys, double* vals, size_t n, size_t k, size_t* m);

// deterministic FP64 sum / dot reductions
int reduce_sum_sq(Ctx& c, const double* a, size_t n, double* out);

// device -> host readback of a few words through pinned memory (synchronises)
int read_words(Ctx& c, const void* dptr, size_t nbytes, void* host);

}  // namespace sfci

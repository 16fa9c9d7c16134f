// Sparse-vector algebra on device-resident, key-sorted vectors: the GB300
// replacement of dynVec's serial merges and sorts (src/all.h:249-623).
//
// Vectors keep dynVec's invariant (ascending key order).  Two sorted inputs are
// merged with merge-path partitioning (equal keys: first input first), runs of
// equal keys are summed in input order (merge_bucket, src/functions.cpp:429-464),
// and the top-cap by |amp| is taken with a radix select followed by a stable
// compaction, so the result stays in key order without the reference's second
// full sort.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gen.cuh"
#include "prims.cuh"
#include "spmspv.h"

namespace sfci {

constexpr int MP_THREADS = 256;
constexpr int MP_ITEMS = 8;

template <class KT>
__device__ __forceinline__ u64 merge_path(const KT* A, u64 na, const KT* B, u64 nb, u64 diag) {
  u64 lo = diag > nb ? diag - nb : 0, hi = diag < na ? diag : na;
  while (lo < hi) {
    u64 mid = (lo + hi) >> 1;
    if (!key_lt(B[diag - 1 - mid], A[mid])) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// out = merge(alpha*A, beta*B), ties: A first
template <class KT>
__global__ void k_merge(const KT* __restrict__ A, const double* __restrict__ Aa, u64 na, double alpha,
                        const KT* __restrict__ B, const double* __restrict__ Ba, u64 nb, double beta,
                        KT* __restrict__ ok, double* __restrict__ oa, int scaleA) {
  const u64 n = na + nb;
  u64 d = ((u64)blockIdx.x * blockDim.x + threadIdx.x) * MP_ITEMS;
  if (d >= n) return;
  u64 i = merge_path(A, na, B, nb, d), j = d - i;
#pragma unroll
  for (int t = 0; t < MP_ITEMS; ++t) {
    u64 o = d + t;
    if (o >= n) break;
    bool takeA = (j >= nb) || (i < na && !key_lt(B[j], A[i]));
    if (takeA) {
      ok[o] = A[i];
      oa[o] = scaleA ? alpha * Aa[i] : Aa[i];
      ++i;
    } else {
      ok[o] = B[j];
      oa[o] = beta * Ba[j];
      ++j;
    }
  }
}

// dot over common keys (keys unique within each vector)
template <class KT>
__global__ void k_dot(const KT* __restrict__ A, const double* __restrict__ Aa, u64 na, const KT* __restrict__ B,
                      const double* __restrict__ Ba, u64 nb, double* __restrict__ part) {
  __shared__ double sh[32];
  const u64 n = na + nb;
  u64 d = ((u64)blockIdx.x * blockDim.x + threadIdx.x) * MP_ITEMS;
  double acc = 0.0;
  if (d < n) {
    u64 i = merge_path(A, na, B, nb, d), j = d - i;
    for (int t = 0; t < MP_ITEMS && d + t < n; ++t) {
      bool takeA = (j >= nb) || (i < na && !key_lt(B[j], A[i]));
      if (takeA) {
        ++i;
      } else {
        if (i > 0 && key_eq(A[i - 1], B[j])) acc += Aa[i - 1] * Ba[j];
        ++j;
      }
    }
  }
  double t = block_sum<MP_THREADS>(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_sum_serial(const double* __restrict__ p, u64 n, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (u64 i = 0; i < n; ++i) s += __ldcg(p + i);
    *out = s;
  }
}

// ---- segmented reduction of runs of equal keys (sorted input) -------------
constexpr int SR_THREADS = 256;
constexpr int SR_CHUNKS = 16;
constexpr int SR_TILE = SR_THREADS * SR_CHUNKS;

template <class KT>
__device__ __forceinline__ bool is_head(const KT* k, u64 i) {
  return i == 0 || !key_eq(k[i], k[i - 1]);
}

template <class KT, bool WRITE>
__global__ void k_segred(const KT* __restrict__ ik, const double* __restrict__ ia, u64 n, u64* __restrict__ cnt,
                         const u64* __restrict__ off, KT* __restrict__ ok, double* __restrict__ oa) {
  __shared__ u64 sh[SR_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const u64 wb = (u64)blockIdx.x * SR_TILE + (u64)warp * (SR_CHUNKS * 32);
  u64 wc = 0;
  for (int ch = 0; ch < SR_CHUNKS; ++ch) {
    u64 i = wb + (u64)ch * 32 + lane;
    wc += __popc(__ballot_sync(0xffffffffu, i < n && is_head(ik, i)));
  }
  if (lane == 0) sh[warp] = wc;
  __syncthreads();
  if (!WRITE) {
    if (threadIdx.x == 0) {
      u64 t = 0;
      for (int w = 0; w < SR_THREADS / 32; ++w) t += sh[w];
      cnt[blockIdx.x] = t;
    }
    return;
  }
  u64 run = off[blockIdx.x];
  for (int w = 0; w < warp; ++w) run += sh[w];
  for (int ch = 0; ch < SR_CHUNKS; ++ch) {
    u64 i = wb + (u64)ch * 32 + lane;
    bool h = i < n && is_head(ik, i);
    unsigned hb = __ballot_sync(0xffffffffu, h);
    if (h) {
      double s = ia[i];
      for (u64 j = i + 1; j < n && key_eq(ik[j], ik[i]); ++j) s += ia[j];
      u64 p = run + __popc(hb & lt);
      ok[p] = ik[i];
      oa[p] = s;
    }
    run += __popc(hb);
  }
}

template <int W>
static int segreduce(Ctx& c, const typename KeyOf<W>::T* ik, const double* ia, u64 n, typename KeyOf<W>::T* ok,
                     double* oa, u64* m) {
  typedef typename KeyOf<W>::T KT;
  if (n == 0) {
    *m = 0;
    return SFCI_OK;
  }
  u64 nt = (n + SR_TILE - 1) / SR_TILE;
  u64* cnt = (u64*)scratch_get(c, "sr_cnt", (nt + 1) * sizeof(u64));
  if (!cnt) return SFCI_ERR_NOMEM;
  SFCI_LAUNCH(c, (k_segred<KT, false>), (unsigned)nt, SR_THREADS, 0, ik, ia, n, cnt, (const u64*)nullptr,
              (KT*)nullptr, (double*)nullptr);
  int st = scan_excl(c, cnt, cnt, nt);
  if (st) return st;
  SFCI_LAUNCH(c, (k_segred<KT, true>), (unsigned)nt, SR_THREADS, 0, ik, ia, n, (u64*)nullptr, (const u64*)cnt, ok,
              oa);
  return read_words(c, cnt + nt, sizeof(u64), m);
}

template <int W>
static int merge2(Ctx& c, const typename KeyOf<W>::T* A, const double* Aa, u64 na, double alpha, int scaleA,
                  const typename KeyOf<W>::T* B, const double* Ba, u64 nb, double beta, typename KeyOf<W>::T* ok,
                  double* oa) {
  typedef typename KeyOf<W>::T KT;
  u64 n = na + nb;
  if (n == 0) return SFCI_OK;
  u64 threads = (n + MP_ITEMS - 1) / MP_ITEMS;
  unsigned grid = (unsigned)((threads + MP_THREADS - 1) / MP_THREADS);
  SFCI_LAUNCH(c, k_merge<KT>, grid, MP_THREADS, 0, A, Aa, na, alpha, B, Ba, nb, beta, ok, oa, scaleA);
  return SFCI_OK;
}

template <int W>
int dot_impl(Ctx& c, const Vec& x, const Vec& y, double* out) {
  typedef typename KeyOf<W>::T KT;
  if (x.len == 0 || y.len == 0) {
    *out = 0.0;
    return SFCI_OK;
  }
  u64 n = x.len + y.len;
  u64 threads = (n + MP_ITEMS - 1) / MP_ITEMS;
  u64 grid = (threads + MP_THREADS - 1) / MP_THREADS;
  double* part = (double*)scratch_get(c, "dot_part", (grid + 1) * sizeof(double));
  if (!part) return SFCI_ERR_NOMEM;
  SFCI_LAUNCH(c, k_dot<KT>, (unsigned)grid, MP_THREADS, 0, (const KT*)x.keys, x.amps, x.len, (const KT*)y.keys,
              y.amps, y.len, part);
  SFCI_LAUNCH(c, k_sum_serial, 1, 32, 0, (const double*)part, grid, part + grid);
  return read_words(c, part + grid, sizeof(double), out);
}

template <int W>
int add_two_impl(Ctx& c, Vec& v, const Vec& w, double a) {
  typedef typename KeyOf<W>::T KT;
  u64 n = v.len + w.len;
  KT* mk = (KT*)scratch_get(c, "va_mk", (n ? n : 1) * sizeof(KT));
  double* ma = (double*)scratch_get(c, "va_ma", (n ? n : 1) * sizeof(double));
  if (!mk || !ma) return SFCI_ERR_NOMEM;
  int st = merge2<W>(c, (const KT*)v.keys, v.amps, v.len, 1.0, 0, (const KT*)w.keys, w.amps, w.len, a, mk, ma);
  if (st) return st;
  KT* rk = (KT*)scratch_get(c, "va_rk", (n ? n : 1) * sizeof(KT));
  double* ra = (double*)scratch_get(c, "va_ra", (n ? n : 1) * sizeof(double));
  if (!rk || !ra) return SFCI_ERR_NOMEM;
  u64 m = 0;
  if ((st = segreduce<W>(c, mk, ma, n, rk, ra, &m))) return st;
  size_t r = 0;
  if ((st = top_k_stable<W>(c, rk, ra, m, v.cap, -1.0, (KT*)v.keys, v.amps, &r))) return st;
  v.len = r;
  return SFCI_OK;
}

template <int W>
int add_three_impl(Ctx& c, Vec& v, const Vec& x, const Vec& y, const Vec& z, double a, double b, double cc) {
  typedef typename KeyOf<W>::T KT;
  u64 nxy = x.len + y.len, n = nxy + z.len;
  KT* tk = (KT*)scratch_get(c, "va_tk", (nxy ? nxy : 1) * sizeof(KT));
  double* ta = (double*)scratch_get(c, "va_ta", (nxy ? nxy : 1) * sizeof(double));
  KT* mk = (KT*)scratch_get(c, "va_mk", (n ? n : 1) * sizeof(KT));
  double* ma = (double*)scratch_get(c, "va_ma", (n ? n : 1) * sizeof(double));
  if (!tk || !ta || !mk || !ma) return SFCI_ERR_NOMEM;
  int st = merge2<W>(c, (const KT*)x.keys, x.amps, x.len, a, 1, (const KT*)y.keys, y.amps, y.len, b, tk, ta);
  if (st) return st;
  if ((st = merge2<W>(c, tk, ta, nxy, 1.0, 0, (const KT*)z.keys, z.amps, z.len, cc, mk, ma))) return st;
  u64 m = 0;
  // the x/y merge buffer is free again and holds n - z.len <= n entries; reuse
  // the dedicated result buffers instead so the reduction never runs in place
  KT* rk = (KT*)scratch_get(c, "va_rk", (n ? n : 1) * sizeof(KT));
  double* ra = (double*)scratch_get(c, "va_ra", (n ? n : 1) * sizeof(double));
  if (!rk || !ra) return SFCI_ERR_NOMEM;
  if ((st = segreduce<W>(c, mk, ma, n, rk, ra, &m))) return st;
  mk = rk;
  ma = ra;
  // addThree keeps the global Nd largest, then drops |a| <= 1e-14 (src/all.h:589-603)
  size_t r = 0;
  u64 k = std::min<u64>(c.opts.Nd, v.cap);
  if ((st = top_k_stable<W>(c, mk, ma, m, k, 1e-14, (KT*)v.keys, v.amps, &r))) return st;
  v.len = r;
  return SFCI_OK;
}

template <int W>
int shrink_impl(Ctx& c, Vec& dst, const Vec& src) {
  typedef typename KeyOf<W>::T KT;
  size_t r = 0;
  int st = top_k_stable<W>(c, (KT*)src.keys, src.amps, src.len, dst.cap, -1.0, (KT*)dst.keys, dst.amps, &r);
  if (st) return st;
  dst.len = r;
  return SFCI_OK;
}

__global__ void k_scale_copy(const double* __restrict__ a, u64 n, double s, double* __restrict__ o) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) o[i] = s * a[i];
}

template <int W>
int combine_impl(Ctx& c, Vec& dst, const Vec* const* vs, const double* coef, int nv) {
  typedef typename KeyOf<W>::T KT;
  u64 n = 0;
  for (int i = 0; i < nv; ++i) n += vs[i]->len;
  KT* ck = (KT*)scratch_get(c, "cb_k", (n ? n : 1) * sizeof(KT));
  double* ca = (double*)scratch_get(c, "cb_a", (n ? n : 1) * sizeof(double));
  if (!ck || !ca) return SFCI_ERR_NOMEM;
  u64 o = 0;
  for (int i = 0; i < nv; ++i) {
    u64 l = vs[i]->len;
    if (!l) continue;
    SFCI_CUDA(cudaMemcpyAsync(ck + o, vs[i]->keys, l * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
    unsigned grid = (unsigned)std::min<u64>((l + 255) / 256, (u64)c.sm_count * 8);
    SFCI_LAUNCH(c, k_scale_copy, grid, 256, 0, (const double*)vs[i]->amps, l, coef[i], ca + o);
    o += l;
  }
  int st = radix_sort_pairs<W>(c, ck, ca, n, c.N);
  if (st) return st;
  u64 m = 0;
  KT* rk = (KT*)scratch_get(c, "va_rk", (n ? n : 1) * sizeof(KT));
  double* ra = (double*)scratch_get(c, "va_ra", (n ? n : 1) * sizeof(double));
  if (!rk || !ra) return SFCI_ERR_NOMEM;
  if ((st = segreduce<W>(c, ck, ca, n, rk, ra, &m))) return st;
  if (m > dst.cap) return set_error(SFCI_ERR_CAPACITY, "combine: destination capacity too small");
  SFCI_CUDA(cudaMemcpyAsync(dst.keys, rk, m * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
  SFCI_CUDA(cudaMemcpyAsync(dst.amps, ra, m * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  dst.len = m;
  return SFCI_OK;
}

template <class KT>
__global__ void k_unsorted(const KT* __restrict__ k, u64 n, unsigned* __restrict__ flag) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += (u64)gridDim.x * blockDim.x)
    if (key_lt(k[i], k[i - 1])) {
      *flag = 1;
      return;
    }
}

template <int W>
int sort_vec_impl(Ctx& c, Vec& v) {
  typedef typename KeyOf<W>::T KT;
  if (v.len < 2) return SFCI_OK;
  unsigned* flag = (unsigned*)scratch_get(c, "sv_flag", sizeof(unsigned));
  if (!flag) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned), c.stream));
  unsigned grid = (unsigned)std::min<u64>((v.len + 255) / 256, (u64)c.sm_count * 8);
  SFCI_LAUNCH(c, k_unsorted<KT>, grid, 256, 0, (const KT*)v.keys, v.len, flag);
  unsigned h = 0;
  int st = read_words(c, flag, sizeof(unsigned), &h);
  if (st) return st;
  if (!h) return SFCI_OK;
  return radix_sort_pairs<W>(c, (KT*)v.keys, v.amps, v.len, c.N);
}

__global__ void k_scale(double* __restrict__ a, u64 n, double s) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) a[i] *= s;
}

int scale_impl(Ctx& c, Vec& v, double s) {
  if (!v.len) return SFCI_OK;
  unsigned grid = (unsigned)std::min<u64>((v.len + 255) / 256, (u64)c.sm_count * 8);
  SFCI_LAUNCH(c, k_scale, grid, 256, 0, v.amps, v.len, s);
  return SFCI_OK;
}

int norm_impl(Ctx& c, const Vec& v, double* out) {
  double s = 0.0;
  if (v.len) {
    int st = reduce_sum_sq(c, v.amps, v.len, &s);
    if (st) return st;
  }
  *out = std::sqrt(s);
  return SFCI_OK;
}

template int dot_impl<1>(Ctx&, const Vec&, const Vec&, double*);
template int dot_impl<2>(Ctx&, const Vec&, const Vec&, double*);
template int add_two_impl<1>(Ctx&, Vec&, const Vec&, double);
template int add_two_impl<2>(Ctx&, Vec&, const Vec&, double);
template int add_three_impl<1>(Ctx&, Vec&, const Vec&, const Vec&, const Vec&, double, double, double);
template int add_three_impl<2>(Ctx&, Vec&, const Vec&, const Vec&, const Vec&, double, double, double);
template int shrink_impl<1>(Ctx&, Vec&, const Vec&);
template int shrink_impl<2>(Ctx&, Vec&, const Vec&);
template int combine_impl<1>(Ctx&, Vec&, const Vec* const*, const double*, int);
template int combine_impl<2>(Ctx&, Vec&, const Vec* const*, const double*, int);
template int sort_vec_impl<1>(Ctx&, Vec&);
template int sort_vec_impl<2>(Ctx&, Vec&);

}  // namespace sfci

namespace sfci {

// first position of each instance tag t = 0..n in a key-sorted two-word vector
// (the tag is the top INST_BITS of the high word, so the vector is sorted by it)
__global__ void k_inst_bounds(const K128* __restrict__ keys, u64 len, int n, u64* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t > n) return;
  const u64 hi_t = (u64)t << INST_SHIFT;
  u64 lo = 0, hi = len;  // first key with hi word >= hi_t
  while (lo < hi) {
    const u64 mid = (lo + hi) >> 1;
    if (keys[mid].hi < hi_t) lo = mid + 1; else hi = mid;
  }
  out[t] = t == n ? len : lo;
}

int inst_bounds(Ctx& c, const Vec& v, int n, u64* out_host) {
  if (c.W != 2) return set_error(SFCI_ERR_ARG, "instance bounds need two-word keys");
  u64* d = (u64*)scratch_get(c, "ib_out", (n + 1) * sizeof(u64));
  if (!d) return SFCI_ERR_NOMEM;
  SFCI_LAUNCH(c, k_inst_bounds, 1, 64, 0, (const K128*)v.keys, (u64)v.len, n, d);
  return read_words(c, d, (n + 1) * sizeof(u64), out_host);
}

}  // namespace sfci

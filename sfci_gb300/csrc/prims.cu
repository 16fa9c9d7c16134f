// Device primitives (see prims.cuh).
#include <algorithm>
#include <cstring>

#include "prims.cuh"

namespace sfci {

// ============================================================================
// exclusive scan (reduce-then-scan, recursive over block sums)
// ============================================================================

template <typename T>
__global__ void k_scan_reduce(const T* __restrict__ in, size_t n, T* __restrict__ bsum) {
  __shared__ T sh[SCAN_THREADS / 32 + 1];
  size_t base = (size_t)blockIdx.x * SCAN_TILE;
  T s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    size_t idx = base + (size_t)i * SCAN_THREADS + threadIdx.x;
    if (idx < n) s += __ldcg(in + idx);  // counts may come from atomics of the previous kernel
  }
  T tot;
  block_excl_scan<T, SCAN_THREADS>(s, &tot, sh);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

template <typename T>
__global__ void k_scan_down(const T* in, T* out, size_t n, const T* __restrict__ boff) {
  __shared__ T sh[SCAN_THREADS / 32 + 1];
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  T v[SCAN_ITEMS];
  T s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = (base + i < n) ? __ldcg(in + base + i) : T(0);
    s += v[i];
  }
  T off = block_excl_scan<T, SCAN_THREADS>(s, nullptr, sh) + (boff ? boff[blockIdx.x] : T(0));
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) out[base + i] = off;
    off += v[i];
  }
  if (n > 0 && base <= n - 1 && n - 1 < base + SCAN_ITEMS) out[n] = off;
}

template <typename T>
static int scan_impl(Ctx& c, const T* in, T* out, size_t n, int depth) {
  if (n == 0) {
    SFCI_CUDA(cudaMemsetAsync(out, 0, sizeof(T), c.stream));
    return SFCI_OK;
  }
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 1) {
    SFCI_LAUNCH(c, k_scan_down<T>, 1, SCAN_THREADS, 0, in, out, n, (const T*)nullptr);
    return SFCI_OK;
  }
  char name[32];
  snprintf(name, sizeof name, "scan_%d_%d", (int)sizeof(T), depth);
  T* bs = (T*)scratch_get(c, name, (nb + 1) * sizeof(T));
  if (!bs) return SFCI_ERR_NOMEM;
  SFCI_LAUNCH(c, k_scan_reduce<T>, (unsigned)nb, SCAN_THREADS, 0, in, n, bs);
  int st = scan_impl<T>(c, bs, bs, nb, depth + 1);
  if (st) return st;
  SFCI_LAUNCH(c, k_scan_down<T>, (unsigned)nb, SCAN_THREADS, 0, in, out, n, (const T*)bs);
  return SFCI_OK;
}

int scan_excl(Ctx& c, const u64* in, u64* out, size_t n) { return scan_impl<u64>(c, in, out, n, 0); }
int scan_excl_u32(Ctx& c, const uint32_t* in, uint32_t* out, size_t n) {
  return scan_impl<uint32_t>(c, in, out, n, 0);
}

// ============================================================================
// LSD radix sort, 8-bit digits, 4096-item tiles, stable warp-ordered ranking
// ============================================================================

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_CHUNKS = 16;
constexpr int RS_TILE = RS_THREADS * RS_CHUNKS;  // 4096

template <class KT>
__global__ void k_rs_hist(const KT* __restrict__ keys, size_t n, int shift, uint32_t* __restrict__ counts,
                          size_t ntiles) {
  __shared__ uint32_t hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * RS_TILE;
#pragma unroll 4
  for (int i = 0; i < RS_CHUNKS; ++i) {
    size_t idx = base + (size_t)i * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&hist[key_digit(keys[idx], shift)], 1u);
  }
  __syncthreads();
  counts[(size_t)threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

template <class KT>
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const KT* __restrict__ kin, const double* __restrict__ vin,
                                                          KT* __restrict__ kout, double* __restrict__ vout, size_t n,
                                                          int shift, const uint32_t* __restrict__ offs, size_t ntiles) {
  __shared__ uint32_t whist[RS_WARPS][256];
  __shared__ uint32_t base[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < RS_WARPS * 256; d += RS_THREADS) (&whist[0][0])[d] = 0;
  base[threadIdx.x] = offs[(size_t)threadIdx.x * ntiles + blockIdx.x];
  __syncthreads();
  const size_t wbase = (size_t)blockIdx.x * RS_TILE + (size_t)warp * (RS_CHUNKS * 32);
  KT k[RS_CHUNKS];
  double v[RS_CHUNKS];
  int dg[RS_CHUNKS];
#pragma unroll
  for (int c = 0; c < RS_CHUNKS; ++c) {
    size_t idx = wbase + (size_t)c * 32 + lane;
    bool valid = idx < n;
    if (valid) {
      k[c] = kin[idx];
      v[c] = vin[idx];
      dg[c] = (int)key_digit(k[c], shift);
    } else {
      dg[c] = 256 + lane;
    }
    unsigned peers = __match_any_sync(0xffffffffu, dg[c]);
    if (valid && lane == __ffs(peers) - 1) whist[warp][dg[c]] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      uint32_t t = whist[w][d];
      whist[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int c = 0; c < RS_CHUNKS; ++c) {
    size_t idx = wbase + (size_t)c * 32 + lane;
    bool valid = idx < n;
    unsigned peers = __match_any_sync(0xffffffffu, dg[c]);
    if (valid) {
      uint32_t pos = base[dg[c]] + whist[warp][dg[c]] + __popc(peers & lt);
      kout[pos] = k[c];
      vout[pos] = v[c];
    }
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) whist[warp][dg[c]] += __popc(peers);
    __syncwarp();
  }
}

template <int W>
int radix_sort_pairs(Ctx& c, typename KeyOf<W>::T* keys, double* vals, size_t n, int nbits) {
  typedef typename KeyOf<W>::T KT;
  if (n <= 1 || nbits <= 0) return SFCI_OK;
  if (n >= (1ull << 32)) return set_error(SFCI_ERR_UNSUPPORTED, "radix sort beyond 2^32 items");
  size_t ntiles = (n + RS_TILE - 1) / RS_TILE;
  KT* k2 = (KT*)scratch_get(c, "rs_keys", n * sizeof(KT));
  double* v2 = (double*)scratch_get(c, "rs_vals", n * sizeof(double));
  uint32_t* cnt = (uint32_t*)scratch_get(c, "rs_cnt", (256 * ntiles + 1) * sizeof(uint32_t));
  if (!k2 || !v2 || !cnt) return SFCI_ERR_NOMEM;
  KT* ka = keys;
  double* va = vals;
  KT* kb = k2;
  double* vb = v2;
  int passes = (nbits + 7) / 8;
  for (int p = 0; p < passes; ++p) {
    int shift = 8 * p;
    SFCI_LAUNCH(c, k_rs_hist<KT>, (unsigned)ntiles, RS_THREADS, 0, ka, n, shift, cnt, ntiles);
    int st = scan_excl_u32(c, cnt, cnt, 256 * ntiles);
    if (st) return st;
    SFCI_LAUNCH(c, k_rs_scatter<KT>, (unsigned)ntiles, RS_THREADS, 0, ka, va, kb, vb, n, shift,
                (const uint32_t*)cnt, ntiles);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    SFCI_CUDA(cudaMemcpyAsync(keys, ka, n * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
    SFCI_CUDA(cudaMemcpyAsync(vals, va, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  }
  return SFCI_OK;
}

template int radix_sort_pairs<1>(Ctx&, u64*, double*, size_t, int);
template int radix_sort_pairs<2>(Ctx&, K128*, double*, size_t, int);

// ============================================================================
// radix select on |amp|
// ============================================================================

__global__ void k_sel_hist(const double* __restrict__ a, size_t n, int shift, int width, u64 prefix,
                           int pshift, uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[4096];
  const int nb = 1 << width;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const u64 mask = (u64)nb - 1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    u64 b = abs_bits(a[i]);
    if (pshift >= 64 || (b >> pshift) == prefix) atomicAdd(&sh[(b >> shift) & mask], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

int select_threshold(Ctx& c, const double* amps, size_t n, size_t k, u64* tau, size_t* gt) {
  if (k == 0 || k >= n) return set_error(SFCI_ERR_ARG, "select_threshold needs 0 < k < n");
  uint32_t* hist = (uint32_t*)scratch_get(c, "sel_hist", 4096 * sizeof(uint32_t));
  if (!hist) return SFCI_ERR_NOMEM;
  std::vector<uint32_t> h(4096);
  // 63 magnitude bits: five 12-bit digits (bits 62..3) then the last 3 bits
  const int shifts[6] = {51, 39, 27, 15, 3, 0};
  const int widths[6] = {12, 12, 12, 12, 12, 3};
  u64 prefix = 0;
  size_t need = k;  // how many still to take from items matching prefix
  size_t above = 0;
  unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)c.sm_count * 8);
  if (grid == 0) grid = 1;
  for (int r = 0; r < 6; ++r) {
    int nb = 1 << widths[r];
    SFCI_CUDA(cudaMemsetAsync(hist, 0, nb * sizeof(uint32_t), c.stream));
    int pshift = shifts[r] + widths[r];
    SFCI_LAUNCH(c, k_sel_hist, grid, 256, 0, amps, n, shifts[r], widths[r], prefix, r == 0 ? 64 : pshift, hist);
    int st = read_words(c, hist, nb * sizeof(uint32_t), h.data());
    if (st) return st;
    size_t acc = 0;
    int b = nb - 1;
    for (; b >= 0; --b) {
      if (acc + h[b] >= need) break;
      acc += h[b];
    }
    if (b < 0) return set_error(SFCI_ERR_NUMERIC, "radix select lost items (NaN amplitudes?)");
    above += acc;
    need -= acc;
    prefix = (prefix << widths[r]) | (u64)b;
  }
  *tau = prefix;
  *gt = above;
  return SFCI_OK;
}

// ============================================================================
// stable compaction (warp-ballot ranking over 4096-item tiles)
// ============================================================================

constexpr int CP_THREADS = 256;
constexpr int CP_CHUNKS = 16;
constexpr int CP_TILE = CP_THREADS * CP_CHUNKS;

// mode 0: keep |a| > cut
// mode 1: keep |a| > tau or (|a| == tau and eq-rank >= eq_skip), then |a| > tiny if tiny >= 0.
// Ties at the threshold are kept from the end of the index order (the largest keys
// of a key-sorted vector), as a stable ascending sort by |a| followed by "keep the
// last k" does.
// The magnitude tests compare the bits of |a| as integers (cut_key: -1 keeps
// everything), which orders finite doubles as their values do and keeps these
// passes off the FP64 pipe.
struct KeepRule {
  int mode;
  u64 tau;
  u64 eq_skip;
  long long cut_key;   // mode 0: keep |a| > cut
  long long tiny_key;  // mode 1: then |a| > tiny (-1: no such filter)
};

__device__ __forceinline__ bool keep_of(const KeepRule& r, double a, u64 eq_rank, bool& is_eq) {
  u64 b = abs_bits(a);
  if (r.mode == 0) {
    is_eq = false;
    return (long long)b > r.cut_key;
  }
  is_eq = (b == r.tau);
  bool k = b > r.tau || (is_eq && eq_rank >= r.eq_skip);
  return k && (long long)b > r.tiny_key;
}

// stage 0: per-tile count of |a| == tau
__global__ void k_cp_eqcount(const double* __restrict__ a, size_t n, u64 tau, u64* __restrict__ eqc) {
  __shared__ u64 sh[CP_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  size_t wb = (size_t)blockIdx.x * CP_TILE + (size_t)warp * (CP_CHUNKS * 32);
  u64 cnt = 0;
  for (int ch = 0; ch < CP_CHUNKS; ++ch) {
    size_t i = wb + (size_t)ch * 32 + lane;
    bool e = i < n && abs_bits(a[i]) == tau;
    cnt += __popc(__ballot_sync(0xffffffffu, e));
  }
  if (lane == 0) sh[warp] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    u64 t = 0;
    for (int w = 0; w < CP_THREADS / 32; ++w) t += sh[w];
    eqc[blockIdx.x] = t;
  }
}

// stage 1 (write=false): per-tile keep counts; stage 2 (write=true): scatter
template <class KT, bool WRITE>
__global__ void k_cp_pass(const KT* __restrict__ ik, const double* __restrict__ ia, size_t n, KeepRule rule,
                          const u64* __restrict__ eqoff, u64* __restrict__ keepc, const u64* __restrict__ keepoff,
                          KT* __restrict__ ok, double* __restrict__ oa) {
  __shared__ u64 sh_eq[CP_THREADS / 32], sh_kp[CP_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  size_t wb = (size_t)blockIdx.x * CP_TILE + (size_t)warp * (CP_CHUNKS * 32);
  // warp-level eq counts (for eq rank) and keep counts
  u64 weq = 0, wkp = 0;
  if (rule.mode == 1) {
    for (int ch = 0; ch < CP_CHUNKS; ++ch) {
      size_t i = wb + (size_t)ch * 32 + lane;
      bool e = i < n && abs_bits(ia[i]) == rule.tau;
      weq += __popc(__ballot_sync(0xffffffffu, e));
    }
  }
  if (lane == 0) sh_eq[warp] = weq;
  __syncthreads();
  u64 eq_run = rule.mode == 1 ? eqoff[blockIdx.x] : 0;
  for (int w = 0; w < warp; ++w) eq_run += sh_eq[w];
  u64 kp_run = 0;
  if (WRITE) {
    // need the keep offsets of earlier warps: recompute counts first
    u64 e2 = eq_run;
    for (int ch = 0; ch < CP_CHUNKS; ++ch) {
      size_t i = wb + (size_t)ch * 32 + lane;
      bool valid = i < n;
      double a = valid ? ia[i] : 0.0;
      bool ise = false;
      unsigned eb = __ballot_sync(0xffffffffu, valid && rule.mode == 1 && abs_bits(a) == rule.tau);
      bool k = valid && keep_of(rule, a, e2 + __popc(eb & lt), ise);
      e2 += __popc(eb);
      wkp += __popc(__ballot_sync(0xffffffffu, k));
    }
    if (lane == 0) sh_kp[warp] = wkp;
    __syncthreads();
    kp_run = keepoff[blockIdx.x];
    for (int w = 0; w < warp; ++w) kp_run += sh_kp[w];
  }
  u64 e2 = eq_run;
  u64 cnt = 0;
  for (int ch = 0; ch < CP_CHUNKS; ++ch) {
    size_t i = wb + (size_t)ch * 32 + lane;
    bool valid = i < n;
    double a = valid ? ia[i] : 0.0;
    bool ise = false;
    unsigned eb = __ballot_sync(0xffffffffu, valid && rule.mode == 1 && abs_bits(a) == rule.tau);
    bool k = valid && keep_of(rule, a, e2 + __popc(eb & lt), ise);
    e2 += __popc(eb);
    unsigned kb = __ballot_sync(0xffffffffu, k);
    if (WRITE) {
      if (k) {
        u64 pos = kp_run + __popc(kb & lt);
        ok[pos] = ik[i];
        oa[pos] = a;
      }
      kp_run += __popc(kb);
    } else {
      cnt += __popc(kb);
    }
  }
  if (!WRITE) {
    if (lane == 0) sh_kp[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      u64 t = 0;
      for (int w = 0; w < CP_THREADS / 32; ++w) t += sh_kp[w];
      keepc[blockIdx.x] = t;
    }
  }
}

template <int W>
static int compact_rule(Ctx& c, const typename KeyOf<W>::T* ik, const double* ia, size_t n, KeepRule rule,
                        typename KeyOf<W>::T* ok, double* oa, size_t* m) {
  typedef typename KeyOf<W>::T KT;
  if (n == 0) {
    *m = 0;
    return SFCI_OK;
  }
  size_t nt = (n + CP_TILE - 1) / CP_TILE;
  u64* eqo = (u64*)scratch_get(c, "cp_eq", (nt + 1) * sizeof(u64));
  u64* kpo = (u64*)scratch_get(c, "cp_kp", (nt + 1) * sizeof(u64));
  if (!eqo || !kpo) return SFCI_ERR_NOMEM;
  int st;
  if (rule.mode == 1) {
    SFCI_LAUNCH(c, k_cp_eqcount, (unsigned)nt, CP_THREADS, 0, ia, n, rule.tau, eqo);
    if ((st = scan_excl(c, eqo, eqo, nt))) return st;
    // eq_skip arrives as the number of ties to keep; turn it into ties to skip
    u64 tot_eq = 0;
    if ((st = read_words(c, eqo + nt, sizeof(u64), &tot_eq))) return st;
    rule.eq_skip = rule.eq_skip >= tot_eq ? 0 : tot_eq - rule.eq_skip;
  }
  SFCI_LAUNCH(c, (k_cp_pass<KT, false>), (unsigned)nt, CP_THREADS, 0, ik, ia, n, rule, (const u64*)eqo, kpo,
              (const u64*)nullptr, (KT*)nullptr, (double*)nullptr);
  if ((st = scan_excl(c, kpo, kpo, nt))) return st;
  SFCI_LAUNCH(c, (k_cp_pass<KT, true>), (unsigned)nt, CP_THREADS, 0, ik, ia, n, rule, (const u64*)eqo,
              (u64*)nullptr, (const u64*)kpo, ok, oa);
  u64 tot = 0;
  if ((st = read_words(c, kpo + nt, sizeof(u64), &tot))) return st;
  *m = (size_t)tot;
  return SFCI_OK;
}

template <int W>
int compact_top(Ctx& c, const typename KeyOf<W>::T* ik, const double* ia, size_t n, u64 tau, size_t need_eq,
                double tiny, typename KeyOf<W>::T* ok, double* oa, size_t* m) {
  KeepRule r{1, tau, (u64)need_eq, -1ll, cut_key(tiny)};
  return compact_rule<W>(c, ik, ia, n, r, ok, oa, m);
}

template <int W>
int compact_cut(Ctx& c, const typename KeyOf<W>::T* ik, const double* ia, size_t n, double cut,
                typename KeyOf<W>::T* ok, double* oa, size_t* m) {
  KeepRule r{0, 0, 0, cut_key(cut), -1ll};
  return compact_rule<W>(c, ik, ia, n, r, ok, oa, m);
}

template <int W>
int top_k_stable(Ctx& c, typename KeyOf<W>::T* ik, double* ia, size_t n, size_t k, double tiny,
                 typename KeyOf<W>::T* ok, double* oa, size_t* m) {
  typedef typename KeyOf<W>::T KT;
  if (n <= k) {
    if (tiny >= 0.0) {
      // filter only: keep |a| > tiny (all of them pass the selection)
      // tau = 0 keeping all n ties keeps everything before the tiny filter
      KeepRule r{1, 0ull, (u64)n, -1ll, cut_key(tiny)};
      return compact_rule<W>(c, ik, ia, n, r, ok, oa, m);
    }
    if (ok != ik) {
      SFCI_CUDA(cudaMemcpyAsync(ok, ik, n * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
      SFCI_CUDA(cudaMemcpyAsync(oa, ia, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    }
    *m = n;
    return SFCI_OK;
  }
  u64 tau;
  size_t gt;
  int st = select_threshold(c, ia, n, k, &tau, &gt);
  if (st) return st;
  size_t need_eq = k - gt;
  if (ok == ik) {
    // compaction may not run in place across tiles; stage through scratch
    KT* tk = (KT*)scratch_get(c, "topk_k", n * sizeof(KT));
    double* ta = (double*)scratch_get(c, "topk_a", n * sizeof(double));
    if (!tk || !ta) return SFCI_ERR_NOMEM;
    if ((st = compact_top<W>(c, ik, ia, n, tau, need_eq, tiny, tk, ta, m))) return st;
    SFCI_CUDA(cudaMemcpyAsync(ok, tk, *m * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
    SFCI_CUDA(cudaMemcpyAsync(oa, ta, *m * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    return SFCI_OK;
  }
  return compact_top<W>(c, ik, ia, n, tau, need_eq, tiny, ok, oa, m);
}

template <int W>
int select_sorted(Ctx& c, typename KeyOf<W>::T* keys, double* vals, size_t n, size_t k, size_t* m) {
  typedef typename KeyOf<W>::T KT;
  int st = radix_sort_pairs<W>(c, keys, vals, n, c.N);
  if (st) return st;
  if (n <= k) {
    *m = n;
    return SFCI_OK;
  }
  KT* tk = (KT*)scratch_get(c, "rs_keys", n * sizeof(KT));
  double* ta = (double*)scratch_get(c, "rs_vals", n * sizeof(double));
  if (!tk || !ta) return SFCI_ERR_NOMEM;
  if ((st = top_k_stable<W>(c, keys, vals, n, k, -1.0, tk, ta, m))) return st;
  SFCI_CUDA(cudaMemcpyAsync(keys, tk, *m * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
  SFCI_CUDA(cudaMemcpyAsync(vals, ta, *m * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  return SFCI_OK;
}

template int select_sorted<1>(Ctx&, u64*, double*, size_t, size_t, size_t*);
template int select_sorted<2>(Ctx&, K128*, double*, size_t, size_t, size_t*);
template int compact_top<1>(Ctx&, const u64*, const double*, size_t, u64, size_t, double, u64*, double*, size_t*);
template int compact_top<2>(Ctx&, const K128*, const double*, size_t, u64, size_t, double, K128*, double*,
                            size_t*);
template int compact_cut<1>(Ctx&, const u64*, const double*, size_t, double, u64*, double*, size_t*);
template int compact_cut<2>(Ctx&, const K128*, const double*, size_t, double, K128*, double*, size_t*);
template int top_k_stable<1>(Ctx&, u64*, double*, size_t, size_t, double, u64*, double*, size_t*);
template int top_k_stable<2>(Ctx&, K128*, double*, size_t, size_t, double, K128*, double*, size_t*);

// ============================================================================
// deterministic sum of squares
// ============================================================================

constexpr int RED_BLOCKS = 512;

__global__ void k_sumsq_part(const double* __restrict__ a, size_t n, double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += a[i] * a[i];
  double t = block_sum<256>(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_sum_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < np; ++i) s += __ldcg(part + i);
    *out = s;
  }
}

int reduce_sum_sq(Ctx& c, const double* a, size_t n, double* out) {
  double* part = (double*)scratch_get(c, "red_part", (RED_BLOCKS + 1) * sizeof(double));
  if (!part) return SFCI_ERR_NOMEM;
  SFCI_LAUNCH(c, k_sumsq_part, RED_BLOCKS, 256, 0, a, n, part);
  SFCI_LAUNCH(c, k_sum_final, 1, 32, 0, (const double*)part, RED_BLOCKS, part + RED_BLOCKS);
  return read_words(c, part + RED_BLOCKS, sizeof(double), out);
}

}  // namespace sfci

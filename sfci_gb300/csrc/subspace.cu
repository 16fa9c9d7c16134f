// Hamiltonian on a determinant subspace, for the reference's two dense
// diagonalisation utilities:
//   * calc_CISD (src/sparse_solver.cpp:15-114): the block spanned by a
//     reference determinant and every determinant it connects to (its singles
//     and doubles), diagonalised with Eigen's SelfAdjointEigenSolver; the
//     result is eigenvector `state_idx` over the block, sorted by key (:113);
//   * fci (src/dense_algo.cpp:77-124) over generateBasis / comb_det (:14-74):
//     every determinant with as many alpha as beta electrons; it reports the
//     ground-state energy.
// Neither block is formed densely here.  Its off-diagonal elements come from the
// per-determinant enumeration of the SpMSpV (gen.cuh) and are stored once as a
// CSR matrix in HBM: row i holds, in term order, (k, <basis_k|H|basis_i>) for
// every generated target basis_k inside the block (a key -> index hash table
// answers membership), and the diagonal is kept beside it.  Lanczos with full
// reorthogonalisation (two classical Gram-Schmidt passes against all previous
// vectors, dense device vectors of the block's length) converges the lowest
// eigenpairs; the tridiagonal eigenproblem is solved on the host by Sturm
// bisection and inverse iteration.  Eigenvector signs are fixed so that the
// component of largest magnitude is positive (Eigen's sign is arbitrary).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gen.cuh"
#include "prims.cuh"
#include "spmspv.h"
#include "hostla.h"
#include "table.cuh"

namespace sfci {

constexpr int SS_THREADS = 256;  // row kernels: one CTA per basis determinant
constexpr int VD_THREADS = 256;  // dense vector kernels
constexpr int VD_EPT = 8;        // elements per thread of a dot chunk
constexpr int VD_CHUNK = VD_THREADS * VD_EPT;
constexpr int VD_JB = 16;        // vectors per CTA of a block dot
constexpr int LZ_MAX = 1000;     // Lanczos vectors at most

SFCI_HD size_t ss_al16(size_t x) { return (x + 15) & ~(size_t)15; }

template <class KT>
SFCI_HD size_t row_smem_bytes() {
  return ss_al16(sizeof(DetInfo<KT>)) + ss_al16(2016 * sizeof(unsigned short));
}

// ---------------------------------------------------------------------------
// bases
// ---------------------------------------------------------------------------
// every term target of one determinant; term 0 is the determinant itself
template <class KT>
__global__ void __launch_bounds__(SS_THREADS) k_targets(KT key, HamView h, u64 T, KT* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  DetInfo<KT>& d = *reinterpret_cast<DetInfo<KT>*>(smem);
  unsigned short* pt = reinterpret_cast<unsigned short*>(smem + ss_al16(sizeof(DetInfo<KT>)));
  fill_pair_table(pt);
  if (threadIdx.x < 32) det_setup_warp(d, key, 1.0, 0.0, 0.0, h.M);
  __syncthreads();
  det_fill_singles(d, threadIdx.x, SS_THREADS);
  __syncthreads();
  const DetHead<KT> dh = d.h;
  for (u64 l = (u64)blockIdx.x * SS_THREADS + threadIdx.x; l < T; l += (u64)gridDim.x * SS_THREADS)
    out[l] = target_key(dh, d, decode(dh, pt, (unsigned)l));
}

// r-subset of {0 .. M-1} with colex rank `rank`: for j = r .. 1 the largest c
// with C(c, j) <= rank (binom[n * (M + 1) + k] = C(n, k))
SFCI_HD u64 unrank_colex(u64 rank, int M, int r, const u64* binom) {
  u64 bits = 0;
  int c = M - 1;
  for (int j = r; j >= 1; --j) {
    while (binom[(size_t)c * (M + 1) + j] > rank) --c;
    bits |= 1ull << c;
    rank -= binom[(size_t)c * (M + 1) + j];
    --c;
  }
  return bits;
}

// determinant r of the (alpha rank, beta rank) enumeration of the space with na
// alpha and nb beta electrons in M spatial orbitals (spin orbital 2o + s)
template <class KT>
__global__ void k_fci_keys(const u64* __restrict__ binom, int M, int na, int nb, u64 nbeta, u64 n,
                           KT* __restrict__ out) {
  for (u64 r = (u64)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (u64)gridDim.x * blockDim.x) {
    const u64 ra = r / nbeta, rb = r - ra * nbeta;
    const u64 a = unrank_colex(ra, M, na, binom), b = unrank_colex(rb, M, nb, binom);
    KT k = key_zero<KT>();
    for (int o = 0; o < M; ++o) {
      if ((a >> o) & 1ull) key_flip(k, 2 * o);
      if ((b >> o) & 1ull) key_flip(k, 2 * o + 1);
    }
    out[r] = k;
  }
}

// ---------------------------------------------------------------------------
// key -> basis index table
// ---------------------------------------------------------------------------
template <class KT>
__global__ void k_index_clear(KT* tk, u64 n) {
  const KT empty = key_empty<KT>();
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) tk[i] = empty;
}

// the table has at least twice as many slots as keys, so a probe sequence
// always meets a free slot
template <class KT>
__global__ void k_index_build(const KT* __restrict__ keys, u64 n, KT* tk, uint32_t* tv, unsigned mask) {
  const KT empty = key_empty<KT>();
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    unsigned slot = (unsigned)slot_hash(keys[i]) & mask;
    for (unsigned probe = 0; probe <= mask; ++probe) {
      const KT prev = cas_key(&tk[slot], empty, keys[i]);
      if (key_eq(prev, empty) || key_eq(prev, keys[i])) {
        tv[slot] = (uint32_t)i;
        break;
      }
      slot = (slot + 1) & mask;
    }
  }
}

// ---------------------------------------------------------------------------
// CSR rows of the block
// ---------------------------------------------------------------------------
// FILL = false: diagonal element and number of in-block targets of each row;
// FILL = true: the row's (column, element) pairs in term order.
template <class KT, bool FILL>
__global__ void __launch_bounds__(SS_THREADS) k_rows(const KT* __restrict__ basis, u64 n, HamView h, const KT* tk,
                                                    const uint32_t* tv, unsigned mask, u64* __restrict__ rowcnt,
                                                    const u64* __restrict__ rowptr, uint32_t* __restrict__ col,
                                                    double* __restrict__ val, double* __restrict__ diag) {
  extern __shared__ __align__(16) unsigned char smem[];
  DetInfo<KT>& d = *reinterpret_cast<DetInfo<KT>*>(smem);
  unsigned short* pt = reinterpret_cast<unsigned short*>(smem + ss_al16(sizeof(DetInfo<KT>)));
  __shared__ uint32_t s_scan[SS_THREADS / 32 + 1];
  const int tid = threadIdx.x, lane = tid & 31;
  fill_pair_table(pt);
  for (u64 row = blockIdx.x; row < n; row += gridDim.x) {
    const KT key = basis[row];
    if (tid < 32) {
      det_setup_warp(d, key, 1.0, 0.0, 0.0, h.M);
      if (!FILL) {
        const double D = diag_element_warp(key, h);
        if (lane == 0) diag[row] = D;
      }
    }
    __syncthreads();
    det_fill_singles(d, tid, SS_THREADS);
    __syncthreads();
    const DetHead<KT> dh = d.h;
    const unsigned T = dh.c[5];
    if (!FILL) {
      uint32_t cnt = 0;
      for (unsigned l = 1 + tid; l < T; l += SS_THREADS)
        cnt += table_find_global(tk, mask, target_key(dh, d, decode(dh, pt, l))) >= 0 ? 1u : 0u;
      uint32_t tot;
      block_excl_scan<uint32_t, SS_THREADS>(cnt, &tot, s_scan);
      if (tid == 0) rowcnt[row] = tot;
    } else {
      u64 base = rowptr[row];
      for (unsigned l0 = 1; l0 < T; l0 += SS_THREADS) {
        const unsigned l = l0 + tid;
        Exc e{};
        int slot = -1;
        if (l < T) {
          e = decode(dh, pt, l);
          slot = table_find_global(tk, mask, target_key(dh, d, e));
        }
        uint32_t tot;
        const uint32_t ex = block_excl_scan<uint32_t, SS_THREADS>(slot >= 0 ? 1u : 0u, &tot, s_scan);
        if (slot >= 0) {
          col[base + ex] = __ldcg(tv + slot);
          val[base + ex] = term_amp(dh, d, e, h);
        }
        base += tot;
      }
    }
    __syncthreads();
  }
}

// y = H x on the block: one warp per row, lanes striding the row's entries with
// four independent accumulators (four index loads, gathers and FMAs in flight
// per lane instead of one dependent chain), combined in a fixed order
__global__ void k_csr_spmv(const u64* __restrict__ rowptr, const uint32_t* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ diag,
                           const double* __restrict__ x, double* __restrict__ y, u64 n) {
  const int lane = threadIdx.x & 31;
  const u64 nw = ((u64)gridDim.x * blockDim.x) >> 5;
  for (u64 w = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += nw) {
    const u64 b = rowptr[w], e = rowptr[w + 1];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    u64 p = b + lane;
    for (; p + 96 < e; p += 128) {
      const uint32_t c0 = col[p], c1 = col[p + 32], c2 = col[p + 64], c3 = col[p + 96];
      const double v0 = val[p], v1 = val[p + 32], v2 = val[p + 64], v3 = val[p + 96];
      s0 = fma(v0, x[c0], s0);
      s1 = fma(v1, x[c1], s1);
      s2 = fma(v2, x[c2], s2);
      s3 = fma(v3, x[c3], s3);
    }
    for (; p < e; p += 32) s0 = fma(val[p], x[col[p]], s0);
    const double s = warp_sum((s0 + s1) + (s2 + s3));
    if (lane == 0) y[w] = fma(diag[w], x[w], s);
  }
}

// ---------------------------------------------------------------------------
// dense vectors (block length n, vector j at V + j * ld)
// ---------------------------------------------------------------------------
// part[j * gridDim.x + b] = sum over chunk b of V_j . w, for j in this CTA's group
__global__ void __launch_bounds__(VD_THREADS) k_vdot_part(const double* __restrict__ V, u64 ld, int nv,
                                                         const double* __restrict__ w, u64 n,
                                                         double* __restrict__ part) {
  __shared__ double s_red[VD_THREADS / 32];
  const u64 i0 = (u64)blockIdx.x * VD_CHUNK + threadIdx.x;
  double wr[VD_EPT];
#pragma unroll
  for (int t = 0; t < VD_EPT; ++t) {
    const u64 i = i0 + (u64)t * VD_THREADS;
    wr[t] = i < n ? w[i] : 0.0;
  }
  const int j0 = blockIdx.y * VD_JB, j1 = min(nv, j0 + VD_JB);
  for (int j = j0; j < j1; ++j) {
    const double* vj = V + (u64)j * ld;
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < VD_EPT; ++t) {
      const u64 i = i0 + (u64)t * VD_THREADS;
      if (i < n) s = fma(vj[i], wr[t], s);
    }
    s = block_sum<VD_THREADS>(s, s_red);
    if (threadIdx.x == 0) part[(u64)j * gridDim.x + blockIdx.x] = s;
  }
}

// h[j] = sum_b part[j * nblk + b], in chunk order
__global__ void k_vdot_fin(const double* __restrict__ part, int nblk, int nv, double* __restrict__ h) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nv) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += part[(u64)j * nblk + b];
    h[j] = s;
  }
}

// w += alpha * sum_j V_j h[j]
__global__ void k_vcomb(const double* __restrict__ V, u64 ld, int nv, const double* __restrict__ h, double alpha,
                        double* __restrict__ w, u64 n) {
  extern __shared__ double s_h[];
  for (int j = threadIdx.x; j < nv; j += blockDim.x) s_h[j] = h[j];
  __syncthreads();
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < nv; ++j) s = fma(V[(u64)j * ld + i], s_h[j], s);
    w[i] = fma(alpha, s, w[i]);
  }
}

__global__ void k_vscale(const double* __restrict__ src, double s, double* __restrict__ dst, u64 n) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
    dst[i] = src[i] * s;
}

// deterministic start vector: a hash of each key mapped to [-1, 1)
template <class KT>
__global__ void k_vstart(const KT* __restrict__ keys, u64 n, double* __restrict__ out) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    const u64 z = mix64(slot_hash(keys[i]) ^ 0x2545f4914f6cdd1dull);
    out[i] = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
}

// per-CTA largest |x| and its lowest index
__global__ void __launch_bounds__(VD_THREADS) k_amax_part(const double* __restrict__ x, u64 n,
                                                         double* __restrict__ pv, u64* __restrict__ pi) {
  __shared__ double sv[VD_THREADS];
  __shared__ u64 si[VD_THREADS];
  double bv = -1.0;
  u64 bi = ~0ull;
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    const double a = fabs(x[i]);
    if (a > bv) {
      bv = a;
      bi = i;
    }
  }
  sv[threadIdx.x] = bv;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int o = VD_THREADS / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) {
      const double v2 = sv[threadIdx.x + o];
      const u64 i2 = si[threadIdx.x + o];
      if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    pv[blockIdx.x] = sv[0];
    pi[blockIdx.x] = si[0];
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

// device allocations owned by one call
struct DevArena {
  std::vector<void*> ps;
  ~DevArena() {
    for (void* p : ps) cudaFree(p);
  }
  void* get(size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
      cudaGetLastError();
      set_error(SFCI_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes for the subspace failed");
      return nullptr;
    }
    ps.push_back(p);
    return p;
  }
};

HamView ss_ham_view(Ctx& c) {
  HamView h;
  h.N = c.N;
  h.M = c.M;
  h.P = c.P;
  h.h1 = c.d_h1;
  h.V = c.d_V;
  h.ecore = c.ham.ecore;
  return h;
}

unsigned grid_for(Ctx& c, u64 n, int threads, int per_sm) {
  u64 g = (n + threads - 1) / threads;
  const u64 cap = (u64)c.sm_count * per_sm;
  if (g > cap) g = cap;
  return (unsigned)(g ? g : 1);
}

}  // namespace

// Lowest eigenpairs of H on the block spanned by the sorted, distinct keys
// basis[0..n).  evals[0..nev) receives the lowest eigenvalues (NaN where the
// Krylov space ended before reaching them); x (device, n) the unit eigenvector
// of eigenvalue `want` with its largest component positive; *resid the norm of
// H x - evals[want] x.
template <int W>
static int subspace_eigs(Ctx& c, DevArena& A, const typename KeyOf<W>::T* basis, u64 n, int nev, int want,
                         double* evals, double* x, double* resid) {
  typedef typename KeyOf<W>::T KT;
  if (n >= (1ull << 31)) return set_error(SFCI_ERR_UNSUPPORTED, "subspace larger than 2^31 determinants");
  const HamView h = ss_ham_view(c);
  // 1. key -> index table
  u64 tsz = 64;
  while (tsz < 2 * n) tsz <<= 1;
  KT* tk = (KT*)A.get(tsz * sizeof(KT));
  uint32_t* tv = (uint32_t*)A.get(tsz * sizeof(uint32_t));
  u64* rowptr = (u64*)A.get((n + 1) * sizeof(u64));
  double* diag = (double*)A.get(n * sizeof(double));
  if (!tk || !tv || !rowptr || !diag) return SFCI_ERR_NOMEM;
  SFCI_LAUNCH(c, k_index_clear<KT>, grid_for(c, tsz, 256, 8), 256, 0, tk, tsz);
  SFCI_LAUNCH(c, k_index_build<KT>, grid_for(c, n, 256, 8), 256, 0, basis, n, tk, tv, (unsigned)(tsz - 1));
  // 2. row counts and diagonal, scan, then the CSR rows
  const size_t rsm = row_smem_bytes<KT>();
  SFCI_CUDA(cudaFuncSetAttribute(k_rows<KT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
  SFCI_CUDA(cudaFuncSetAttribute(k_rows<KT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
  const unsigned rg = (unsigned)std::min<u64>(n, (u64)c.sm_count * 4);
  SFCI_LAUNCH(c, (k_rows<KT, false>), rg, SS_THREADS, rsm, basis, n, h, tk, tv, (unsigned)(tsz - 1), rowptr,
              (const u64*)nullptr, (uint32_t*)nullptr, (double*)nullptr, diag);
  int st = scan_excl(c, rowptr, rowptr, n);
  if (st) return st;
  u64 nnz = 0;
  if ((st = read_words(c, rowptr + n, sizeof(u64), &nnz))) return st;
  size_t fr = 0, tot = 0;
  SFCI_CUDA(cudaMemGetInfo(&fr, &tot));
  const double csr_bytes = (double)nnz * (sizeof(uint32_t) + sizeof(double));
  if (csr_bytes > 0.8 * (double)fr)
    return set_error(SFCI_ERR_NOMEM, "subspace Hamiltonian with " + std::to_string(nnz) +
                                         " off-diagonal elements does not fit in device memory");
  uint32_t* col = (uint32_t*)A.get(nnz * sizeof(uint32_t));
  double* val = (double*)A.get(nnz * sizeof(double));
  if (!col || !val) return SFCI_ERR_NOMEM;
  SFCI_LAUNCH(c, (k_rows<KT, true>), rg, SS_THREADS, rsm, basis, n, h, tk, tv, (unsigned)(tsz - 1), (u64*)nullptr,
              (const u64*)rowptr, col, val, (double*)nullptr);
  // 3. Lanczos vectors: as many as memory allows, up to LZ_MAX and n
  SFCI_CUDA(cudaMemGetInfo(&fr, &tot));
  u64 mcap = std::min<u64>((u64)LZ_MAX, n);
  const u64 fit = (u64)(0.8 * (double)fr / (8.0 * (double)n));
  if (fit < 3) return set_error(SFCI_ERR_NOMEM, "no device memory left for the Lanczos vectors");
  mcap = std::min<u64>(mcap, fit - 2);
  const int nb = (int)((n + VD_CHUNK - 1) / VD_CHUNK);
  double* V = (double*)A.get((mcap + 1) * n * sizeof(double));
  double* w = (double*)A.get(n * sizeof(double));
  double* hv = (double*)A.get((mcap + 2) * sizeof(double));
  double* part = (double*)A.get((size_t)(mcap + 1) * nb * sizeof(double));
  double* pv = (double*)A.get(1024 * sizeof(double));
  u64* pi = (u64*)A.get(1024 * sizeof(u64));
  if (!V || !w || !hv || !part || !pv || !pi) return SFCI_ERR_NOMEM;
  const unsigned vg = grid_for(c, n, 256, 8);
  const unsigned sg = grid_for(c, n * 32, 256, 8);
  auto spmv = [&](const double* xin, double* yout) -> int {
    SFCI_LAUNCH(c, k_csr_spmv, sg, 256, 0, (const u64*)rowptr, (const uint32_t*)col, (const double*)val,
                (const double*)diag, xin, yout, n);
    return SFCI_OK;
  };
  // hv[0..nv) = V[0..nv)^T y
  auto vdots = [&](const double* Vb, int nv, const double* y) -> int {
    dim3 g((unsigned)nb, (unsigned)((nv + VD_JB - 1) / VD_JB));
    SFCI_LAUNCH(c, k_vdot_part, g, VD_THREADS, 0, Vb, n, nv, y, n, part);
    SFCI_LAUNCH(c, k_vdot_fin, (unsigned)((nv + 127) / 128), 128, 0, (const double*)part, nb, nv, hv);
    return SFCI_OK;
  };
  auto vcomb = [&](const double* Vb, int nv, const double* coef, double alpha, double* y) -> int {
    SFCI_LAUNCH(c, k_vcomb, vg, 256, (size_t)nv * sizeof(double), Vb, n, nv, coef, alpha, y, n);
    return SFCI_OK;
  };
  auto norm2 = [&](const double* y, double* out) -> int {
    int s2 = vdots(y, 1, y);
    if (s2) return s2;
    double q = 0.0;
    if ((s2 = read_words(c, hv, sizeof(double), &q))) return s2;
    *out = std::sqrt(q);
    return SFCI_OK;
  };
  // start vector
  SFCI_LAUNCH(c, k_vstart<KT>, vg, 256, 0, basis, n, V);
  double nr = 0.0;
  if ((st = norm2(V, &nr))) return st;
  SFCI_LAUNCH(c, k_vscale, vg, 256, 0, (const double*)V, 1.0 / nr, V, n);
  std::vector<double> al, be, th;
  std::vector<std::vector<double>> sv;
  const double tol = 1e-11;
  int m = 0;
  double anorm = 0.0;
  for (u64 j = 0;; ++j) {
    double* vj = V + j * n;
    if ((st = spmv(vj, w))) return st;
    double alpha = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
      if ((st = vdots(V, (int)j + 1, w))) return st;
      if ((st = vcomb(V, (int)j + 1, hv, -1.0, w))) return st;
      double hj = 0.0;
      if ((st = read_words(c, hv + j, sizeof(double), &hj))) return st;
      alpha += hj;
    }
    double beta = 0.0;
    if ((st = norm2(w, &beta))) return st;
    al.push_back(alpha);
    be.push_back(beta);
    m = (int)j + 1;
    anorm = std::max(anorm, std::fabs(alpha) + beta + (j ? be[j - 1] : 0.0));
    const bool ended = (u64)m == n || (u64)m == mcap || beta <= 1e-13 * anorm;
    const int k = std::min(nev, m);
    if (ended || (m >= nev && m % 5 == 0)) {
      hostla::tri_lowest(al, be, m, k, th, sv);
      bool conv = k == nev;
      for (int q = 0; q < k && conv; ++q)
        if (beta * std::fabs(sv[q][m - 1]) > tol * std::max(1.0, std::fabs(th[q]))) conv = false;
      if (conv || ended) break;
    }
    SFCI_LAUNCH(c, k_vscale, vg, 256, 0, (const double*)w, 1.0 / beta, V + (j + 1) * n, n);
  }
  const int k = std::min(nev, m);
  for (int q = 0; q < nev; ++q) evals[q] = q < k ? th[q] : std::nan("");
  if (want >= k) return set_error(SFCI_ERR_NUMERIC, "the subspace has fewer eigenvalues than the state asked for");
  // 4. Ritz vector, unit norm, largest component positive; its true residual
  SFCI_CUDA(cudaMemcpyAsync(hv, sv[want].data(), m * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  SFCI_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), c.stream));
  if ((st = vcomb(V, m, hv, 1.0, x))) return st;
  SFCI_CUDA(cudaStreamSynchronize(c.stream));
  if ((st = norm2(x, &nr))) return st;
  const unsigned ag = std::min<unsigned>(vg, 1024);
  SFCI_LAUNCH(c, k_amax_part, ag, VD_THREADS, 0, (const double*)x, n, pv, pi);
  std::vector<double> hpv(ag);
  std::vector<u64> hpi(ag);
  if ((st = read_words(c, pv, ag * sizeof(double), hpv.data()))) return st;
  if ((st = read_words(c, pi, ag * sizeof(u64), hpi.data()))) return st;
  u64 bi = ~0ull;
  double bv = -1.0;
  for (unsigned q = 0; q < ag; ++q)
    if (hpv[q] > bv || (hpv[q] == bv && hpi[q] < bi)) {
      bv = hpv[q];
      bi = hpi[q];
    }
  double xb = 0.0;
  if ((st = read_words(c, x + bi, sizeof(double), &xb))) return st;
  SFCI_LAUNCH(c, k_vscale, vg, 256, 0, (const double*)x, (xb < 0 ? -1.0 : 1.0) / nr, x, n);
  if ((st = spmv(x, w))) return st;
  const double mth = -th[want];
  SFCI_CUDA(cudaMemcpyAsync(hv, &mth, sizeof(double), cudaMemcpyHostToDevice, c.stream));
  if ((st = vcomb(x, 1, hv, 1.0, w))) return st;
  double r = 0.0;
  if ((st = norm2(w, &r))) return st;
  if (resid) *resid = r;
  return SFCI_OK;
}

template <int W>
static int copy_out(Ctx& c, Vec& out, const typename KeyOf<W>::T* keys, const double* x, u64 n) {
  typedef typename KeyOf<W>::T KT;
  if (out.cap < n) return set_error(SFCI_ERR_CAPACITY, "output vector capacity below the subspace dimension");
  SFCI_CUDA(cudaMemcpyAsync(out.keys, keys, n * sizeof(KT), cudaMemcpyDeviceToDevice, c.stream));
  SFCI_CUDA(cudaMemcpyAsync(out.amps, x, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  SFCI_CUDA(cudaStreamSynchronize(c.stream));
  out.len = n;
  return SFCI_OK;
}

template <int W>
int cisd_impl(Ctx& c, const u64* ref_key, int state_idx, int n_evals, double* evals, Vec& out, double* resid,
              u64* block_size) {
  typedef typename KeyOf<W>::T KT;
  KT key;
  std::memcpy(&key, ref_key, sizeof(KT));
  unsigned cnt[2] = {0, 0};
  for (int b = 0; b < 64 * W; ++b) {
    const bool set = (ref_key[b >> 6] >> (b & 63)) & 1ull;
    if (set && b >= c.N) return set_error(SFCI_ERR_ARG, "reference determinant has bits beyond num_orb");
    if (set) ++cnt[b & 1];
  }
  if ((int)(cnt[0] + cnt[1]) != c.ne)
    return set_error(SFCI_ERR_ARG, "reference determinant does not hold num_e electrons");
  const u64 T = det_terms(cnt[0], c.M - cnt[0], cnt[1], c.M - cnt[1]);
  if (block_size) *block_size = T;
  if (out.cap < T) return set_error(SFCI_ERR_CAPACITY, "output vector capacity below the CISD block size");
  const int nev = std::max(state_idx + 1, n_evals);
  DevArena A;
  KT* keys = (KT*)A.get(T * sizeof(KT));
  double* tmp = (double*)A.get(T * sizeof(double));
  double* x = (double*)A.get(T * sizeof(double));
  if (!keys || !tmp || !x) return SFCI_ERR_NOMEM;
  const size_t rsm = row_smem_bytes<KT>();
  SFCI_CUDA(cudaFuncSetAttribute(k_targets<KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
  const unsigned g = (unsigned)std::min<u64>((T + SS_THREADS * 8 - 1) / (SS_THREADS * 8), (u64)c.sm_count * 2);
  SFCI_LAUNCH(c, k_targets<KT>, g, SS_THREADS, rsm, key, ss_ham_view(c), T, keys);
  SFCI_CUDA(cudaMemsetAsync(tmp, 0, T * sizeof(double), c.stream));
  int st = radix_sort_pairs<W>(c, keys, tmp, T, c.N);
  if (st) return st;
  std::vector<double> ev(nev);
  if ((st = subspace_eigs<W>(c, A, keys, T, nev, state_idx, ev.data(), x, resid))) return st;
  for (int q = 0; q < n_evals; ++q) evals[q] = ev[q];
  return copy_out<W>(c, out, keys, x, T);
}

template <int W>
int fci_impl(Ctx& c, int n_evals, double* evals, Vec* ground, double* resid, u64* dim) {
  typedef typename KeyOf<W>::T KT;
  if (c.ne % 2) return set_error(SFCI_ERR_ARG, "the FCI space is the Sz = 0 block: num_e must be even");
  const int M = c.M, na = c.ne / 2, nb = c.ne / 2;
  if (na > M || M > 64) return set_error(SFCI_ERR_ARG, "electron count does not fit the orbitals");
  std::vector<u64> binom((size_t)(M + 1) * (M + 1), 0);
  for (int i = 0; i <= M; ++i) {
    binom[(size_t)i * (M + 1)] = 1;
    for (int k = 1; k <= i; ++k) {
      const u64 a = binom[(size_t)(i - 1) * (M + 1) + k - 1], b = k <= i - 1 ? binom[(size_t)(i - 1) * (M + 1) + k] : 0;
      binom[(size_t)i * (M + 1) + k] = (a > ~0ull - b) ? ~0ull : a + b;  // saturates
    }
  }
  const u64 nalpha = binom[(size_t)M * (M + 1) + na], nbeta = binom[(size_t)M * (M + 1) + nb];
  const double nd = (double)nalpha * (double)nbeta;
  if (nd >= 2147483648.0) return set_error(SFCI_ERR_UNSUPPORTED, "FCI space larger than 2^31 determinants");
  const u64 n = nalpha * nbeta;
  if (dim) *dim = n;
  if (ground && ground->cap < n) return set_error(SFCI_ERR_CAPACITY, "ground vector capacity below the FCI dimension");
  DevArena A;
  u64* dbin = (u64*)A.get(binom.size() * sizeof(u64));
  KT* keys = (KT*)A.get(n * sizeof(KT));
  double* tmp = (double*)A.get(n * sizeof(double));
  double* x = (double*)A.get(n * sizeof(double));
  if (!dbin || !keys || !tmp || !x) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemcpyAsync(dbin, binom.data(), binom.size() * sizeof(u64), cudaMemcpyHostToDevice, c.stream));
  SFCI_LAUNCH(c, k_fci_keys<KT>, grid_for(c, n, 256, 8), 256, 0, (const u64*)dbin, M, na, nb, nbeta, n, keys);
  SFCI_CUDA(cudaMemsetAsync(tmp, 0, n * sizeof(double), c.stream));
  int st = radix_sort_pairs<W>(c, keys, tmp, n, c.N);
  if (st) return st;
  const int nev = std::max(1, n_evals);
  std::vector<double> ev(nev);
  if ((st = subspace_eigs<W>(c, A, keys, n, nev, 0, ev.data(), x, resid))) return st;
  for (int q = 0; q < n_evals; ++q) evals[q] = ev[q];
  if (ground) return copy_out<W>(c, *ground, keys, x, n);
  SFCI_CUDA(cudaStreamSynchronize(c.stream));
  return SFCI_OK;
}

template int cisd_impl<1>(Ctx&, const u64*, int, int, double*, Vec&, double*, u64*);
template int cisd_impl<2>(Ctx&, const u64*, int, int, double*, Vec&, double*, u64*);
template int fci_impl<1>(Ctx&, int, double*, Vec*, double*, u64*);
template int fci_impl<2>(Ctx&, int, double*, Vec*, double*, u64*);

}  // namespace sfci

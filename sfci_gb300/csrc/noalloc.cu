// sfci_dot_noalloc: the sparse dot product for callers that cannot allocate
// device memory.
//
// Some callers must not call cudaMalloc. One example is code that runs inside
// another framework's device-memory pool, where the framework has reserved
// nearly all of the GPU up front, so a new allocation fails or fragments the
// pool. Another is a host whose hot loop forbids allocation, because it has a
// fixed memory budget decided at start-up. sfci_dot (vecops.cu) keeps its
// per-block partial sums in context scratch that grows with cudaMalloc. This
// variant keeps them in a fixed file-scope device array instead. The caller
// supplies inputs and the output in its own device memory, and nothing is
// allocated or freed.
//
// Limits and sharing:
//  * The array holds DOT_NOALLOC_BLOCKS partial sums. That bounds a call to
//    nx + ny <= DOT_NOALLOC_MAX_ENTRIES merged entries; larger calls are
//    rejected with SFCI_ERR_ARG before anything is launched.
//  * Every GPU that loads the library holds the array (64 KiB) until the
//    process exits.
//  * All calls share the one array. Each call overwrites every slot it reads,
//    so nothing needs clearing between calls. Calls whose kernels overlap on
//    the GPU (different streams, or different host threads) race on the array.
//    Order them on one stream, or serialise them.
//  * On each device, the first call looks up the array's device address with
//    cudaGetSymbolAddress while that device is current. Make that first call
//    before any stream capture begins.
#include <cstdint>
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace sfci {

constexpr int DOT_NOALLOC_THREADS = 256;
constexpr int DOT_NOALLOC_ITEMS = 8;
constexpr unsigned DOT_NOALLOC_BLOCKS = 8192;
constexpr uint64_t DOT_NOALLOC_MAX_ENTRIES =
    (uint64_t)DOT_NOALLOC_BLOCKS * DOT_NOALLOC_THREADS * DOT_NOALLOC_ITEMS;  // 16,777,216

// the fixed scratch: one partial sum per block
static __device__ __align__(256) double g_dot_noalloc_part[DOT_NOALLOC_BLOCKS];

template <class KT>
__device__ __forceinline__ uint64_t na_merge_path(const KT* A, uint64_t na, const KT* B, uint64_t nb, uint64_t diag) {
  uint64_t lo = diag > nb ? diag - nb : 0, hi = diag < na ? diag : na;
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (!key_lt(B[diag - 1 - mid], A[mid])) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// merge-path dot over common keys, one partial per block into `part`
template <class KT>
__global__ void k_dot_noalloc(const KT* __restrict__ A, const double* __restrict__ Aa, uint64_t na,
                              const KT* __restrict__ B, const double* __restrict__ Ba, uint64_t nb, double* part) {
  __shared__ double sh[DOT_NOALLOC_THREADS / 32];
  const uint64_t n = na + nb;
  uint64_t d = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * DOT_NOALLOC_ITEMS;
  double acc = 0.0;
  if (d < n) {
    uint64_t i = na_merge_path(A, na, B, nb, d), j = d - i;
    for (int t = 0; t < DOT_NOALLOC_ITEMS && d + t < n; ++t) {
      bool takeA = (j >= nb) || (i < na && !key_lt(B[j], A[i]));
      if (takeA) {
        ++i;
      } else {
        if (i > 0 && key_eq(A[i - 1], B[j])) acc += Aa[i - 1] * Ba[j];
        ++j;
      }
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < DOT_NOALLOC_THREADS / 32; ++w) s += sh[w];
    part[blockIdx.x] = s;
  }
}

__global__ void k_dot_noalloc_final(const double* part, unsigned np, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (unsigned i = 0; i < np; ++i) s += __ldcg(part + i);
    *out = s;
  }
}

__global__ void k_dot_noalloc_zero(double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = 0.0;
}

// device address of the fixed array, looked up once per device
static std::mutex g_na_mu;
static double* g_na_ptr[128];

static int noalloc_scratch(double** p) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 128) return set_error(SFCI_ERR_UNSUPPORTED, "device ordinal beyond 127");
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* q = nullptr;
    e = cudaGetSymbolAddress(&q, g_dot_noalloc_part);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_dot_noalloc_part)");
    g_na_ptr[dev] = (double*)q;
  }
  *p = g_na_ptr[dev];
  return SFCI_OK;
}

template <class KT>
static int dot_noalloc(const void* xk, const double* xa, uint64_t nx, const void* yk, const double* ya, uint64_t ny,
                       double* d_out, cudaStream_t s) {
  double* part = nullptr;
  int st = noalloc_scratch(&part);
  if (st) return st;
  if (nx == 0 || ny == 0) {
    k_dot_noalloc_zero<<<1, 32, 0, s>>>(d_out);
  } else {
    uint64_t n = nx + ny;
    uint64_t threads = (n + DOT_NOALLOC_ITEMS - 1) / DOT_NOALLOC_ITEMS;
    unsigned grid = (unsigned)((threads + DOT_NOALLOC_THREADS - 1) / DOT_NOALLOC_THREADS);
    k_dot_noalloc<KT><<<grid, DOT_NOALLOC_THREADS, 0, s>>>((const KT*)xk, xa, nx, (const KT*)yk, ya, ny, part);
    k_dot_noalloc_final<<<1, 32, 0, s>>>(part, grid, d_out);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sfci_dot_noalloc launch");
  return SFCI_OK;
}

}  // namespace sfci

extern "C" int sfci_dot_noalloc(const uint64_t* x_keys, const double* x_amps, uint64_t nx, const uint64_t* y_keys,
                                const double* y_amps, uint64_t ny, int key_words, double* d_out, void* stream) {
  using namespace sfci;
  if (!d_out || (nx && (!x_keys || !x_amps)) || (ny && (!y_keys || !y_amps)))
    return set_error(SFCI_ERR_ARG, "sfci_dot_noalloc: null device pointer");
  if (key_words != 1 && key_words != 2) return set_error(SFCI_ERR_ARG, "sfci_dot_noalloc: key_words must be 1 or 2");
  if (nx + ny > DOT_NOALLOC_MAX_ENTRIES || nx > DOT_NOALLOC_MAX_ENTRIES || ny > DOT_NOALLOC_MAX_ENTRIES)
    return set_error(SFCI_ERR_ARG,
                     "sfci_dot_noalloc: nx + ny exceeds the fixed scratch limit of 16777216 entries; use sfci_dot");
  cudaStream_t s = (cudaStream_t)stream;
  return key_words == 1 ? dot_noalloc<u64>(x_keys, x_amps, nx, y_keys, y_amps, ny, d_out, s)
                        : dot_noalloc<K128>(x_keys, x_amps, nx, y_keys, y_amps, ny, d_out, s);
}

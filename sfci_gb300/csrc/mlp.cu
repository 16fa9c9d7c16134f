// The learned excitation screen: a 3-layer BF16 MLP (hidden width 256, FP32
// accumulation, sigmoid output) that predicts, for a term group of a source
// determinant (screen.cuh), whether any of its terms lands on a determinant
// that survives the product's cut and cap.  It has no counterpart in the
// reference; it screens the generator of OffDiagGen_bit (src/bitstr.cpp:162-302).
//
// Layer 1 has sparse inputs (the source's occupancy bits, one-hot p, q, r and
// class, two scalars).  Inference runs in two kernels: a pre-pass
// (k_screen_classify) that keeps the groups the guard keeps, skips those under
// the floor and lists the rest with their features, and the network
// (k_mlp_infer), which runs layer 1's 0/1 part on the tensor cores, an MMA of
// the tile's input rows with W1^T streamed in K chunks by bulk copies, and
// adds the class row and the scalar rows in the epilogue.  The training
// forward sums the about 25 rows of W1 on CUDA cores, the occupancy part
// shared by the rows of a tile that come from one source.  Layer 2 (256 x 256)
// runs on the tensor cores in both: tiles of 128 groups, tcgen05.mma with the
// BF16 weight chunks in shared memory, the FP32 accumulator in TMEM.  Layer 3
// and the sigmoid are the epilogue.
//
// Training (hand-written, four kernels per step): a forward kernel that also
// forms the output error and the layer-2 error Delta2; a backward kernel with
// Delta1 = (Delta2 W2) .* relu'(z1) on the tensor cores (W2^T image); a split-K
// gradient kernel computing dW2 = Delta2^T H1 and dW1 = Delta1^T X on the
// tensor cores over the batch; and an Adam update that rewrites the BF16
// images.  Operands of the gradient products are written by the forward and
// backward kernels as K-major tiles whose K is the batch row.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "prims.cuh"
#include "screen.cuh"
#include "spmspv.h"
#include "umma.cuh"

namespace sfci {

int read_words(Ctx& c, const void* dptr, size_t nbytes, void* host);

namespace mlp {

constexpr int HID = 256;
constexpr int KIN = 576;  // layer-1 input rows, padded to a multiple of 64
constexpr int IN_OCC = 0, IN_P = 128, IN_Q = 256, IN_R = 384, IN_CLS = 512, IN_LC = 516, IN_LV = 517;
constexpr int TILE = 128;  // groups per tile (MMA M)
constexpr int THREADS = 128;
constexpr float FEAT_SCALE = 0.1f;  // log10 features scaled into about [-3, 0]

// parameter block (FP32), offsets in floats
constexpr size_t OFF_W1 = 0;                          // [KIN][HID], row = input
constexpr size_t OFF_B1 = OFF_W1 + (size_t)KIN * HID;  // [HID]
constexpr size_t OFF_W2 = OFF_B1 + HID;                // [HID out][HID in]
constexpr size_t OFF_B2 = OFF_W2 + (size_t)HID * HID;  // [HID]
constexpr size_t OFF_W3 = OFF_B2 + HID;                // [HID]
constexpr size_t OFF_B3 = OFF_W3 + HID;                // [1]
constexpr size_t NPARAM = OFF_B3 + 4;

constexpr uint32_t W2_BYTES = HID * HID * 2;         // 131072: K-major image of a 256 x 256 BF16 matrix
constexpr uint32_t A_BYTES = TILE * HID * 2;         // 65536: one 128 x 256 activation tile
constexpr uint32_t T256_BYTES = HID * TILE * 2;      // 65536: a 256 x 128 transposed tile (K = batch row)
constexpr uint32_t XT_BYTES = KIN * TILE * 2;        // 147456: the 576 x 128 transposed input tile
constexpr uint32_t MASK_WORDS = TILE * HID / 32;     // relu'(z1) bits of a tile
constexpr int MAX_SYSTEMS = 64;                      // Hamiltonians one training set may mix
// inference: the 0/1 rows of W1 (occupancy, p, q, r: rows 0..511) and all of
// W2 go through the tensor cores as B operands streamed by bulk copies, in K
// chunks of 32 through a ring of shared-memory stages
constexpr int IKC = 32;                              // K chunk
constexpr int NCH1 = (IN_R + 128 - IN_OCC) / IKC;    // 16 chunks of W1^T (inputs 0..511: occupancy, p, q, r)
constexpr int NCH2 = HID / IKC;                      // 8 chunks of W2
constexpr int NCHT = NCH1 + NCH2;                    // chunks per tile
constexpr uint32_t IB_BYTES = HID * IKC * 2;         // 16384: K-major image of a 256 x 32 B chunk
constexpr uint32_t IA_BYTES = TILE * IKC * 2;        // 8192: a 128 x 32 input chunk
constexpr uint32_t ISTAGE = IB_BYTES + IA_BYTES;
constexpr int ISTAGES = 6;
constexpr int ROW_THREADS = 256;                     // inference: 8 row warps, two per row quarter of TMEM lanes
constexpr int INF_THREADS = ROW_THREADS + 32;        // and one copy warp

}  // namespace mlp

using namespace mlp;

// ---------------------------------------------------------------------------
// examples: (source, group) pairs enumerated source by source
// ---------------------------------------------------------------------------
struct ExView {
  const u64* keys;     // W words per source
  const double* cc;    // |coefficient| feature of the source (its amplitude in the product input)
  const u64* goff;     // [nsrc + 1] exclusive prefix of groups per source (group 0 excluded)
  u64 nsrc, nex;
  int W, N, M, P;
  const float* const* vmaxs;  // integral-bound tables [4][P][M], one per Hamiltonian
  const uint8_t* sys;         // nullable: table of each source (else table 0)
};

__device__ __forceinline__ u64 source_of(const ExView& x, u64 e) {
  u64 lo = 0, hi = x.nsrc;  // largest j with goff[j] <= e
  while (hi - lo > 1) {
    const u64 mid = (lo + hi) >> 1;
    if (__ldg(x.goff + mid) <= e) lo = mid; else hi = mid;
  }
  return lo;
}

template <class KT>
__device__ __forceinline__ KT load_key(const u64* keys, u64 j);
template <>
__device__ __forceinline__ u64 load_key<u64>(const u64* keys, u64 j) { return __ldg(keys + j); }
template <>
__device__ __forceinline__ K128 load_key<K128>(const u64* keys, u64 j) {
  K128 k;
  k.lo = __ldg(keys + 2 * j);
  k.hi = __ldg(keys + 2 * j + 1);
  return k;
}

struct Feat {
  int cls, p, q, r;
  float lc, lv;
  unsigned gstart, gsize;
};

template <class KT>
__device__ Feat example_feat(const ExView& x, const KT& key, double cc, unsigned g, u64 j) {
  unsigned a0, a1;
  spin_counts(key, x.N, a0, a1);
  const unsigned v0 = x.M - a0, v1 = x.M - a1;
  const GroupCounts gc = group_counts(a0, v0, a1, v1);
  unsigned c[6];
  c[0] = 1;
  c[1] = c[0] + a0 * v0;
  c[2] = c[1] + a1 * v1;
  c[3] = c[2] + c2(a0) * c2(v0);
  c[4] = c[3] + c2(a1) * c2(v1);
  c[5] = c[4] + a0 * v0 * a1 * v1;
  const GroupDesc d = group_desc(gc, c, g);
  Feat f;
  group_orbitals(key, x.N, gc, d, f.p, f.q, f.r);
  f.cls = d.cls;
  f.gstart = d.start;
  f.gsize = d.size;
  const float* vmax = x.vmaxs[x.sys ? x.sys[j] : 0];
  const float vb = group_vbound(vmax, x.M, x.P, d.cls, f.p, f.q, f.r);
  f.lc = FEAT_SCALE * log10f(fmaxf((float)fabs(cc), 1e-30f));
  f.lv = FEAT_SCALE * log10f(fmaxf(vb, 1e-30f));
  return f;
}

// sum of W1's occupancy rows of a key: thread t of 128 writes columns t and t + 128
template <class KT>
__device__ void occ_sum(const KT& key, int N, const __nv_bfloat16* __restrict__ W1b, float* u) {
  float s0 = 0.f, s1 = 0.f;
  for (int o = 0; o < N; ++o) {
    if (!key_test(key, o)) continue;
    const __nv_bfloat16* row = W1b + (size_t)(IN_OCC + o) * HID;
    s0 += __bfloat162float(row[threadIdx.x]);
    s1 += __bfloat162float(row[threadIdx.x + 128]);
  }
  u[threadIdx.x] = s0;
  u[threadIdx.x + 128] = s1;
}

// 8 BF16 weights starting at a 16-byte boundary, added to acc[0..7] with scale s
__device__ __forceinline__ void add_row8(float* acc, const __nv_bfloat16* p, float s) {
  const uint4 q = __ldg(reinterpret_cast<const uint4*>(p));
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(h[i]);
    acc[2 * i] += s * f.x;
    acc[2 * i + 1] += s * f.y;
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// Layer 1 of this thread's row into the K-major A tile (BF16, relu applied);
// the relu'(z1) bits (8 words of 32 columns) go to mask (nullable)
__device__ __forceinline__ void layer1_row(const Feat& f, bool valid, const float* u,
                                           const __nv_bfloat16* __restrict__ W1b, const float* __restrict__ b1,
                                           uint8_t* A, int row, uint32_t* mask) {
#pragma unroll
  for (int k = 0; k < HID / 32; ++k) {
    uint32_t word = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c0 = 32 * k + 8 * q;
      float acc[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) acc[i] = valid ? (__ldg(b1 + c0 + i) + u[c0 + i]) : 0.f;
      if (valid) {
        add_row8(acc, W1b + (size_t)(IN_P + f.p) * HID + c0, 1.f);
        add_row8(acc, W1b + (size_t)(IN_Q + f.q) * HID + c0, 1.f);
        add_row8(acc, W1b + (size_t)(IN_R + f.r) * HID + c0, 1.f);
        add_row8(acc, W1b + (size_t)(IN_CLS + f.cls) * HID + c0, 1.f);
        add_row8(acc, W1b + (size_t)IN_LC * HID + c0, f.lc);
        add_row8(acc, W1b + (size_t)IN_LV * HID + c0, f.lv);
      }
      float h[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        h[i] = fmaxf(acc[i], 0.f);
        word |= (acc[i] > 0.f ? 1u : 0u) << (8 * q + i);
      }
      uint4 o;
      o.x = pack_bf16(h[0], h[1]);
      o.y = pack_bf16(h[2], h[3]);
      o.z = pack_bf16(h[4], h[5]);
      o.w = pack_bf16(h[6], h[7]);
      *reinterpret_cast<uint4*>(A + umma::tile_offset(row, c0, HID)) = o;
    }
    if (mask) mask[k] = word;
  }
}

// Copy a K-major 128 x 256 tile in shared memory to a 256 x 128 K-major tile
// (its transpose, K = the batch row) in global memory; 16-byte stores.
__device__ void export_transposed(const uint8_t* A, uint8_t* __restrict__ out) {
  for (unsigned q = threadIdx.x; q < HID * TILE / 8; q += THREADS) {
    // chunk q: column c (0..255), rows 8g..8g+7
    const unsigned c7 = q & 7, g = (q >> 3) & 15, chi = q >> 7;
    const unsigned c = chi * 8 + c7;
    uint16_t v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = *reinterpret_cast<const uint16_t*>(A + umma::tile_offset(8 * g + i, c, HID));
    uint4 o;
    o.x = v[0] | ((uint32_t)v[1] << 16);
    o.y = v[2] | ((uint32_t)v[3] << 16);
    o.z = v[4] | ((uint32_t)v[5] << 16);
    o.w = v[6] | ((uint32_t)v[7] << 16);
    *reinterpret_cast<uint4*>(out + umma::tile_offset(c, 8 * g, TILE)) = o;
  }
}

// butterfly reduction over the 32 lanes of 32 values: lane l returns the sum of v[l]
__device__ __forceinline__ float lane_column_sum(float* v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool up = lane & s;
#pragma unroll
    for (int i = 0; i < s; ++i) {
      const float send = up ? v[i] : v[i + s];
      const float recv = __shfl_xor_sync(0xffffffffu, send, s);
      v[i] = (up ? v[i + s] : v[i]) + recv;
    }
  }
  return v[0];
}

// ---------------------------------------------------------------------------
// forward: training (loss, Delta2, gradient operands) in k_mlp_fwd, inference
// (keep bits) in k_mlp_infer
// ---------------------------------------------------------------------------
struct FwdArgs {
  ExView x;
  const __nv_bfloat16* W1b;
  const float* params;   // FP32 masters: b1, b2, w3, b3 read from here
  const uint8_t* W2img;  // K-major image of W2 (B = W2, N = out, K = in)
  const uint8_t* Wc;     // inference: NCHT K-major 256 x 32 chunks, W1^T rows 0..511 then W2
  const u64* list_e;     // inference: the examples the network decides (in any order) ...
  const uint32_t* list_j;  // ... their sources ...
  const uint4* list_f;     // ... and their features (ListFeat)
  u64 nlist;
  unsigned ntiles;
  const u64* tile_start;  // training: first example of each tile (nullptr: tile t starts at 128 t)
  // inference
  float thr;
  float lguard;           // log10 of the guard: a group with log10(|c_j| * vbound) >= lguard is kept
  float lfloor;           // log10 of the floor: a group with log10(|c_j| * vbound) < lfloor is skipped
  uint32_t* keep;         // one bit per example
  u64* kept_terms;        // per source
  u64* kept_groups;       // per source
  u64* all_terms;         // nullable: terms of every group (one counter)
  float* prob;            // nullable: per example
  // training
  const uint32_t* labels;
  float pos_weight, inv_batch;
  uint8_t* H1T;           // [ntiles] 256 x 128 tiles of H1^T
  uint8_t* D2img;         // [ntiles] 128 x 256 tiles of Delta2
  uint8_t* D2T;           // [ntiles] 256 x 128 tiles of Delta2^T
  uint8_t* XT;            // [ntiles] 576 x 128 tiles of X^T
  uint32_t* mask1;        // [ntiles] relu'(z1) bits
  float* grads;           // b2, w3, b3 gradients accumulate here
  double* loss;           // sum of weighted BCE over the batch
  unsigned* err;          // [0] = a wait timed out
};

template <class KT>
__global__ void __launch_bounds__(THREADS, 1) k_mlp_fwd(FwdArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sW2 = smem;                        // 128 KB
  uint8_t* sA = smem + W2_BYTES;              // 64 KB
  float* su = reinterpret_cast<float*>(sA + A_BYTES);  // [2][256] occupancy sums
  float* sb2 = su + 2 * HID;                  // [256]
  float* sw3 = sb2 + HID;                     // [256]
  float* sg_b2 = sw3 + HID;                   // [256] gradient partials
  float* sg_w3 = sg_b2 + HID;                 // [256]
  __shared__ __align__(8) uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ u64 s_src[2];
  __shared__ float s_gb3;
  __shared__ double s_loss[THREADS / 32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  bool failed = false;

  if (tid == 0) {
    umma::mbar_init(&bar_load, 1);
    umma::mbar_init(&bar_mma, 1);
    umma::fence_mbar_init();
  }
  for (int i = tid; i < HID; i += THREADS) {
    sb2[i] = a.params[OFF_B2 + i];
    sw3[i] = a.params[OFF_W3 + i];
    sg_b2[i] = 0.f;
    sg_w3[i] = 0.f;
  }
  if (tid == 0) s_gb3 = 0.f;
  __syncthreads();
  if (warp == 0) umma::tmem_alloc(&tmem_slot, 256);
  if (tid == 0) {
    umma::mbar_arrive_expect_tx(&bar_load, W2_BYTES);
    for (uint32_t o = 0; o < W2_BYTES; o += 16384) umma::bulk_g2s(sW2 + o, a.W2img + o, 16384, &bar_load);
  }
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  failed = __syncthreads_or(!umma::mbar_wait(&bar_load, 0)) != 0;
  const float b3 = a.params[OFF_B3];
  const uint32_t idesc = umma::idesc_bf16_f32(TILE, HID);
  double lacc = 0.0;
  uint32_t mma_phase = 0;

  for (unsigned t = blockIdx.x; t < a.ntiles && !failed; t += gridDim.x) {
    const u64 e0 = a.tile_start ? a.tile_start[t] : (u64)t * TILE;
    const u64 e = e0 + tid;
    const bool valid = e < a.x.nex;
    // the tile's first and last sources: their occupancy sums are shared
    if (tid == 0) s_src[0] = source_of(a.x, e0 < a.x.nex ? e0 : a.x.nex - 1);
    if (tid == 1) {
      const u64 el = e0 + TILE - 1 < a.x.nex ? e0 + TILE - 1 : a.x.nex - 1;
      s_src[1] = source_of(a.x, el);
    }
    __syncthreads();
    occ_sum(load_key<KT>(a.x.keys, s_src[0]), a.x.N, a.W1b, su);
    if (s_src[1] != s_src[0]) occ_sum(load_key<KT>(a.x.keys, s_src[1]), a.x.N, a.W1b, su + HID);
    __syncthreads();
    u64 j = 0;
    Feat f{};
    KT key{};
    if (valid) {
      // sources are in example order: walk forward from the tile's first one
      j = s_src[0];
      while (j + 1 < a.x.nsrc && __ldg(a.x.goff + j + 1) <= e) ++j;
      key = load_key<KT>(a.x.keys, j);
      f = example_feat(a.x, key, a.x.cc[j], (unsigned)(e - a.x.goff[j]) + 1u, j);
    }
    float ubuf[HID];
    const float* u = su;
    if (valid && j == s_src[1] && j != s_src[0]) u = su + HID;
    if (valid && j != s_src[0] && j != s_src[1]) {  // a source strictly inside the tile: its own sum
      for (int c = 0; c < HID; ++c) ubuf[c] = 0.f;
      for (int o = 0; o < a.x.N; ++o)
        if (key_test(key, o))
          for (int c = 0; c < HID; ++c) ubuf[c] += __bfloat162float(a.W1b[(size_t)(IN_OCC + o) * HID + c]);
      u = ubuf;
    }
    uint32_t mbits[8];
    layer1_row(f, valid, u, a.W1b, a.params + OFF_B1, sA, tid, mbits);
    umma::fence_async_smem();
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
    if (tid == 0) {
      umma::gemm_tile(tmem, umma::smem_u32(sA), umma::smem_u32(sW2), HID, idesc, false);
      umma::mma_commit(&bar_mma);
    }
    {
      // while the tensor cores run: the gradient operands that need only layer 1
      uint8_t* xt = a.XT + (size_t)t * XT_BYTES;
      export_transposed(sA, a.H1T + (size_t)t * T256_BYTES);
      for (uint32_t o = tid * 16; o < XT_BYTES; o += THREADS * 16) *reinterpret_cast<uint4*>(xt + o) = make_uint4(0, 0, 0, 0);
      uint32_t* mk = a.mask1 + (size_t)t * MASK_WORDS + tid * 8;
#pragma unroll
      for (int w = 0; w < 8; ++w) mk[w] = mbits[w];
      __syncthreads();  // zero fill before the scattered ones
      if (valid) {
        const __nv_bfloat16 one = __float2bfloat16(1.f);
        auto put = [&](int in, __nv_bfloat16 v) {
          *reinterpret_cast<__nv_bfloat16*>(xt + umma::tile_offset(in, tid, TILE)) = v;
        };
        for (int o = 0; o < a.x.N; ++o)
          if (key_test(key, o)) put(IN_OCC + o, one);
        put(IN_P + f.p, one);
        put(IN_Q + f.q, one);
        put(IN_R + f.r, one);
        put(IN_CLS + f.cls, one);
        put(IN_LC, __float2bfloat16(f.lc));
        put(IN_LV, __float2bfloat16(f.lv));
      }
    }
    failed = __syncthreads_or(!umma::mbar_wait(&bar_mma, mma_phase)) != 0;
    mma_phase ^= 1u;
    umma::tc_fence_after();
    // epilogue pass 1: layer 3
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
    float logit = b3;
    for (int k = 0; k < HID / 32 && !failed; ++k) {
      float z[32];
      umma::tmem_ld32(trow + 32 * k, z);
#pragma unroll
      for (int i = 0; i < 32; ++i) logit += fmaxf(z[i] + sb2[32 * k + i], 0.f) * sw3[32 * k + i];
    }
    const float p = 1.f / (1.f + __expf(-logit));
    {
      const bool y = valid && ((a.labels[e >> 5] >> (e & 31)) & 1u);
      const float wgt = valid ? (y ? a.pos_weight : 1.f) : 0.f;
      const float d3 = wgt * (p - (y ? 1.f : 0.f)) * a.inv_batch;
      if (valid) {
        const float pc = fminf(fmaxf(p, 1e-7f), 1.f - 1e-7f);
        lacc += (double)(wgt * -(y ? __logf(pc) : __logf(1.f - pc)));
      }
      // the A tile is free once the MMA has completed (waited above) and the
      // H1^T export has finished
      __syncthreads();
      for (int k = 0; k < HID / 32 && !failed; ++k) {
        float z[32], g2[32], gw[32];
        umma::tmem_ld32(trow + 32 * k, z);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float zz = z[i] + sb2[32 * k + i];
          const float h2 = fmaxf(zz, 0.f);
          g2[i] = zz > 0.f ? d3 * sw3[32 * k + i] : 0.f;
          gw[i] = d3 * h2;
        }
        // Delta2 row chunk into the A tile (K-major [row][out])
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint4 o;
          o.x = pack_bf16(g2[8 * q + 0], g2[8 * q + 1]);
          o.y = pack_bf16(g2[8 * q + 2], g2[8 * q + 3]);
          o.z = pack_bf16(g2[8 * q + 4], g2[8 * q + 5]);
          o.w = pack_bf16(g2[8 * q + 6], g2[8 * q + 7]);
          *reinterpret_cast<uint4*>(sA + umma::tile_offset(tid, 32 * k + 8 * q, HID)) = o;
        }
        const float cb = lane_column_sum(g2), cw = lane_column_sum(gw);
        atomicAdd(sg_b2 + 32 * k + lane, cb);
        atomicAdd(sg_w3 + 32 * k + lane, cw);
      }
      const float d3s = warp_sum(d3);
      if (lane == 0) atomicAdd(&s_gb3, d3s);
      __syncthreads();
      // Delta2 (K-major, for the backward kernel) and Delta2^T (for dW2)
      uint8_t* d2 = a.D2img + (size_t)t * A_BYTES;
      for (uint32_t o = tid * 16; o < A_BYTES; o += THREADS * 16)
        *reinterpret_cast<uint4*>(d2 + o) = *reinterpret_cast<const uint4*>(sA + o);
      export_transposed(sA, a.D2T + (size_t)t * T256_BYTES);
    }
    umma::tc_fence_before();
    __syncthreads();  // the A tile and TMEM are rewritten by the next tile
    umma::tc_fence_after();
  }
  {
    __syncthreads();
    for (int i = tid; i < HID; i += THREADS) {
      atomicAdd(a.grads + OFF_B2 + i, sg_b2[i]);
      atomicAdd(a.grads + OFF_W3 + i, sg_w3[i]);
    }
    if (tid == 0) atomicAdd(a.grads + OFF_B3, s_gb3);
    double l = warp_sum(lacc);
    if (lane == 0) s_loss[warp] = l;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < THREADS / 32; ++w) s += s_loss[w];
      atomicAdd(a.loss, s);
    }
  }
  if (failed && tid == 0) atomicOr(a.err, 1u);
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

// Decides the groups the network need not see: a group whose largest possible
// term, |c_j| times its integral bound, reaches the guard is kept; one below the
// floor is skipped (the training labels call a group alive only through a term
// above their minimum, so a floor at that minimum skips only groups the labels
// call dead); the rest join the network's list (example and source), in any
// order.  Writes every keep word (the guard's bits), the guard-kept groups and
// terms per source and the terms of all groups.  A warp takes CW consecutive
// keep words (32 examples each) per round, one lane per example; one atomic per
// block round claims the list positions.
constexpr int CW = 4;
// a list entry's features, 16 bytes: p | q << 7 | r << 14 | class << 21, log|c|, log bound, terms
__device__ __forceinline__ uint4 pack_feat(const Feat& f) {
  return make_uint4((unsigned)f.p | ((unsigned)f.q << 7) | ((unsigned)f.r << 14) | ((unsigned)f.cls << 21),
                    __float_as_uint(f.lc), __float_as_uint(f.lv), f.gsize);
}
__device__ __forceinline__ Feat unpack_feat(const uint4 v) {
  Feat f;
  f.p = (int)(v.x & 127u);
  f.q = (int)((v.x >> 7) & 127u);
  f.r = (int)((v.x >> 14) & 127u);
  f.cls = (int)((v.x >> 21) & 3u);
  f.lc = __uint_as_float(v.y);
  f.lv = __uint_as_float(v.z);
  f.gstart = 0;
  f.gsize = v.w;
  return f;
}

template <class KT>
__global__ void __launch_bounds__(256) k_screen_classify(FwdArgs a, u64 wbeg, u64 nwords, u64* __restrict__ list_e,
                                                         uint32_t* __restrict__ list_j, uint4* __restrict__ list_f,
                                                         u64* __restrict__ nlist) {
  __shared__ unsigned s_cnt[8];
  __shared__ u64 s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const u64 step = (u64)gridDim.x * 8 * CW;
  for (u64 wb = wbeg + (u64)blockIdx.x * 8 * CW; wb < nwords; wb += step) {
    const u64 w0 = wb + (u64)warp * CW;
    unsigned unsure_bits = 0, total = 0;
    u64 js[CW];
    uint4 fs[CW];
    for (int k = 0; k < CW; ++k) {
      const u64 w = w0 + k;
      js[k] = 0;
      fs[k] = make_uint4(0, 0, 0, 0);
      if (w >= nwords) continue;  // warp-uniform
      const u64 e = (w << 5) + lane;
      const bool valid = e < a.x.nex;
      u64 j = 0;
      if (lane == 0) j = source_of(a.x, w << 5);
      j = __shfl_sync(0xffffffffu, j, 0);
      Feat f{};
      if (valid) {
        while (j + 1 < a.x.nsrc && __ldg(a.x.goff + j + 1) <= e) ++j;
        f = example_feat(a.x, load_key<KT>(a.x.keys, j), a.x.cc[j], (unsigned)(e - a.x.goff[j]) + 1u, j);
      }
      js[k] = j;
      fs[k] = pack_feat(f);
      const float lb = 10.f * (f.lc + f.lv);
      const bool gk = valid && lb >= a.lguard;
      const bool unsure = valid && !gk && lb >= a.lfloor;
      const unsigned m = __ballot_sync(0xffffffffu, gk);
      if (lane == 0) a.keep[w] = m;
      const unsigned at = warp_sum(valid ? f.gsize : 0u);
      if (lane == 0 && at) atomicAdd(a.all_terms, (u64)at);
      const u64 jj = valid ? j : ~0ull;
      const unsigned same = __match_any_sync(0xffffffffu, jj);
      const unsigned nt = gk ? f.gsize : 0u, ng = gk ? 1u : 0u;
      if (same == 0xffffffffu) {
        const unsigned st = warp_sum(nt), sg = warp_sum(ng);
        if (lane == 0 && st) {
          atomicAdd(a.kept_terms + j, (u64)st);
          atomicAdd(a.kept_groups + j, (u64)sg);
        }
      } else if (gk) {
        atomicAdd(a.kept_terms + j, (u64)nt);
        atomicAdd(a.kept_groups + j, (u64)ng);
      }
      const unsigned bu = __ballot_sync(0xffffffffu, unsure);
      if (unsure) unsure_bits |= 1u << k;
      total += __popc(bu);
    }
    if (lane == 0) s_cnt[warp] = total;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned t = 0;
      for (int i = 0; i < 8; ++i) {
        const unsigned c = s_cnt[i];
        s_cnt[i] = t;
        t += c;
      }
      s_base = t ? atomicAdd(nlist, (u64)t) : 0ull;
    }
    __syncthreads();
    u64 pos = s_base + s_cnt[warp];
    for (int k = 0; k < CW; ++k) {
      const u64 w = w0 + k;
      if (w >= nwords) break;  // warp-uniform
      const bool unsure = (unsure_bits >> k) & 1u;
      const unsigned bu = __ballot_sync(0xffffffffu, unsure);
      if (unsure) {
        const u64 q = pos + __popc(bu & lt);
        list_e[q] = (w << 5) + lane;
        list_j[q] = (uint32_t)js[k];
        list_f[q] = fs[k];
      }
      pos += __popc(bu);
    }
    __syncthreads();  // s_cnt and s_base are rewritten next round
  }
}

// ---------------------------------------------------------------------------
// inference: both hidden layers on the tensor cores
// ---------------------------------------------------------------------------
// The rows of a tile are entries of the pre-pass's list (example, source,
// features), in any order.  Warps 0-7 are row warps: warp w holds rows
// 32 (w % 4) .. + 31 of the tile (the TMEM lane quarter it may read) and the
// column half w / 4 of every 256-wide epilogue, so two warps share each row
// and each scheduler has two.  Warp 8 is a copy warp.  Every tile takes the
// same 24 B-operand chunks (256 x 32, 16 KB): 16 of W1^T for the 0/1 inputs
// (occupancy, p, q, r: W1 rows 0..511) and 8 of W2, through a ring of 6
// stages; the copy warp streams them ahead of use, across tile boundaries and
// through the epilogues.  Layer 1: per W1 chunk the row warps write the tile's
// 0/1 input chunk (the source's occupancy bits or a one-hot index) into the
// stage and one thread issues its two MMAs into TMEM columns 0..255.  The
// layer-1 epilogue adds b1, the class row and the two scalar rows (kept in
// shared memory as FP32 copies of the BF16 weights), applies the ReLU and
// writes the BF16 layer-2 operand (64 KB); layer 2 accumulates into TMEM
// columns 256..511; layer 3 and the sigmoid are the last epilogue, its two
// column halves added through shared memory.  The same function as the
// training forward (layer1_row), summed in another order.
//
// Barrier phases: chunk g of the CTA's sequence uses stage g % 6; its use
// u = g / 6 completes `full` (copy landed) and, after the MMAs that read the
// stage, `freed` (tcgen05.commit), both with parity u & 1.  The row warps sync
// among themselves on named barrier 1 and vote on failures with bar.red.or, so
// every branch is uniform; every mbarrier wait is bounded.
__device__ __forceinline__ void rows_sync() { asm volatile("bar.sync 1, %0;" ::"r"(ROW_THREADS) : "memory"); }
// named barrier 1 over the row warps that also ORs a flag across them
__device__ __forceinline__ bool rows_or(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(ROW_THREADS)
      : "memory");
  return r != 0;
}

template <class KT>
__global__ void __launch_bounds__(INF_THREADS, 1) k_mlp_infer(FwdArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA2 = smem;                                                  // 64 KB layer-2 operand
  uint8_t* sStg = smem + A_BYTES;                                       // ISTAGES x (B chunk, input chunk)
  float* sb1 = reinterpret_cast<float*>(sStg + ISTAGES * ISTAGE);       // [256] b1
  float* scls = sb1 + 2 * HID;                                          // [4][256] class rows
  float* slc = scls + 4 * HID;                                          // [256] log|c| row
  float* slv = slc + HID;                                               // [256] log bound row
  float* sb2 = slv + HID;                                               // [256]
  float* sw3 = sb2 + HID;                                               // [256]
  float* slog = sw3 + HID;                                              // [128] second-half logits
  __shared__ __align__(8) uint64_t bar_full[ISTAGES], bar_free[ISTAGES], bar_done, bar_fin;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < ISTAGES; ++i) {
      umma::mbar_init(&bar_full[i], 1);
      umma::mbar_init(&bar_free[i], 1);
    }
    umma::mbar_init(&bar_done, 1);
    umma::mbar_init(&bar_fin, 1);
    umma::fence_mbar_init();
    s_fail = 0;
  }
  for (int i = tid; i < HID; i += INF_THREADS) {
    sb1[i] = a.params[OFF_B1 + i];
    for (int k = 0; k < 4; ++k) scls[k * HID + i] = __bfloat162float(a.W1b[(size_t)(IN_CLS + k) * HID + i]);
    slc[i] = __bfloat162float(a.W1b[(size_t)IN_LC * HID + i]);
    slv[i] = __bfloat162float(a.W1b[(size_t)IN_LV * HID + i]);
    sb2[i] = a.params[OFF_B2 + i];
    sw3[i] = a.params[OFF_W3 + i];
  }
  __syncthreads();
  if (warp == 0) umma::tmem_alloc(&tmem_slot, 512);
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == ROW_THREADS / 32) {
    // ---- copy warp: the B chunks of every tile, in order, ISTAGES ahead
    if (lane == 0) {
      uint32_t g = 0;
      for (unsigned t = blockIdx.x; t < a.ntiles && !s_fail; t += gridDim.x) {
        for (int c = 0; c < NCHT; ++c) {
          const uint32_t st = g % ISTAGES, use = g / ISTAGES;
          if (use > 0 && !umma::mbar_wait(&bar_free[st], (use - 1) & 1u)) s_fail = 1;
          if (s_fail) break;
          umma::mbar_arrive_expect_tx(&bar_full[st], IB_BYTES);
          umma::bulk_g2s(sStg + st * ISTAGE, a.Wc + (size_t)c * IB_BYTES, IB_BYTES, &bar_full[st]);
          ++g;
        }
      }
      // the copies this warp started have landed (the row warps waited for
      // them already unless a wait timed out)
      for (uint32_t st = 0; st < (uint32_t)ISTAGES; ++st) {
        const uint32_t uses = g / ISTAGES + (st < g % ISTAGES ? 1u : 0u);
        if (uses) umma::mbar_wait(&bar_full[st], (uses - 1) & 1u);
      }
    }
  } else {
    // ---- row warps
    const int row = 32 * (warp & 3) + lane, half = warp >> 2, c0h = 128 * half;
    const float b3 = a.params[OFF_B3];
    const uint32_t idesc = umma::idesc_bf16_f32(TILE, HID);
    const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    const uint16_t ONE = 0x3f80;  // BF16 1.0
    uint32_t g = 0, done_phase = 0;
    bool fail = false;  // this thread's; every decision takes it through rows_or
    const int N = a.x.N;
    const u64 nmask0 = N >= 64 ? ~0ull : ((1ull << N) - 1ull);
    const u64 nmask1 = N >= 128 ? ~0ull : (N > 64 ? ((1ull << (N - 64)) - 1ull) : 0ull);
    for (unsigned t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
      // row `row` of the tile: an entry of the network's list (example, source)
      const u64 idx = (u64)t * TILE + row;
      const bool valid = idx < a.nlist;
      u64 e = 0, j = 0;
      Feat f{};
      u64 occ[2] = {0ull, 0ull};
      if (valid) {
        e = __ldg(a.list_e + idx);
        j = __ldg(a.list_j + idx);
        f = unpack_feat(__ldg(a.list_f + idx));  // computed by the pre-pass
        const KT key = load_key<KT>(a.x.keys, j);
        occ[0] = kword(key, 0) & nmask0;
        if (sizeof(KT) > 8) occ[1] = kword(key, 1) & nmask1;
      }
      // ---- layer 1, one-hot part: NCH1 chunks
      for (int c = 0; c < NCH1; ++c, ++g) {
        const uint32_t st = g % ISTAGES, use = g / ISTAGES;
        uint8_t* sB = sStg + st * ISTAGE;
        uint8_t* sX = sB + IB_BYTES;
        if (use > 0 && !umma::mbar_wait(&bar_free[st], (use - 1) & 1u)) fail = true;
        // this row's 32 inputs of chunk c: occupancy bits (c < 4), then p, q or r
        // as a one-hot index; each of the row's two threads writes 16 of them
        unsigned bits = 0;
        if (valid) {
          if (c < 4) {
            bits = (unsigned)(occ[c >> 1] >> (32 * (c & 1)));
          } else {
            const int cc = c - 4;
            const int oh = cc < 4 ? f.p : (cc < 8 ? f.q : f.r);
            const int lo = IKC * (cc & 3);
            if (oh >= lo && oh < lo + IKC) bits = 1u << (oh - lo);
          }
        }
#pragma unroll
        for (int qq = 0; qq < IKC / 16; ++qq) {
          const int q = 2 * half + qq;
          const unsigned by = (bits >> (8 * q)) & 0xffu;
          uint32_t w[4];
#pragma unroll
          for (int h = 0; h < 4; ++h)
            w[h] = ((by >> (2 * h)) & 1u ? ONE : 0u) | (((by >> (2 * h + 1)) & 1u ? ONE : 0u) << 16);
          *reinterpret_cast<uint4*>(sX + umma::tile_offset(row, 8 * q, IKC)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
        umma::fence_async_smem();
        umma::tc_fence_before();
        if (rows_or(fail)) {
          fail = true;
          break;
        }
        if (tid == 0) {
          umma::tc_fence_after();
          if (umma::mbar_wait(&bar_full[st], use & 1u))
            umma::gemm_tile(tmem, umma::smem_u32(sX), umma::smem_u32(sB), IKC, idesc, c > 0);
          else
            fail = true;
          umma::mma_commit(&bar_free[st]);
          if (c == NCH1 - 1) umma::mma_commit(&bar_done);
        }
      }
      if (rows_or(fail)) {
        fail = true;
        break;
      }
      // ---- layer-1 epilogue, this thread's 128 columns
      if (!umma::mbar_wait(&bar_done, done_phase)) fail = true;
      done_phase ^= 1u;
      if (rows_or(fail)) {
        fail = true;
        break;
      }
      umma::tc_fence_after();
      {
        const float* u = sb1;
        const float* rc = scls + (valid ? f.cls : 0) * HID;
        for (int k = 0; k < HID / 64; ++k) {
          const int cb = c0h + 32 * k;
          float z[32];
          umma::tmem_ld32(trow + cb, z);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int c8 = cb + 8 * q;
            float h[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const float x = z[8 * q + i] + u[c8 + i] + rc[c8 + i] + f.lc * slc[c8 + i] + f.lv * slv[c8 + i];
              h[i] = valid ? fmaxf(x, 0.f) : 0.f;
            }
            uint4 o;
            o.x = pack_bf16(h[0], h[1]);
            o.y = pack_bf16(h[2], h[3]);
            o.z = pack_bf16(h[4], h[5]);
            o.w = pack_bf16(h[6], h[7]);
            *reinterpret_cast<uint4*>(sA2 + umma::tile_offset(row, c8, HID)) = o;
          }
        }
      }
      umma::fence_async_smem();
      umma::tc_fence_before();
      rows_sync();
      // ---- layer 2: NCH2 chunks of W2 against the K stripes of the operand
      if (tid == 0) {
        umma::tc_fence_after();
        for (int c = 0; c < NCH2; ++c) {
          const uint32_t gg = g + (uint32_t)c, st = gg % ISTAGES, use = gg / ISTAGES;
          if (!fail && umma::mbar_wait(&bar_full[st], use & 1u)) {
            const uint32_t sB = umma::smem_u32(sStg + st * ISTAGE), sa = umma::smem_u32(sA2);
#pragma unroll
            for (int k = 0; k < IKC; k += 16)
              umma::mma_bf16(tmem + HID, umma::sdesc(sa + ((IKC * c + k) >> 3) * umma::CORE_BYTES, HID),
                             umma::sdesc(sB + (k >> 3) * umma::CORE_BYTES, IKC), idesc, c > 0 || k > 0);
          } else {
            fail = true;
          }
          umma::mma_commit(&bar_free[st]);
        }
        umma::mma_commit(&bar_done);
      }
      g += NCH2;
      if (!umma::mbar_wait(&bar_done, done_phase)) fail = true;
      done_phase ^= 1u;
      if (rows_or(fail)) {
        fail = true;
        break;
      }
      umma::tc_fence_after();
      // ---- layer 3: each half's 128 columns, the second half's sum through shared memory
      float logit = 0.f;
      for (int k = 0; k < HID / 64; ++k) {
        const int cb = c0h + 32 * k;
        float z[32];
        umma::tmem_ld32(trow + HID + cb, z);
#pragma unroll
        for (int i = 0; i < 32; ++i) logit += fmaxf(z[i] + sb2[cb + i], 0.f) * sw3[cb + i];
      }
      if (half) slog[row] = logit;
      rows_sync();
      if (!half) {
        logit += slog[row] + b3;
        const float p = 1.f / (1.f + __expf(-logit));
        const bool kept = valid && p >= a.thr;
        if (kept) atomicOr(a.keep + (e >> 5), 1u << (e & 31));
        if (valid && a.prob) a.prob[e] = p;
        const u64 jj = valid ? j : ~0ull;
        const unsigned same = __match_any_sync(0xffffffffu, jj);
        const unsigned nt = kept ? f.gsize : 0u, ng = kept ? 1u : 0u;
        if (same == 0xffffffffu) {
          const unsigned sm_ = warp_sum(nt), sg = warp_sum(ng);
          if (lane == 0 && valid && sm_) {
            atomicAdd(a.kept_terms + j, (u64)sm_);
            atomicAdd(a.kept_groups + j, (u64)sg);
          }
        } else if (valid && kept) {
          atomicAdd(a.kept_terms + j, (u64)nt);
          atomicAdd(a.kept_groups + j, (u64)ng);
        }
      }
      umma::tc_fence_before();
      rows_sync();  // the operand, the logits and TMEM are rewritten by the next tile
      umma::tc_fence_after();
    }
    if (fail) {
      s_fail = 1;  // stops the copy warp
      if (tid == 0) {
        atomicOr(a.err, 1u);
        umma::mma_commit(&bar_fin);  // arrives once every MMA issued before has completed
        umma::mbar_wait(&bar_fin, 0);
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// backward: Delta1 = (Delta2 W2) .* relu'(z1), exported as Delta1^T tiles
// ---------------------------------------------------------------------------
struct BwdArgs {
  const uint8_t* W2Timg;  // K-major image of W2^T (B = W2^T: N = in, K = out)
  const uint8_t* D2img;
  const uint32_t* mask1;
  uint8_t* D1T;
  float* grads;           // b1 gradient
  unsigned ntiles;
  unsigned* err;
};

__global__ void __launch_bounds__(THREADS, 1) k_mlp_bwd(BwdArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sW = smem;
  uint8_t* sA = smem + W2_BYTES;
  float* sg_b1 = reinterpret_cast<float*>(sA + A_BYTES);
  __shared__ __align__(8) uint64_t bar_load, bar_a, bar_mma;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  bool failed = false;
  if (tid == 0) {
    umma::mbar_init(&bar_load, 1);
    umma::mbar_init(&bar_a, 1);
    umma::mbar_init(&bar_mma, 1);
    umma::fence_mbar_init();
  }
  for (int i = tid; i < HID; i += THREADS) sg_b1[i] = 0.f;
  __syncthreads();
  if (warp == 0) umma::tmem_alloc(&tmem_slot, 256);
  if (tid == 0) {
    umma::mbar_arrive_expect_tx(&bar_load, W2_BYTES);
    for (uint32_t o = 0; o < W2_BYTES; o += 16384) umma::bulk_g2s(sW + o, a.W2Timg + o, 16384, &bar_load);
  }
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  failed = __syncthreads_or(!umma::mbar_wait(&bar_load, 0)) != 0;
  const uint32_t idesc = umma::idesc_bf16_f32(TILE, HID);
  uint32_t ph_a = 0, ph_m = 0;
  for (unsigned t = blockIdx.x; t < a.ntiles && !failed; t += gridDim.x) {
    if (tid == 0) {
      umma::mbar_arrive_expect_tx(&bar_a, A_BYTES);
      const uint8_t* src = a.D2img + (size_t)t * A_BYTES;
      for (uint32_t o = 0; o < A_BYTES; o += 16384) umma::bulk_g2s(sA + o, src + o, 16384, &bar_a);
    }
    failed = __syncthreads_or(!umma::mbar_wait(&bar_a, ph_a)) != 0;
    ph_a ^= 1u;
    umma::tc_fence_after();
    if (tid == 0 && !failed) {
      umma::gemm_tile(tmem, umma::smem_u32(sA), umma::smem_u32(sW), HID, idesc, false);
      umma::mma_commit(&bar_mma);
    }
    if (failed) break;
    failed = __syncthreads_or(!umma::mbar_wait(&bar_mma, ph_m)) != 0;
    ph_m ^= 1u;
    umma::tc_fence_after();
    const uint32_t* mk = a.mask1 + (size_t)t * MASK_WORDS + tid * 8;
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
    for (int k = 0; k < HID / 32 && !failed; ++k) {
      float z[32];
      umma::tmem_ld32(trow + 32 * k, z);
      const uint32_t m = mk[k];
#pragma unroll
      for (int i = 0; i < 32; ++i) z[i] = ((m >> i) & 1u) ? z[i] : 0.f;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint4 o;
        o.x = pack_bf16(z[8 * q + 0], z[8 * q + 1]);
        o.y = pack_bf16(z[8 * q + 2], z[8 * q + 3]);
        o.z = pack_bf16(z[8 * q + 4], z[8 * q + 5]);
        o.w = pack_bf16(z[8 * q + 6], z[8 * q + 7]);
        *reinterpret_cast<uint4*>(sA + umma::tile_offset(tid, 32 * k + 8 * q, HID)) = o;
      }
      const float cb = lane_column_sum(z);
      atomicAdd(sg_b1 + 32 * k + lane, cb);
    }
    __syncthreads();
    export_transposed(sA, a.D1T + (size_t)t * T256_BYTES);
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
  }
  __syncthreads();
  for (int i = tid; i < HID; i += THREADS) atomicAdd(a.grads + OFF_B1 + i, sg_b1[i]);
  if (failed && tid == 0) atomicOr(a.err, 1u);
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------------------
// split-K gradient products over the batch
// ---------------------------------------------------------------------------
// job 0: dW2[out][in] = sum_rows Delta2[row][out] H1[row][in]   (A = Delta2^T, B = H1^T)
// jobs 1..3: dW1[in][h] = sum_rows X[row][in] Delta1[row][h]    (A = Delta1^T, B = rows of X^T)
struct GradArgs {
  const uint8_t* D2T;
  const uint8_t* H1T;
  const uint8_t* D1T;
  const uint8_t* XT;
  float* grads;
  unsigned ntiles, ksplit;
  unsigned* err;
};

__global__ void __launch_bounds__(THREADS, 1) k_mlp_grad(GradArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;            // 256 x 128 (64 KB)
  uint8_t* sB = smem + T256_BYTES;  // up to 256 x 128 (64 KB)
  __shared__ __align__(8) uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned job = blockIdx.x / a.ksplit, part = blockIdx.x % a.ksplit;
  const unsigned nin = job == 0 ? HID : (job < 3 ? 256u : (unsigned)(KIN - 512));
  const unsigned in0 = job == 0 ? 0u : 256u * (job - 1);
  bool failed = false;
  if (tid == 0) {
    umma::mbar_init(&bar_load, 1);
    umma::mbar_init(&bar_mma, 1);
    umma::fence_mbar_init();
  }
  __syncthreads();
  if (warp == 0) umma::tmem_alloc(&tmem_slot, 512);
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const unsigned t0 = (unsigned)((u64)a.ntiles * part / a.ksplit), t1 = (unsigned)((u64)a.ntiles * (part + 1) / a.ksplit);
  const uint32_t idesc = umma::idesc_bf16_f32(128, nin);
  const uint32_t bbytes = nin * TILE * 2;
  uint32_t ph_l = 0, ph_m = 0;
  for (unsigned t = t0; t < t1 && !failed; ++t) {
    if (tid == 0) {
      const uint8_t* A = (job == 0 ? a.D2T : a.D1T) + (size_t)t * T256_BYTES;
      const uint8_t* B = job == 0 ? a.H1T + (size_t)t * T256_BYTES
                                  : a.XT + (size_t)t * XT_BYTES + (size_t)in0 * TILE * 2;
      umma::mbar_arrive_expect_tx(&bar_load, T256_BYTES + bbytes);
      for (uint32_t o = 0; o < T256_BYTES; o += 16384) umma::bulk_g2s(sA + o, A + o, 16384, &bar_load);
      for (uint32_t o = 0; o < bbytes; o += 16384)
        umma::bulk_g2s(sB + o, B + o, bbytes - o < 16384 ? bbytes - o : 16384, &bar_load);
    }
    failed = __syncthreads_or(!umma::mbar_wait(&bar_load, ph_l)) != 0;
    ph_l ^= 1u;
    umma::tc_fence_after();
    if (tid == 0 && !failed) {
      // two M = 128 halves of the 256 output rows; K = the tile's 128 batch rows
      for (int h = 0; h < 2; ++h)
        umma::gemm_tile(tmem + 256u * h, umma::smem_u32(sA) + h * (T256_BYTES / 2), umma::smem_u32(sB), TILE,
                        idesc, t > t0);
      umma::mma_commit(&bar_mma);
    }
    failed = __syncthreads_or(!umma::mbar_wait(&bar_mma, ph_m)) != 0;
    ph_m ^= 1u;
    umma::tc_fence_before();
    __syncthreads();  // smem operands are reloaded next
    umma::tc_fence_after();
  }
  if (!failed && t1 > t0) {
    for (int h = 0; h < 2; ++h) {
      const unsigned row = 128u * h + 32u * warp + (threadIdx.x & 31);  // out (job 0) or hidden unit (jobs 1-3)
      for (unsigned k = 0; k < nin; k += 32) {
        float z[32];
        umma::tmem_ld32(tmem + 256u * h + ((uint32_t)(32 * warp) << 16) + k, z);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          if (job == 0)
            atomicAdd(a.grads + OFF_W2 + (size_t)row * HID + k + i, z[i]);
          else
            atomicAdd(a.grads + OFF_W1 + (size_t)(in0 + k + i) * HID + row, z[i]);
        }
      }
    }
  }
  if (failed && tid == 0) atomicOr(a.err, 1u);
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// Adam and the BF16 images
// ---------------------------------------------------------------------------
__global__ void k_mlp_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float b1c, float b2c) {
  const float B1 = 0.9f, B2 = 0.999f, EPS = 1e-8f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = B1 * m[i] + (1.f - B1) * gi, vi = B2 * v[i] + (1.f - B2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / b1c) / (sqrtf(vi / b2c) + EPS);
  }
}

__global__ void k_mlp_images(const float* p, __nv_bfloat16* W1b, uint8_t* W2img, uint8_t* W2Timg, uint8_t* Wc) {
  const size_t n1 = (size_t)KIN * HID;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n1 + (size_t)HID * HID;
       i += (size_t)gridDim.x * blockDim.x) {
    if (i < n1) {
      const __nv_bfloat16 w = __float2bfloat16(p[OFF_W1 + i]);
      W1b[i] = w;
      // W1 row `in` (an input), column `h` (a hidden unit): element (h, in % IKC)
      // of the inference chunk in / IKC
      const unsigned in = (unsigned)(i / HID), h = (unsigned)(i % HID);
      if (in < (unsigned)(IN_OCC + NCH1 * IKC)) {
        const unsigned r = in - IN_OCC;
        *reinterpret_cast<__nv_bfloat16*>(Wc + (size_t)(r / IKC) * IB_BYTES + umma::tile_offset(h, r % IKC, IKC)) = w;
      }
    } else {
      const size_t k = i - n1;
      const unsigned o = (unsigned)(k / HID), in = (unsigned)(k % HID);
      const __nv_bfloat16 w = __float2bfloat16(p[OFF_W2 + k]);
      *reinterpret_cast<__nv_bfloat16*>(W2img + umma::tile_offset(o, in, HID)) = w;
      *reinterpret_cast<__nv_bfloat16*>(W2Timg + umma::tile_offset(in, o, HID)) = w;
      // inference chunk NCH1 + in / IKC: element (o, in % IKC)
      *reinterpret_cast<__nv_bfloat16*>(Wc + (size_t)(NCH1 + in / IKC) * IB_BYTES +
                                        umma::tile_offset(o, in % IKC, IKC)) = w;
    }
  }
}

// row maxima of the two-body table, both orientations: vmax[blk][pair][o]
__global__ void k_vmax(const double* __restrict__ V, int M, int P, float* __restrict__ vmax) {
  const size_t n = (size_t)4 * P * M;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int o = (int)(i % M);
    const size_t bp = i / M;
    const int pr = (int)(bp % P), blk = (int)(bp / P);
    double mx = 0.0;
    for (int o2 = 0; o2 < M; ++o2) {
      const int q = spatial_pair(o, o2);
      const double x = fabs(V[((size_t)blk * P + pr) * P + q]), y = fabs(V[((size_t)blk * P + q) * P + pr]);
      mx = fmax(mx, fmax(x, y));
    }
    vmax[i] = (float)mx;
  }
}

}  // namespace sfci

// ===========================================================================
// host side
// ===========================================================================
namespace sfci {

struct Screen {
  Ctx* ctx = nullptr;
  float* params = nullptr;  // NPARAM FP32 masters
  float* grads = nullptr;
  float* am = nullptr;      // Adam moments
  float* av = nullptr;
  __nv_bfloat16* W1b = nullptr;
  uint8_t* W2img = nullptr;
  uint8_t* W2Timg = nullptr;
  uint8_t* Wc = nullptr;     // NCHT B-operand chunks of the inference MMAs
  float* vmax = nullptr;     // this context's table (system 0)
  std::vector<float*> vmaxs;  // one per logged system; [0] = vmax
  float** d_vmaxs = nullptr;  // device copy of the pointers
  uint8_t* ex_sys = nullptr;  // system of each logged source
  unsigned* err = nullptr;
  double* loss = nullptr;
  // training set: sources, group offsets, label bits (grown by appending)
  u64* ex_keys = nullptr;
  double* ex_cc = nullptr;
  u64* ex_goff = nullptr;
  uint32_t* ex_labels = nullptr;
  u64 nsrc = 0, nex = 0, cap_src = 0, cap_ex = 0, npos = 0;
  // per-step training scratch
  uint8_t* tr_buf = nullptr;
  unsigned tr_tiles = 0;
  u64* tile_start = nullptr;
  u64 step = 0;
  uint64_t rng = 0;
  std::vector<void*> owned;
};

static int dev_alloc(Screen& s, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
    cudaGetLastError();
    return set_error(SFCI_ERR_NOMEM, "screen: device allocation failed");
  }
  s.owned.push_back(*p);
  return SFCI_OK;
}
static void dev_free(Screen& s, void* p) {
  if (!p) return;
  for (auto& q : s.owned)
    if (q == p) q = nullptr;
  cudaFree(p);
}

static uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double unif(uint64_t& x) { return (double)(splitmix(x) >> 11) * (1.0 / 9007199254740992.0); }
static double gauss(uint64_t& x) {
  const double u1 = unif(x) + 1e-300, u2 = unif(x);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

static int screen_images(Screen& s) {
  Ctx& c = s.ctx[0];
  SFCI_LAUNCH(c, k_mlp_images, c.sm_count * 4, 256, 0, (const float*)s.params, s.W1b, s.W2img, s.W2Timg, s.Wc);
  return SFCI_OK;
}

static int fwd_smem_bytes() { return (int)(W2_BYTES + A_BYTES + 6 * HID * sizeof(float)); }
static int infer_smem_bytes() { return (int)(A_BYTES + ISTAGES * ISTAGE + (10 * HID + TILE) * sizeof(float)); }
static int bwd_smem_bytes() { return (int)(W2_BYTES + A_BYTES + HID * sizeof(float)); }
static int grad_smem_bytes() { return (int)(2 * T256_BYTES); }

static int screen_kernel_attrs() {
  static bool done = false;
  if (done) return SFCI_OK;
  SFCI_CUDA(cudaFuncSetAttribute(k_mlp_infer<u64>, cudaFuncAttributeMaxDynamicSharedMemorySize, infer_smem_bytes()));
  SFCI_CUDA(cudaFuncSetAttribute(k_mlp_fwd<u64>, cudaFuncAttributeMaxDynamicSharedMemorySize, fwd_smem_bytes()));
  SFCI_CUDA(cudaFuncSetAttribute(k_mlp_infer<K128>, cudaFuncAttributeMaxDynamicSharedMemorySize, infer_smem_bytes()));
  SFCI_CUDA(cudaFuncSetAttribute(k_mlp_fwd<K128>, cudaFuncAttributeMaxDynamicSharedMemorySize, fwd_smem_bytes()));
  SFCI_CUDA(cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, bwd_smem_bytes()));
  SFCI_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, grad_smem_bytes()));
  done = true;
  return SFCI_OK;
}

static int screen_init(Screen& s, uint64_t seed) {
  Ctx& c = *s.ctx;
  int st;
  if ((st = screen_kernel_attrs())) return st;
  void* p = nullptr;
  if ((st = dev_alloc(s, &p, NPARAM * 4 * sizeof(float)))) return st;
  s.params = (float*)p;
  s.grads = s.params + NPARAM;
  s.am = s.grads + NPARAM;
  s.av = s.am + NPARAM;
  if ((st = dev_alloc(s, &p, (size_t)KIN * HID * 2 + 2 * (size_t)W2_BYTES + (size_t)NCHT * IB_BYTES))) return st;
  s.W1b = (__nv_bfloat16*)p;
  s.W2img = (uint8_t*)p + (size_t)KIN * HID * 2;
  s.W2Timg = s.W2img + W2_BYTES;
  s.Wc = s.W2Timg + W2_BYTES;
  if ((st = dev_alloc(s, &p, (size_t)4 * c.P * c.M * sizeof(float)))) return st;
  s.vmax = (float*)p;
  s.vmaxs.push_back(s.vmax);
  if ((st = dev_alloc(s, &p, MAX_SYSTEMS * sizeof(float*)))) return st;
  s.d_vmaxs = (float**)p;
  if ((st = dev_alloc(s, &p, 64))) return st;
  s.err = (unsigned*)p;
  s.loss = (double*)((char*)p + 32);
  // He-style initialisation: about 25 active layer-1 inputs per group
  std::vector<float> h(NPARAM, 0.f);
  s.rng = seed * 0x2545f4914f6cdd1dull + 1;
  for (size_t i = 0; i < (size_t)KIN * HID; ++i) h[OFF_W1 + i] = (float)(gauss(s.rng) * std::sqrt(2.0 / 25.0));
  for (size_t i = 0; i < (size_t)HID * HID; ++i) h[OFF_W2 + i] = (float)(gauss(s.rng) * std::sqrt(2.0 / HID));
  for (int i = 0; i < HID; ++i) h[OFF_W3 + i] = (float)(gauss(s.rng) * std::sqrt(1.0 / HID));
  h[OFF_B3] = -2.0f;  // most groups are dead
  SFCI_CUDA(cudaMemcpyAsync(s.params, h.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice, c.stream));
  SFCI_CUDA(cudaMemsetAsync(s.am, 0, 2 * NPARAM * sizeof(float), c.stream));
  SFCI_CUDA(cudaMemsetAsync(s.err, 0, 64, c.stream));
  SFCI_LAUNCH(c, k_vmax, c.sm_count * 4, 256, 0, (const double*)c.d_V, c.M, c.P, s.vmax);
  SFCI_CUDA(cudaMemcpyAsync(s.d_vmaxs, s.vmaxs.data(), sizeof(float*), cudaMemcpyHostToDevice, c.stream));
  if ((st = screen_images(s))) return st;
  SFCI_CUDA(cudaStreamSynchronize(c.stream));
  return SFCI_OK;
}

static ExView ex_view(Ctx& c, const Screen& s, const u64* keys, const double* cc, const u64* goff, u64 nsrc, u64 nex,
                      const uint8_t* sys = nullptr) {
  ExView x;
  x.keys = keys;
  x.cc = cc;
  x.goff = goff;
  x.nsrc = nsrc;
  x.nex = nex;
  x.W = c.W;
  x.N = c.N;
  x.M = c.M;
  x.P = c.P;
  x.vmaxs = s.d_vmaxs;
  x.sys = sys;
  return x;
}

template <int W>
static int group_offsets(Ctx& c, const u64* keys, u64 n, u64* goff) {
  return group_offsets_impl<W>(c, (const typename KeyOf<W>::T*)keys, n, goff);
}

static int check_err(Screen& s) {
  unsigned e = 0;
  int st = read_words(*s.ctx, s.err, sizeof(unsigned), &e);
  if (st) return st;
  if (e) {
    cudaMemsetAsync(s.err, 0, sizeof(unsigned), s.ctx->stream);
    return set_error(SFCI_ERR_CUDA, "screen: a tensor-core wait timed out");
  }
  return SFCI_OK;
}

// inference over the groups of n sources: keep bits, kept groups and terms per source
static int screen_infer(Ctx& c, Screen& s, const u64* keys, const double* amps, u64 n, double thr, double guard,
                        double floor_, u64** goff_out, uint32_t** keep_out, u64** kterms_out, u64** kgroups_out,
                        u64* nex_out, float* prob) {
  int st;
  u64* goff = (u64*)scratch_get(c, "sc_goff", (n + 1) * sizeof(u64));
  if (!goff) return SFCI_ERR_NOMEM;
  if ((st = c.W == 1 ? group_offsets<1>(c, keys, n, goff) : group_offsets<2>(c, keys, n, goff))) return st;
  u64 nex = 0;
  if ((st = read_words(c, goff + n, sizeof(u64), &nex))) return st;
  const u64 nwords = (nex + 31) / 32;
  // the network's list is built and run in chunks of examples (whole keep words)
  const u64 CHW = (1ull << 25) / 32;
  const u64 chunk = std::min<u64>(nwords, CHW) * 32;
  uint32_t* keep = (uint32_t*)scratch_get(c, "sc_keep", (nwords + 1) * sizeof(uint32_t));
  u64* kt = (u64*)scratch_get(c, "sc_kterms", (2 * (n + 1) + 1) * sizeof(u64));
  u64* le = (u64*)scratch_get(c, "sc_le", (chunk + 1) * sizeof(u64));
  uint32_t* lj = (uint32_t*)scratch_get(c, "sc_lj", (chunk + 1) * sizeof(uint32_t));
  uint4* lf = (uint4*)scratch_get(c, "sc_lf", (chunk + 1) * sizeof(uint4));
  u64* nl = (u64*)scratch_get(c, "sc_nl", sizeof(u64));
  if (!keep || !kt || !le || !lj || !lf || !nl) return SFCI_ERR_NOMEM;
  u64* kg = kt + (n + 1);
  u64* allt = kg + (n + 1);
  SFCI_CUDA(cudaMemsetAsync(kt, 0, (2 * (n + 1) + 1) * sizeof(u64), c.stream));
  FwdArgs a{};
  a.x = ex_view(c, s, keys, amps, goff, n, nex);
  a.W1b = s.W1b;
  a.params = s.params;
  a.W2img = s.W2img;
  a.Wc = s.Wc;
  a.thr = (float)thr;
  a.lguard = guard > 0.0 ? (float)std::log10(guard) : INFINITY;
  a.lfloor = floor_ > 0.0 ? (float)std::log10(floor_) : -INFINITY;
  a.keep = keep;
  a.kept_terms = kt;
  a.kept_groups = kg;
  a.all_terms = allt;
  a.prob = prob;
  a.err = s.err;
  a.list_e = le;
  a.list_j = lj;
  a.list_f = lf;
  for (u64 w0 = 0; w0 < nwords; w0 += CHW) {
    const u64 w1 = std::min<u64>(nwords, w0 + CHW);
    SFCI_CUDA(cudaMemsetAsync(nl, 0, sizeof(u64), c.stream));
    const unsigned cg = (unsigned)std::min<u64>((w1 - w0 + 8 * CW - 1) / (8 * CW), (u64)c.sm_count * 8);
    if (c.W == 1)
      SFCI_LAUNCH(c, k_screen_classify<u64>, cg, 256, 0, a, w0, w1, le, lj, lf, nl);
    else
      SFCI_LAUNCH(c, k_screen_classify<K128>, cg, 256, 0, a, w0, w1, le, lj, lf, nl);
    u64 nlist = 0;
    if ((st = read_words(c, nl, sizeof(u64), &nlist))) return st;
    if (!nlist) continue;
    a.nlist = nlist;
    a.ntiles = (unsigned)((nlist + TILE - 1) / TILE);
    const unsigned grid = std::min<unsigned>(a.ntiles, (unsigned)c.sm_count);
    if (c.W == 1)
      SFCI_LAUNCH(c, k_mlp_infer<u64>, grid, INF_THREADS, infer_smem_bytes(), a);
    else
      SFCI_LAUNCH(c, k_mlp_infer<K128>, grid, INF_THREADS, infer_smem_bytes(), a);
  }
  *goff_out = goff;
  *keep_out = keep;
  *kterms_out = kt;
  *kgroups_out = kg;
  *nex_out = nex;
  return check_err(s);
}

// kept groups of each source in term order: full start and screened start
__global__ void k_screen_lists(const u64* __restrict__ goff, const uint32_t* __restrict__ keep,
                               const u64* __restrict__ koff, const u64* __restrict__ keys, int W, int N, int M, u64 n,
                               uint32_t* __restrict__ kstart, uint32_t* __restrict__ kpre) {
  const int lane = threadIdx.x & 31;
  for (u64 j = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += ((u64)gridDim.x * blockDim.x) >> 5) {
    unsigned a0, a1;
    if (W == 1) {
      spin_counts(keys[j], N, a0, a1);
    } else {
      K128 k;
      k.lo = keys[2 * j];
      k.hi = keys[2 * j + 1];
      spin_counts(k, N, a0, a1);
    }
    const unsigned v0 = M - a0, v1 = M - a1;
    const GroupCounts gc = group_counts(a0, v0, a1, v1);
    unsigned c[6];
    c[0] = 1;
    c[1] = c[0] + a0 * v0;
    c[2] = c[1] + a1 * v1;
    c[3] = c[2] + c2(a0) * c2(v0);
    c[4] = c[3] + c2(a1) * c2(v1);
    c[5] = c[4] + a0 * v0 * a1 * v1;
    const u64 e0 = goff[j], ng = goff[j + 1] - e0;
    u64 out = koff[j];
    uint32_t run = c[2];  // screened index after group 0
    for (u64 b = 0; b < ng; b += 32) {
      const u64 e = e0 + b + lane;
      const bool in = b + lane < ng;
      const bool kept = in && ((keep[e >> 5] >> (e & 31)) & 1u);
      GroupDesc d{};
      if (kept) d = group_desc(gc, c, (unsigned)(b + lane) + 1u);
      const unsigned m = __ballot_sync(0xffffffffu, kept);
      unsigned sz = kept ? d.size : 0u, incl = sz;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (kept) {
        const u64 pos = out + __popc(m & ((1u << lane) - 1u));
        kstart[pos] = d.start;
        kpre[pos] = run + incl - sz;
      }
      run += __shfl_sync(0xffffffffu, incl, 31);
      out += __popc(m);
    }
  }
}

int screen_select(Ctx& c, const void* keys, const double* amps, u64 n, ScreenList* out) {
  Screen& s = *c.screen;
  int st;
  u64 *goff, *kt, *kg, nex = 0;
  uint32_t* keep;
  if ((st = screen_infer(c, s, (const u64*)keys, amps, n, c.screen_thr, c.screen_guard, c.screen_floor, &goff, &keep,
                         &kt, &kg, &nex, nullptr)))
    return st;
  // offsets of the kept-group lists, the largest list, the totals
  u64* koff = (u64*)scratch_get(c, "sc_koff", (n + 1) * sizeof(u64));
  if (!koff) return SFCI_ERR_NOMEM;
  if ((st = scan_excl(c, kg, koff, n))) return st;
  u64 nk = 0;
  if ((st = read_words(c, koff + n, sizeof(u64), &nk))) return st;
  std::vector<u64> kgh(n);
  if ((st = read_words(c, kg, n * sizeof(u64), kgh.data()))) return st;
  u64 gmax = 0;
  for (u64 v : kgh) gmax = std::max(gmax, v);
  u64* kts = (u64*)scratch_get(c, "sc_ktsum", (n + 1) * sizeof(u64));
  if (!kts) return SFCI_ERR_NOMEM;
  if ((st = scan_excl(c, kt, kts, n))) return st;
  u64 tk = 0;
  if ((st = read_words(c, kts + n, sizeof(u64), &tk))) return st;
  uint32_t* ks = (uint32_t*)scratch_get(c, "sc_kstart", (nk + 1) * sizeof(uint32_t));
  uint32_t* kp = (uint32_t*)scratch_get(c, "sc_kpre", (nk + 1) * sizeof(uint32_t));
  if (!ks || !kp) {
    // the previous product's buffers still hold the device: let them go (this
    // product plans after the lists are built) and try once more
    scratch_release_plan(c);
    ks = (uint32_t*)scratch_get(c, "sc_kstart", (nk + 1) * sizeof(uint32_t));
    kp = (uint32_t*)scratch_get(c, "sc_kpre", (nk + 1) * sizeof(uint32_t));
  }
  if (!ks || !kp) return SFCI_ERR_NOMEM;
  if (n) {
    const unsigned grid = (unsigned)std::min<u64>((n * 32 + 255) / 256, (u64)c.sm_count * 16);
    SFCI_LAUNCH(c, k_screen_lists, grid, 256, 0, (const u64*)goff, (const uint32_t*)keep, (const u64*)koff,
                (const u64*)keys, c.W, c.N, c.M, n, ks, kp);
  }
  out->start = ks;
  out->pre = kp;
  out->off = koff;
  out->kept_terms = kt;
  out->gmax = (unsigned)gmax;
  out->groups = nex;
  out->kept_groups = nk;
  out->kept_terms_total = tk;
  u64 all = 0;
  if ((st = read_words(c, kg + (n + 1), sizeof(u64), &all))) return st;
  c.screen_stats[0] += nex;
  c.screen_stats[1] += nk;
  c.screen_stats[2] += tk;
  c.screen_stats[3] += 1;
  c.screen_stats[4] += all;
  return SFCI_OK;
}

// ---- training set --------------------------------------------------------------
template <class T>
static int grow(Screen& s, T** p, u64 used, u64 want, u64& cap, u64 elems_per) {
  if (want <= cap) return SFCI_OK;
  u64 nc = std::max<u64>(want, cap * 2);
  void* q = nullptr;
  int st = dev_alloc(s, &q, nc * elems_per * sizeof(T));
  if (st) return st;
  if (*p && used) SFCI_CUDA(cudaMemcpyAsync(q, *p, used * elems_per * sizeof(T), cudaMemcpyDeviceToDevice, s.ctx->stream));
  SFCI_CUDA(cudaStreamSynchronize(s.ctx->stream));
  dev_free(s, *p);
  *p = (T*)q;
  cap = nc;
  return SFCI_OK;
}

__global__ void k_add_u64(u64* p, u64 n, u64 v) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) p[i] += v;
}
__global__ void k_abs_copy(double* dst, const double* src, u64 n) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) dst[i] = fabs(src[i]);
}

// label log of one product: sources = the product's input (at most its Nd),
// labels from its output.  The vectors may live on another context over a
// Hamiltonian with the same number of orbitals: its term groups are labelled
// there, and its integral-bound table joins the screen's as a new system.
static int screen_log(Screen& s, const Vec& in, const Vec& out, double min_term, u64* nex_out, u64* npos_out) {
  Ctx& c = *s.ctx;
  Ctx& vc = *in.ctx;
  int st;
  if (out.ctx != in.ctx) return set_error(SFCI_ERR_ARG, "screen log: input and output on different contexts");
  if (vc.N != c.N || vc.M != c.M || vc.W != c.W)
    return set_error(SFCI_ERR_ARG, "screen log: the vectors' system has another number of orbitals");
  const u64 n = in.len;
  const u64* keys = in.keys;
  const double* amps = in.amps;
  // the product multiplies the top Nd of its input by |amplitude| only: the
  // logged sources must be exactly the determinants the product used
  if (n > vc.opts.Nd) return set_error(SFCI_ERR_UNSUPPORTED, "screen log: input longer than Nd; log its top-Nd slice");
  if (n == 0) {
    *nex_out = 0;
    *npos_out = 0;
    return SFCI_OK;
  }
  uint8_t sys = 0;
  if (&vc != &c) {
    if (s.vmaxs.size() >= (size_t)MAX_SYSTEMS) return set_error(SFCI_ERR_CAPACITY, "screen log: 64 systems at most");
    void* p = nullptr;
    if ((st = dev_alloc(s, &p, (size_t)4 * c.P * c.M * sizeof(float)))) return st;
    SFCI_LAUNCH(vc, k_vmax, vc.sm_count * 4, 256, 0, (const double*)vc.d_V, vc.M, vc.P, (float*)p);
    SFCI_CUDA(cudaStreamSynchronize(vc.stream));
    s.vmaxs.push_back((float*)p);
    SFCI_CUDA(cudaMemcpyAsync(s.d_vmaxs, s.vmaxs.data(), s.vmaxs.size() * sizeof(float*), cudaMemcpyHostToDevice,
                              c.stream));
    sys = (uint8_t)(s.vmaxs.size() - 1);
  }
  u64* goff = (u64*)scratch_get(vc, "sc_lgoff", (n + 1) * sizeof(u64));
  if (!goff) return SFCI_ERR_NOMEM;
  if ((st = vc.W == 1 ? group_offsets<1>(vc, keys, n, goff) : group_offsets<2>(vc, keys, n, goff))) return st;
  u64 ne = 0;
  if ((st = read_words(vc, goff + n, sizeof(u64), &ne))) return st;
  if ((st = grow(s, &s.ex_keys, s.nsrc * c.W, (s.nsrc + n) * c.W, s.cap_src, 1))) return st;
  // per-source feature, offsets and system: reallocated at the new length
  void* q = nullptr;
  if ((st = dev_alloc(s, &q, (s.nsrc + n) * sizeof(double)))) return st;
  double* ncc = (double*)q;
  if ((st = dev_alloc(s, &q, (s.nsrc + n + 1) * sizeof(u64)))) return st;
  u64* ngo = (u64*)q;
  if ((st = dev_alloc(s, &q, s.nsrc + n))) return st;
  uint8_t* nsy = (uint8_t*)q;
  if (s.nsrc) {
    SFCI_CUDA(cudaMemcpyAsync(ncc, s.ex_cc, s.nsrc * sizeof(double), cudaMemcpyDeviceToDevice, vc.stream));
    SFCI_CUDA(cudaMemcpyAsync(ngo, s.ex_goff, s.nsrc * sizeof(u64), cudaMemcpyDeviceToDevice, vc.stream));
    SFCI_CUDA(cudaMemcpyAsync(nsy, s.ex_sys, s.nsrc, cudaMemcpyDeviceToDevice, vc.stream));
  }
  SFCI_CUDA(cudaMemsetAsync(nsy + s.nsrc, sys, n, vc.stream));
  SFCI_CUDA(cudaMemcpyAsync(s.ex_keys + s.nsrc * c.W, keys, n * c.W * sizeof(u64), cudaMemcpyDeviceToDevice,
                            vc.stream));
  SFCI_LAUNCH(vc, k_abs_copy, vc.sm_count * 4, 256, 0, ncc + s.nsrc, amps, n);
  SFCI_CUDA(cudaMemcpyAsync(ngo + s.nsrc, goff, (n + 1) * sizeof(u64), cudaMemcpyDeviceToDevice, vc.stream));
  SFCI_LAUNCH(vc, k_add_u64, vc.sm_count * 4, 256, 0, ngo + s.nsrc, n + 1, s.nex);
  SFCI_CUDA(cudaStreamSynchronize(vc.stream));
  dev_free(s, s.ex_cc);
  dev_free(s, s.ex_goff);
  dev_free(s, s.ex_sys);
  s.ex_cc = ncc;
  s.ex_goff = ngo;
  s.ex_sys = nsy;
  // label words: the new examples start at bit s.nex; they are computed into a
  // word-aligned scratch and merged bit by bit into the global array
  const u64 words_old = (s.nex + 31) / 32, words_new = (s.nex + ne + 31) / 32 + 1;
  if ((st = grow(s, &s.ex_labels, words_old, words_new, s.cap_ex, 1))) return st;
  SFCI_CUDA(cudaMemsetAsync(s.ex_labels + words_old, 0, (words_new - words_old) * sizeof(uint32_t), c.stream));
  uint32_t* lab = (uint32_t*)scratch_get(vc, "sc_lab", ((ne + 31) / 32 + 1) * sizeof(uint32_t));
  if (!lab) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemsetAsync(lab, 0, ((ne + 31) / 32 + 1) * sizeof(uint32_t), vc.stream));
  if ((st = vc.W == 1 ? label_impl<1>(vc, (const u64*)keys, amps, n, goff, out, lab, min_term)
                      : label_impl<2>(vc, (const K128*)keys, amps, n, goff, out, lab, min_term)))
    return st;
  // shift the new words into place (s.nex is not word-aligned in general)
  {
    std::vector<uint32_t> hl((ne + 31) / 32 + 1), hg(words_new - (s.nex / 32));
    if ((st = read_words(vc, lab, hl.size() * sizeof(uint32_t), hl.data()))) return st;
    if ((st = read_words(c, s.ex_labels + s.nex / 32, hg.size() * sizeof(uint32_t), hg.data()))) return st;
    const unsigned sh = (unsigned)(s.nex & 31);
    u64 pos = 0;
    for (u64 i = 0; i < ne; ++i) {
      if ((hl[i >> 5] >> (i & 31)) & 1u) {
        const u64 b = sh + i;
        hg[b >> 5] |= 1u << (b & 31);
        ++pos;
      }
    }
    SFCI_CUDA(cudaMemcpyAsync(s.ex_labels + s.nex / 32, hg.data(), hg.size() * sizeof(uint32_t),
                              cudaMemcpyHostToDevice, c.stream));
    SFCI_CUDA(cudaStreamSynchronize(c.stream));
    s.npos += pos;
    *npos_out = pos;
  }
  s.nsrc += n;
  s.nex += ne;
  *nex_out = ne;
  return SFCI_OK;
}

static int screen_train(Screen& s, int steps, unsigned batch_tiles, double lr, double pos_weight, int sequential,
                        double* loss_out) {
  Ctx& c = *s.ctx;
  int st;
  if (s.nex < TILE) return set_error(SFCI_ERR_ARG, "screen train: fewer than 128 logged examples");
  if (batch_tiles == 0) return set_error(SFCI_ERR_ARG, "screen train: empty batch");
  if (batch_tiles > s.tr_tiles) {
    dev_free(s, s.tr_buf);
    dev_free(s, s.tile_start);
    s.tr_buf = nullptr;
    s.tile_start = nullptr;
    void* p = nullptr;
    const size_t per = 4 * (size_t)T256_BYTES + XT_BYTES + MASK_WORDS * 4;
    if ((st = dev_alloc(s, &p, per * batch_tiles))) return st;
    s.tr_buf = (uint8_t*)p;
    if ((st = dev_alloc(s, &p, batch_tiles * sizeof(u64)))) return st;
    s.tile_start = (u64*)p;
    s.tr_tiles = batch_tiles;
  }
  const unsigned nt = batch_tiles;
  uint8_t* H1T = s.tr_buf;
  uint8_t* D2img = H1T + (size_t)nt * T256_BYTES;
  uint8_t* D2T = D2img + (size_t)nt * A_BYTES;
  uint8_t* D1T = D2T + (size_t)nt * T256_BYTES;
  uint8_t* XT = D1T + (size_t)nt * T256_BYTES;
  uint32_t* mask1 = (uint32_t*)(XT + (size_t)nt * XT_BYTES);
  std::vector<u64> ts(nt);
  const ExView xv = ex_view(c, s, s.ex_keys, s.ex_cc, s.ex_goff, s.nsrc, s.nex, s.ex_sys);
  double loss_sum = 0.0;
  const unsigned ksplit = std::max<unsigned>(1, std::min<unsigned>(nt, (unsigned)c.sm_count / 4));
  for (int it = 0; it < steps; ++it) {
    for (unsigned t = 0; t < nt; ++t)
      ts[t] = sequential ? ((u64)t * TILE) % s.nex : (u64)(unif(s.rng) * (double)(s.nex - TILE + 1));
    SFCI_CUDA(cudaMemcpyAsync(s.tile_start, ts.data(), nt * sizeof(u64), cudaMemcpyHostToDevice, c.stream));
    SFCI_CUDA(cudaMemsetAsync(s.grads, 0, NPARAM * sizeof(float), c.stream));
    SFCI_CUDA(cudaMemsetAsync(s.loss, 0, sizeof(double), c.stream));
    FwdArgs a{};
    a.x = xv;
    a.W1b = s.W1b;
    a.params = s.params;
    a.W2img = s.W2img;
    a.ntiles = nt;
    a.tile_start = s.tile_start;
    a.labels = s.ex_labels;
    a.pos_weight = (float)pos_weight;
    a.inv_batch = 1.f / (float)(nt * TILE);
    a.H1T = H1T;
    a.D2img = D2img;
    a.D2T = D2T;
    a.XT = XT;
    a.mask1 = mask1;
    a.grads = s.grads;
    a.loss = s.loss;
    a.err = s.err;
    const unsigned grid = std::min<unsigned>(nt, (unsigned)c.sm_count);
    if (c.W == 1)
      SFCI_LAUNCH(c, (k_mlp_fwd<u64>), grid, THREADS, fwd_smem_bytes(), a);
    else
      SFCI_LAUNCH(c, (k_mlp_fwd<K128>), grid, THREADS, fwd_smem_bytes(), a);
    BwdArgs b{};
    b.W2Timg = s.W2Timg;
    b.D2img = D2img;
    b.mask1 = mask1;
    b.D1T = D1T;
    b.grads = s.grads;
    b.ntiles = nt;
    b.err = s.err;
    SFCI_LAUNCH(c, k_mlp_bwd, grid, THREADS, bwd_smem_bytes(), b);
    GradArgs g{};
    g.D2T = D2T;
    g.H1T = H1T;
    g.D1T = D1T;
    g.XT = XT;
    g.grads = s.grads;
    g.ntiles = nt;
    g.ksplit = ksplit;
    g.err = s.err;
    SFCI_LAUNCH(c, k_mlp_grad, 4 * ksplit, THREADS, grad_smem_bytes(), g);
    ++s.step;
    if (lr > 0.0) {
      const float b1c = 1.f - std::pow(0.9f, (float)s.step), b2c = 1.f - std::pow(0.999f, (float)s.step);
      SFCI_LAUNCH(c, k_mlp_adam, c.sm_count * 4, 256, 0, s.params, (const float*)s.grads, s.am, s.av, NPARAM,
                  (float)lr, b1c, b2c);
      if ((st = screen_images(s))) return st;
    }
    double l = 0.0;
    if ((st = read_words(c, s.loss, sizeof(double), &l))) return st;
    loss_sum = l / (double)(nt * TILE);
  }
  if (loss_out) *loss_out = loss_sum;
  return check_err(s);
}

}  // namespace sfci

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct sfci_screen {
  sfci::Screen s;
};

using namespace sfci;

namespace sfci {
void screen_orphan(Screen* s) {
  if (!s) return;
  if (s->ctx) {
    cudaStreamSynchronize(s->ctx->stream);
    if (s->ctx->screen == s) s->ctx->screen = nullptr;
    s->ctx->screens.erase(s);
  }
  for (void*& p : s->owned)
    if (p) {
      cudaFree(p);
      p = nullptr;
    }
  s->ctx = nullptr;
}
}  // namespace sfci

extern "C" int sfci_screen_create(sfci_ctx* ctx, uint64_t seed, sfci_screen** out) {
  if (!ctx || !out) return set_error(SFCI_ERR_ARG, "sfci_screen_create: null argument");
  *out = nullptr;
  sfci_screen* x = new sfci_screen();
  x->s.ctx = &ctx->c;
  int st = screen_init(x->s, seed);
  if (st) {
    for (void* p : x->s.owned)
      if (p) cudaFree(p);
    delete x;
    return st;
  }
  ctx->c.screens.insert(&x->s);
  *out = x;
  return SFCI_OK;
}

// A screen whose context was destroyed first is an orphan: its device memory
// went with the context, and only the handle is left to free.
extern "C" int sfci_screen_destroy(sfci_screen* x) {
  if (!x) return SFCI_OK;
  screen_orphan(&x->s);
  delete x;
  return SFCI_OK;
}

extern "C" int sfci_screen_log(sfci_screen* x, const sfci_vec* in, const sfci_vec* out, double min_term,
                               uint64_t* examples, uint64_t* positives) {
  if (!x || !in || !out) return set_error(SFCI_ERR_ARG, "sfci_screen_log: null argument");
  if (!x->s.ctx) return set_error(SFCI_ERR_ARG, "sfci_screen_log: the screen's context was destroyed");
  if (!in->v.ctx || !out->v.ctx) return set_error(SFCI_ERR_ARG, "sfci_screen_log: vector of a destroyed context");
  u64 ne = 0, np = 0;
  int st = screen_log(x->s, in->v, out->v, min_term, &ne, &np);
  if (examples) *examples = ne;
  if (positives) *positives = np;
  return st;
}

extern "C" int sfci_screen_train(sfci_screen* x, int steps, int batch_tiles, double lr, double pos_weight,
                                 int sequential, double* loss) {
  if (!x || steps < 0 || batch_tiles <= 0) return set_error(SFCI_ERR_ARG, "sfci_screen_train: bad argument");
  if (!x->s.ctx) return set_error(SFCI_ERR_ARG, "sfci_screen_train: the screen's context was destroyed");
  return screen_train(x->s, steps, (unsigned)batch_tiles, lr, pos_weight, sequential, loss);
}

extern "C" int sfci_screen_stats(const sfci_screen* x, uint64_t* sources, uint64_t* examples, uint64_t* positives,
                                 uint64_t* steps) {
  if (!x) return set_error(SFCI_ERR_ARG, "sfci_screen_stats: null screen");
  if (sources) *sources = x->s.nsrc;
  if (examples) *examples = x->s.nex;
  if (positives) *positives = x->s.npos;
  if (steps) *steps = x->s.step;
  return SFCI_OK;
}

extern "C" int sfci_screen_predict(sfci_screen* x, const sfci_vec* in, double threshold, uint64_t* groups,
                                   uint64_t* kept_groups, uint64_t* kept_terms, float* prob_host,
                                   uint64_t prob_cap) {
  if (!x || !in) return set_error(SFCI_ERR_ARG, "sfci_screen_predict: null argument");
  if (!x->s.ctx || in->v.ctx != x->s.ctx)
    return set_error(SFCI_ERR_ARG, "sfci_screen_predict: a vector of the screen's own (live) context");
  Screen& s = x->s;
  Ctx& c = *s.ctx;
  int st;
  u64 *goff, *kt, *kg, nex = 0;
  uint32_t* keep;
  float* prob = nullptr;
  if (prob_host) {
    u64 ng = 0;
    {
      u64* go = (u64*)scratch_get(c, "sc_goff", (in->v.len + 1) * sizeof(u64));
      if (!go) return SFCI_ERR_NOMEM;
      if ((st = c.W == 1 ? group_offsets<1>(c, in->v.keys, in->v.len, go) : group_offsets<2>(c, in->v.keys, in->v.len, go)))
        return st;
      if ((st = read_words(c, go + in->v.len, sizeof(u64), &ng))) return st;
    }
    if (ng > prob_cap) return set_error(SFCI_ERR_CAPACITY, "sfci_screen_predict: prob_cap below the group count");
    prob = (float*)scratch_get(c, "sc_prob", (ng + 1) * sizeof(float));
    if (!prob) return SFCI_ERR_NOMEM;
  }
  if ((st = screen_infer(c, s, in->v.keys, in->v.amps, in->v.len, threshold, 0.0, 0.0, &goff, &keep, &kt, &kg, &nex,
                         prob)))
    return st;
  std::vector<u64> a(in->v.len), b(in->v.len);
  if ((st = read_words(c, kt, in->v.len * sizeof(u64), a.data()))) return st;
  if ((st = read_words(c, kg, in->v.len * sizeof(u64), b.data()))) return st;
  u64 ta = 0, tb = 0;
  for (u64 i = 0; i < in->v.len; ++i) {
    ta += a[i];
    tb += b[i];
  }
  if (groups) *groups = nex;
  if (kept_groups) *kept_groups = tb;
  if (kept_terms) *kept_terms = ta;
  if (prob_host && nex) SFCI_CUDA(cudaMemcpy(prob_host, prob, nex * sizeof(float), cudaMemcpyDeviceToHost));
  return SFCI_OK;
}

extern "C" int sfci_screen_params(sfci_screen* x, float* get, const float* set, uint64_t n) {
  if (!x) return set_error(SFCI_ERR_ARG, "sfci_screen_params: null screen");
  if (n != NPARAM) return set_error(SFCI_ERR_ARG, "sfci_screen_params: n must be the parameter count");
  if (!x->s.ctx) return set_error(SFCI_ERR_ARG, "sfci_screen_params: the screen's context was destroyed");
  Ctx& c = *x->s.ctx;
  if (get) {
    SFCI_CUDA(cudaStreamSynchronize(c.stream));
    SFCI_CUDA(cudaMemcpy(get, x->s.params, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  }
  if (set) {
    SFCI_CUDA(cudaMemcpyAsync(x->s.params, set, NPARAM * sizeof(float), cudaMemcpyHostToDevice, c.stream));
    int st = screen_images(x->s);
    if (st) return st;
    SFCI_CUDA(cudaStreamSynchronize(c.stream));
  }
  return SFCI_OK;
}

extern "C" int sfci_screen_grads(sfci_screen* x, float* get, uint64_t n) {
  if (!x || !get) return set_error(SFCI_ERR_ARG, "sfci_screen_grads: null argument");
  if (n != NPARAM) return set_error(SFCI_ERR_ARG, "sfci_screen_grads: n must be the parameter count");
  if (!x->s.ctx) return set_error(SFCI_ERR_ARG, "sfci_screen_grads: the screen's context was destroyed");
  SFCI_CUDA(cudaStreamSynchronize(x->s.ctx->stream));
  SFCI_CUDA(cudaMemcpy(get, x->s.grads, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  return SFCI_OK;
}

extern "C" uint64_t sfci_screen_param_count(void) { return NPARAM; }

extern "C" int sfci_ctx_set_screen(sfci_ctx* ctx, sfci_screen* x, double threshold) {
  if (!ctx) return set_error(SFCI_ERR_ARG, "sfci_ctx_set_screen: null context");
  if (x && x->s.ctx != &ctx->c) return set_error(SFCI_ERR_ARG, "sfci_ctx_set_screen: screen of another context");
  if (!(threshold >= 0.0 && threshold <= 1.0)) return set_error(SFCI_ERR_ARG, "sfci_ctx_set_screen: threshold in [0, 1]");
  ctx->c.screen = x ? &x->s : nullptr;
  ctx->c.screen_thr = threshold;
  return SFCI_OK;
}

extern "C" int sfci_ctx_set_screen_guard(sfci_ctx* ctx, double guard) {
  if (!ctx) return set_error(SFCI_ERR_ARG, "sfci_ctx_set_screen_guard: null context");
  if (!(guard >= 0.0) || std::isinf(guard)) return set_error(SFCI_ERR_ARG, "sfci_ctx_set_screen_guard: guard >= 0, finite");
  ctx->c.screen_guard = guard;
  return SFCI_OK;
}

extern "C" int sfci_ctx_set_screen_floor(sfci_ctx* ctx, double floor_) {
  if (!ctx) return set_error(SFCI_ERR_ARG, "sfci_ctx_set_screen_floor: null context");
  if (!(floor_ >= 0.0) || std::isinf(floor_)) return set_error(SFCI_ERR_ARG, "sfci_ctx_set_screen_floor: floor >= 0, finite");
  ctx->c.screen_floor = floor_;
  return SFCI_OK;
}

extern "C" int sfci_ctx_screen_stats(const sfci_ctx* ctx, uint64_t* out5) {
  if (!ctx || !out5) return set_error(SFCI_ERR_ARG, "sfci_ctx_screen_stats: null argument");
  for (int i = 0; i < 5; ++i) out5[i] = ctx->c.screen_stats[i];
  return SFCI_OK;
}

// Fifth-generation tensor-core primitives for sm_103a (tcgen05 + TMEM), inline PTX.
//
// Every GEMM here is D[M x N] (+)= A[M x K] * B[N x K]^T with BF16 operands in
// shared memory, both K-major, no swizzle, and an FP32 accumulator in tensor
// memory (TMEM).  An operand tile of R rows and K columns is stored as 8 x 8
// "core matrices" (8 rows of 16 bytes, 128 contiguous bytes): core matrix
// (row group g, column group c) starts at byte g * (K / 8) * 128 + c * 128, and
// element (r, k) lies at byte 16 * (r % 8) + 2 * (k % 8) inside it.  In the
// shared-memory descriptor this is a leading-dimension byte offset (between
// core matrices adjacent in K) of 128 and a stride-dimension byte offset
// (between adjacent 8-row groups) of K * 16.
//
// One elected thread issues the MMAs and commits them to an mbarrier; the
// accumulator row i of an M = 128 tile is TMEM lane i, column j is TMEM column
// base + j, and warp w of the CTA's first warpgroup reads lanes 32w .. 32w+31.
// Every wait on an mbarrier is bounded: on timeout the caller sets an error
// flag and leaves its loops instead of spinning forever.
#pragma once

#include <cstdint>

namespace sfci {
namespace umma {

constexpr int CORE_BYTES = 128;  // one 8 x 8 BF16 core matrix

// byte offset of element (r, k) in a K-major no-swizzle tile with K columns
__host__ __device__ __forceinline__ uint32_t tile_offset(uint32_t r, uint32_t k, uint32_t K) {
  return (r >> 3) * (K >> 3) * CORE_BYTES + (k >> 3) * CORE_BYTES + (r & 7u) * 16u + (k & 7u) * 2u;
}

// instruction descriptor, kind::f16: BF16 x BF16 -> FP32, A and B K-major
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t M, uint32_t N) {
  return (1u << 4)            // D format: F32
         | (1u << 7)          // A format: BF16
         | (1u << 10)         // B format: BF16
         | ((N >> 3) << 17)   // N / 8
         | ((M >> 4) << 24);  // M / 16
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor (K-major, no swizzle) of a tile starting at
// shared address `addr` with K columns
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t K) {
  const uint64_t lbo = CORE_BYTES >> 4, sbo = (uint64_t)(K * 16u) >> 4;
  return (uint64_t)((addr >> 4) & 0x3fffu) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase with parity `phase` to complete
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, uint32_t max_iter = 1u << 24) {
  for (uint32_t i = 0; i < max_iter; ++i) {
    if (mbar_try_wait(bar, phase)) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// bulk (TMA, non-tensor) copy global -> shared, completing on an mbarrier;
// 16-byte aligned addresses, size a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// generic-proxy shared-memory writes -> visible to the tensor core's async proxy
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation by one full warp; the address lands in *slot (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) = A * B^T (+ D when accumulate)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}
// arrive on *bar once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// K-loop of one tile product: A (M x K) at shared address a, B (N x K) at b,
// both K-major no-swizzle; each instruction consumes K = 16 (two core matrices)
__device__ __forceinline__ void gemm_tile(uint32_t d_tmem, uint32_t a, uint32_t b, uint32_t K, uint32_t idesc,
                                          bool accumulate) {
  for (uint32_t k = 0; k < K; k += 16) {
    const uint32_t off = (k >> 3) * CORE_BYTES;
    mma_bf16(d_tmem, sdesc(a + off, K), sdesc(b + off, K), idesc, accumulate || k > 0);
  }
}

// 32 consecutive FP32 columns of this thread's TMEM lane (lane = 32 * warp + lane id)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  // the load and its wait in one statement: no use of r can be scheduled between them
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
#endif  // __CUDACC__

}  // namespace umma
}  // namespace sfci

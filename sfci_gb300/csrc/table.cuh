// Open-addressing key tables in global memory shared by the SpMSpV support set
// and the subspace index: 128-bit compare-and-swap, L2 loads of keys, and the
// lookup of a key's slot.
#pragma once

#include "common.cuh"

namespace sfci {

#ifdef __CUDACC__
// 128-bit compare-and-swap (generic address, sm_90+)
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
  unsigned slot = (unsigned)slot_hash(key) & mask;
  const KT empty = key_empty<KT>();
  for (unsigned probe = 0; probe <= mask; ++probe) {
    KT cur = ldcg_key(tk + slot);
    if (key_eq(cur, key)) return (int)slot;
    if (key_eq(cur, empty)) return -1;
    slot = (slot + 1) & mask;
  }
  return -1;
}

#endif  // __CUDACC__

}  // namespace sfci

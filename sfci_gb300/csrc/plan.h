// Device-memory plan of one SpMSpV (host logic, header-only so that the host
// tests compile it as it is).
#pragma once

#include <algorithm>
#include <vector>

namespace sfci {

typedef unsigned long long plan_u64;

struct MemPlan {
  plan_u64 C1 = 0;  // level-1 term capacity: the terms of one generation pass
  plan_u64 C2 = 0;  // level-2 group capacity (partition ping-pong buffer)
  plan_u64 SC = 0;  // survivor capacity (held twice: the key sort before a cut goes through a copy)
  int passes = 0;
};

// Generation passes over the level-1 bins for a level-1 capacity c1: consecutive
// bins are grouped greedily while their terms fit (binoff: nb1 + 1 offsets).
inline int plan_passes(const std::vector<plan_u64>& binoff, unsigned nb1, plan_u64 c1) {
  int np = 0;
  for (unsigned lo = 0; lo < nb1; ++np) {
    unsigned hi = lo + 1;
    while (hi < nb1 && binoff[hi + 1] - binoff[lo] <= c1) ++hi;
    lo = hi;
  }
  return np;
}

// Split `avail` terms of device memory between the level-1 buffer, the level-2
// buffer and the survivors (cap = output capacity, at most T).  Every generation
// pass regenerates all T terms, so the plan takes the fewest passes first; among
// plans with that many, the largest level-2 groups (fewer, fuller partition and
// merge launches: 1/16 to 1/128 of the budget, at least 2^20 terms).  Without
// partition levels the level-2 buffer is one group buffer of 1/6 of the budget.
// false: the budget cannot hold a single level-1 bin.
inline bool plan_memory(const std::vector<plan_u64>& binoff, unsigned nb1, plan_u64 T, plan_u64 avail, plan_u64 cap,
                        plan_u64 maxbin, bool partition, MemPlan& out) {
  out = MemPlan();
  for (const int div : {6, 16, 24, 32, 48, 64, 96, 128}) {
    if (partition == (div == 6)) continue;
    const plan_u64 share = partition ? std::max<plan_u64>(avail / div, 1ull << 20) : avail / div;
    const plan_u64 c2 = std::max<plan_u64>(maxbin, std::min<plan_u64>(T, share));
    const plan_u64 sc = cap + std::min<plan_u64>(c2, T);
    const plan_u64 l2 = partition ? c2 : 0;
    plan_u64 c1 = T;
    if (c1 + l2 + 2 * sc > avail) {
      if (avail < l2 + 2 * sc + maxbin) continue;
      c1 = avail - l2 - 2 * sc;
    }
    if (c1 < maxbin || c2 < maxbin) continue;
    const int np = plan_passes(binoff, nb1, c1);
    if (out.passes == 0 || np < out.passes) {
      out.C1 = c1;
      out.C2 = c2;
      out.SC = sc;
      out.passes = np;
    }
  }
  return out.passes > 0;
}

// Class passes: the 256 alpha classes' term counts hh, the level-1 capacity c1.
// Passes are runs of aligned blocks of 2^k classes (the generator enumerates a
// pass's spin-0 doubles block by block): k three bits below the widest block
// size whose blocks all fit c1 (0 when even single classes do not), consecutive
// blocks while they fit and while their runs (occupied spin-0 pairs x blocks,
// at most nop_max x blocks) fit run_cap.  A block larger than c1 is a pass of
// its own (the caller splits it further into bin passes).  Empty passes are
// dropped.
struct ClassPass {
  unsigned lo, hi;  // classes [lo, hi): aligned blocks of 2^k
  plan_u64 terms;
  int k;
};

inline std::vector<ClassPass> plan_class_passes(const std::vector<plan_u64>& hh, plan_u64 c1, unsigned nop_max,
                                                unsigned run_cap) {
  const unsigned NC = 256;
  auto block_sum = [&](unsigned lo, int kb) {
    plan_u64 t = 0;
    for (unsigned cc = lo; cc < lo + (1u << kb); ++cc) t += hh[cc];
    return t;
  };
  int kfit = -1;
  for (int kb = 8; kb >= 0 && kfit < 0; --kb) {
    bool fits = true;
    for (unsigned lo = 0; lo < NC && fits; lo += 1u << kb) fits = block_sum(lo, kb) <= c1;
    if (fits) kfit = kb;
  }
  const int kc = std::max(0, kfit - 3);
  const unsigned nblk_cap = std::max(1u, run_cap / std::max(1u, nop_max));
  std::vector<ClassPass> out;
  unsigned lo = 0;
  while (lo < NC) {
    unsigned hi = lo + (1u << kc);
    plan_u64 sum = block_sum(lo, kc);
    while (hi < NC && ((hi - lo) >> kc) < nblk_cap && sum + block_sum(hi, kc) <= c1) {
      sum += block_sum(hi, kc);
      hi += 1u << kc;
    }
    if (sum) out.push_back({lo, hi, sum, kc});
    lo = hi;
  }
  return out;
}

}  // namespace sfci

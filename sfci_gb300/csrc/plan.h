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

}  // namespace sfci

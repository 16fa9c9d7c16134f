// Test harness only: the SpMSpV device-memory plan (csrc/plan.h) behind a C ABI.
#include <vector>

#include "plan.h"

extern "C" int pl_plan(const unsigned long long* binoff, unsigned nb1, unsigned long long T, unsigned long long avail,
                       unsigned long long cap, unsigned long long maxbin, int partition, unsigned long long* out) {
  std::vector<unsigned long long> b(binoff, binoff + nb1 + 1);
  sfci::MemPlan p;
  const bool ok = sfci::plan_memory(b, nb1, T, avail, cap, maxbin, partition != 0, p);
  out[0] = p.C1;
  out[1] = p.C2;
  out[2] = p.SC;
  out[3] = (unsigned long long)p.passes;
  return ok ? 1 : 0;
}

extern "C" int pl_passes(const unsigned long long* binoff, unsigned nb1, unsigned long long c1) {
  std::vector<unsigned long long> b(binoff, binoff + nb1 + 1);
  return sfci::plan_passes(b, nb1, c1);
}

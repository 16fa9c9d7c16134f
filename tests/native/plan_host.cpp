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

// class passes: out[4 * i + 0..3] = lo, hi, terms, k; returns the pass count (at most max_out)
extern "C" int pl_class(const unsigned long long* hh, unsigned long long c1, unsigned nop_max, unsigned run_cap,
                        unsigned long long* out, int max_out) {
  std::vector<unsigned long long> h(hh, hh + 256);
  const std::vector<sfci::ClassPass> p = sfci::plan_class_passes(h, c1, nop_max, run_cap);
  const int n = (int)p.size() < max_out ? (int)p.size() : max_out;
  for (int i = 0; i < n; ++i) {
    out[4 * i] = p[i].lo;
    out[4 * i + 1] = p[i].hi;
    out[4 * i + 2] = p[i].terms;
    out[4 * i + 3] = (unsigned long long)p[i].k;
  }
  return (int)p.size();
}

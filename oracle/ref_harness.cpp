// Test infrastructure only: a C-ABI harness around the reference SFCI SpMSpV
// sources (functions.cpp, bitstr.cpp, introsort.cpp), compiled unmodified from
// the reference tree into oracle/_ref/libsfci_ref.so by oracle/build_ref.sh.
// Tests and the golden-fixture script use it to pin the oracle restatement;
// nothing in the product links or loads it.
//
// The globals below are the ones src/main.cpp:12-40 defines; ref_setup repeats
// the set-up of src/main.cpp:178-223 (bucket geometry, nck table, hard-coded
// caps).  numConnected (src/main.cpp:195) is a fixed 10000 there and overflows
// OffDiagGen_bit_e on larger systems; the harness lets the caller raise it.
#include "all.h"

#include <cstdint>
#include <cstring>
#include <sstream>

Hamiltonian H;
unsigned int nThread;
unsigned int blockDim;
unsigned int threadBcktRatio;
unsigned int bucketNum;
unsigned int bucketSize;
unsigned int spaceDim;
unsigned int bucketSize_bit;
unsigned int numConnected = 20000;
unsigned int Nd = 200000;
unsigned int bucket_unit = 60000;
string filename;
string task;
unsigned int orbitalNum;
unsigned int electronNum;
unsigned int numIteration;
unsigned int numRestart;
DET_TYPE init_hf;
FLOAT_TYPE target_energy;
FLOAT_TYPE SpMSpVFinalResCut;
unsigned int HPsiCap;
vector<vector<unsigned int>> nck_list;
vector<det_bit> basis_bit;
double lambda;

using colvec = dynVec<DET_TYPE, FLOAT_TYPE>;
void introsort(colvec&, int);
void introsort_amp(colvec&, int);
unsigned int merge_bucket(colvec&, unsigned int);
FLOAT_TYPE calc_energy(const colvec&);
void OffDiagGen_bit_e(const DET_TYPE, colvec&);
int make_bucket(const colvec&, vector<colvec>&);
void spmspvm_bucket_linear(const colvec&, colvec&, FLOAT_TYPE, vector<FLOAT_TYPE>&, vector<vector<colvec>>&, int,
                           int);
FLOAT_TYPE spmspvm_bucket_res_norm(const colvec&, colvec&, vector<colvec>&, FLOAT_TYPE, int);

static std::ostringstream g_sink;
static std::streambuf* g_saved = nullptr;

static void quiet(bool on) {
  if (on && !g_saved) g_saved = cout.rdbuf(g_sink.rdbuf());
  if (!on && g_saved) { cout.rdbuf(g_saved); g_saved = nullptr; }
  g_sink.str("");
}

static void fill(colvec& v, const uint64_t* k, const double* a, unsigned len) {
  for (unsigned i = 0; i < len; ++i) { v.basis[i] = k[i]; v.amp[i] = a[i]; }
  v.len = len;
}

static void drain(const colvec& v, uint64_t* k, double* a, unsigned* len) {
  for (unsigned i = 0; i < v.len; ++i) { k[i] = v.basis[i]; a[i] = v.amp[i]; }
  *len = v.len;
}

extern "C" {

int ref_setup(const char* in_path, unsigned norb, unsigned ne, unsigned nd,
              unsigned bunit, unsigned nthread, unsigned num_connected) {
  H = Hamiltonian();
  orbitalNum = norb;
  electronNum = ne;
  Nd = nd;
  bucket_unit = bunit;
  nThread = nthread;
  filename = in_path;
  quiet(true);
  load_integrals(filename);
  unsigned int one = 1;
  blockDim = nck(orbitalNum / 2, electronNum / 2);
  spaceDim = blockDim;
  threadBcktRatio = 4;
  bucketSize_bit = ((unsigned int)log2(blockDim)) / 2;
  bucketSize = one << bucketSize_bit;
  bucketNum = (spaceDim / bucketSize) + 1;
  HPsiCap = 60000000;
  numConnected = num_connected ? num_connected : 10000;
  SpMSpVFinalResCut = 1e-5;
  omp_set_num_threads(nThread);
  nck_list.assign(electronNum / 2, vector<unsigned int>(orbitalNum / 2, 0));
  for (unsigned i = 0; i < electronNum / 2; i++)
    for (unsigned j = 0; j < orbitalNum / 2; j++)
      if (j >= i + 1) nck_list[i][j] = nck(j, i + 1);
  spaceDim = blockDim * blockDim;
  return 0;
}

unsigned ref_bucket_num() { return bucketNum; }
unsigned ref_bucket_bits() { return bucketSize_bit; }
double ref_constant() { return H.constant; }

double ref_diag(uint64_t det) { return DiagCal_bit(det); }
double ref_sign(uint64_t det, int p, int q) { return signCal_bit(det, p, q); }
unsigned long long ref_index(uint64_t det) { return indexCal(det); }

// OffDiagGen_bit_e: raw emitted terms of one determinant (unit coefficient).
unsigned ref_offdiag(uint64_t det, uint64_t* keys, double* amps, unsigned cap) {
  colvec t;
  OffDiagGen_bit_e(det, t);
  unsigned n = t.len < cap ? t.len : cap;
  for (unsigned i = 0; i < n; ++i) { keys[i] = t.basis[i]; amps[i] = t.amp[i]; }
  return t.len;
}

// SpMVMtply_bucket (src/functions.cpp:511-804) on a caller vector.
void ref_spmspv(const uint64_t* ik, const double* ia, unsigned ilen, unsigned icap,
                unsigned ocap, double lam, double coeff, uint64_t* ok, double* oa,
                unsigned* olen, double* diag) {
  colvec in(icap < ilen ? ilen : icap), out(ocap);
  fill(in, ik, ia, ilen);
  FLOAT_TYPE d = 0;
  SpMVMtply_bucket(in, out, lam, coeff, d);
  drain(out, ok, oa, olen);
  *diag = d;
}

double ref_energy(const uint64_t* k, const double* a, unsigned len) {
  colvec v(len ? len : 1);
  fill(v, k, a, len);
  return calc_energy(v);
}

double ref_dot(const uint64_t* k1, const double* a1, unsigned l1,
               const uint64_t* k2, const double* a2, unsigned l2) {
  colvec x(l1 ? l1 : 1), y(l2 ? l2 : 1);
  fill(x, k1, a1, l1);
  fill(y, k2, a2, l2);
  return x.dot(y);
}

double ref_norm(const uint64_t* k, const double* a, unsigned len) {
  colvec v(len ? len : 1);
  fill(v, k, a, len);
  return v.norm();
}

// v.addTwo(w, a) with v.cap = vcap; result written to (ok, oa, olen).
void ref_add_two(const uint64_t* vk, const double* va, unsigned vl, unsigned vcap,
                 const uint64_t* wk, const double* wa, unsigned wl, double a,
                 uint64_t* ok, double* oa, unsigned* olen) {
  unsigned c = vcap > vl + wl ? vcap : vl + wl;
  colvec v(c), w(wl ? wl : 1);
  fill(v, vk, va, vl);
  fill(w, wk, wa, wl);
  v.cap = vcap;
  v.addTwo(w, a);
  drain(v, ok, oa, olen);
}

// v.addThree(x, y, z, a, b, c): result capped at the global Nd.
void ref_add_three(const uint64_t* xk, const double* xa, unsigned xl,
                   const uint64_t* yk, const double* ya, unsigned yl,
                   const uint64_t* zk, const double* za, unsigned zl,
                   double a, double b, double c,
                   uint64_t* ok, double* oa, unsigned* olen) {
  unsigned n = xl + yl + zl;
  colvec v(n ? n : 1), x(xl ? xl : 1), y(yl ? yl : 1), z(zl ? zl : 1);
  fill(x, xk, xa, xl);
  fill(y, yk, ya, yl);
  fill(z, zk, za, zl);
  v.addThree(x, y, z, a, b, c);
  drain(v, ok, oa, olen);
}

// dst.shrinkFrom(src) with dst.cap = dcap.
void ref_shrink_from(const uint64_t* sk, const double* sa, unsigned sl, unsigned dcap,
                     uint64_t* ok, double* oa, unsigned* olen) {
  colvec src(sl ? sl : 1), dst(dcap > sl ? dcap : (sl ? sl : 1));
  fill(src, sk, sa, sl);
  dst.cap = dcap;
  dst.shrinkFrom(src);
  drain(dst, ok, oa, olen);
}

// introsort by key + merge_bucket (the restart-vector merge of the driver).
unsigned ref_sort_merge(uint64_t* k, double* a, unsigned len) {
  colvec v(len ? len : 1);
  fill(v, k, a, len);
  introsort(v, v.len);
  unsigned m = merge_bucket(v, v.len);
  v.len = m;
  unsigned out;
  drain(v, k, a, &out);
  return out;
}

// spmspvm_bucket_linear (src/functions.cpp:858-1094) with input = basis vector
// `cur` of the nb vectors given back to back (lengths blen), as the linear
// driver calls it (src/sparse_solver.cpp:663-669); Hij[0..nb) receives the dots.
void ref_spmspv_linear(const uint64_t* bk, const double* ba, const unsigned* blen, unsigned nb, unsigned cur,
                       double lam, unsigned ocap, uint64_t* ok, double* oa, unsigned* olen, double* hij) {
  std::vector<colvec> basis(nb);
  std::vector<std::vector<colvec>> bb(nb);
  int maxb = 0;
  size_t off = 0;
  for (unsigned j = 0; j < nb; ++j) {
    basis[j].reserveMem(blen[j] ? blen[j] : 1);
    fill(basis[j], bk + off, ba + off, blen[j]);
    off += blen[j];
    int m = make_bucket(basis[j], bb[j]);
    if (m > maxb) maxb = m;
  }
  std::vector<FLOAT_TYPE> h(nb, 0.0);
  colvec out(ocap);
  spmspvm_bucket_linear(basis[cur], out, lam, h, bb, maxb, (int)cur);
  drain(out, ok, oa, olen);
  for (unsigned j = 0; j < nb; ++j) hij[j] = h[j];
}

// spmspvm_bucket_res_norm (src/functions.cpp:1096-1269): r = top-ocap of the cut
// of merge((H - lam) x) - b, sorted; returns |merge((H - lam) x) - b| before the cut.
double ref_res_norm(const uint64_t* xk, const double* xa, unsigned xl, const uint64_t* bk, const double* ba,
                    unsigned bl, double lam, unsigned ocap, uint64_t* ok, double* oa, unsigned* olen) {
  colvec x(xl ? xl : 1), b(bl ? bl : 1), out(ocap);
  fill(x, xk, xa, xl);
  fill(b, bk, ba, bl);
  std::vector<colvec> bb;
  int maxb = make_bucket(b, bb);
  double r = spmspvm_bucket_res_norm(x, out, bb, lam, maxb);
  drain(out, ok, oa, olen);
  return r;
}

}  // extern "C"

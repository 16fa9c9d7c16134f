// Internal types shared by the translation units of libsfci_gb300.
#pragma once

#include <cstdint>
#include <cstdio>
#include <map>
#include <set>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sfci_gb300.h"

namespace sfci {

typedef unsigned long long u64;

// Host copy of the integral tables.  Two-body values are (mn|pq) in chemists'
// notation over spin orbitals, stored per spin block b = 2*spin(m) + spin(p)
// and packed pair indices of the spatial orbitals: V[b][pair(m,n)][pair(p,q)].
// One-body values h1[s][m][n] keep the file's (target, source) orientation.
struct HamHost {
  int M = 0, N = 0, P = 0;
  double ecore = 0.0;
  std::vector<double> h1;  // 2*M*M
  std::vector<double> V;   // 4*P*P
  uint64_t n_two = 0, n_one = 0;
};

// Parse an _IN file (src/functions.cpp:297-395 routing) into dense tables.
int load_in_file(const char* path, int num_orb, HamHost& out, std::string& err);

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

enum Phase { PH_COUNT = 0, PH_SCATTER, PH_PARTITION, PH_MERGE, PH_SELECT, PH_SORT, PH_OTHER, PH_N };

struct Ctx {
  int N = 0, M = 0, ne = 0, W = 1, P = 0;
  sfci_opts opts{};
  HamHost ham;
  double* d_h1 = nullptr;
  double* d_V = nullptr;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  std::map<std::string, Buf> scratch;
  u64 launches = 0;
  cudaEvent_t ev[16] = {};
  // per-phase profiling
  bool profile = false;
  double ph_ms[PH_N] = {};
  u64 ph_launch[PH_N] = {};
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ph_pending;
  uint64_t stats[8] = {};
  bool last_pruned = false;  // the last SpMSpV cut its survivors to the output capacity before the end
  double dup_est = 0.0;  // terms per distinct key of the last SpMSpV (sizes its leaves)
  // vectors created on this context (freed with it; their handles become orphans)
  std::set<struct Vec*> live;
  // pinned host staging for small readbacks
  u64* h_pin = nullptr;
  size_t h_pin_words = 0;
  // batched contexts: one Hamiltonian per instance (device HamView table);
  // ninst = 0 for an ordinary context
  int ninst = 0;
  std::vector<HamHost> inst_ham;
  std::vector<double*> inst_h1, inst_V;
  std::vector<int> inst_N, inst_ne;
  void* d_insts = nullptr;
  std::vector<double> inst_diag;  // <v|Hv> of each instance, from the last product
  // tunables of the product (the autotuner sets them; results do not depend on them)
  int tune_l1_bits = 9;       // level-1 bins of the generation sweep: 2^bits
  int tune_digit_bits = 9;    // most bits per partition level
  int tune_leaf_uniq = 120;   // distinct keys a leaf is sized for
  int tune_gen_ctas = 2;      // generation CTAs per SM
  int tune_class_passes = 0;  // generation passes by target alpha class: 0 when needed, 1 always, -1 never
  // learned excitation screen applied by the products (nullptr: plain products)
  struct Screen* screen = nullptr;
  // screens created on this context (freed with it; their handles become orphans)
  std::set<struct Screen*> screens;
  double screen_thr = 0.5;
  double screen_guard = 0.0;  // a group whose term bound |c_j| * max|V| reaches this is always kept (0: off)
  double screen_floor = 0.0;  // a group whose term bound is below this is skipped without the network (0: off)
  uint64_t screen_stats[5] = {};  // groups, kept groups, kept terms, screened products, terms of all groups
};

struct Vec {
  Ctx* ctx = nullptr;
  uint64_t cap = 0, len = 0;
  u64* keys = nullptr;   // len*W words
  double* amps = nullptr;
};

// release a screen's device memory and detach it from its context (mlp.cu)
void screen_orphan(struct Screen* s);

// growable named device scratch (contents not preserved on growth)
void* scratch_get(Ctx& c, const char* name, size_t bytes);
void scratch_free_all(Ctx& c);
// free one named buffer; free the SpMSpV plan's large buffers (its next call
// re-plans from the memory that is then free)
void scratch_release(Ctx& c, const char* name);
void scratch_release_plan(Ctx& c);
// pinned host words for readbacks
u64* pinned_words(Ctx& c, size_t n);

// error state (thread-local message)
int set_error(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// phase timing: begin returns a token; end closes it
int phase_begin(Ctx& c, Phase p);
void phase_end(Ctx& c, int token);
void phase_collect(Ctx& c);

}  // namespace sfci

struct sfci_ctx {
  sfci::Ctx c;
};
struct sfci_vec {
  sfci::Vec v;
};

// A vector passed to an entry point with a context must belong to that
// context: another context's vectors may hold keys of another width or tags of
// another batch.  SFCI_OK, or SFCI_ERR_ARG with the error text set.
inline int vec_of(const sfci_ctx* x, const sfci_vec* v) {
  if (!v || !v->v.ctx) return sfci::set_error(SFCI_ERR_ARG, "null vector");
  if (v->v.ctx != &x->c) return sfci::set_error(SFCI_ERR_ARG, "vector belongs to another context");
  return SFCI_OK;
}

#define SFCI_CUDA(call)                                         \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return ::sfci::cuda_fail(e_, #call); \
  } while (0)

// launch with error check and launch accounting
#define SFCI_LAUNCH(ctx, kern, grid, block, smem, ...)                          \
  do {                                                                          \
    kern<<<(grid), (block), (smem), (ctx).stream>>>(__VA_ARGS__);               \
    (ctx).launches++;                                                           \
    cudaError_t e_ = cudaGetLastError();                                        \
    if (e_ != cudaSuccess) return ::sfci::cuda_fail(e_, #kern);                 \
  } while (0)

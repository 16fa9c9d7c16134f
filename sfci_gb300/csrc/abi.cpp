// C ABI of libsfci_gb300 (declarations and reference citations in
// include/sfci_gb300.h).  Host-side plumbing: contexts, device vectors,
// scratch memory, error state, timing; the hot path lives in the .cu files.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gen.cuh"
#include "internal.h"
#include "spmspv.h"

namespace sfci {

static thread_local std::string g_err;

int set_error(int status, const std::string& msg) {
  g_err = msg;
  return status;
}

int cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return SFCI_ERR_NOMEM;
  return SFCI_ERR_CUDA;
}

void* scratch_get(Ctx& c, const char* name, size_t bytes) {
  if (bytes == 0) bytes = 16;
  Buf& b = c.scratch[name];
  if (b.bytes >= bytes) return b.p;
  if (b.p) {
    cudaStreamSynchronize(c.stream);
    cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
  }
  // headroom against regrowth, for buffers under 1 GiB only: the large ones
  // are sized by the product's memory plan, which the headroom would overrun
  size_t want = bytes < ((size_t)1 << 30) ? bytes + bytes / 8 : bytes;
  void* p = nullptr;
  if (cudaMalloc(&p, want) != cudaSuccess) {
    cudaGetLastError();
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      set_error(SFCI_ERR_NOMEM, std::string("device allocation of ") + std::to_string(bytes) + " bytes for " + name +
                                    " failed");
      return nullptr;
    }
    want = bytes;
  }
  b.p = p;
  b.bytes = want;
  return p;
}

void scratch_free_all(Ctx& c) {
  for (auto& kv : c.scratch)
    if (kv.second.p) cudaFree(kv.second.p);
  c.scratch.clear();
}

void scratch_release(Ctx& c, const char* name) {
  auto it = c.scratch.find(name);
  if (it == c.scratch.end() || !it->second.p) return;
  cudaStreamSynchronize(c.stream);
  cudaFree(it->second.p);
  c.scratch.erase(it);
}

void scratch_release_plan(Ctx& c) {
  for (const char* nm : {"sp_l1k", "sp_l1a", "sp_l2k", "sp_l2a", "sp_sk", "sp_sa", "rs_keys", "rs_vals", "topk_k",
                         "topk_a"})
    scratch_release(c, nm);
}

u64* pinned_words(Ctx& c, size_t n) {
  if (c.h_pin_words >= n) return c.h_pin;
  if (c.h_pin) cudaFreeHost(c.h_pin);
  c.h_pin = nullptr;
  c.h_pin_words = 0;
  size_t want = n < 4096 ? 4096 : n;
  if (cudaMallocHost(&c.h_pin, want * sizeof(u64)) != cudaSuccess) {
    cudaGetLastError();
    c.h_pin = nullptr;
    return nullptr;
  }
  c.h_pin_words = want;
  return c.h_pin;
}

int read_words(Ctx& c, const void* dptr, size_t nbytes, void* host) {
  size_t words = (nbytes + 7) / 8;
  u64* pin = pinned_words(c, words);
  if (!pin) {
    SFCI_CUDA(cudaMemcpyAsync(host, dptr, nbytes, cudaMemcpyDeviceToHost, c.stream));
    SFCI_CUDA(cudaStreamSynchronize(c.stream));
    return SFCI_OK;
  }
  SFCI_CUDA(cudaMemcpyAsync(pin, dptr, nbytes, cudaMemcpyDeviceToHost, c.stream));
  SFCI_CUDA(cudaStreamSynchronize(c.stream));
  memcpy(host, pin, nbytes);
  return SFCI_OK;
}

// ---- phase timing ----------------------------------------------------------
static cudaEvent_t pool_event(Ctx& c) {
  if (!c.ev_pool.empty()) {
    cudaEvent_t e = c.ev_pool.back();
    c.ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

struct OpenPhase {
  int phase;
  cudaEvent_t start;
  u64 launches0;
};
static thread_local std::vector<OpenPhase> g_open;

int phase_begin(Ctx& c, Phase p) {
  if (!c.profile) return -1;
  OpenPhase o{(int)p, pool_event(c), c.launches};
  cudaEventRecord(o.start, c.stream);
  g_open.push_back(o);
  return (int)g_open.size() - 1;
}

void phase_end(Ctx& c, int token) {
  if (!c.profile || token < 0 || token >= (int)g_open.size()) return;
  OpenPhase o = g_open[token];
  cudaEvent_t stop = pool_event(c);
  cudaEventRecord(stop, c.stream);
  c.ph_pending.push_back({o.phase, {o.start, stop}});
  c.ph_launch[o.phase] += c.launches - o.launches0;
  g_open.resize(token);
}

void phase_collect(Ctx& c) {
  if (c.ph_pending.empty()) return;
  cudaStreamSynchronize(c.stream);
  for (auto& p : c.ph_pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.second.first, p.second.second);
    c.ph_ms[p.first] += ms;
    c.ev_pool.push_back(p.second.first);
    c.ev_pool.push_back(p.second.second);
  }
  c.ph_pending.clear();
}

// ---- width dispatch --------------------------------------------------------
#define SFCI_W(c, fn, ...) ((c).W == 1 ? fn<1>(__VA_ARGS__) : fn<2>(__VA_ARGS__))

int op_spmspv(Ctx& c, const Vec& in, Vec& out, double lambda, double coeff, double* diag) {
  int st = SFCI_W(c, spmspv_impl, c, in, out, lambda, coeff, diag);
  phase_collect(c);
  return st;
}
int op_energy(Ctx& c, const Vec& psi, double* E) { return SFCI_W(c, energy_impl, c, psi, E); }
int op_dot(Ctx& c, const Vec& x, const Vec& y, double* out) { return SFCI_W(c, dot_impl, c, x, y, out); }
int op_add_two(Ctx& c, Vec& v, const Vec& w, double a) { return SFCI_W(c, add_two_impl, c, v, w, a); }
int op_add_three(Ctx& c, Vec& v, const Vec& x, const Vec& y, const Vec& z, double a, double b, double cc) {
  return SFCI_W(c, add_three_impl, c, v, x, y, z, a, b, cc);
}
int op_shrink(Ctx& c, Vec& dst, const Vec& src) { return SFCI_W(c, shrink_impl, c, dst, src); }
int op_combine(Ctx& c, Vec& dst, const Vec* const* vs, const double* coef, int n) {
  return SFCI_W(c, combine_impl, c, dst, vs, coef, n);
}
int op_copy(Ctx& c, Vec& dst, const Vec& src) {
  if (&dst == &src) return SFCI_OK;
  if (src.len > dst.cap) return set_error(SFCI_ERR_CAPACITY, "copy: destination capacity too small");
  if (src.len) {
    SFCI_CUDA(cudaMemcpyAsync(dst.keys, src.keys, src.len * c.W * sizeof(u64), cudaMemcpyDeviceToDevice, c.stream));
    SFCI_CUDA(cudaMemcpyAsync(dst.amps, src.amps, src.len * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  }
  dst.len = src.len;
  return SFCI_OK;
}

int op_spmspv_linear(Ctx& c, const Vec& in, Vec& out, double lambda, const Vec* const* basis, int nb, double* hij) {
  int st = SFCI_W(c, spmspv_linear_impl, c, in, out, lambda, basis, nb, hij);
  phase_collect(c);
  return st;
}

int op_res_norm(Ctx& c, const Vec& x, Vec& r, const Vec& b, double lambda, double* res) {
  int st = SFCI_W(c, res_norm_impl, c, x, r, b, lambda, res);
  phase_collect(c);
  return st;
}

}  // namespace sfci

using namespace sfci;

static int vec_check(const sfci_vec* v) {
  if (!v || !v->v.ctx) return set_error(SFCI_ERR_ARG, "null vector");
  return SFCI_OK;
}

extern "C" {

const char* sfci_last_error(void) { return g_err.c_str(); }

const char* sfci_status_name(int s) {
  switch (s) {
    case SFCI_OK: return "SFCI_OK";
    case SFCI_ERR_ARG: return "SFCI_ERR_ARG";
    case SFCI_ERR_IO: return "SFCI_ERR_IO";
    case SFCI_ERR_NOMEM: return "SFCI_ERR_NOMEM";
    case SFCI_ERR_CUDA: return "SFCI_ERR_CUDA";
    case SFCI_ERR_CAPACITY: return "SFCI_ERR_CAPACITY";
    case SFCI_ERR_UNSUPPORTED: return "SFCI_ERR_UNSUPPORTED";
    case SFCI_ERR_NUMERIC: return "SFCI_ERR_NUMERIC";
  }
  return "SFCI_ERR_UNKNOWN";
}

int sfci_version(void) { return 10000; }

int sfci_ctx_create(const char* in_path, int num_orb, int num_e, const sfci_opts* opts, sfci_ctx** out) {
  if (!out || !in_path) return set_error(SFCI_ERR_ARG, "null argument");
  *out = nullptr;
  if (num_orb <= 0 || num_orb > 128 || (num_orb & 1))
    return set_error(SFCI_ERR_ARG, "num_orb must be even and in [2, 128]");
  if (num_e < 0 || num_e >= num_orb) return set_error(SFCI_ERR_ARG, "num_e must be in [0, num_orb)");
  sfci_ctx* x = new sfci_ctx();
  Ctx& c = x->c;
  c.N = num_orb;
  c.M = num_orb / 2;
  c.ne = num_e;
  c.W = num_orb <= 64 ? 1 : 2;
  c.P = c.M * (c.M + 1) / 2;
  if (opts) c.opts = *opts;
  if (!c.opts.Nd) c.opts.Nd = 200000;
  if (!c.opts.hpsi_cap) c.opts.hpsi_cap = 60000000;
  // 0 (or NaN): the reference's 1e-5; a negative cut keeps every merged determinant
  if (c.opts.coeff_cut == 0.0 || c.opts.coeff_cut != c.opts.coeff_cut) c.opts.coeff_cut = 1e-5;
  std::string err;
  int st = load_in_file(in_path, num_orb, c.ham, err);
  if (st) {
    delete x;
    return set_error(st, err);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c.d_h1, c.ham.h1.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&c.d_V, c.ham.V.size() * sizeof(double));
  if (e == cudaSuccess)
    e = cudaMemcpy(c.d_h1, c.ham.h1.data(), c.ham.h1.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c.d_V, c.ham.V.data(), c.ham.V.size() * sizeof(double), cudaMemcpyHostToDevice);
  for (int i = 0; i < 16 && e == cudaSuccess; ++i) e = cudaEventCreate(&c.ev[i]);
  if (e != cudaSuccess) {
    int s2 = cuda_fail(e, "context set-up");
    sfci_ctx_destroy(x);
    return s2;
  }
  *out = x;
  return SFCI_OK;
}

int sfci_batch_create(int n, const char* const* in_paths, const int* num_orb, const int* num_e,
                      const sfci_opts* opts, sfci_ctx** out) {
  if (!out || !in_paths || !num_orb || !num_e) return set_error(SFCI_ERR_ARG, "null argument");
  *out = nullptr;
  if (n < 1 || n > INST_MAX) return set_error(SFCI_ERR_ARG, "a batch holds 1 to 32 instances");
  for (int i = 0; i < n; ++i) {
    if (!in_paths[i]) return set_error(SFCI_ERR_ARG, "null integral path");
    if (num_orb[i] <= 0 || num_orb[i] > INST_MAX_ORB || (num_orb[i] & 1))
      return set_error(SFCI_ERR_ARG, "batched instances need an even num_orb in [2, 120]");
    if (num_e[i] < 0 || num_e[i] >= num_orb[i]) return set_error(SFCI_ERR_ARG, "num_e must be in [0, num_orb)");
  }
  sfci_ctx* x = new sfci_ctx();
  Ctx& c = x->c;
  c.ninst = n;
  c.W = 2;
  c.N = 128;  // sorts cover the instance tag
  c.M = 0;
  c.ne = 0;
  for (int i = 0; i < n; ++i) {
    c.M = std::max(c.M, num_orb[i] / 2);
    c.ne = std::max(c.ne, num_e[i]);
  }
  c.P = c.M * (c.M + 1) / 2;
  if (opts) c.opts = *opts;
  if (!c.opts.Nd) c.opts.Nd = 200000;
  if (!c.opts.hpsi_cap) c.opts.hpsi_cap = 60000000;
  // 0 (or NaN): the reference's 1e-5; a negative cut keeps every merged determinant
  if (c.opts.coeff_cut == 0.0 || c.opts.coeff_cut != c.opts.coeff_cut) c.opts.coeff_cut = 1e-5;
  c.inst_ham.resize(n);
  for (int i = 0; i < n; ++i) {
    std::string err;
    int st = load_in_file(in_paths[i], num_orb[i], c.inst_ham[i], err);
    if (st) {
      delete x;
      return set_error(st, std::string("instance ") + std::to_string(i) + ": " + err);
    }
    c.inst_N.push_back(num_orb[i]);
    c.inst_ne.push_back(num_e[i]);
  }
  c.ham = c.inst_ham[0];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
  std::vector<HamView> views(n);
  c.inst_h1.assign(n, nullptr);
  c.inst_V.assign(n, nullptr);
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    const HamHost& h = c.inst_ham[i];
    e = cudaMalloc(&c.inst_h1[i], h.h1.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c.inst_V[i], h.V.size() * sizeof(double));
    if (e == cudaSuccess)
      e = cudaMemcpy(c.inst_h1[i], h.h1.data(), h.h1.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c.inst_V[i], h.V.data(), h.V.size() * sizeof(double), cudaMemcpyHostToDevice);
    views[i].N = h.N;
    views[i].M = h.M;
    views[i].P = h.P;
    views[i].h1 = c.inst_h1[i];
    views[i].V = c.inst_V[i];
    views[i].ecore = h.ecore;
    views[i].inst = nullptr;
  }
  c.d_h1 = c.inst_h1[0];
  c.d_V = c.inst_V[0];
  if (e == cudaSuccess) e = cudaMalloc(&c.d_insts, n * sizeof(HamView));
  if (e == cudaSuccess) e = cudaMemcpy(c.d_insts, views.data(), n * sizeof(HamView), cudaMemcpyHostToDevice);
  for (int i = 0; i < 16 && e == cudaSuccess; ++i) e = cudaEventCreate(&c.ev[i]);
  if (e != cudaSuccess) {
    int s2 = cuda_fail(e, "batched context set-up");
    sfci_ctx_destroy(x);
    return s2;
  }
  *out = x;
  return SFCI_OK;
}

int sfci_batch_lanczos(sfci_ctx* x, sfci_vec* const* v, int n, int Nl, int restarts, double* energies,
                       double* final_e) {
  if (!x || !v || !energies || !final_e) return set_error(SFCI_ERR_ARG, "null argument");
  if (!x->c.ninst || x->c.W != 2) return set_error(SFCI_ERR_ARG, "batched Lanczos needs a batched context");
  if (n != x->c.ninst) return set_error(SFCI_ERR_ARG, "batched Lanczos: one vector per instance");
  std::vector<Vec*> vs(n);
  for (int i = 0; i < n; ++i) {
    if (!v[i] || v[i]->v.ctx != &x->c) return set_error(SFCI_ERR_ARG, "batched Lanczos: vector of another context");
    if (v[i]->v.len == 0) return set_error(SFCI_ERR_ARG, "batched Lanczos: an empty start vector");
    vs[i] = &v[i]->v;
  }
  // vector i must hold instance i's keys only: vectors are sorted by key and the
  // tag is the key's top field, so the first and last keys carry every key's tag
  for (int i = 0; i < n; ++i) {
    const Vec& w = v[i]->v;
    u64 hi[2] = {0ull, 0ull};
    SFCI_CUDA(cudaMemcpyAsync(&hi[0], w.keys + 1, sizeof(u64), cudaMemcpyDeviceToHost, x->c.stream));
    SFCI_CUDA(cudaMemcpyAsync(&hi[1], w.keys + 2 * (w.len - 1) + 1, sizeof(u64), cudaMemcpyDeviceToHost, x->c.stream));
    SFCI_CUDA(cudaStreamSynchronize(x->c.stream));
    if ((hi[0] >> INST_SHIFT) != (u64)i || (hi[1] >> INST_SHIFT) != (u64)i)
      return set_error(SFCI_ERR_ARG, "batched Lanczos: vector " + std::to_string(i) + " holds keys of another instance");
  }
  return lanczos_batched(x->c, vs.data(), n, Nl, restarts, energies, final_e);
}

int sfci_ctx_set_tuning(sfci_ctx* x, const int* t4) {
  if (!x || !t4) return set_error(SFCI_ERR_ARG, "null argument");
  if (t4[0] < 4 || t4[0] > 9 || t4[1] < 6 || t4[1] > 9 || t4[2] < 16 || t4[2] > 120 || t4[3] < 1 || t4[3] > 2)
    return set_error(SFCI_ERR_ARG, "tuning out of range: l1 bits 4-9, digit bits 6-9, leaf keys 16-120, CTAs/SM 1-2");
  Ctx& c = x->c;
  c.tune_l1_bits = t4[0];
  c.tune_digit_bits = t4[1];
  c.tune_leaf_uniq = t4[2];
  c.tune_gen_ctas = t4[3];
  return SFCI_OK;
}

int sfci_ctx_set_class_passes(sfci_ctx* x, int mode) {
  if (!x || mode < -1 || mode > 1) return set_error(SFCI_ERR_ARG, "class-pass mode is -1, 0 or 1");
  x->c.tune_class_passes = mode;
  return SFCI_OK;
}

int sfci_ctx_get_tuning(const sfci_ctx* x, int* t4) {
  if (!x || !t4) return set_error(SFCI_ERR_ARG, "null argument");
  const Ctx& c = x->c;
  t4[0] = c.tune_l1_bits;
  t4[1] = c.tune_digit_bits;
  t4[2] = c.tune_leaf_uniq;
  t4[3] = c.tune_gen_ctas;
  return SFCI_OK;
}

int sfci_autotune(sfci_ctx* x, const sfci_vec* in, sfci_vec* out, int* best4, double* best_ms) {
  if (!x || !in || !out) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, in) || vec_of(x, out)) return SFCI_ERR_ARG;
  Ctx& c = x->c;
  // candidates: level-1 bins, partition digit width, leaf size, generation occupancy
  static const int cand[][4] = {{9, 9, 120, 2}, {9, 8, 120, 2}, {8, 9, 120, 2}, {9, 9, 80, 2},
                                {9, 9, 60, 2},  {9, 9, 120, 1}, {7, 8, 120, 2}, {9, 8, 80, 2}};
  const int save[4] = {c.tune_l1_bits, c.tune_digit_bits, c.tune_leaf_uniq, c.tune_gen_ctas};
  double best = 1e300;
  int bi = 0;
  uint64_t ref_len = 0;
  double ref_diag = 0.0;
  for (int k = 0; k < (int)(sizeof(cand) / sizeof(cand[0])); ++k) {
    int st = sfci_ctx_set_tuning(x, cand[k]);
    if (st) return st;
    double dg = 0.0;
    if ((st = op_spmspv(c, in->v, out->v, 0.0, 1.0, &dg))) return st;  // warm-up: scratch at this plan's sizes
    cudaEvent_t e0 = c.ev[14], e1 = c.ev[15];
    SFCI_CUDA(cudaEventRecord(e0, c.stream));
    if ((st = op_spmspv(c, in->v, out->v, 0.0, 1.0, &dg))) return st;
    SFCI_CUDA(cudaEventRecord(e1, c.stream));
    SFCI_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    SFCI_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    // the merge is exact: every plan must give the same product
    if (k == 0) {
      ref_len = out->v.len;
      ref_diag = dg;
    } else if (out->v.len != ref_len || std::fabs(dg - ref_diag) > 1e-12 * std::fabs(ref_diag) + 1e-14) {
      sfci_ctx_set_tuning(x, save);
      return set_error(SFCI_ERR_NUMERIC, "autotune: plans disagree on the product");
    }
    if (ms < best) {
      best = ms;
      bi = k;
    }
  }
  sfci_ctx_set_tuning(x, cand[bi]);
  if (best4)
    for (int i = 0; i < 4; ++i) best4[i] = cand[bi][i];
  if (best_ms) *best_ms = best;
  return SFCI_OK;
}

int sfci_ctx_destroy(sfci_ctx* x) {
  if (!x) return SFCI_OK;
  Ctx& c = x->c;
  if (c.stream) cudaStreamSynchronize(c.stream);
  for (Vec* v : c.live) {  // orphan vectors that outlive their context
    if (v->keys) cudaFree(v->keys);
    if (v->amps) cudaFree(v->amps);
    v->keys = nullptr;
    v->amps = nullptr;
    v->ctx = nullptr;
    v->cap = v->len = 0;
  }
  c.live.clear();
  for (Screen* s : std::set<Screen*>(c.screens)) screen_orphan(s);  // screens that outlive their context
  c.screens.clear();
  c.screen = nullptr;
  scratch_free_all(c);
  if (c.d_h1) cudaFree(c.d_h1);
  if (c.d_V) cudaFree(c.d_V);
  for (size_t i = 1; i < c.inst_h1.size(); ++i) {  // instance 0's tables are d_h1 / d_V
    if (c.inst_h1[i]) cudaFree(c.inst_h1[i]);
    if (c.inst_V[i]) cudaFree(c.inst_V[i]);
  }
  if (c.d_insts) cudaFree(c.d_insts);
  for (int i = 0; i < 16; ++i)
    if (c.ev[i]) cudaEventDestroy(c.ev[i]);
  for (auto e : c.ev_pool) cudaEventDestroy(e);
  for (auto& p : c.ph_pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  if (c.h_pin) cudaFreeHost(c.h_pin);
  if (c.stream) cudaStreamDestroy(c.stream);
  delete x;
  return SFCI_OK;
}

int sfci_key_words(const sfci_ctx* x) { return x ? x->c.W : 0; }

int sfci_ctx_stream(const sfci_ctx* x, void** s) {
  if (!x || !s) return set_error(SFCI_ERR_ARG, "null argument");
  *s = (void*)x->c.stream;
  return SFCI_OK;
}

int sfci_ctx_set_nd(sfci_ctx* x, uint64_t Nd) {
  if (!x || !Nd) return set_error(SFCI_ERR_ARG, "Nd must be positive");
  x->c.opts.Nd = Nd;
  return SFCI_OK;
}

int sfci_ctx_trim(sfci_ctx* x) {
  if (!x) return set_error(SFCI_ERR_ARG, "null context");
  SFCI_CUDA(cudaStreamSynchronize(x->c.stream));
  scratch_free_all(x->c);
  return SFCI_OK;
}

int sfci_ctx_launch_count(const sfci_ctx* x, uint64_t* n) {
  if (!x || !n) return set_error(SFCI_ERR_ARG, "null argument");
  *n = x->c.launches;
  return SFCI_OK;
}

int sfci_ctx_event_record(sfci_ctx* x, int slot) {
  if (!x || slot < 0 || slot >= 16) return set_error(SFCI_ERR_ARG, "event slot out of range");
  SFCI_CUDA(cudaEventRecord(x->c.ev[slot], x->c.stream));
  return SFCI_OK;
}

int sfci_ctx_event_elapsed(sfci_ctx* x, int a, int b, float* ms) {
  if (!x || a < 0 || a >= 16 || b < 0 || b >= 16 || !ms) return set_error(SFCI_ERR_ARG, "bad event slots");
  SFCI_CUDA(cudaEventSynchronize(x->c.ev[b]));
  SFCI_CUDA(cudaEventElapsedTime(ms, x->c.ev[a], x->c.ev[b]));
  return SFCI_OK;
}

int sfci_ctx_profile(sfci_ctx* x, int enable) {
  if (!x) return set_error(SFCI_ERR_ARG, "null context");
  x->c.profile = enable != 0;
  return SFCI_OK;
}

static const char* kPhaseNames[PH_N] = {"count", "scatter", "partition", "merge", "select", "sort", "other"};

int sfci_ctx_profile_read(sfci_ctx* x, const char* phase, double* ms, uint64_t* launches) {
  if (!x || !phase) return set_error(SFCI_ERR_ARG, "null argument");
  phase_collect(x->c);
  for (int i = 0; i < PH_N; ++i)
    if (!strcmp(phase, kPhaseNames[i])) {
      if (ms) *ms = x->c.ph_ms[i];
      if (launches) *launches = x->c.ph_launch[i];
      return SFCI_OK;
    }
  return set_error(SFCI_ERR_ARG, std::string("unknown phase ") + phase);
}

int sfci_ctx_profile_reset(sfci_ctx* x) {
  if (!x) return set_error(SFCI_ERR_ARG, "null context");
  phase_collect(x->c);
  for (int i = 0; i < PH_N; ++i) {
    x->c.ph_ms[i] = 0;
    x->c.ph_launch[i] = 0;
  }
  return SFCI_OK;
}

int sfci_ctx_last_stats(const sfci_ctx* x, uint64_t stats[8]) {
  if (!x || !stats) return set_error(SFCI_ERR_ARG, "null argument");
  for (int i = 0; i < 8; ++i) stats[i] = x->c.stats[i];
  return SFCI_OK;
}

// ---- vectors ----------------------------------------------------------------

int sfci_vec_create(sfci_ctx* x, uint64_t cap, sfci_vec** out) {
  if (!x || !out) return set_error(SFCI_ERR_ARG, "null argument");
  *out = nullptr;
  // bounds the byte sizes below far from overflow (2^40 entries: 26 TB)
  if (cap > (1ull << 40)) return set_error(SFCI_ERR_ARG, "vector capacity beyond 2^40 entries");
  sfci_vec* v = new sfci_vec();
  v->v.ctx = &x->c;
  v->v.cap = cap;
  x->c.live.insert(&v->v);
  size_t n = cap ? cap : 1;
  cudaError_t e = cudaMalloc(&v->v.keys, n * x->c.W * sizeof(u64));
  if (e == cudaSuccess) e = cudaMalloc(&v->v.amps, n * sizeof(double));
  if (e != cudaSuccess) {
    int st = cuda_fail(e, "sfci_vec_create");
    sfci_vec_destroy(v);
    return st;
  }
  *out = v;
  return SFCI_OK;
}

int sfci_vec_destroy(sfci_vec* v) {
  if (!v) return SFCI_OK;
  if (v->v.ctx) {
    if (v->v.ctx->stream) cudaStreamSynchronize(v->v.ctx->stream);
    v->v.ctx->live.erase(&v->v);
  }
  if (v->v.keys) cudaFree(v->v.keys);
  if (v->v.amps) cudaFree(v->v.amps);
  delete v;
  return SFCI_OK;
}

int sfci_vec_len(const sfci_vec* v, uint64_t* len) {
  if (vec_check(v) || !len) return set_error(SFCI_ERR_ARG, "null argument");
  *len = v->v.len;
  return SFCI_OK;
}

int sfci_vec_cap(const sfci_vec* v, uint64_t* cap) {
  if (vec_check(v) || !cap) return set_error(SFCI_ERR_ARG, "null argument");
  *cap = v->v.cap;
  return SFCI_OK;
}

int sfci_vec_upload(sfci_vec* v, const uint64_t* keys, const double* amps, uint64_t len) {
  if (vec_check(v)) return SFCI_ERR_ARG;
  if (len && (!keys || !amps)) return set_error(SFCI_ERR_ARG, "null host buffers");
  if (len > v->v.cap) return set_error(SFCI_ERR_CAPACITY, "upload longer than vector capacity");
  Ctx& c = *v->v.ctx;
  if (len && c.ninst) {
    const u64 bad = first_bad_batched_key((const u64*)keys, len, c.inst_N.data(), c.ninst);
    if (bad < len)
      return set_error(SFCI_ERR_ARG, "key " + std::to_string(bad) +
                                         " names no instance of the batch or sets a bit beyond its instance's "
                                         "spin orbitals");
  }
  if (len) {
    SFCI_CUDA(cudaMemcpyAsync(v->v.keys, keys, len * c.W * sizeof(u64), cudaMemcpyHostToDevice, c.stream));
    SFCI_CUDA(cudaMemcpyAsync(v->v.amps, amps, len * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  }
  v->v.len = len;
  int st = SFCI_W(c, sort_vec_impl, c, v->v);
  if (st) return st;
  SFCI_CUDA(cudaStreamSynchronize(c.stream));
  return SFCI_OK;
}

int sfci_vec_download(const sfci_vec* v, uint64_t* keys, double* amps, uint64_t cap, uint64_t* len) {
  if (vec_check(v)) return SFCI_ERR_ARG;
  Ctx& c = *v->v.ctx;
  uint64_t n = v->v.len < cap ? v->v.len : cap;
  if (n && (!keys || !amps)) return set_error(SFCI_ERR_ARG, "null host buffers");
  if (n) {
    SFCI_CUDA(cudaMemcpyAsync(keys, v->v.keys, n * c.W * sizeof(u64), cudaMemcpyDeviceToHost, c.stream));
    SFCI_CUDA(cudaMemcpyAsync(amps, v->v.amps, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  }
  SFCI_CUDA(cudaStreamSynchronize(c.stream));
  if (len) *len = v->v.len;
  return SFCI_OK;
}

int sfci_vec_copy(sfci_vec* dst, const sfci_vec* src) {
  if (vec_check(dst) || vec_check(src)) return SFCI_ERR_ARG;
  if (dst->v.ctx != src->v.ctx) return set_error(SFCI_ERR_ARG, "copy between vectors of different contexts");
  return op_copy(*dst->v.ctx, dst->v, src->v);
}

int sfci_vec_clear(sfci_vec* v) {
  if (vec_check(v)) return SFCI_ERR_ARG;
  v->v.len = 0;
  return SFCI_OK;
}

// ---- hot path -----------------------------------------------------------------

int sfci_spmspv(sfci_ctx* x, const sfci_vec* in, sfci_vec* out, double lambda, double coeff, double* diag) {
  if (!x || !diag) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, in) || vec_of(x, out)) return SFCI_ERR_ARG;
  if (in == out) return set_error(SFCI_ERR_ARG, "spmspv input and output must differ");
  return op_spmspv(x->c, in->v, out->v, lambda, coeff, diag);
}

int sfci_diag_elements(sfci_ctx* x, const uint64_t* keys, uint64_t n, double* out) {
  if (!x || (n && (!keys || !out))) return set_error(SFCI_ERR_ARG, "null argument");
  if (!n) return SFCI_OK;
  if (n > (1ull << 40)) return set_error(SFCI_ERR_ARG, "more than 2^40 keys");
  Ctx& c = x->c;
  if (c.ninst) {
    const u64 bad = first_bad_batched_key((const u64*)keys, n, c.inst_N.data(), c.ninst);
    if (bad < n)
      return set_error(SFCI_ERR_ARG, "key " + std::to_string(bad) +
                                         " names no instance of the batch or sets a bit beyond its instance's "
                                         "spin orbitals");
  }
  void* dk = scratch_get(c, "de_keys", n * c.W * sizeof(u64));
  if (!dk) return SFCI_ERR_NOMEM;
  SFCI_CUDA(cudaMemcpyAsync(dk, keys, n * c.W * sizeof(u64), cudaMemcpyHostToDevice, c.stream));
  return c.W == 1 ? diag_elements_impl<1>(c, (const u64*)dk, n, out) : diag_elements_impl<2>(c, (const K128*)dk, n, out);
}

int sfci_energy(sfci_ctx* x, const sfci_vec* psi, double* E) {
  if (!x || !E) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, psi)) return SFCI_ERR_ARG;
  return op_energy(x->c, psi->v, E);
}

// ---- linear solver products ------------------------------------------------------

int sfci_spmspv_linear(sfci_ctx* x, const sfci_vec* in, sfci_vec* out, double lambda, const sfci_vec* const* basis,
                       int nbasis, double* hij) {
  if (!x || !basis || nbasis < 1 || nbasis > 64 || !hij) return set_error(SFCI_ERR_ARG, "bad spmspv_linear arguments");
  if (vec_of(x, in) || vec_of(x, out)) return SFCI_ERR_ARG;
  if (in == out) return set_error(SFCI_ERR_ARG, "spmspv_linear input and output must differ");
  std::vector<const Vec*> bp(nbasis);
  for (int j = 0; j < nbasis; ++j) {
    if (vec_of(x, basis[j])) return SFCI_ERR_ARG;
    if (basis[j] == out) return set_error(SFCI_ERR_ARG, "spmspv_linear output is one of the basis vectors");
    bp[j] = &basis[j]->v;
  }
  return op_spmspv_linear(x->c, in->v, out->v, lambda, bp.data(), nbasis, hij);
}

int sfci_res_norm(sfci_ctx* x, const sfci_vec* xv, sfci_vec* r, const sfci_vec* b, double lambda, double* res) {
  if (!x || !res) return set_error(SFCI_ERR_ARG, "bad res_norm arguments");
  if (vec_of(x, xv) || vec_of(x, r) || vec_of(x, b)) return SFCI_ERR_ARG;
  if (r == xv || r == b) return set_error(SFCI_ERR_ARG, "res_norm output must differ from its inputs");
  return op_res_norm(x->c, xv->v, r->v, b->v, lambda, res);
}

// ---- subspace eigenproblems -----------------------------------------------------

int sfci_cisd(sfci_ctx* x, const uint64_t* ref_key, int state_idx, int n_evals, double* evals, sfci_vec* out,
              double* resid, uint64_t* block_size) {
  if (!x || !ref_key || vec_check(out) || state_idx < 0 || n_evals < 0 || (n_evals && !evals))
    return set_error(SFCI_ERR_ARG, "bad cisd arguments");
  if (out->v.ctx != &x->c) return set_error(SFCI_ERR_ARG, "output vector belongs to another context");
  Ctx& c = x->c;
  if (c.ninst) return set_error(SFCI_ERR_UNSUPPORTED, "cisd takes an ordinary (single-Hamiltonian) context");
  return SFCI_W(c, cisd_impl, c, (const u64*)ref_key, state_idx, n_evals, evals, out->v, resid, (u64*)block_size);
}

int sfci_fci(sfci_ctx* x, int n_evals, double* evals, sfci_vec* ground, double* resid, uint64_t* dim) {
  if (!x || n_evals < 0 || (n_evals && !evals)) return set_error(SFCI_ERR_ARG, "bad fci arguments");
  if (ground && (vec_check(ground) || ground->v.ctx != &x->c))
    return set_error(SFCI_ERR_ARG, "ground vector belongs to another context");
  Ctx& c = x->c;
  if (c.ninst) return set_error(SFCI_ERR_UNSUPPORTED, "fci takes an ordinary (single-Hamiltonian) context");
  return SFCI_W(c, fci_impl, c, n_evals, evals, ground ? &ground->v : nullptr, resid, (u64*)dim);
}

int sfci_dot(sfci_ctx* x, const sfci_vec* a, const sfci_vec* b, double* out) {
  if (!x || !out) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, a) || vec_of(x, b)) return SFCI_ERR_ARG;
  return op_dot(x->c, a->v, b->v, out);
}

int sfci_norm(sfci_ctx* x, const sfci_vec* v, double* out) {
  if (!x || !out) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, v)) return SFCI_ERR_ARG;
  return norm_impl(x->c, v->v, out);
}

int sfci_scale(sfci_ctx* x, sfci_vec* v, double a) {
  if (!x) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, v)) return SFCI_ERR_ARG;
  return scale_impl(x->c, v->v, a);
}

int sfci_normalize(sfci_ctx* x, sfci_vec* v) {
  if (!x) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, v)) return SFCI_ERR_ARG;
  double n = 0;
  int st = norm_impl(x->c, v->v, &n);
  if (st) return st;
  return scale_impl(x->c, v->v, 1.0 / n);
}

int sfci_add_two(sfci_ctx* x, sfci_vec* v, const sfci_vec* w, double a) {
  if (!x) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, v) || vec_of(x, w)) return SFCI_ERR_ARG;
  return op_add_two(x->c, v->v, w->v, a);
}

int sfci_add_three(sfci_ctx* x, sfci_vec* v, const sfci_vec* a, const sfci_vec* b, const sfci_vec* cc, double ca,
                   double cb, double c3) {
  if (!x) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, v) || vec_of(x, a) || vec_of(x, b) || vec_of(x, cc)) return SFCI_ERR_ARG;
  return op_add_three(x->c, v->v, a->v, b->v, cc->v, ca, cb, c3);
}

int sfci_shrink_from(sfci_ctx* x, sfci_vec* dst, const sfci_vec* src) {
  if (!x) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, dst) || vec_of(x, src)) return SFCI_ERR_ARG;
  if (dst == src) return set_error(SFCI_ERR_ARG, "shrink_from needs distinct vectors");
  return op_shrink(x->c, dst->v, src->v);
}

int sfci_combine(sfci_ctx* x, sfci_vec* dst, const sfci_vec* const* vs, const double* coef, int n) {
  if (!x || n < 0 || (n && (!vs || !coef))) return set_error(SFCI_ERR_ARG, "null argument");
  if (vec_of(x, dst)) return SFCI_ERR_ARG;
  std::vector<const Vec*> p(n);
  for (int i = 0; i < n; ++i) {
    if (vec_of(x, vs[i])) return SFCI_ERR_ARG;
    p[i] = &vs[i]->v;
  }
  return op_combine(x->c, dst->v, p.data(), coef, n);
}

}  // extern "C"

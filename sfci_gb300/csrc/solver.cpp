// Krylov drivers on device-resident sparse vectors, and the FP64 generalised
// symmetric eigensolver they use.
//
// sfci_lanczos_ground follows sparse_krylov_solve_eigenval
// (src/sparse_solver.cpp:246-548) step for step; sfci_minres follows minres_sp
// (src/minres.cpp:73-225), including its quirk of comparing the squared
// residual with the unsquared tolerance (:211); sfci_krylov_linear follows
// sparse_krylov_solve_linear (src/sparse_solver.cpp:561-730) and
// sfci_shift_invert sparse_solve_SI (:732-771).  Every sparse-vector operation
// runs on the GPU; only the Nl x Nl projected matrices and scalars live on the
// host.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <limits>
#include <memory>
#include <vector>

#include "hostla.h"
#include "internal.h"
#include "spmspv.h"

namespace sfci {

// ---- K c = E S c ----------------------------------------------------------------
// Cholesky S = L L^T, C = L^-1 K L^-T, cyclic Jacobi on C, x = L^-T y: the
// eigenvectors come out S-orthonormal, as Eigen's GeneralizedSelfAdjointEigenSolver
// returns them (Ax_lBx mode).  Column-major n x n arrays.
static int gsaes_impl(int n, const double* K, const double* S, double* ev, double* X) {
  std::vector<double> L((size_t)n * n, 0.0), C((size_t)n * n), V((size_t)n * n, 0.0);
  auto at = [n](std::vector<double>& A, int i, int j) -> double& { return A[(size_t)j * n + i]; };
  for (int j = 0; j < n; ++j) {
    double d = S[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) d -= at(L, j, k) * at(L, j, k);
    if (!(d > 0.0)) return set_error(SFCI_ERR_NUMERIC, "overlap matrix is not positive definite");
    double ljj = std::sqrt(d);
    at(L, j, j) = ljj;
    for (int i = j + 1; i < n; ++i) {
      double s = S[(size_t)j * n + i];
      for (int k = 0; k < j; ++k) s -= at(L, i, k) * at(L, j, k);
      at(L, i, j) = s / ljj;
    }
  }
  // T = L^-1 K  (forward substitution per column), C = T L^-T = (L^-1 T^T)^T
  std::vector<double> T((size_t)n * n);
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) {
      double s = K[(size_t)c * n + i];
      for (int k = 0; k < i; ++k) s -= at(L, i, k) * T[(size_t)c * n + k];
      T[(size_t)c * n + i] = s / at(L, i, i);
    }
  for (int r = 0; r < n; ++r)  // C(r, :) = L^-1 applied to row r of T
    for (int i = 0; i < n; ++i) {
      double s = T[(size_t)i * n + r];
      for (int k = 0; k < i; ++k) s -= at(L, i, k) * at(C, r, k);
      at(C, r, i) = s / at(L, i, i);
    }
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      double m = 0.5 * (at(C, i, j) + at(C, j, i));
      at(C, i, j) = at(C, j, i) = m;
    }
  for (int i = 0; i < n; ++i) at(V, i, i) = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += at(C, p, q) * at(C, p, q);
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = at(C, p, q);
        if (std::fabs(apq) < 1e-300) continue;
        double theta = (at(C, q, q) - at(C, p, p)) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = at(C, k, p), akq = at(C, k, q);
          at(C, k, p) = c * akp - s * akq;
          at(C, k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = at(C, p, k), aqk = at(C, q, k);
          at(C, p, k) = c * apk - s * aqk;
          at(C, q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = at(V, k, p), vkq = at(V, k, q);
          at(V, k, p) = c * vkp - s * vkq;
          at(V, k, q) = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int a, int b) { return at(C, a, a) < at(C, b, b); });
  for (int k = 0; k < n; ++k) {
    int src = ord[k];
    ev[k] = at(C, src, src);
    // x = L^-T y  (back substitution)
    for (int i = n - 1; i >= 0; --i) {
      double s = at(V, i, src);
      for (int r = i + 1; r < n; ++r) s -= at(L, r, i) * X[(size_t)k * n + r];
      X[(size_t)k * n + i] = s / at(L, i, i);
    }
    // deterministic sign: largest-magnitude component positive
    int im = 0;
    for (int i = 1; i < n; ++i)
      if (std::fabs(X[(size_t)k * n + i]) > std::fabs(X[(size_t)k * n + im])) im = i;
    if (X[(size_t)k * n + im] < 0)
      for (int i = 0; i < n; ++i) X[(size_t)k * n + i] = -X[(size_t)k * n + i];
  }
  return SFCI_OK;
}

// ---- RAII device vectors for the drivers -----------------------------------------
struct DVec {
  Ctx* c = nullptr;
  Vec v;
  int alloc(Ctx& ctx, uint64_t cap) {
    c = &ctx;
    v.ctx = &ctx;
    v.cap = cap;
    v.len = 0;
    size_t n = cap ? cap : 1;
    // the products keep their scratch between calls (up to most of the
    // device); a driver vector that finds no room releases it and retries, and
    // the next product plans with what is left
    for (int attempt = 0; attempt < 2; ++attempt) {
      if (cudaMalloc(&v.keys, n * ctx.W * sizeof(u64)) == cudaSuccess &&
          cudaMalloc(&v.amps, n * sizeof(double)) == cudaSuccess)
        return SFCI_OK;
      cudaGetLastError();
      if (v.keys) cudaFree(v.keys);
      v.keys = nullptr;
      v.amps = nullptr;
      if (attempt == 0) {
        cudaStreamSynchronize(ctx.stream);
        scratch_free_all(ctx);
      }
    }
    return set_error(SFCI_ERR_NOMEM, "driver vector allocation failed");
  }
  ~DVec() {
    if (v.keys) cudaFree(v.keys);
    if (v.amps) cudaFree(v.amps);
  }
};

#define TRY(x)              \
  do {                      \
    int s_ = (x);           \
    if (s_) return s_;      \
  } while (0)

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

static int norm_of(Ctx& c, const Vec& v, double* n) { return norm_impl(c, v, n); }

int lanczos_ground(Ctx& c, Vec& v, int Nl, int restarts, double* energies, double* final_e) {
  const bool vb = c.opts.verbose != 0;
  const uint64_t Nd = c.opts.Nd, cap = c.opts.hpsi_cap;
  std::vector<std::unique_ptr<DVec>> KB(Nl);
  for (int i = 0; i < Nl; ++i) {
    KB[i].reset(new DVec);
    TRY(KB[i]->alloc(c, Nd));
  }
  DVec u, temp, temp_u, v_next, vv;
  TRY(u.alloc(c, cap));
  TRY(temp.alloc(c, cap));
  TRY(temp_u.alloc(c, cap));
  TRY(v_next.alloc(c, Nd));
  TRY(vv.alloc(c, (uint64_t)Nl * Nd));
  std::vector<double> KM((size_t)Nl * Nl, 0.0), S((size_t)Nl * Nl, 0.0), ev(Nl), X((size_t)Nl * Nl);
  auto km = [&](int i, int j) -> double& { return KM[(size_t)j * Nl + i]; };
  auto sm = [&](int i, int j) -> double& { return S[(size_t)j * Nl + i]; };
  const double deltaE = 1e-5;
  double previousE = 0.0, nearestE = -1000000.0;
  for (int r = 0; r < restarts; ++r) energies[r] = std::numeric_limits<double>::quiet_NaN();
  for (int res = 0; res < restarts; ++res) {
    if (vb) printf("\n*****************block %d starts*****************\n", res);
    TRY(op_copy(c, KB[0]->v, v));
    double alpha = 0.0;
    TRY(op_spmspv(c, v, u.v, 0.0, 1.0, &alpha));
    if (vb) printf("H * phi_0 len:%llu\n", (unsigned long long)u.v.len);
    km(0, 0) = alpha;
    double beta = 0.0;
    for (int i = 1; i < Nl; ++i) {
      double t_it = now_s();
      TRY(op_copy(c, temp.v, u.v));
      TRY(op_add_two(c, temp.v, v, -alpha));
      TRY(op_shrink(c, v_next.v, temp.v));
      double gamma = 0.0;
      TRY(norm_of(c, v_next.v, &gamma));
      beta = gamma;
      TRY(scale_impl(c, v_next.v, 1.0 / gamma));
      double t_sp = now_s();
      TRY(op_spmspv(c, v_next.v, temp_u.v, 0.0, 1.0, &alpha));
      cudaStreamSynchronize(c.stream);
      if (vb) printf("Single spmspvm time:%.6f\n", now_s() - t_sp);
      km(i, i) = alpha;
      for (int j = 0; j < i; ++j) {
        double d = 0.0;
        TRY(op_dot(c, KB[j]->v, temp_u.v, &d));
        km(j, i) = d;
        km(i, j) = d;
      }
      TRY(op_add_two(c, temp_u.v, v, -beta));
      TRY(op_copy(c, u.v, temp_u.v));
      TRY(op_copy(c, v, v_next.v));
      TRY(op_copy(c, KB[i]->v, v));
      temp.v.len = 0;
      temp_u.v.len = 0;
      if (vb) printf("time of current iter:%.6f\n", now_s() - t_it);
    }
    for (int i = 0; i < Nl; ++i)
      for (int j = i; j < Nl; ++j) {
        double d = 0.0;
        TRY(op_dot(c, KB[i]->v, KB[j]->v, &d));
        sm(i, j) = d;
        sm(j, i) = d;
      }
    TRY(gsaes_impl(Nl, KM.data(), S.data(), ev.data(), X.data()));
    int idx = 0;
    double gap = std::fabs(nearestE - ev[0]);
    for (int i = 1; i < Nl; ++i)
      if (std::fabs(nearestE - ev[i]) < gap) {
        gap = std::fabs(nearestE - ev[i]);
        idx = i;
      }
    nearestE = ev[idx];
    std::vector<const Vec*> ptr(Nl);
    for (int i = 0; i < Nl; ++i) ptr[i] = &KB[i]->v;
    TRY(op_combine(c, vv.v, ptr.data(), X.data() + (size_t)idx * Nl, Nl));
    TRY(op_shrink(c, v, vv.v));
    double nv = 0.0;
    TRY(norm_of(c, v, &nv));
    TRY(scale_impl(c, v, 1.0 / nv));
    if (vb) {
      double et = 0.0;
      TRY(op_energy(c, v, &et));
      printf("energy Psi_res after truncation:%.12f\n", et);
    }
    std::fill(KM.begin(), KM.end(), 0.0);
    for (int i = 0; i < Nl; ++i) KB[i]->v.len = 0;
    energies[res] = ev[idx];
    if (vb) printf("gsaes energy:%.12f\n*****************block %d ends*****************\n", ev[idx], res);
    if (previousE - ev[idx] < deltaE) break;
    previousE = ev[idx];
  }
  double fe = 0.0;
  TRY(op_energy(c, v, &fe));
  if (vb) printf("final e:%.12f\n", fe);
  *final_e = fe;
  return SFCI_OK;
}

int krylov_linear(Ctx& c, const Vec& b, Vec& result, double target_energy, int num_iter, int num_restart,
                  double* residues) {
  const bool vb = c.opts.verbose != 0;
  const uint64_t Nd = c.opts.Nd;
  if (b.len > Nd) return set_error(SFCI_ERR_CAPACITY, "right-hand side longer than Nd");
  const int n1 = num_iter + 1;
  std::vector<std::unique_ptr<DVec>> V(n1);
  for (int i = 0; i < n1; ++i) {
    V[i].reset(new DVec);
    TRY(V[i]->alloc(c, Nd));
  }
  DVec w, r0, xm, sum;
  TRY(w.alloc(c, Nd));
  TRY(r0.alloc(c, Nd));
  TRY(xm.alloc(c, Nd));
  TRY(sum.alloc(c, (uint64_t)num_iter * Nd));
  std::vector<double> hess((size_t)n1 * n1, 0.0), S((size_t)n1 * n1, 0.0), hij(n1, 0.0);
  auto hm = [&](int i, int j) -> double& { return hess[(size_t)j * n1 + i]; };
  auto sm = [&](int i, int j) -> double& { return S[(size_t)j * n1 + i]; };
  TRY(op_copy(c, r0.v, b));  // x0 = 0: r0 = b (:615-616)
  for (int res = 0; res < num_restart; ++res) {
    double beta = 0.0;
    TRY(norm_of(c, r0.v, &beta));
    TRY(op_copy(c, V[0]->v, r0.v));
    if (beta > 0.0) TRY(scale_impl(c, V[0]->v, 1.0 / beta));
    if (vb) printf("initial residue: %.12g\n", beta);
    std::vector<const Vec*> bp;
    for (int i = 0; i < n1; ++i) {
      bp.push_back(&V[i]->v);
      std::fill(hij.begin(), hij.end(), 0.0);
      TRY(op_spmspv_linear(c, V[i]->v, w.v, target_energy, bp.data(), i + 1, hij.data()));
      for (int j = i; j >= 0; --j) {
        hm(j, i) = hij[j];
        hm(i, j) = hij[j];
        double d = 0.0;
        TRY(op_dot(c, V[j]->v, V[i]->v, &d));
        sm(i, j) = d;
        sm(j, i) = d;
      }
      double wn = 0.0;
      TRY(norm_of(c, w.v, &wn));
      if (!(wn > 0.0)) return set_error(SFCI_ERR_NUMERIC, "linear solver: the Krylov vector vanished");
      TRY(scale_impl(c, w.v, 1.0 / wn));
      if (i < num_iter) TRY(op_copy(c, V[i + 1]->v, w.v));
    }
    // (S H_rec) y = beta S e_0 in the least-squares sense (:679-692)
    std::vector<double> A((size_t)n1 * num_iter, 0.0), e(n1);
    for (int i = 0; i < n1; ++i) {
      e[i] = sm(i, 0) * beta;
      for (int j = 0; j < num_iter; ++j) {
        double t = 0.0;
        for (int k = 0; k < n1; ++k) t += sm(i, k) * hm(k, j);
        A[(size_t)j * n1 + i] = t;
      }
    }
    std::vector<double> y;
    hostla::lstsq_qr(n1, num_iter, A, e, y);
    // x_m += V_m y: merged, no cut (add_bucketed_vec, src/functions.cpp:807-856),
    // then addTwo's top-Nd
    TRY(op_combine(c, sum.v, bp.data(), y.data(), num_iter));
    TRY(op_add_two(c, xm.v, sum.v, 1.0));
    double rn = 0.0;
    TRY(op_res_norm(c, xm.v, r0.v, b, target_energy, &rn));
    TRY(scale_impl(c, r0.v, -1.0));
    if (residues) residues[res] = rn;
    if (vb) printf("residue after truncation: %.12g\n*************************restart %d ends*************************\n",
                   rn, res);
  }
  return op_copy(c, result, xm.v);
}

int shift_invert(Ctx& c, Vec& b, double target_energy, int num_iter, int num_restart, double* energy) {
  DVec result;
  TRY(result.alloc(c, c.opts.Nd));
  TRY(krylov_linear(c, b, result.v, target_energy, num_iter, num_restart, nullptr));
  TRY(op_copy(c, b, result.v));
  double nb = 0.0;
  TRY(norm_of(c, b, &nb));
  if (nb > 0.0) TRY(scale_impl(c, b, 1.0 / nb));
  return op_energy(c, b, energy);
}

int minres(Ctx& c, const Vec& rhs, const Vec& guess, Vec& result, int iters, double tol, double lambda,
           int* iters_done) {
  const uint64_t N = c.opts.Nd;
  double rhsn = 0.0;
  TRY(norm_of(c, rhs, &rhsn));
  DVec x, v_old, v, v_new, w, w_new, p_oold, p_old, p;
  for (DVec* d : {&x, &v_old, &v, &v_new, &w, &w_new, &p_oold, &p_old, &p}) TRY(d->alloc(c, N));
  TRY(op_copy(c, x.v, guess));
  double diag = 0.0;
  TRY(op_spmspv(c, x.v, v_new.v, lambda, -1.0, &diag));
  TRY(op_add_two(c, v_new.v, rhs, 1.0));
  double nr = 0.0;
  TRY(norm_of(c, v_new.v, &nr));
  double residualNorm2 = nr * nr;
  TRY(op_copy(c, w_new.v, v_new.v));
  double beta_new2 = 0.0;
  TRY(op_dot(c, v_new.v, w_new.v, &beta_new2));
  double beta_new = std::sqrt(beta_new2), beta_one = beta_new;
  TRY(scale_impl(c, v_new.v, 1.0 / beta_new));
  TRY(scale_impl(c, w_new.v, 1.0 / beta_new));
  double cs = 1.0, c_old = 1.0, s = 0.0, s_old = 0.0, eta = 1.0;
  p_old.v.len = 0;
  p.v.len = 0;
  int it = 0, done = 0;
  while (it < iters) {
    double beta = beta_new;
    TRY(op_copy(c, v_old.v, v.v));
    TRY(op_copy(c, v.v, v_new.v));
    TRY(op_copy(c, w.v, w_new.v));
    TRY(op_spmspv(c, w.v, v_new.v, lambda, 1.0, &diag));
    TRY(op_add_two(c, v_new.v, v_old.v, -beta));
    double alpha = 0.0;
    TRY(op_dot(c, v_new.v, w.v, &alpha));
    TRY(op_add_two(c, v_new.v, v.v, -alpha));
    TRY(op_copy(c, w_new.v, v_new.v));
    TRY(op_dot(c, v_new.v, w_new.v, &beta_new2));
    beta_new = std::sqrt(beta_new2);
    TRY(scale_impl(c, v_new.v, 1.0 / beta_new));
    TRY(scale_impl(c, w_new.v, 1.0 / beta_new));
    const double r2 = s * alpha + cs * c_old * beta;
    const double r3 = s_old * beta;
    const double r1_hat = cs * alpha - c_old * s * beta;
    const double r1 = std::sqrt(r1_hat * r1_hat + beta_new * beta_new);
    c_old = cs;
    s_old = s;
    cs = r1_hat / r1;
    s = beta_new / r1;
    TRY(op_copy(c, p_oold.v, p_old.v));
    TRY(op_copy(c, p_old.v, p.v));
    TRY(op_add_three(c, p.v, w.v, p_old.v, p_oold.v, 1.0 / r1, -r2 / r1, -r3 / r1));
    TRY(op_add_two(c, x.v, p.v, beta_one * cs * eta));
    residualNorm2 *= s * s;
    ++done;
    if (c.opts.verbose) printf("res norm:%.12g\n%d is done\n", residualNorm2, it);
    if (residualNorm2 < tol) break;
    eta = -s * eta;
    ++it;
  }
  if (iters_done) *iters_done = done;
  return op_copy(c, result, x.v);
}

}  // namespace sfci

using namespace sfci;

extern "C" {

int sfci_gsaes(int n, const double* K, const double* S, double* evals, double* evecs) {
  if (n <= 0 || !K || !S || !evals || !evecs) return set_error(SFCI_ERR_ARG, "bad gsaes arguments");
  return gsaes_impl(n, K, S, evals, evecs);
}

int sfci_lanczos_ground(sfci_ctx* x, sfci_vec* v, int Nl, int restarts, double* energies, double* final_e) {
  if (!x || !v || !energies || !final_e || Nl < 1 || restarts < 1)
    return set_error(SFCI_ERR_ARG, "bad lanczos arguments");
  if (vec_of(x, v)) return SFCI_ERR_ARG;
  if (v->v.len == 0) return set_error(SFCI_ERR_ARG, "lanczos start vector is empty");
  return lanczos_ground(x->c, v->v, Nl, restarts, energies, final_e);
}

int sfci_krylov_linear(sfci_ctx* x, const sfci_vec* b, sfci_vec* result, double target_energy, int num_iter,
                       int num_restart, double* residues) {
  if (!x || !b || !result || num_iter < 1 || num_iter > 63 || num_restart < 1 || b == result)
    return set_error(SFCI_ERR_ARG, "bad krylov_linear arguments");
  if (vec_of(x, b) || vec_of(x, result)) return SFCI_ERR_ARG;
  if (b->v.len == 0) return set_error(SFCI_ERR_ARG, "krylov_linear right-hand side is empty");
  return krylov_linear(x->c, b->v, result->v, target_energy, num_iter, num_restart, residues);
}

int sfci_shift_invert(sfci_ctx* x, sfci_vec* b, double target_energy, int num_iter, int num_restart, double* energy) {
  if (!x || !b || !energy || num_iter < 1 || num_iter > 63 || num_restart < 1)
    return set_error(SFCI_ERR_ARG, "bad shift_invert arguments");
  if (vec_of(x, b)) return SFCI_ERR_ARG;
  if (b->v.len == 0) return set_error(SFCI_ERR_ARG, "shift_invert start vector is empty");
  return shift_invert(x->c, b->v, target_energy, num_iter, num_restart, energy);
}

int sfci_minres(sfci_ctx* x, const sfci_vec* rhs, const sfci_vec* guess, sfci_vec* result, int iters, double tol,
                double lambda, int* iters_done) {
  if (!x || !rhs || !guess || !result || iters < 0) return set_error(SFCI_ERR_ARG, "bad minres arguments");
  if (vec_of(x, rhs) || vec_of(x, guess) || vec_of(x, result)) return SFCI_ERR_ARG;
  return minres(x->c, rhs->v, guess->v, result->v, iters, tol, lambda, iters_done);
}

}  // extern "C"

namespace sfci {

// ---- batched instances ------------------------------------------------------------
// sparse_krylov_solve_eigenval (src/sparse_solver.cpp:246-548) on n instances
// of a batched context at once.  Every Krylov step is ONE product over all
// active instances: their vectors (keys tagged by instance, so concatenation in
// instance order is key order) are concatenated, multiplied by one pass of the
// product pipeline, and the result is split at the instance tags.  Each
// instance's <v|Hv> comes from the same pass.  The rest of the step (dots,
// axpys, truncation to the instance's Nd = its vector capacity, the Nl x Nl
// eigenproblem) is per instance, as in the single-instance driver.  The merge is
// exact, so each instance's product equals its unbatched product bit for bit;
// energies agree with unbatched runs to the rounding of the <v|Hv> partial sums.
namespace {
struct GrowVec {
  DVec d;
  uint64_t phys = 0;  // allocated entries
  // room for at least `want` entries; the vector's capacity, which is what caps
  // an axpy or a product into it, is min(allocated, limit)
  int need(Ctx& c, uint64_t want, uint64_t limit = ~0ull) {
    if (!d.v.keys || phys < want) {
      if (d.v.keys) cudaFree(d.v.keys);
      if (d.v.amps) cudaFree(d.v.amps);
      d.v.keys = nullptr;
      d.v.amps = nullptr;
      TRY(d.alloc(c, std::max<uint64_t>(want, 1024)));
      phys = d.v.cap;
    }
    d.v.cap = std::min(phys, limit);
    return SFCI_OK;
  }
};
struct Inst {
  Vec* v = nullptr;
  uint64_t Nd = 0;
  std::vector<std::unique_ptr<DVec>> KB;
  GrowVec u, temp, temp_u;
  DVec v_next, vv;
  std::vector<double> KM, S, ev, X;
  double previousE = 0.0, nearestE = -1000000.0, alpha = 0.0, beta = 0.0;
  bool active = true;
};
}  // namespace

// one product over the instances in `idx` (inputs in[i]), outputs split into out[i]
static int batched_product(Ctx& c, std::vector<Inst>& S, const std::vector<int>& idx, GrowVec& all_in,
                           GrowVec& all_out, bool use_next, int nin) {
  uint64_t tot = 0;
  for (int i : idx) tot += use_next ? S[i].v_next.v.len : S[i].v->len;
  TRY(all_in.need(c, tot));
  uint64_t o = 0;
  for (int i : idx) {
    const Vec& x = use_next ? S[i].v_next.v : *S[i].v;
    if (x.len) {
      SFCI_CUDA(cudaMemcpyAsync(all_in.d.v.keys + o * 2, x.keys, x.len * 2 * sizeof(u64), cudaMemcpyDeviceToDevice,
                                c.stream));
      SFCI_CUDA(cudaMemcpyAsync(all_in.d.v.amps + o, x.amps, x.len * sizeof(double), cudaMemcpyDeviceToDevice,
                                c.stream));
    }
    o += x.len;
  }
  all_in.d.v.len = tot;
  // The product's output capacity is a cap over the whole batch, but each
  // instance's cap is hpsi_cap, as in its own driver.  So the batch output
  // holds every survivor (the capacity grows, and the product is redone, when
  // the survivors outgrow it), and each instance's slice is cut to hpsi_cap by
  // the same stable top-k rule the product's own cap applies.
  const uint64_t hcap = c.opts.hpsi_cap;
  uint64_t want = std::max<uint64_t>(hcap, all_out.d.v.cap);
  double dg = 0.0;
  const uint64_t Nd = c.opts.Nd;
  for (int attempt = 0;; ++attempt) {
    TRY(all_out.need(c, want));
    c.opts.Nd = std::max<uint64_t>(Nd, tot);  // each instance is already truncated to its own Nd
    int st = op_spmspv(c, all_in.d.v, all_out.d.v, 0.0, 1.0, &dg);
    c.opts.Nd = Nd;
    TRY(st);
    const uint64_t surv = c.stats[3];
    if (!c.last_pruned && surv <= all_out.d.v.cap) break;
    if (attempt >= 8) return set_error(SFCI_ERR_NOMEM, "batched SpMSpV: survivors keep outgrowing the output");
    want = std::max<uint64_t>(surv + surv / 4, 2 * all_out.d.v.cap);
  }
  std::vector<u64> b(nin + 1);
  TRY(inst_bounds(c, all_out.d.v, nin, b.data()));
  for (int i : idx) {
    GrowVec& dst = use_next ? S[i].temp_u : S[i].u;
    const uint64_t n = b[i + 1] - b[i];
    // room for the axpy that follows (at most Nd more entries), as the single
    // driver's HPsiCap-sized vectors have
    TRY(dst.need(c, std::min<uint64_t>(hcap, n + S[i].Nd), hcap));
    Vec slice;
    slice.ctx = &c;
    slice.keys = all_out.d.v.keys + b[i] * 2;
    slice.amps = all_out.d.v.amps + b[i];
    slice.len = slice.cap = n;
    if (n > hcap) {
      Vec cut = dst.d.v;
      cut.cap = hcap;
      TRY(op_shrink(c, cut, slice));
      dst.d.v.len = cut.len;
    } else {
      if (n) {
        SFCI_CUDA(cudaMemcpyAsync(dst.d.v.keys, slice.keys, n * 2 * sizeof(u64), cudaMemcpyDeviceToDevice, c.stream));
        SFCI_CUDA(cudaMemcpyAsync(dst.d.v.amps, slice.amps, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
      }
      dst.d.v.len = n;
    }
    S[i].alpha = c.inst_diag.size() > (size_t)i ? c.inst_diag[i] : 0.0;
  }
  return SFCI_OK;
}

int lanczos_batched(Ctx& c, Vec* const* v, int n, int Nl, int restarts, double* energies, double* final_e) {
  if (!c.ninst || c.W != 2) return set_error(SFCI_ERR_ARG, "batched Lanczos needs a batched context");
  if (n != c.ninst) return set_error(SFCI_ERR_ARG, "batched Lanczos: one vector per instance");
  if (Nl < 2 || restarts < 1) return set_error(SFCI_ERR_ARG, "batched Lanczos: Nl >= 2 and restarts >= 1");
  std::vector<Inst> S(n);
  for (int i = 0; i < n; ++i) {
    Inst& s = S[i];
    s.v = v[i];
    s.Nd = v[i]->cap;
    s.KB.resize(Nl);
    for (int k = 0; k < Nl; ++k) {
      s.KB[k].reset(new DVec);
      TRY(s.KB[k]->alloc(c, s.Nd));
    }
    TRY(s.v_next.alloc(c, s.Nd));
    TRY(s.vv.alloc(c, (uint64_t)Nl * s.Nd));
    s.KM.assign((size_t)Nl * Nl, 0.0);
    s.S.assign((size_t)Nl * Nl, 0.0);
    s.ev.assign(Nl, 0.0);
    s.X.assign((size_t)Nl * Nl, 0.0);
    for (int r = 0; r < restarts; ++r) energies[(size_t)i * restarts + r] = std::numeric_limits<double>::quiet_NaN();
  }
  GrowVec all_in, all_out;
  const double deltaE = 1e-5;
  for (int res = 0; res < restarts; ++res) {
    std::vector<int> idx;
    for (int i = 0; i < n; ++i)
      if (S[i].active) idx.push_back(i);
    if (idx.empty()) break;
    for (int i : idx) TRY(op_copy(c, S[i].KB[0]->v, *S[i].v));
    TRY(batched_product(c, S, idx, all_in, all_out, false, n));
    for (int i : idx) {
      auto km = [&](int a, int b) -> double& { return S[i].KM[(size_t)b * Nl + a]; };
      km(0, 0) = S[i].alpha;
    }
    for (int it = 1; it < Nl; ++it) {
      for (int i : idx) {
        Inst& s = S[i];
        TRY(s.temp.need(c, std::min<uint64_t>(c.opts.hpsi_cap, s.u.d.v.len + s.v->len), c.opts.hpsi_cap));
        TRY(op_copy(c, s.temp.d.v, s.u.d.v));
        TRY(op_add_two(c, s.temp.d.v, *s.v, -s.alpha));
        TRY(op_shrink(c, s.v_next.v, s.temp.d.v));
        double gamma = 0.0;
        TRY(norm_of(c, s.v_next.v, &gamma));
        s.beta = gamma;
        TRY(scale_impl(c, s.v_next.v, 1.0 / gamma));
      }
      TRY(batched_product(c, S, idx, all_in, all_out, true, n));
      for (int i : idx) {
        Inst& s = S[i];
        auto km = [&](int a, int b) -> double& { return s.KM[(size_t)b * Nl + a]; };
        km(it, it) = s.alpha;
        for (int j = 0; j < it; ++j) {
          double d = 0.0;
          TRY(op_dot(c, s.KB[j]->v, s.temp_u.d.v, &d));
          km(j, it) = d;
          km(it, j) = d;
        }
        TRY(op_add_two(c, s.temp_u.d.v, *s.v, -s.beta));
        TRY(s.u.need(c, s.temp_u.d.v.len, c.opts.hpsi_cap));
        TRY(op_copy(c, s.u.d.v, s.temp_u.d.v));
        TRY(op_copy(c, *s.v, s.v_next.v));
        TRY(op_copy(c, s.KB[it]->v, *s.v));
      }
    }
    for (int i : idx) {
      Inst& s = S[i];
      auto sm = [&](int a, int b) -> double& { return s.S[(size_t)b * Nl + a]; };
      for (int a = 0; a < Nl; ++a)
        for (int b = a; b < Nl; ++b) {
          double d = 0.0;
          TRY(op_dot(c, s.KB[a]->v, s.KB[b]->v, &d));
          sm(a, b) = d;
          sm(b, a) = d;
        }
      TRY(gsaes_impl(Nl, s.KM.data(), s.S.data(), s.ev.data(), s.X.data()));
      int k = 0;
      double gap = std::fabs(s.nearestE - s.ev[0]);
      for (int a = 1; a < Nl; ++a)
        if (std::fabs(s.nearestE - s.ev[a]) < gap) {
          gap = std::fabs(s.nearestE - s.ev[a]);
          k = a;
        }
      s.nearestE = s.ev[k];
      std::vector<const Vec*> ptr(Nl);
      for (int a = 0; a < Nl; ++a) ptr[a] = &s.KB[a]->v;
      TRY(op_combine(c, s.vv.v, ptr.data(), s.X.data() + (size_t)k * Nl, Nl));
      TRY(op_shrink(c, *s.v, s.vv.v));
      double nv = 0.0;
      TRY(norm_of(c, *s.v, &nv));
      TRY(scale_impl(c, *s.v, 1.0 / nv));
      std::fill(s.KM.begin(), s.KM.end(), 0.0);
      for (int a = 0; a < Nl; ++a) s.KB[a]->v.len = 0;
      energies[(size_t)i * restarts + res] = s.ev[k];
      if (s.previousE - s.ev[k] < deltaE) s.active = false;  // the signed test of :535
      s.previousE = s.ev[k];
    }
  }
  for (int i = 0; i < n; ++i) TRY(op_energy(c, *S[i].v, &final_e[i]));
  return SFCI_OK;
}

}  // namespace sfci

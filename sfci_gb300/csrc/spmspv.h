// Entry points of the device hot path, one instantiation per key width W.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace sfci {

// Extra input of spmspv_impl: each listed vector enters the merge as one term
// per entry, amplitude coef * amp (before the cut); when sumsq is set it
// receives the sum over merged determinants of their squared amplitude, before
// the cut.
struct SpExtra {
  const Vec* vecs[2] = {nullptr, nullptr};
  double coef[2] = {0.0, 0.0};
  int n = 0;
  double* sumsq = nullptr;
};

template <int W> int spmspv_impl(Ctx& c, const Vec& in, Vec& out, double lambda, double coeff, double* diag,
                                 const SpExtra* ex = nullptr);
template <int W> int project_impl(Ctx& c, const Vec& src, double lambda, const Vec* const* basis, int nv,
                                  double* out);
template <int W> int spmspv_linear_impl(Ctx& c, const Vec& in, Vec& out, double lambda, const Vec* const* basis,
                                        int nb, double* hij);
template <int W> int res_norm_impl(Ctx& c, const Vec& x, Vec& r, const Vec& b, double lambda, double* res);
template <int W> int energy_impl(Ctx& c, const Vec& psi, double* E);
template <int W> int diag_elements_impl(Ctx& c, const typename KeyOf<W>::T* dkeys, u64 n, double* out_host);

template <int W> int dot_impl(Ctx& c, const Vec& x, const Vec& y, double* out);
template <int W> int add_two_impl(Ctx& c, Vec& v, const Vec& w, double a);
template <int W> int add_three_impl(Ctx& c, Vec& v, const Vec& x, const Vec& y, const Vec& z, double a, double b,
                                    double cc);
template <int W> int shrink_impl(Ctx& c, Vec& dst, const Vec& src);
template <int W> int combine_impl(Ctx& c, Vec& dst, const Vec* const* vs, const double* coef, int n);
template <int W> int sort_vec_impl(Ctx& c, Vec& v);
int scale_impl(Ctx& c, Vec& v, double a);

// subspace eigenproblems (subspace.cu)
template <int W> int cisd_impl(Ctx& c, const u64* ref_key, int state_idx, int n_evals, double* evals, Vec& out,
                               double* resid, u64* block_size);
template <int W> int fci_impl(Ctx& c, int n_evals, double* evals, Vec* ground, double* resid, u64* dim);
int norm_impl(Ctx& c, const Vec& v, double* out);

// learned excitation screen (mlp.cu, screen.cuh): the kept term groups of each
// source determinant of a product, in the screened term index space
struct ScreenList {
  const uint32_t* start = nullptr;  // full term index of each kept group's first term
  const uint32_t* pre = nullptr;    // screened term index of each kept group's first term
  const u64* off = nullptr;         // [n + 1] exclusive prefix of kept groups per source
  const u64* kept_terms = nullptr;  // per source: terms of its kept groups (group 0 not counted)
  unsigned gmax = 0;                // most kept groups of one source
  u64 groups = 0, kept_groups = 0, kept_terms_total = 0;
};
// run the screen on n sources (keys: W words each; amps: the product's input amplitudes)
int screen_select(Ctx& c, const void* keys, const double* amps, u64 n, ScreenList* out);
// groups per source (group 0 excluded), exclusive prefix in goff[0..n]
template <int W> int group_offsets_impl(Ctx& c, const typename KeyOf<W>::T* keys, u64 n, u64* goff);
// label bits of the groups of n sources: a group is alive when one of its terms,
// of magnitude above min_term, lands on a key of `out` (the product's output);
// bit goff[j] + g - 1 of labels
template <int W> int label_impl(Ctx& c, const typename KeyOf<W>::T* keys, const double* amps, u64 n,
                                const u64* goff, const Vec& out, uint32_t* labels, double min_term);

// batched contexts: first position of each instance tag 0..n in a key-sorted
// vector (n + 1 entries, host)
int inst_bounds(Ctx& c, const Vec& v, int n, u64* out_host);
// the truncated Lanczos driver on n instances of a batched context, one batched
// product per Krylov step (solver.cpp)
int lanczos_batched(Ctx& c, Vec* const* v, int n, int Nl, int restarts, double* energies, double* final_e);

// width dispatch used by the ABI and the drivers
int op_spmspv(Ctx& c, const Vec& in, Vec& out, double lambda, double coeff, double* diag);
int op_energy(Ctx& c, const Vec& psi, double* E);
int op_dot(Ctx& c, const Vec& x, const Vec& y, double* out);
int op_add_two(Ctx& c, Vec& v, const Vec& w, double a);
int op_add_three(Ctx& c, Vec& v, const Vec& x, const Vec& y, const Vec& z, double a, double b, double cc);
int op_shrink(Ctx& c, Vec& dst, const Vec& src);
int op_combine(Ctx& c, Vec& dst, const Vec* const* vs, const double* coef, int n);
int op_copy(Ctx& c, Vec& dst, const Vec& src);
int op_spmspv_linear(Ctx& c, const Vec& in, Vec& out, double lambda, const Vec* const* basis, int nb, double* hij);
int op_res_norm(Ctx& c, const Vec& x, Vec& r, const Vec& b, double lambda, double* res);

// linear Krylov driver (solver.cpp)
int krylov_linear(Ctx& c, const Vec& b, Vec& result, double target_energy, int num_iter, int num_restart,
                  double* residues);
int shift_invert(Ctx& c, Vec& b, double target_energy, int num_iter, int num_restart, double* energy);

}  // namespace sfci

/*
 * sfci_gb300 — C ABI of the GB300 (sm_103a) truncated-Krylov hot path of SFCI.
 *
 * The reference (wlj89/SFCI) is a C++/OpenMP program whose hot path is the
 * on-the-fly Hamiltonian sparse-matrix x sparse-vector product over bitstring
 * determinants (SpMVMtply_bucket) and the sparse-vector algebra and Krylov
 * drivers around it.  Its functions are plain C++ on global state; this header
 * is the drop-in replacement boundary: plain pointers and sizes, status codes,
 * opaque handles, device-resident vectors, one CUDA stream per context.
 *
 * Keys: a determinant is an occupation bitstring over num_orb spin orbitals
 * (spin orbital b: spatial b >> 1, spin b & 1).  Keys cross the ABI as
 * key_words() uint64 words per determinant, low word first (1 word for
 * num_orb <= 64, 2 words for num_orb <= 128).
 *
 * Every call returns SFCI_OK (0) or a negative status; sfci_last_error()
 * returns a message for the calling thread's last failure.  A context is used
 * from one host thread at a time.  Vectors passed to a call together with a
 * context must have been created on it (SFCI_ERR_ARG otherwise: another
 * context's keys may have another width); sfci_vec_copy needs both vectors on
 * one context.  The screen's label log alone takes vectors of another context
 * over the same number of orbitals.
 */
#ifndef SFCI_GB300_H
#define SFCI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum sfci_status {
  SFCI_OK = 0,
  SFCI_ERR_ARG = -1,        /* invalid argument / size */
  SFCI_ERR_IO = -2,         /* integral file missing or malformed */
  SFCI_ERR_NOMEM = -3,      /* device memory budget exceeded (never an overflow) */
  SFCI_ERR_CUDA = -4,       /* CUDA runtime error */
  SFCI_ERR_CAPACITY = -5,   /* a vector's capacity is smaller than its contents */
  SFCI_ERR_UNSUPPORTED = -6,/* input the implementation does not handle */
  SFCI_ERR_NUMERIC = -7     /* non-positive-definite overlap, NaN, ... */
};

typedef struct sfci_ctx sfci_ctx;
typedef struct sfci_vec sfci_vec;

/* Options: the sfci.input keys that shape the hot path (src/main.cpp:58-124)
 * plus the constants src/main.cpp:194-196 hard-codes.  Zero fields take the
 * reference defaults. */
typedef struct sfci_opts {
  uint64_t Nd;             /* Krylov truncation (default 200000, src/main.cpp:23) */
  uint64_t hpsi_cap;       /* capacity of H*v products (default 6e7, src/main.cpp:194) */
  double coeff_cut;        /* post-merge magnitude cut (0: the default 1e-5, src/main.cpp:196;
                              negative: no cut, every merged determinant is kept) */
  uint64_t bucket_unit;    /* accepted and ignored: sizes come from prefix sums */
  uint64_t mem_budget;     /* bytes of device scratch the SpMSpV may use (0: 90% of free) */
  int verbose;             /* 1: print the reference's progress lines */
  int reserved[7];
} sfci_opts;

const char* sfci_last_error(void);
const char* sfci_status_name(int status);
int sfci_version(void);

/* ---- context ---------------------------------------------------------------
 * Replaces load_integrals + the global set-up of src/main.cpp:170-223
 * (src/functions.cpp:398-418, src/all.h:628).  Reads an _IN integral file. */
int sfci_ctx_create(const char* in_path, int num_orb, int num_e, const sfci_opts* opts,
                    sfci_ctx** out);
int sfci_ctx_destroy(sfci_ctx* ctx);
int sfci_key_words(const sfci_ctx* ctx);
/* CUDA stream (cudaStream_t) all of the context's work is queued on. */
int sfci_ctx_stream(const sfci_ctx* ctx, void** stream);
int sfci_ctx_set_nd(sfci_ctx* ctx, uint64_t Nd);
/* Frees the device scratch the context's products keep between calls (it grows
 * to most of the free device memory); the next product allocates it again. */
int sfci_ctx_trim(sfci_ctx* ctx);
/* Kernel launches issued by this context so far (monotone counter). */
int sfci_ctx_launch_count(const sfci_ctx* ctx, uint64_t* n);
/* Timing probe: record CUDA event `slot` (0..15) on the context stream, and
 * read the elapsed milliseconds between two recorded slots (synchronises). */
int sfci_ctx_event_record(sfci_ctx* ctx, int slot);
int sfci_ctx_event_elapsed(sfci_ctx* ctx, int slot_a, int slot_b, float* ms);
/* Per-phase device time of the SpMSpV (ms, accumulated since the last reset);
 * names: "count", "scatter", "partition", "merge", "select", "sort", "other". */
int sfci_ctx_profile(sfci_ctx* ctx, int enable);
int sfci_ctx_profile_read(sfci_ctx* ctx, const char* phase, double* ms, uint64_t* launches);
int sfci_ctx_profile_reset(sfci_ctx* ctx);
/* Statistics of the last SpMSpV: [0] input dets used, [1] generated terms,
 * [2] merged unique dets, [3] survivors of the cut, [4] output length,
 * [5] passes, [6] leaves, [7] leaves that took the global-memory path. */
int sfci_ctx_last_stats(const sfci_ctx* ctx, uint64_t stats[8]);

/* ---- sparse vectors (dynVec, src/all.h:150-625) ------------------------------ */
/* A device vector of capacity cap (at most 2^40 entries, else SFCI_ERR_ARG). */
int sfci_vec_create(sfci_ctx* ctx, uint64_t cap, sfci_vec** out);
int sfci_vec_destroy(sfci_vec* v);
int sfci_vec_len(const sfci_vec* v, uint64_t* len);
int sfci_vec_cap(const sfci_vec* v, uint64_t* cap);
/* Host -> device: keys (len * key_words words) and amplitudes.  The vector is
 * sorted by key on the device if it is not already (dynVec keeps key order).
 * In a batched context every key must carry the tag of one of its instances
 * and no bit at or above that instance's num_orb, else SFCI_ERR_ARG before any
 * copy. */
int sfci_vec_upload(sfci_vec* v, const uint64_t* keys, const double* amps, uint64_t len);
/* Device -> host: copies min(len, cap) entries, reports len. */
int sfci_vec_download(const sfci_vec* v, uint64_t* keys, double* amps, uint64_t cap,
                      uint64_t* len);
/* Restart-vector text files in the reference's wf_self_as_guess.out format
 * (writer src/minres.cpp:59-70, reader readPsi src/main.cpp:288-307): the
 * length on the first line, then "key amplitude" per line, the key in decimal
 * (the whole 128-bit value for two-word keys) and the amplitude with 12
 * significant digits.  sfci_vec_load checks keys against num_orb, returns
 * SFCI_ERR_CAPACITY when the file holds more than the vector's capacity and
 * sorts the vector by key.  The sfci_psi_* forms work on host arrays and need
 * no GPU; sfci_psi_read with keys and amps NULL and cap 0 reports the length. */
int sfci_vec_save(const sfci_vec* v, const char* path);
int sfci_vec_load(sfci_vec* v, const char* path);
int sfci_psi_write(const uint64_t* keys, const double* amps, uint64_t n, int key_words, const char* path);
int sfci_psi_read(const char* path, int key_words, int num_orb, uint64_t* keys, double* amps, uint64_t cap,
                  uint64_t* len);
/* dynVec::naiveCopy (src/all.h:610-623); dst->cap must hold src->len. */
int sfci_vec_copy(sfci_vec* dst, const sfci_vec* src);
int sfci_vec_clear(sfci_vec* v);                                   /* setZeroVec :244 */

/* ---- hot path ----------------------------------------------------------------
 * SpMVMtply_bucket (src/functions.cpp:511-804, declared src/all.h:642):
 *   out = top_cap( { k : |a_k| > coeff_cut } of merge( coeff * (H - lambda) * top_Nd(in) ) )
 * sorted by key, with *diag = coeff * <top_Nd(in)| (H - lambda) |top_Nd(in)>
 * evaluated before the cut.  An empty input leaves *diag untouched and
 * empties out, as the reference does (:529-533).  Each term is rounded to the
 * nearest multiple of 2^-64 (an unbiased error of at most 2.7e-20), the rounded
 * terms of a determinant are summed exactly, whatever their order, and the sum
 * is rounded once to double; a term with |amplitude| >= 2^24 (or not finite) gives
 * SFCI_ERR_NUMERIC, and determinants connected to more than 2^19 others give
 * SFCI_ERR_UNSUPPORTED. */
int sfci_spmspv(sfci_ctx* ctx, const sfci_vec* in, sfci_vec* out, double lambda, double coeff,
                double* diag);
/* DiagCal_bit (src/bitstr.cpp:433-476) for `n` host keys (checked like
 * sfci_vec_upload's in a batched context). */
int sfci_diag_elements(sfci_ctx* ctx, const uint64_t* keys, uint64_t n, double* out);
/* calc_energy (src/functions.cpp:1272-1313): <psi|H|psi> on psi's support. */
int sfci_energy(sfci_ctx* ctx, const sfci_vec* psi, double* energy);

/* ---- sparse-vector algebra (src/all.h) ---------------------------------------- */
int sfci_dot(sfci_ctx* ctx, const sfci_vec* x, const sfci_vec* y, double* out);   /* dot :317 */
int sfci_norm(sfci_ctx* ctx, const sfci_vec* v, double* out);                      /* norm :249 */
int sfci_scale(sfci_ctx* ctx, sfci_vec* v, double alpha);                          /* scalarMtply :260 */
int sfci_normalize(sfci_ctx* ctx, sfci_vec* v);                                    /* normalize :267 */
/* v = v + a*w, merged, top-v.cap by |amp|, key order (addTwo :407-480). */
int sfci_add_two(sfci_ctx* ctx, sfci_vec* v, const sfci_vec* w, double a);
/* v = a*x + b*y + c*z, merged, top-Nd by |amp|, drop |amp| <= 1e-14 (addThree :482-608). */
int sfci_add_three(sfci_ctx* ctx, sfci_vec* v, const sfci_vec* x, const sfci_vec* y,
                   const sfci_vec* z, double a, double b, double c);
/* dst = top-dst.cap of src by |amp|, key order (shrinkFrom :281-299; src is left intact). */
int sfci_shrink_from(sfci_ctx* ctx, sfci_vec* dst, const sfci_vec* src);
/* dst = merge(sum_i coef[i] * vs[i]) (the restart combination, src/sparse_solver.cpp:492-509). */
int sfci_combine(sfci_ctx* ctx, sfci_vec* dst, const sfci_vec* const* vs, const double* coef,
                 int n);

/* ---- Krylov drivers ------------------------------------------------------------
 * sparse_krylov_solve_eigenval (src/sparse_solver.cpp:246-548): truncated
 * Lanczos with full projected H and overlap S, generalised eigensolve, nearest
 * root, restart vector truncated to Nd.  v is the start vector on entry and the
 * final restart vector on return; energies[0..restarts) receive the per-restart
 * "gsaes energy" (unused entries NaN); *final_e the closing calc_energy. */
int sfci_lanczos_ground(sfci_ctx* ctx, sfci_vec* v, int Nl, int restarts, double* energies,
                        double* final_e);
/* minres_sp (src/minres.cpp:73-225, declared src/all.h:635-638): MINRES on
 * (H - lambda) x = rhs with truncated sparse vectors.  *iters_done receives the
 * iterations run. */
int sfci_minres(sfci_ctx* ctx, const sfci_vec* rhs, const sfci_vec* guess, sfci_vec* result,
                int iters, double tol, double lambda, int* iters_done);

/* ---- linear (shift-invert) solver ------------------------------------------------
 * spmspvm_bucket_linear (src/functions.cpp:858-1094) with current_idx =
 * nbasis - 1: w = (H - lambda) in merged over the whole input (no top-Nd slice);
 * hij[j] = <w, basis[j]> for j < nbasis (1..64), before anything is removed;
 * out = top-out.cap of { |a| > cut } of w - hij[nb-1] basis[nb-1] - hij[nb-2]
 * basis[nb-2], keys ascending.  An empty input gives an empty out and leaves hij
 * as it was (:880-884). */
int sfci_spmspv_linear(sfci_ctx* ctx, const sfci_vec* in, sfci_vec* out, double lambda,
                       const sfci_vec* const* basis, int nbasis, double* hij);
/* spmspvm_bucket_res_norm (src/functions.cpp:1096-1269): r = top-r.cap of the cut
 * of merge((H - lambda) x) - b; *res = |merge((H - lambda) x) - b| before the cut. */
int sfci_res_norm(sfci_ctx* ctx, const sfci_vec* x, sfci_vec* r, const sfci_vec* b, double lambda,
                  double* res);
/* sparse_krylov_solve_linear (src/sparse_solver.cpp:561-730): (H - E_t) x = b with
 * x0 = 0, num_iter + 1 non-orthogonal Krylov vectors per restart (num_iter <= 63),
 * least squares on the projected system, x truncated to Nd; residues[r] (nullable)
 * receives |A x - b| after restart r. */
int sfci_krylov_linear(sfci_ctx* ctx, const sfci_vec* b, sfci_vec* result, double target_energy,
                       int num_iter, int num_restart, double* residues);
/* sparse_solve_SI (src/sparse_solver.cpp:732-771): one shift-invert step; b is
 * replaced by the normalised solution and *energy receives its calc_energy. */
int sfci_shift_invert(sfci_ctx* ctx, sfci_vec* b, double target_energy, int num_iter, int num_restart,
                      double* energy);

/* ---- subspace eigenproblems ----------------------------------------------------
 * calc_CISD (src/sparse_solver.cpp:15-114): lowest eigenpairs of H on the block
 * spanned by ref_key (key_words words) and every determinant it connects to.
 * `out` receives eigenvector state_idx over the whole block, keys ascending
 * (capacity >= *block_size, which is set before the capacity check); evals
 * [0..n_evals) the lowest eigenvalues ascending (the reference prints 10);
 * *resid (nullable) the norm of H x - E x.  The eigenvector sign is fixed so that
 * its largest component is positive.  Ordinary contexts only (a batched context
 * is SFCI_ERR_UNSUPPORTED), as for sfci_fci. */
int sfci_cisd(sfci_ctx* ctx, const uint64_t* ref_key, int state_idx, int n_evals, double* evals,
              sfci_vec* out, double* resid, uint64_t* block_size);
/* fci (src/dense_algo.cpp:77-124) over generateBasis (:55-74): lowest eigenvalues
 * of H on every determinant with num_e/2 alpha and num_e/2 beta electrons
 * (num_e even).  `ground` (nullable) receives the ground state, keys ascending;
 * *dim (nullable) the dimension. */
int sfci_fci(sfci_ctx* ctx, int n_evals, double* evals, sfci_vec* ground, double* resid, uint64_t* dim);

/* ---- allocation-free variant (no counterpart in the reference) -----------------
 * Sparse dot product of two key-sorted vectors held in caller-owned DEVICE arrays
 * (keys: n * key_words uint64 words; amplitudes: n doubles).  The result goes to
 * the device double *d_out, queued on `stream` (a cudaStream_t; NULL = the
 * default stream); the call does not synchronise.  It allocates no device memory:
 * its per-block partial sums live in a fixed 64 KiB device array that every GPU
 * loading the library holds until the process exits.  It is meant for callers
 * that cannot allocate: code running inside another framework's device-memory
 * pool that has reserved the GPU up front (a new cudaMalloc fails or fragments
 * the pool), or hosts whose hot loop must not allocate.  Limit: nx + ny <=
 * 16,777,216 entries, otherwise SFCI_ERR_ARG before any launch.  All calls share
 * the array, so calls whose kernels overlap on the GPU race; order them on one
 * stream.  The first call on a device looks up the array's address with that
 * device current (cudaGetSymbolAddress) and keeps it for the life of the
 * process; make that first call before any stream capture begins.  A
 * cudaDeviceReset (or a release and re-creation of the device's primary
 * context) reloads the module and leaves that cached address stale: calls on a
 * device after such a reset are not supported. */
int sfci_dot_noalloc(const uint64_t* x_keys, const double* x_amps, uint64_t nx, const uint64_t* y_keys,
                     const double* y_amps, uint64_t ny, int key_words, double* d_out, void* stream);

/* ---- batched instances (no counterpart in the reference) -------------------------
 * A batched context holds n <= 32 Hamiltonians (each <= 120 spin orbitals, keys
 * of two words): a key's top five bits (bits 123..127) name its instance, so
 * vectors of different instances never merge and one product multiplies the
 * vectors of every instance at once, each by its own Hamiltonian.  Tag keys with
 * the instance before upload.  sfci_batch_lanczos runs sparse_krylov_solve_eigenval
 * (src/sparse_solver.cpp:246-548) on every instance with one batched product
 * per Krylov step; each instance's Nd is its vector's capacity, and opts.hpsi_cap
 * caps each instance's products (not the batch's: the batched product's output
 * grows to hold every survivor, and each instance's slice is cut to hpsi_cap by
 * the single driver's rule); energies[i * restarts + r], final_e[i] per instance. */
int sfci_batch_create(int n, const char* const* in_paths, const int* num_orb, const int* num_e,
                      const sfci_opts* opts, sfci_ctx** out);
int sfci_batch_lanczos(sfci_ctx* ctx, sfci_vec* const* v, int n, int Nl, int restarts, double* energies,
                       double* final_e);
/* Product plan tunables {level-1 bits 4-9, partition digit bits 6-9, distinct keys
 * per leaf 16-120, generation CTAs per SM 1-2}: they change speed, never results
 * (the merge is exact).  sfci_autotune times candidate plans on the product of
 * `in` (into `out`), checks that they agree, and keeps the fastest. */
int sfci_ctx_set_tuning(sfci_ctx* ctx, const int* tuning4);
/* Generation passes of a product whose terms exceed the device budget: by ranges
 * of the targets' alpha class (mode 0: when three or more passes are needed; 1:
 * whenever the product can be split so; -1: never), each pass generating only
 * its own terms, or by hash bins, each pass regenerating every term.  Results
 * never depend on the mode. */
int sfci_ctx_set_class_passes(sfci_ctx* ctx, int mode);
int sfci_ctx_get_tuning(const sfci_ctx* ctx, int* tuning4);
int sfci_autotune(sfci_ctx* ctx, const sfci_vec* in, sfci_vec* out, int* best4, double* best_ms);

/* ---- learned excitation screen (no counterpart in the reference) ---------------
 * A BF16 MLP (3 layers, hidden width 256, FP32 accumulation, sigmoid output),
 * trained and run on the tensor cores, that predicts for each term group of a
 * source determinant whether any of its terms lands on a determinant that
 * survives the product's cut and cap.  A group is a source determinant's
 * excitations sharing one prefix: same-spin doubles with a given occupied pair
 * and larger hole, or opposite-spin doubles with a given spin-0 single and spin-1
 * occupied orbital; the diagonal and singles are never screened.  Features: the
 * source's occupancy bits, one-hot (p, q, r) of the prefix and its class,
 * log10 |c_j| and log10 of a bound on the group's two-body elements.  With a
 * screen attached (sfci_ctx_set_screen), sfci_spmspv and the drivers built on
 * it skip the groups predicted dead (probability below the threshold): the
 * generator of OffDiagGen_bit (src/bitstr.cpp:162-302) restricted to the kept
 * groups.  Threshold 0 keeps every group and gives the plain product exactly;
 * products with extra sources (sfci_spmspv_linear, sfci_res_norm) and
 * sfci_energy are never screened, so calc_energy stays an unscreened check of a
 * screened run's energy. */
typedef struct sfci_screen sfci_screen;
/* A screen lives on the context it is created on; destroying that context first
 * frees the screen's device memory and leaves a handle that only
 * sfci_screen_destroy accepts. */
int sfci_screen_create(sfci_ctx* ctx, uint64_t seed, sfci_screen** out);
int sfci_screen_destroy(sfci_screen* s);
/* Appends labelled examples: every term group of the determinants of `in` (at
 * most Nd of them: the sources of a product), alive when one of its terms of
 * magnitude above min_term (0: any) lands on a key of `out`, the product's output.  `in` and `out` may belong to another
 * context with the same number of orbitals (another Hamiltonian, up to 64 of
 * them per screen); the screen keeps that Hamiltonian's integral bounds for the
 * examples' features. */
int sfci_screen_log(sfci_screen* s, const sfci_vec* in, const sfci_vec* out, double min_term, uint64_t* examples,
                    uint64_t* positives);
/* `steps` Adam steps on batches of batch_tiles x 128 logged examples (random
 * windows, or consecutive from the first example when `sequential`), binary
 * cross-entropy with positives weighted by pos_weight; lr 0 computes the
 * gradients of one batch without updating.  *loss: the last batch's mean. */
int sfci_screen_train(sfci_screen* s, int steps, int batch_tiles, double lr, double pos_weight, int sequential,
                      double* loss);
int sfci_screen_stats(const sfci_screen* s, uint64_t* sources, uint64_t* examples, uint64_t* positives,
                      uint64_t* steps);
/* Runs the MLP on the groups of the determinants of `in`: counts of groups, of
 * groups with probability >= threshold and of their terms; prob_host (nullable,
 * prob_cap entries) receives each group's probability, source by source. */
int sfci_screen_predict(sfci_screen* s, const sfci_vec* in, double threshold, uint64_t* groups,
                        uint64_t* kept_groups, uint64_t* kept_terms, float* prob_host, uint64_t prob_cap);
/* FP32 parameters (sfci_screen_param_count floats: W1[576][256] by input row,
 * b1, W2[256 out][256 in], b2, w3, b3, padding); get and/or set (nullable). */
uint64_t sfci_screen_param_count(void);
int sfci_screen_params(sfci_screen* s, float* get, const float* set, uint64_t n);
/* the gradients of the last training step (same layout) */
int sfci_screen_grads(sfci_screen* s, float* get, uint64_t n);
/* Attach (s non-null) or detach the screen of the context's products. */
int sfci_ctx_set_screen(sfci_ctx* ctx, sfci_screen* s, double threshold);
/* Guard of the context's screened products: a group whose largest possible
 * term, |c_j| times its two-body integral bound (the feature log|(pq|rs)|), is
 * at least `guard` is kept whatever the network predicts; 0 switches it off
 * (the default).  As the guard goes to 0+ the screened product becomes the
 * plain one. */
int sfci_ctx_set_screen_guard(sfci_ctx* ctx, double guard);
/* Floor of the context's screened products: a group whose largest possible
 * term is below `floor` is skipped without running the network (0 switches it
 * off, the default).  With the floor at the training labels' minimum term
 * (sfci_screen_log's min_term) it skips only groups the labels call dead. */
int sfci_ctx_set_screen_floor(sfci_ctx* ctx, double floor_);
/* groups seen, groups kept, terms kept, screened products, terms of all groups,
 * since the context was made (five counters) */
int sfci_ctx_screen_stats(const sfci_ctx* ctx, uint64_t* out5);

/* Generalised symmetric eigensolve K c = E S c (Eigen GSAES as used at
 * src/sparse_solver.cpp:450), FP64 on the host: eigenvalues ascending,
 * eigenvectors column-major with c^T S c = 1. */
int sfci_gsaes(int n, const double* K, const double* S, double* evals, double* evecs);

#ifdef __cplusplus
}
#endif

#endif /* SFCI_GB300_H */

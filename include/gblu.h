/*
 * gblu.h -- C ABI of libgblu, the GB300 (sm_103a) dense LU library.
 *
 * libgblu is the device side of LinearSolve.jl's dense LU path: getrf
 * (partial-pivot LU) and getrs (the back-solve), plus mixed-precision
 * factorization with FP64 iterative refinement.  A host binding calls it the
 * way LinearSolve.jl calls OpenBLAS: symbols resolved once, plain pointers and
 * sizes, LAPACK conventions (column-major, leading dimensions, 1-based int64
 * ipiv, int64 info).  No torch, CUDA or C++ types cross this boundary; the
 * stream getter returns an opaque pointer.
 *
 * Conventions shared by every entry point
 *   - Return value: int32 status, GBLU_OK (0) on success.  A failed call leaves
 *     a message readable with gblu_last_error(ctx).
 *   - `info` follows LAPACK getrf: 0 = success, k > 0 = U(k,k) is exactly zero
 *     (the first such column, 1-based).  A singular matrix is a *successful*
 *     call with info > 0, as in the reference (src/factorization.jl:716-722).
 *   - Every call is synchronous on return unless its name ends in _async.
 *   - Threading: a context serialises its own calls with an internal mutex;
 *     use one context per host thread for concurrency.
 *   - Device waits inside kernels are bounded; an expired wait returns
 *     GBLU_ETIMEOUT instead of hanging.
 */
#ifndef GBLU_H
#define GBLU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define GBLU_OK 0
#define GBLU_EINVAL 1        /* bad argument (LAPACK info < 0 / chkargsok)   */
#define GBLU_ECUDA 2         /* CUDA runtime error                          */
#define GBLU_ENOMEM 3        /* device allocation failed or budget exceeded */
#define GBLU_ETIMEOUT 4      /* a bounded device-side wait expired          */
#define GBLU_ENOTFACTORED 5  /* getrs before a successful getrf            */
#define GBLU_ESTALL 6        /* refinement stalled and fallback disabled    */
#define GBLU_EUNSUPPORTED 7  /* size/precision outside what is implemented */
#define GBLU_ENODEVICE 8     /* no usable CUDA device                       */

/* ---- factor precisions ---------------------------------------------------- */
#define GBLU_FP64 0 /* plain FP64 LU, FP64 getrs                              */
#define GBLU_FP32 1 /* FP32 LU, FP64 iterative refinement                      */
#define GBLU_BF16 2 /* FP32 LU whose trailing updates run on tcgen05 with BF16
                       operands (FP32 accumulation), FP64 refinement         */
#define GBLU_FP16 3 /* as GBLU_BF16 with FP16 operands, each column of the
                       right operand scaled by a power of two              */

/* ---- buffer locations ---------------------------------------------------- */
#define GBLU_HOST 0
#define GBLU_DEVICE 1

typedef struct gblu_ctx gblu_ctx;
typedef struct gblu_factor gblu_factor;

/* Library version, (major << 16) | minor. */
int32_t gblu_version(void);

/* ---- context --------------------------------------------------------------
 * A context binds one CUDA device, one CUDA stream and an HBM budget for all
 * device memory it allocates (0 = no budget beyond the device's free memory).
 * Replaces: the per-process BLAS handle of src/openblas.jl:48-72 (dlopen +
 * dlsym once, then fixed pointers). */
int32_t gblu_create(gblu_ctx** out, int32_t device, uint64_t hbm_budget_bytes);
int32_t gblu_destroy(gblu_ctx* ctx);
/* Message of the last failed call on this context ("" if none).  With ctx ==
 * NULL: the last failure of gblu_create or of the LAPACK-shaped entries. */
const char* gblu_last_error(const gblu_ctx* ctx);
/* The context's cudaStream_t, for callers that time or order work around it. */
int32_t gblu_ctx_stream(gblu_ctx* ctx, void** stream_out);
/* Device bytes currently held by the context's objects, and its budget. */
int32_t gblu_ctx_memory(gblu_ctx* ctx, uint64_t* in_use, uint64_t* budget);

/* ---- launch accounting ---------------------------------------------------------
 * Counts every kernel the context launches and, when enabled, times each
 * launch with CUDA events on the context's stream.  Kinds (index into the
 * arrays): 0 trailing GEMM update, 1 panel getf2, 2 row interchanges, 3 TRSM,
 * 4 permutation build, 5 getrs sweeps, 6 refinement kernels, 7 batched,
 * 8 other.  flops/bytes are the algorithmic work the launches were given.
 * Measurement utility; no counterpart in the reference. */
#define GBLU_PROFILE_KINDS 9
typedef struct gblu_profile {
  uint64_t launches;
  uint64_t count[GBLU_PROFILE_KINDS];
  double ms[GBLU_PROFILE_KINDS];
  double flops[GBLU_PROFILE_KINDS];
  double bytes[GBLU_PROFILE_KINDS];
} gblu_profile;
/* Enable (1) or disable (0) event timing; always resets the counters. */
int32_t gblu_profile_enable(gblu_ctx* ctx, int32_t enable);
/* Synchronise the stream and read the counters (reset != 0 clears them). */
int32_t gblu_profile_read(gblu_ctx* ctx, gblu_profile* out, int32_t reset);

/* ---- factorization objects -------------------------------------------------
 * A factor owns, in HBM, everything getrf/getrs need for an m x n matrix:
 * the factors, ipiv, the row permutation, and all scratch.  It is the
 * device-resident counterpart of LinearCache.cacheval (src/common.jl:281-306;
 * the OpenBLASLUCache of src/openblas.jl:318-360).  Refactoring reuses it
 * without allocating, as src/factorization.jl:630-641 does with ipiv.
 * precision: GBLU_FP64 or GBLU_FP32 (mixed: FP32 factors, FP64 refinement;
 * the FP64 copy of A is kept on the device for residuals). */
int32_t gblu_factor_create(gblu_ctx* ctx, int64_t m, int64_t n, int32_t precision,
                           gblu_factor** out);
int32_t gblu_factor_destroy(gblu_ctx* ctx, gblu_factor* f);

/* getrf: factor A (m x n, leading dimension lda) into f.  A is read, never
 * written; a_loc = GBLU_HOST copies it to the device first (a pageable A of
 * 32 MB or more, or of 4 MB or more while another such copy is running in the
 * process, goes through the context's pinned staging chunks; pinned memory
 * is copied directly; GBLU_HOST_STAGING=0 copies every A directly).
 * Replaces: LAPACK.getrf! reached from solve!(cache, ::LUFactorization)
 * (src/factorization.jl:643-736, do_factorization :738-751) and the
 * dgetrf_ ccall of src/openblas.jl:131-154. */
int32_t gblu_getrf(gblu_ctx* ctx, gblu_factor* f, const double* A, int64_t lda,
                   int32_t a_loc, int64_t* info);

/* How getrs applies the triangular factors (gblu_factor_set_solve).
 * GBLU_SOLVE_EXACT (default): each row of the two sweeps accumulates its
 *   updates in the reference back-solve's order (src/factorization.jl:433-457),
 *   bit-identical to it; a chain of n dependent steps per sweep.
 * GBLU_SOLVE_FAST: the same two sweeps with the 64 x 64 diagonal blocks of L
 *   and U inverted once after each getrf and applied as matrix-vector
 *   products, and independent partial sums elsewhere; backward-error accurate
 *   (not bit-identical), several times shorter critical path.  For a mixed
 *   factor it selects the low-precision solve inside refinement (the
 *   default for mixed factors: refinement makes either FP64-accurate); the
 *   FP64 fallback solve stays exact.  An FP64 factor allocates n x 128
 *   doubles on its first switch to GBLU_SOLVE_FAST. */
#define GBLU_SOLVE_EXACT 0
#define GBLU_SOLVE_FAST 1
int32_t gblu_factor_set_solve(gblu_ctx* ctx, gblu_factor* f, int32_t mode);

/* How a mixed-precision factor (GBLU_FP32 / BF16 / FP16) pivots its
 * low-precision LU, from the next getrf on (gblu_factor_set_pivoting).
 * GBLU_PIVOT_PARTIAL (default): partial pivoting, the reference's order
 *   (blocked_lufact.jl), per 32-column leaf.
 * GBLU_PIVOT_TOURNAMENT: tournament pivoting (CALU's tall-skinny panel) for
 *   leaves taller than 512 rows.
 * GBLU_PIVOT_RBT: no pivoting, after a depth-2 random butterfly transform of
 *   both sides, Ar = U^T A V / 4 (Parker 1995; Baboulin, Dongarra, Herrmann
 *   and Tomov 2013): the leaves need no pivot search and no interchanges.
 *   Refinement still solves the original system (residuals against the FP64
 *   A; corrections V (LU)^-1 U^T r); the pivot-growth check and the FP64
 *   fallback (with partial pivoting) catch a factorization the transform
 *   did not stabilise.  Square factors of order 4 or more: the butterflies
 *   cover the leading n - n mod 4 rows and columns (U, V = diag(W, I)).
 * GBLU_EUNSUPPORTED for GBLU_FP64 factors and for RBT on other shapes.
 * No counterpart in the reference. */
#define GBLU_PIVOT_PARTIAL 0
#define GBLU_PIVOT_TOURNAMENT 1
#define GBLU_PIVOT_RBT 2
int32_t gblu_factor_set_pivoting(gblu_ctx* ctx, gblu_factor* f, int32_t mode);

/* getrs: solve op(A) X = B in place for nrhs columns of B (ldb), with
 * trans = 'N' or 'T'.  For a GBLU_FP32 factor this is the refined solve
 * (gblu_solve_refined with default options), so the result is FP64-accurate.
 * Replaces: _smart_lu_ldiv! / ldiv! -> getrs (src/factorization.jl:603-611,
 * :727-728) and the dgetrs_ ccall of src/openblas.jl:247-278. */
int32_t gblu_getrs(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, double* B,
                   int64_t ldb, int32_t b_loc);

/* Copies of the factorization result, for parity checks against LAPACK. */
int32_t gblu_get_ipiv(gblu_ctx* ctx, gblu_factor* f, int64_t* ipiv_host);
/* The packed L\U factors (FP64; low-precision factors are widened). */
int32_t gblu_get_factors(gblu_ctx* ctx, gblu_factor* f, double* host, int64_t ld);
/* info of the last getrf on f. */
int32_t gblu_get_info(gblu_ctx* ctx, gblu_factor* f, int64_t* info);
/* Pivot growth max_ij |U_ij| / max_ij |A_ij| of the last getrf on a
 * mixed-precision factor (GBLU_FP32 / BF16 / FP16), computed on the device:
 * max |A| over the FP64 input as it is converted, max |U| over the
 * low-precision factors after getrf (0 for GBLU_FP64 factors).  The refined
 * solve compares it with gblu_refine_opts.growth_limit.  No counterpart in
 * the reference. */
int32_t gblu_get_growth(gblu_ctx* ctx, gblu_factor* f, double* growth);

/* ---- mixed precision and iterative refinement --------------------------------
 * A GBLU_FP32 factor holds FP32 L\U factors; solves reach FP64 accuracy by
 * refinement: r = b - A x in FP64 (A kept in FP64 on the device), a
 * correction solved with the FP32 factors, x += d in FP64.  mode
 * GBLU_REFINE_IR is classic iterative refinement; GBLU_REFINE_GMRES is
 * GMRES-IR (the correction equation solved by FP64 GMRES left-preconditioned
 * by the FP32 LU).  When the backward error stops decreasing, or after
 * max_iter iterations, the library factors A in FP64 and solves with that
 * (fallback != 0), or returns GBLU_ESTALL (fallback == 0).
 * No counterpart in the reference: its *32Mixed* types stop after the FP32
 * solve (src/openblas.jl:487-543, ext/LinearSolveCUDAExt.jl:211-242). */
#define GBLU_REFINE_IR 0
#define GBLU_REFINE_GMRES 1

typedef struct gblu_refine_opts {
  int32_t mode;          /* GBLU_REFINE_IR or GBLU_REFINE_GMRES              */
  int32_t max_iter;      /* outer refinement iterations                      */
  double tol;            /* stop when backward error <= tol (<= 0: n * eps)  */
  int32_t fallback;      /* nonzero: FP64 LU when refinement stalls          */
  int32_t gmres_restart; /* GMRES basis size (<= 30)                          */
  double gmres_tol;      /* relative residual target of each GMRES solve     */
  double growth_limit;   /* pivot growth max|U| / max|A| of the low-precision
                            factors above which the solve goes to the FP64
                            LU at once, without refining (<= 0: 1 / u of the
                            factorization's arithmetic: 2^24 for FP32, 2^11
                            for FP16 operands, 2^8 for BF16 operands, the
                            growth at which its rounding errors reach the size
                            of A's entries)                                   */
} gblu_refine_opts;

/* Why the FP64 fallback produced an answer (gblu_refine_stats.fallback_reason). */
#define GBLU_FALLBACK_NONE 0
#define GBLU_FALLBACK_STALL 1      /* backward error stopped decreasing / max_iter */
#define GBLU_FALLBACK_GROWTH 2     /* pivot growth above growth_limit             */
#define GBLU_FALLBACK_ZERO_PIVOT 3 /* exact zero pivot in the low-precision LU    */

typedef struct gblu_refine_stats {
  int32_t iterations;       /* outer iterations taken (max over columns)     */
  int32_t inner_iterations; /* total GMRES iterations                        */
  int32_t converged;        /* 1 if every column met tol                     */
  int32_t fell_back;        /* 1 if the FP64 fallback produced the answer    */
  double backward_error;    /* final max_j ||b-Ax||/(||A|| ||x|| + ||b||), inf-norms */
  double growth;            /* pivot growth of the factors (gblu_get_growth) */
  int32_t fallback_reason;  /* GBLU_FALLBACK_*                                */
  int32_t pad_;
} gblu_refine_stats;

int32_t gblu_refine_opts_default(gblu_refine_opts* opts);
/* Solve op(A) X = B (in place) to FP64 accuracy with the factor f.  For a
 * GBLU_FP64 factor this is the plain getrs followed by one residual that
 * fills stats.  opts may be NULL (defaults); stats may be NULL. */
int32_t gblu_solve_refined(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, double* B,
                           int64_t ldb, int32_t b_loc, const gblu_refine_opts* opts,
                           gblu_refine_stats* stats);

/* ---- a-posteriori residual check ---------------------------------------------
 * res_norm = ||B - op(A) X||_F and b_norm = ||B||_F (the 2-norms for one
 * column), computed in FP64 on the device from the FP64 matrix of f's last
 * getrf, with a fixed summation order.  A mixed-precision factor keeps that
 * matrix anyway; a GBLU_FP64 factor factors A in place, so it keeps a copy
 * only after gblu_factor_keep_matrix(ctx, f, 1) (the copy is taken at each
 * later getrf; keep = 0 frees it).  X and B are n x nrhs (ldx, ldb) in host
 * or device memory (loc).  A caller compares res_norm with
 * abstol + reltol * b_norm.
 * Replaces: _check_residual_safety (src/factorization.jl:127-156: mul!, axpy!
 * and norm on the backed-up A), which solve!(cache, ::LUFactorization) runs
 * after each refactorization when residualsafety = true (:647-651, :729-732). */
int32_t gblu_factor_keep_matrix(gblu_ctx* ctx, gblu_factor* f, int32_t keep);
int32_t gblu_residual_norm(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs,
                           const double* X, int64_t ldx, const double* B, int64_t ldb,
                           int32_t loc, double* res_norm, double* b_norm);

/* The trailing-update contraction of the mixed-precision getrf on its own:
 * C (m x n, FP32) -= A (m x k) * B (k x n), all column-major FP32 in memory.
 * precision GBLU_BF16 / GBLU_FP16: operands rounded to 16 bits (FP16 with a
 * power-of-two scale per column of B), products accumulated in FP32 on the
 * tensor cores (tcgen05, TMEM accumulator); GBLU_FP32: the FP32 SIMT kernel,
 * each C element updated by fma in k order.  loc: GBLU_HOST or GBLU_DEVICE
 * for all three matrices.
 * Replaces: the Schur update of src/blocked_lufact.jl:186-656 as a standalone
 * call (A22 -= L21 * U12). */
int32_t gblu_gemm_update(gblu_ctx* ctx, int32_t precision, int64_t m, int64_t n, int64_t k,
                         const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                         int64_t ldc, int32_t loc);

/* ---- batched uneven LU ------------------------------------------------------
 * `count` independent square systems A_i x_i = b_i, 1 <= n_i <= 256, one RHS
 * each, packed back to back: A_i column-major (lda = n_i) at element offset
 * sum_{k<i} n_k^2 of A, b_i at sum_{k<i} n_k of B.  gblu_batch_create sorts
 * the systems into size buckets and captures one CUDA graph holding one
 * persistent kernel per bucket (each takes systems from a queue, largest
 * first); gblu_batch_solve copies the inputs, launches the graph once and
 * overwrites B with the solutions.  precision GBLU_FP64: per-system getrf +
 * getrs in FP64 (bit-identical to src/blocked_lufact.jl + the back-solve of
 * src/factorization.jl:433-457 applied to each system); GBLU_FP32: FP32
 * factors + FP64 refinement per system, systems that do not converge re-solved
 * in FP64 by a second kernel of the same graph.  info_host (may be NULL)
 * receives each system's getrf info.
 * No counterpart in the reference (LinearProblem holds one A); it batches
 * what a caller of solve(LinearProblem(A_i, b_i), LUFactorization()) loops over. */
typedef struct gblu_batch gblu_batch;
int32_t gblu_batch_create(gblu_ctx* ctx, int64_t count, const int64_t* sizes, int32_t precision,
                          gblu_batch** out);
/* Replace the bucket schedule (from the autotuner): nbuckets (<= 8) buckets
 * with inclusive upper size edges (the last must be 256), threads per CTA and
 * panel width per bucket ((64, 8), (128|256, 8|16) or (512, 16)), CTAs per bucket
 * (NULL or <= 0 entries: fill the GPU).  Re-captures the graph. */
int32_t gblu_batch_schedule(gblu_ctx* ctx, gblu_batch* b, int32_t nbuckets, const int32_t* upper,
                            const int32_t* threads, const int32_t* panel, const int32_t* ctas);
int32_t gblu_batch_solve(gblu_ctx* ctx, gblu_batch* b, const double* A, double* B, int32_t loc,
                         int64_t* info_host);
/* Per system, the refinement iterations of the last GBLU_FP32 solve (-1: the
 * system was re-solved by the FP64 kernel; 0 for GBLU_FP64 batches). */
int32_t gblu_batch_iterations(gblu_ctx* ctx, gblu_batch* b, int32_t* iterations_host);
int32_t gblu_batch_destroy(gblu_ctx* ctx, gblu_batch* b);

/* ---- serving loop ----------------------------------------------------------------
 * Continuous batching over factorizations kept resident in HBM.  A request
 * carries a key and either a new matrix A for that key (factor, then solve) or
 * only a right-hand side for a key whose factors are resident (solve).
 * `workers` host threads, each with its own stream, take the oldest runnable
 * request (its key idle; a new factorization object admitted within
 * hbm_budget_bytes, evicting least recently used idle ones); requests on one
 * key keep submission order; up to max_rhs_batch consecutive solve-only
 * requests on a key are merged into one multi-RHS solve.  A result depends
 * only on its own inputs, never on what else is in flight.
 * No counterpart in the reference (one LinearProblem per solve call). */
typedef struct gblu_server gblu_server;
typedef struct gblu_serve_config {
  int32_t workers;           /* concurrent slots                                   */
  int32_t precision;         /* factor precision of new matrices (GBLU_FP64 .. FP16) */
  int32_t refine_mode;       /* GBLU_REFINE_IR / GBLU_REFINE_GMRES (mixed precisions) */
  uint64_t hbm_budget_bytes; /* resident factorizations (0: no limit)             */
  int32_t max_rhs_batch;     /* solve-only requests merged per key                 */
  int32_t small_n;           /* requests with n <= small_n (<= 256; 0: none) go to
                                the small-system lane: whatever of them is queued,
                                across keys, is factored and solved in one launch
                                of the batched kernels (the key keeps its matrix
                                in host memory, not its factors)                   */
  int32_t solve_mode;        /* GBLU_SOLVE_EXACT / GBLU_SOLVE_FAST for the factors
                                the server creates                                 */
  int32_t max_small_batch;   /* systems per small-lane launch                      */
  int32_t large_n;           /* factorizations of n >= large_n count as large ...  */
  int32_t max_large;         /* ... and at most max_large of them run at once (0: no
                                limit; defaults 2048 and 1): large factorizations
                                running together slow each other down, and they
                                are the latency tail                               */
  int32_t pivoting;          /* GBLU_PIVOT_* of the mixed-precision factors the
                                server creates (default GBLU_PIVOT_PARTIAL;
                                GBLU_PIVOT_RBT for n >= 4, partial below)          */
} gblu_serve_config;
typedef struct gblu_request {
  uint64_t key;      /* factorization key                                        */
  int64_t n;
  const double* A;   /* host n x n column-major (lda = n), or NULL: solve only   */
  const double* b;   /* host, n                                                  */
  double* x;         /* host, n: the solution, written before completion         */
  uint64_t tag;      /* caller's identifier, returned in the completion          */
} gblu_request;
typedef struct gblu_completion {
  uint64_t tag;
  int32_t status;         /* GBLU_OK, GBLU_ENOTFACTORED (key not resident), ...   */
  int32_t refactored;     /* this request factored its matrix                    */
  int32_t fell_back;      /* refinement fell back to the FP64 LU                 */
  int32_t iterations;     /* refinement iterations                               */
  int64_t info;           /* getrf info of a factoring request                   */
  double backward_error;  /* final backward error (-1: not computed, FP64)       */
  double latency_us;      /* submit -> solution in host memory                   */
  double queue_us;        /* submit -> start of work                             */
} gblu_completion;
typedef struct gblu_serve_stats {
  int64_t submitted, completed, failed, factorizations, solves, merged_solves, evictions;
  int64_t resident_factors, queued, in_flight;
  uint64_t resident_bytes;
  int64_t small_launches;   /* launches of the small-system lane                */
  int64_t small_systems;    /* requests solved by it                             */
  int64_t admission_waits;  /* times a request waited for memory to be admitted  */
} gblu_serve_stats;
int32_t gblu_serve_config_default(gblu_serve_config* cfg);
int32_t gblu_serve_create(gblu_ctx* ctx, const gblu_serve_config* cfg, gblu_server** out);
/* Non-blocking; the request's buffers must stay valid until its completion. */
int32_t gblu_serve_submit(gblu_server* s, const gblu_request* req);
/* Up to max completions into out (waiting up to wait_ms for the first one). */
int32_t gblu_serve_poll(gblu_server* s, gblu_completion* out, int32_t max, int32_t* n_out,
                        int32_t wait_ms);
int32_t gblu_serve_get_stats(gblu_server* s, gblu_serve_stats* out);
/* Finishes every submitted request, then releases the factorizations. */
int32_t gblu_serve_destroy(gblu_server* s);

/* ---- LAPACK-shaped entries ---------------------------------------------------
 * Same argument lists as LAPACK dgetrf_/dgetrs_/sgetrf_/sgetrs_ with 64-bit
 * integers (the ILP64 BlasInt of src/LinearSolve.jl:52-63), so a binding can
 * swap the symbol in the ccall of src/openblas.jl:144-153,267-276.  Host
 * buffers; each call copies to and from a process-wide default context on
 * the current device.  info < 0 reports a bad argument as LAPACK does;
 * info = -1000 - status reports a library failure (see gblu_last_error(NULL)). */
void gblu_dgetrf_(const int64_t* m, const int64_t* n, double* A, const int64_t* lda,
                  int64_t* ipiv, int64_t* info);
void gblu_dgetrs_(const char* trans, const int64_t* n, const int64_t* nrhs,
                  const double* A, const int64_t* lda, const int64_t* ipiv, double* B,
                  const int64_t* ldb, int64_t* info, long trans_len);
void gblu_sgetrf_(const int64_t* m, const int64_t* n, float* A, const int64_t* lda,
                  int64_t* ipiv, int64_t* info);
void gblu_sgetrs_(const char* trans, const int64_t* n, const int64_t* nrhs,
                  const float* A, const int64_t* lda, const int64_t* ipiv, float* B,
                  const int64_t* ldb, int64_t* info, long trans_len);

/* ---- allocation-free solve -------------------------------------------------
 * No counterpart in the reference.  For callers that must not allocate device
 * memory: per-step solver loops (e.g. Newton iterations inside an ODE
 * integrator) where cudaMalloc/cudaFree would synchronise the device, and
 * hosts that committed all device memory to a budget.  (It is meant for a
 * non-blocking caller stream; with stream NULL it runs on the legacy default
 * stream, and it reads one error word back with a synchronising copy, so it
 * is not meant for use while a global-mode stream capture is open.)
 * Solves op(A) X = B in place with factors dLU (lda) and 1-based int64 pivots
 * d_ipiv from getrf, all three in device memory, on `stream` (NULL: the
 * default stream); returns when the solve has finished.  It allocates
 * nothing: its scratch is one fixed ~1.1 MB device array compiled into the
 * library, held on every device that loads it until the process exits.
 * Limit: n <= 16384 (larger n returns GBLU_EUNSUPPORTED); any nrhs.  The first
 * call on a device looks up that array's address; make that call before any
 * stream capture.  All calls share the one array, so calls that overlap on
 * the GPU (different streams or threads at once) race; serialise them.
 * Errors are reported through gblu_last_error(NULL).  An invalid pivot is
 * detected on the device after the solve was queued, so after a non-OK
 * return the contents of dB are unspecified. */
int32_t gblu_dgetrs_noalloc(char trans, int64_t n, int64_t nrhs, const double* dLU, int64_t lda,
                            const int64_t* d_ipiv, double* dB, int64_t ldb, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBLU_H */

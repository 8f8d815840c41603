/*
 * cpals.h -- C ABI of the GB300 CP-ALS engine (libcpals.so).
 *
 * This is the drop-in boundary for ITensorCPD.jl's normal-equation ALS path.
 * Julia binds it with `ccall`, the way ITensorCPD binds its one native helper
 * (src/algebra/SEQRCS.jl:41-60, library located in src/ITensorCPD.jl:25-36).
 * Python binds it with ctypes.
 *
 * Conventions
 *  - Every entry point returns an int status: CPALS_OK (0) or a negative code.
 *    No entry point aborts or traps.
 *  - Tensors and matrices crossing the boundary are column-major (first index
 *    fastest), as ITensor Dense storage and Julia Arrays are.
 *    A factor F_n is I_n x R, an MTTKRP M_n is I_n x R, a Gram is R x R.
 *  - Modes are 0-based here; the Julia shim passes `fact - 1`.
 *    Sample indices (pivots) are 1-based Int64, as Julia stores them
 *    (src/math_tools/probability.jl:25).
 *  - Host pointers: the library copies in and out; it owns every device buffer
 *    of a handle.  The one exception, cpals_set_tensor_device, borrows a device
 *    buffer, which must outlive its use.
 *  - One CUDA stream per handle.  A handle must not be used from two threads
 *    at once.
 */
#ifndef CPALS_H
#define CPALS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define CPALS_OK 0
#define CPALS_E_ARG (-1)         /* bad argument: sizes, mode, index out of range, null pointer */
#define CPALS_E_CUDA (-2)        /* a CUDA runtime call failed */
#define CPALS_E_NAN (-3)         /* the fit became NaN: fit_check.jl:40-42 throws "Error NAN" */
#define CPALS_E_STATE (-4)       /* call out of order, e.g. a sweep before the tensor is set */
#define CPALS_E_UNSUPPORTED (-5) /* shape or option this build does not handle */
#define CPALS_E_DEVICE (-6)      /* a kernel reported an error status (bounded wait expired, bad index) */

/* ---- tensor element types ---- */
#define CPALS_DTYPE_F64 0
#define CPALS_DTYPE_F32 1

/* ---- MTTKRP arithmetic ---- */
#define CPALS_MTTKRP_FP64 0   /* plain FP64 on CUDA cores: the parity / comparator path */
#define CPALS_MTTKRP_BF16X3 1 /* tcgen05 split-BF16 (hi*hi + hi*lo + lo*hi), FP32 accumulate */

/* ---- create flags ---- */
#define CPALS_FLAG_NO_GRAPH 1 /* launch sweeps kernel by kernel instead of replaying a CUDA graph */
#define CPALS_FLAG_DIMTREE 2  /* dimension-tree MTTKRP (order >= 3): two passes over T per sweep */
#define CPALS_FLAG_FUSED_TAIL 8 /* per-mode tail (solve, Gram, lambda, normalisation, fit) as one cooperative
                                  launch instead of three kernels; measured slower on GB300 (2341 against 2374
                                  sweeps/s at 512^3 R=64, 1222 against 1249 at 128^4 R=128) */
#define CPALS_FLAG_LOWMEM 4   /* split-BF16 engine: one tile stream buffer, each mode's stream built from T
                                 just before its MTTKRP (2x the tensor's bytes on the device instead of
                                 (N + 1)x; about 0.43 ms per GB of tensor per mode more) */

/* ---- convergence checks ---- */
#define CPALS_CHECK_NONE 0 /* NoCheck, src/converge_checks/no_check.jl:1-20 */
#define CPALS_CHECK_FIT 1  /* FitCheck, src/converge_checks/fit_check.jl:5-68 */
#define CPALS_CHECK_DIFF 2 /* CPDiffCheck, src/converge_checks/cp_diff_check.jl:6-68 */
#define CPALS_CHECK_ANGLE 3 /* CPAngleCheck, src/converge_checks/cp_angle_check.jl:6-68 */

#define CPALS_MAX_ORDER 8

typedef struct cpals_ctx cpals_ctx;

/* Mirror of the mutable check structs (fit_check.jl:5-20, no_check.jl:1-9,
 * cp_diff_check.jl:6-18, cp_angle_check.jl:6-18).  cpals_optimize reads it on entry and
 * writes the updated fields back, so a check object can be reused across calls as in the
 * reference.  The previous iterate that CPDiffCheck / CPAngleCheck keep (PrevCP) stays
 * on the device, in the handle; `has_prev` says whether it is set (PrevCP !== nothing),
 * and cpals_get_prev / cpals_set_prev move it between handles. */
typedef struct cpals_check {
  int32_t kind;        /* CPALS_CHECK_NONE, _FIT, _DIFF or _ANGLE */
  int32_t iter;        /* in/out */
  int32_t counter;     /* in/out (FitCheck, CPDiffCheck, CPAngleCheck) */
  int32_t max_counter; /* sweeps allowed */
  double tolerance;    /* tol on |delta fit| (|delta angle| for CPAngleCheck) */
  double ref_norm;     /* FitCheck norm(T) */
  double lastfit;      /* in/out; starts at 1 (CPAngleCheck: lastangle) */
  double final_fit;    /* out */
  int32_t total_iter;  /* out */
  int32_t sweeps_run;  /* out: sweeps executed by this call */
  double norm_prev;    /* in/out: norm_prev_iter (CPDiffCheck ||prev||^2, CPAngleCheck ||prev||) */
  int32_t has_prev;    /* in/out: 1 when the handle holds the previous iterate */
  int32_t reserved;
} cpals_check;

/* Library version (major*10000 + minor*100 + patch). */
int cpals_version(void);
/* Static message for a status code. */
const char* cpals_status_string(int status);

/* Create a handle for an order-`order` tensor of extents dims[0..order-1] and CP
 * rank `rank` on CUDA device `device`.  Replaces the state that compute_als builds
 * (src/optimizers/als_optimizers/als_optimizer.jl:37-55,
 *  optimizers/als_optimizers/standard/tensor.jl:3-14). */
int cpals_create(cpals_ctx** out, int device, int order, const int64_t* dims, int64_t rank,
                 int tensor_dtype, int mttkrp_mode, int flags);
int cpals_destroy(cpals_ctx* ctx);

/* Copy the column-major target tensor in (the ALS `target`, als_optimizer.jl:5-10). */
int cpals_set_tensor(cpals_ctx* ctx, const void* host_tensor);
/* Use a column-major tensor already resident on the handle's device (borrowed). */
int cpals_set_tensor_device(cpals_ctx* ctx, const void* device_tensor);

/* The device copy of the target the handle uses (owned or borrowed), for another handle's
 * cpals_set_tensor_device: the rank-adaptive decompose (decompose.jl:32-69) runs one
 * handle per rank on one upload.  The pointer lives as long as this handle (owned) or the
 * caller's buffer (borrowed).  CPALS_E_STATE before a tensor is set. */
int cpals_tensor_device(cpals_ctx* ctx, const void** device_tensor);

/* Copy factors (each I_n x R column-major) and lambda (R) in / out.  Setting
 * factors also recomputes the Grams, as compute_als does
 * (optimizers/als_optimizers/standard/tensor.jl:3-14). */
int cpals_set_factors(cpals_ctx* ctx, const double* const* host_factors, const double* host_lambda);
int cpals_get_factors(cpals_ctx* ctx, double* const* host_factors, double* host_lambda);
/* Gram G_n = F_n^T F_n (R x R) of the current factors. */
int cpals_get_gram(cpals_ctx* ctx, int mode, double* host_gram);

/* MTTKRP of `mode` with the current factors: M_n = T_(n) (KRP of the other factors),
 * I_n x R column-major.  Replaces matricize_tensor(::KRPFreeNormal / ::KRPNormal)
 * (src/algorithms/als_algorithms/standard/tensor.jl:12-44). */
int cpals_mttkrp(cpals_ctx* ctx, int mode, double* host_out);

/* Run ALS sweeps with the given check: the loop of optimize
 * (src/optimizers/als_optimizers/optimize.jl:6-35) with compute_krp, solve_ls_problem,
 * row_norm, post_solve and check_converge on the device.  `fit_trajectory`
 * (may be NULL) receives one fit per sweep run, up to `traj_capacity` entries:
 * for CPDiffCheck the fit between consecutive iterates, for CPAngleCheck their angle,
 * NaN for a sweep whose check only stored the iterate (PrevCP was nothing).
 * Returns CPALS_E_NAN if a FitCheck fit became NaN (fit_check.jl:41). */
int cpals_optimize(cpals_ctx* ctx, cpals_check* check, double* fit_trajectory, int64_t traj_capacity);

/* One mode of an ALS sweep on the device, for a sweep loop the caller drives (optimize,
 * src/optimizers/als_optimizers/optimize.jl:19-27): compute_krp (the Hadamard product of the
 * other modes' Grams, MttkrpAlgorithm.jl:18-31), matricize_tensor (the MTTKRP,
 * standard/tensor.jl:12-44), solve_ls_problem (MttkrpAlgorithm.jl:34-41, ldiv_solve.jl:4-29),
 * row_norm (row_norm.jl:4-24) and post_solve (standard/tensor.jl:22-25, 46-49).  M_n stays on
 * the device.  On the last mode the terms of the fit are saved for cpals_check_converge, as
 * save_mttkrp does (MttkrpAlgorithm.jl:5-14, fit_check.jl:22).  host_solution (may be NULL)
 * receives the solve's result before normalisation, X = F_n diag(lambda), I_n x R
 * column-major, for a caller that keeps its own copy of the factors; with NULL the call
 * returns once the work is enqueued.  `order` calls (modes 0..order-1) followed by
 * cpals_check_converge equal one sweep of cpals_optimize bit for bit. */
int cpals_mode_update(cpals_ctx* ctx, int mode, double* host_solution);

/* One check_converge call on the handle's current state (MttkrpAlgorithm.jl:5-14), for
 * loops that update the factors themselves.  FitCheck / NoCheck (fit_check.jl:24-66,
 * no_check.jl:11-20): the fit from the terms the last cpals_mode_update of the last mode
 * saved (CPALS_E_STATE when there is none newer than the last check); CPALS_E_NAN when a
 * FitCheck fit is NaN.  CPDiffCheck / CPAngleCheck (cp_diff_check.jl:20-68,
 * cp_angle_check.jl:20-68): on the handle's current factors and lambda, as the sampled
 * solvers' loop needs (ProjectionAlgorithm.jl:15-54 passes these checks through).
 * *converged receives the check's return value and *value (may be NULL) the fit (angle)
 * it computed, NaN when it only stored the iterate. */
int cpals_check_converge(cpals_ctx* ctx, cpals_check* check, int* converged, double* value);

/* norm(T) of the handle's tensor, from ||T||^2 computed on the device as a double-double
 * when the tensor was set (what FitCheck's ref_norm is given, fit_check.jl:14-19).  norm2
 * (may be NULL, 2 entries) receives ||T||^2 as hi + lo.  CPALS_E_NAN for a non-finite tensor. */
int cpals_tensor_norm(cpals_ctx* ctx, double* norm, double* norm2);
/* The previous iterate held for CPDiffCheck / CPAngleCheck (PrevCP): factors I_n x R
 * column-major and lambda.  get returns CPALS_E_STATE when none is held; set makes the
 * handle hold the given one. */
int cpals_get_prev(cpals_ctx* ctx, double* const* host_factors, double* host_lambda);
int cpals_set_prev(cpals_ctx* ctx, const double* const* host_factors, const double* host_lambda);

/* ---- sparse sign embeddings and sketched matricization ---- */

/* An l x n oblivious sparse sign embedding Omega, zeta nonzeros per column, each +-1/sqrt(zeta),
 * generated on the device and written to host arrays of n*zeta entries: column c's entries
 * are rows[c*zeta + k] (0-based, as the reference's C generators leave them) and
 * vals[c*zeta + k]; colstarts (n+1 entries, may be NULL) receives c*zeta, as theirs does.
 * injective = 0: zeta distinct uniform rows per column (sparse_sign, src/algebra/sparse_sign.c);
 * injective = 1: one uniform row in each of zeta near-equal row blocks (sparsestack,
 * src/algebra/sparsestack.c).  zeta is clamped to l.  The draws come from a counter-based
 * generator keyed by `seed`, so the same seed gives the same embedding on any device; the
 * reference's rand() stream is not reproduced.  Replaces sparse_sign_call
 * (src/algebra/SEQRCS.jl:41-60). */
int cpals_sparse_sign(int device, int64_t l, int64_t n, int zeta, int injective, uint64_t seed, int32_t* rows,
                      double* vals, int32_t* colstarts);

/* A_sk = T_(mode) Omega^T (I_mode x l, column-major FP64) for the handle's tensor, with Omega
 * given by host arrays of n*zeta entries as above (n = product of the other extents, their
 * indices fused first-fastest): sketched_matricization(T, k, l, rows, vals, s)
 * (src/algebra/pivot_mapping.jl:111-140).  Each output column sums its entries in entry order,
 * as the reference does. */
int cpals_sketched_matricization(cpals_ctx* ctx, int mode, int64_t l, int zeta, const int32_t* rows,
                                 const double* vals, double* host_out);

/* ---- column-pivoted QR and SE-QRCS (the QR-pivoted projection solvers' pivots) ----
 * QR with column pivoting in FP64 on the device, with LAPACK xGEQP3's pivot rule (largest
 * partial column norm, lowest position on ties) and norm downdating, replacing
 * qr(A, ColumnNorm()) where the reference takes pivots from it
 * (src/optimizers/als_optimizers/randomized/qr_lev_score_sampled.jl:23, 127, 243;
 * src/algebra/SEQRCS.jl:101, 117, 152, 166, 198, 221).  Common arguments:
 *   ncand      pivots are chosen among the first ncand columns (<= 0: all); the other
 *              columns only receive the reflectors (so R's columns past ncand are Q^T A_rest);
 *   max_steps  at most this many Householder steps (<= 0: min(m, ncand));
 *   stop_ratio stop after the first step whose |r_jj| <= stop_ratio |r_00| (< 0: never);
 *              positions past the steps run keep their swap order;
 *   perm       n entries, 1-based: perm[k] is the matrix column at position k (Julia's F.p);
 *   rdiag      the diagonal of R for the steps run (LAPACK's signs); steps = how many;
 *   R          NULL, or steps x n column-major, zero below the diagonal;
 *   Q          NULL, or m x steps column-major, orthonormal columns. */
int cpals_qrcp(int device, int64_t m, int64_t n, const double* A, int64_t ncand, int64_t max_steps,
               double stop_ratio, int64_t* perm, double* rdiag, int64_t* steps, double* R, double* Q);
/* The same on columns of the resident tensor's mode unfolding T_(mode) (I_mode x prod of the
 * other extents, columns numbered as Julia's reshape(array(T, (i, Ris...)), ...) does):
 * the ncols columns cols (1-based), or every column when cols is NULL.  Replaces the
 * qr(Tmat, ColumnNorm()) of qr_lev_score_sampled.jl:22-23, 126-127 and the A_subset QR of
 * SEQRCS.jl:117, 166. */
int cpals_unfolding_qrcp(cpals_ctx* ctx, int mode, int64_t ncols, const int64_t* cols, int64_t ncand,
                         int64_t max_steps, double stop_ratio, int64_t* perm, double* rdiag, int64_t* steps,
                         double* R, double* Q);
/* The same on columns of the transposed Khatri-Rao product of the held factors other than
 * `mode` (R x prod of the other extents; qr_lev_score_sampled.jl:240-243). */
int cpals_krp_qrcp(cpals_ctx* ctx, int mode, int64_t ncols, const int64_t* cols, int64_t ncand, int64_t max_steps,
                   double stop_ratio, int64_t* perm, double* rdiag, int64_t* steps, double* R, double* Q);
/* omega_hadamard (src/algebra/had_contract.jl:300-326): Omega times the Khatri-Rao product of
 * the held factors other than `mode`, l x R column-major, for the embedding in rows (0-based) /
 * vals (n*zeta entries as cpals_sparse_sign writes them). */
int cpals_omega_hadamard(cpals_ctx* ctx, int mode, int64_t l, int zeta, const int32_t* rows, const double* vals,
                         double* host_out);
/* SE-QRCS (src/algebra/SEQRCS.jl:83-240).  source 0: the mode unfolding of the resident
 * tensor (m = I_mode); source 1: the transposed Khatri-Rao product of the held factors other
 * than `mode` (m = R).  n = prod of the other extents.  Stage 1 sketches with the embedding
 * (rows 0-based, vals) and takes the first t pivots of the pivoted QR of the m x l sketch;
 * the columns of Omega with an entry in one of those rows form the subset, in pivot order
 * then column order with repeats dropped (sorted_subset = 0, SEQRCS.jl:158-159) or in column
 * order (sorted_subset = 1, SEQRCS.jl:109-111, 205-207); *nsubset = its size.  Stage 2 is the
 * pivoted QR of the subset's columns: perm (n, 1-based) = vcat(subset[p_subset], the other
 * columns ascending), rdiag its diagonal (up to min(m, nsubset) entries).  compute_r != 0 also
 * returns R (steps x n: the subset's R, then Q^T times the other columns) and Q (m x steps)
 * and runs every step; otherwise stop_ratio applies. */
int cpals_seqrcs(cpals_ctx* ctx, int source, int mode, int64_t l, int zeta, const int32_t* rows, const double* vals,
                 int64_t t, int sorted_subset, int compute_r, double stop_ratio, int64_t* perm, double* rdiag,
                 int64_t* steps, int64_t* nsubset, double* R, double* Q);
/* The SE-QRCS column subset alone (host only, no device call): the columns of Omega (n * zeta
 * entries, 0-based rows as cpals_sparse_sign writes them) with an entry in one of the t rows
 * psk (1-based, the sketch's first pivots), in pivot order then column order with repeats
 * dropped (sorted_subset = 0, SEQRCS.jl:158-159) or in column order (sorted_subset = 1,
 * SEQRCS.jl:109-111, 205-207).  subset (capacity n) receives them 1-based; *nsubset their
 * count.  cpals_seqrcs selects its subset with the same code. */
int cpals_seqrcs_subset(int64_t l, int64_t n, int zeta, const int32_t* rows, int64_t t, const int64_t* psk,
                        int sorted_subset, int64_t* subset, int64_t* nsubset);

/* Number of normal-equation solves so far that took the pivoted-QR fallback
 * because the pivoted Cholesky was rank deficient (ldiv_solve.jl:17-22). */
int cpals_fallback_count(cpals_ctx* ctx, int64_t* count);

/* Synchronise the handle's stream (for timing). */
int cpals_synchronize(cpals_ctx* ctx);

/* ---- measurement helpers (no counterpart in the reference) ---- */

/* CUDA-event timer on the handle's stream: start, then stop returns the elapsed ms. */
int cpals_timer_start(cpals_ctx* ctx);
int cpals_timer_stop(cpals_ctx* ctx, double* elapsed_ms);
/* Profiling mode: sweeps are launched kernel by kernel (no CUDA graph) with a CUDA
 * event pair around every MTTKRP launch.  cpals_profile_read returns the summed MTTKRP
 * kernel time and the number of timed launches since profiling was switched on. */
int cpals_set_profiling(cpals_ctx* ctx, int on);
int cpals_profile_read(cpals_ctx* ctx, double* mttkrp_ms, int64_t* launches);
/* In profiling mode every cpals_sampled_update also records CUDA events: *update_ms receives
 * the summed device time of the updates (pivot upload to the new factor), *gather_ms that of
 * their two gathers (sampled KRP rows and fibres), *updates how many were timed. */
int cpals_profile_read_sampled(cpals_ctx* ctx, double* update_ms, double* gather_ms, int64_t* updates);
/* Kernel launches enqueued by this handle so far (every libcpals kernel). */
int cpals_launch_count(cpals_ctx* ctx, int64_t* launches);
/* Smallest rank whose FP64 factorisation (pivoted Cholesky / sweep of the normal equations)
 * runs over a cluster of CTAs instead of one CTA; both give bit-identical results.  Process
 * wide; a value above 256 keeps every factorisation on one CTA.  Returns the previous value. */
int cpals_set_cluster_sweep_min_rank(int min_rank);

/* ---- MTTKRP without any allocation (no counterpart in the reference) ---- */

/* FP64 MTTKRP of `mode` for callers that cannot allocate GPU memory when they need it:
 * code running under a caching allocator's lock or inside a fixed memory budget, and
 * plugins that are handed a stream and device buffers by their host, where a
 * cudaMalloc could fail, block, or synchronise the device.  Nothing is allocated: the
 * caller passes device buffers and the split-K partial sums use a fixed 16 MiB device
 * array that every GPU loading the library keeps until the process exits.
 *   d_tensor     column-major tensor on the current device (CPALS_DTYPE_F64 or _F32)
 *   d_factors    host array of `order` device pointers, F_m column-major I_m x rank (FP64);
 *                the entry for `mode` is not read
 *   d_out        device buffer, I_mode x rank column-major FP64
 *   stream       cudaStream_t the work is enqueued on (NULL = default stream); the call
 *                returns once the work is enqueued
 * Limit: I_mode * rank <= 2^21 (the array holds at least one split's partial sums);
 * larger sizes return CPALS_E_ARG.  The first call on a device looks up the array's
 * device address, so make it before any stream capture.  Calls share the array: two
 * calls that can overlap on the GPU (different streams, or different threads without
 * ordering) race and corrupt each other's result. */
int cpals_mttkrp_fp64_noalloc(int order, const int64_t* dims, int64_t rank, int mode, int tensor_dtype,
                              const void* d_tensor, const double* const* d_factors, double* d_out, void* stream);

/* ---- randomized leverage-score path (LevScoreSampled) ---- */

/* Sampled Khatri-Rao rows: out(s, r) = prod_{m != mode, in mode order} F_m(pivots(s, j_m), r),
 * multiplied left to right from 1 as pivot_hadamard does (src/algebra/had_contract.jl:277-295).
 * pivots: nsamps x (order-1) column-major, 1-based.  out: nsamps x R column-major FP64. */
int cpals_pivot_hadamard(cpals_ctx* ctx, int mode, const int64_t* pivots, int64_t nsamps, double* host_out);

/* Sampled fibres of the tensor: out(i, s) = T(p_1, .., i at `mode`, .., p_{N-1}),
 * as fused_flatten_sample (src/algebra/pivot_mapping.jl:59-85).
 * out: I_mode x nsamps column-major, in the tensor's element type. */
int cpals_fused_flatten_sample(cpals_ctx* ctx, int mode, const int64_t* pivots, int64_t nsamps, void* host_out);

/* Leverage-score probabilities of factor `mode` (I_mode values):
 * compute_leverage_score_probabilitiy (src/math_tools/probability.jl:3-10). */
int cpals_leverage_scores(cpals_ctx* ctx, int mode, double* host_probs);

/* One LevScoreSampled mode update with host-drawn pivots: sampled KRP gather,
 * sampled fibre gather, solve_ls_problem(::ProjectionAlgorithm) (normal != 0:
 * (S^T S) X = (T_s S)^T; else the tall least-squares problem), row_norm
 * (randomized/ProjectionAlgorithm.jl:57-68, randomized/krp_lev_score_sampled.jl:20-57). */
int cpals_sampled_update(cpals_ctx* ctx, int mode, const int64_t* pivots, int64_t nsamps, int normal);

/* ---- batched small decompositions ----
 * Many independent order-3 CP-ALS problems (uneven shapes, ranks up to 64, mode sizes up
 * to 4096 within the shared-memory budget) solved together: one persistent kernel launch
 * per ALS sweep, each CTA running whole sweeps of the tensors it pulls from a device queue.
 * No single counterpart in the reference: it replaces a host loop of decompose(A, rank)
 * calls (src/decompose.jl:1-30) with FitCheck(tol, max_iter, norm(A)) each
 * (src/converge_checks/fit_check.jl:5-66).  dims: count x 3 (row per tensor); tensors are
 * concatenated column-major FP32; factors per tensor are F0, F1, F2 (I_m x R column-major)
 * then lambda (R), concatenated. */
typedef struct cpals_batch cpals_batch;
int cpals_batch_create(cpals_batch** out, int device, int64_t count, const int64_t* dims, const int64_t* ranks,
                       const double* ref_norms);
int cpals_batch_destroy(cpals_batch* b);
int cpals_batch_set_tensors(cpals_batch* b, const float* host_concat);
/* New reference norms (count entries, each finite and > 0), e.g. with a new set of tensors of
 * the same shapes; the FitCheck of the next set_factors / optimize uses them. */
int cpals_batch_set_norms(cpals_batch* b, const double* ref_norms);
/* Initial factors (resets every tensor's FitCheck state). */
int cpals_batch_set_factors(cpals_batch* b, const double* host_concat);
int cpals_batch_get_factors(cpals_batch* b, double* host_concat);
/* Threads per CTA: 128, 256 or 512. */
int cpals_batch_set_threads(cpals_batch* b, int threads);
/* Sweeps per tensor in one launch of cpals_batch_optimize: 0 (the default) runs every tensor to
 * its own stop in a single launch; k >= 1 launches k sweeps at a time (the host polls the
 * active count between launches).  The results are the same either way. */
int cpals_batch_set_sweeps_per_launch(cpals_batch* b, int k);
/* Sweeps until every tensor's FitCheck(tol, max_iter) has stopped.  Per tensor: sweeps run,
 * final fit, flags (1 NaN fit, 2 rank-deficient normal equations met, 4 stopped). */
int cpals_batch_optimize(cpals_batch* b, double tol, int max_iter, int* sweeps_out, double* fits_out, int* flags_out,
                         int64_t* launches_out);
/* Autotuner of the launch schedule, timing `sweeps` sweeps from host_factors per candidate (and
 * restoring host_factors): one class of every tensor at 128, 256 and 512 threads per CTA
 * (ms_out, 3 entries, may be null), and a split into size classes by the CTAs per SM each
 * tensor's shared-memory layout allows (1 to 4), each class with its own layout, thread count
 * (chosen by timing the class alone) and stream, the classes running concurrently.  The
 * fastest schedule is kept; threads_out receives its largest thread count. */
int cpals_batch_autotune(cpals_batch* b, const double* host_factors, int sweeps, int* threads_out, double* ms_out);
/* The schedule in use: *nclass classes; info (6 entries per class, may be null): tensors,
 * largest extent, largest rank, threads per CTA, resident CTAs per SM, and the class's time
 * alone in microseconds (0 when not timed); *ms_split (may be null) the split schedule's time
 * in the last autotune (< 0 when not tried). */
int cpals_batch_schedule(cpals_batch* b, int* nclass, int64_t* info, double* ms_split);

/* ---- seeded synthetic tensors on the device (no counterpart in the reference) ----
 * T = sum_r w_r F_0(:,r) o F_1(:,r) o ... + Gaussian noise at snr_db (counter-based, from
 * `seed`), FP32 column-major into the device buffer d_out (prod(dims) floats).  Factors:
 * FP64 I_m x R column-major, concatenated.  snr_db <= -1000 disables the noise. */
int cpals_synth_lowrank(int device, int order, const int64_t* dims, int64_t rank, const double* host_factors,
                        const double* host_weights, double snr_db, uint64_t seed, float* d_out);

/* ---- the warm-start network (no counterpart in the reference) ----
 * A 3-layer MLP, widths[4] = {in, hidden1, hidden2, out}: BF16 weights and activations,
 * FP32 accumulation, trained on the device (MSE loss, Adam).  Parameters are FP32:
 * W1 [h1][in], b1, W2 [h2][h1], b2, W3 [out][h2], b3. */
typedef struct cpals_mlp cpals_mlp;
int cpals_mlp_create(cpals_mlp** out, int device, const int* widths);
int cpals_mlp_destroy(cpals_mlp* m);
int64_t cpals_mlp_num_params(cpals_mlp* m);
int cpals_mlp_set_params(cpals_mlp* m, const float* host_params);
int cpals_mlp_get_params(cpals_mlp* m, float* host_params);
int cpals_mlp_forward(cpals_mlp* m, const float* host_x, int batch, float* host_y);
int cpals_mlp_gradients(cpals_mlp* m, const float* host_x, const float* host_t, int batch, float* host_grads,
                        double* loss_out);
int cpals_mlp_set_dataset(cpals_mlp* m, const float* host_x, const float* host_t, int64_t n);
int cpals_mlp_train(cpals_mlp* m, const int* host_idx, int steps, int batch, float lr, double* losses);
/* Device time of the last cpals_mlp_train call (ms, CUDA events on the network's stream around
 * its launches) and the tensor-core flops of one training step of B rows. */
int cpals_mlp_train_stats(cpals_mlp* m, int B, double* ms, double* flops_per_step);

#ifdef __cplusplus
}
#endif
#endif /* CPALS_H */

/*
 * rbrp_gb300.h - C ABI of the GB300-native adaptive RBRP column ID.
 *
 * Adaptive Robust Blockwise Random Pivoting selects k columns S of an m x n
 * matrix A (column major) and an interpolation matrix T (k x (n-k)) with
 * A(:, rd) ~= A(:, S) T, stopping once the squared relative residual falls
 * below tol.  Every entry point takes plain pointers and sizes, returns an
 * rbrp_status, never exits, throws or prints, and runs its kernels on the
 * stream set on the handle (default: the legacy default stream).
 *
 * Pointers named d* are device pointers on the handle's device.
 *
 * Reference interfaces replaced (reference repository paths):
 *   RBRP(m, n, A, blk, ranks, error, t_ranks, t_rbrp, flops)   gpu/rbrp.hpp:6-8
 *       -> rbrp_RBRP (drop-in; runs to min(m, n) like the reference loop
 *          gpu/rbrp.cu:367) and rbrp_id_f64 (adds tol and the S/T outputs).
 *   RandAdapLUPP(A, m, n, sk, rd, T, rank, flops, tol, blk)    gpu/rid.hpp:5-7
 *       (declared, never defined in the reference) -> rbrp_RandAdapRBRP, the
 *          same argument meaning with callee-allocated device sk/rd/T as the
 *          sibling RandLUPP does (gpu/randLUPP.cu:25-30).
 *   Compute_interpolation_matrix(r, n, k, Y, P, T)             gpu/interp.hpp:7
 *       -> rbrp_copy_T (T = R11^{-1} R12 of the RBRP factor, k x (n-k), ld >= k).
 *   Handle_t::instance() singletons                            gpu/handle.hpp:28-61
 *       -> rbrp_handle (one per thread / stream; no process-global state).
 */
#ifndef RBRP_GB300_H
#define RBRP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RBRP_GB300_ABI_VERSION 1

typedef enum {
  RBRP_OK = 0,
  RBRP_ERR_INVALID_ARG = 1,   /* bad size, pointer, alignment or parameter */
  RBRP_ERR_CUDA = 2,          /* a CUDA runtime call failed (see rbrp_last_error) */
  RBRP_ERR_ALLOC = 3,         /* device or pinned allocation failed */
  RBRP_ERR_NOT_COMPUTED = 4,  /* result requested before a successful run */
  RBRP_ERR_NUMERIC = 5,       /* non-finite input or breakdown detected on device */
  RBRP_ERR_CAPACITY = 6,      /* caller buffer too small for the result */
  RBRP_ERR_DEVICE_TIMEOUT = 7 /* a bounded device-side wait expired; the kernel exited cleanly */
} rbrp_status;

typedef enum {
  RBRP_SAMPLER_NP = 0,      /* numpy Generator.choice(replace=False, p) semantics over the
                               Philox4x64 stream (python/RBRP.ipynb cell 11 line 108) */
  RBRP_SAMPLER_ES = 1,      /* exponential-key top-b (Efraimidis-Spirakis) over Philox */
  RBRP_SAMPLER_GREEDY = 2   /* top-b residual norms (mode='gp', cell 11 line 112) */
} rbrp_sampler;

typedef enum {
  RBRP_PREC_F64 = 0,        /* FP64 throughout: the plain form */
  RBRP_PREC_F32_MIXED = 1   /* FP32 storage and projections; double-float (pairs of FP32,
                               ~48-bit) panels, sums and T solve; FP64 sampler weights */
} rbrp_precision;

typedef struct {
  double tol;          /* stop when residual < tol * ||A||_F^2 (SQUARED relative
                          residual, python/RBRP.ipynb cell 11 line 164); <= 0: no tol */
  int b;               /* block size (>= 1) */
  int kmax;            /* rank cap; <= 0 means min(m, n) */
  uint64_t seed;       /* Philox key word 0 */
  int sampler;         /* rbrp_sampler */
  int precision;       /* rbrp_precision (rbrp_id_f32 always uses F32_MIXED) */
  double tol_loc;      /* robust-filter tolerance; <= 0 means 1/b (cell 11 line 90) */
  int compute_T;       /* nonzero: compute T = R11^{-1} R12 after the loop */
  int recompute;       /* F32_MIXED: recompute residual norms near tol (1 = on) */
} rbrp_params;

typedef struct {
  int k;               /* rank found (|S|) */
  int nblocks;         /* blocks completed */
  double res0;         /* ||A||_F^2 (FP64 sum of squared column norms) */
  double err_est;      /* final squared relative residual estimate */
  uint64_t draws;      /* uniforms consumed from the np-compat stream */
  double ms_total;     /* device time of the whole call (CUDA events), ms */
  double ms_loop;      /* device time of the pivoting loop, ms */
  double ms_T;         /* device time of the T solve, ms */
  int recomputes;      /* residual-norm recomputations (F32_MIXED) */
} rbrp_result;

typedef struct rbrp_handle_st* rbrp_handle;

/* Defaults: b = 64, tol = 1e-12, kmax = 0, seed = 0, NP sampler, F64, tol_loc = 1/b, T on. */
void rbrp_params_default(rbrp_params* p);

rbrp_status rbrp_create(rbrp_handle* h, int device);
rbrp_status rbrp_destroy(rbrp_handle h);
/* cudaStream_t passed as void* so this header needs no CUDA headers. */
rbrp_status rbrp_set_stream(rbrp_handle h, void* stream);
const char* rbrp_status_string(rbrp_status s);
const char* rbrp_last_error(rbrp_handle h);
int rbrp_abi_version(void);

/* Adaptive RBRP column ID of a device matrix (column major, lda >= m).
 * dPerm (n ints, device or NULL) receives the column permutation: its first
 * k entries are the skeleton S (in selection order), the rest are rd.
 * T stays in the handle until the next run (rbrp_copy_T / rbrp_T_device). */
rbrp_status rbrp_id_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda,
                        const rbrp_params* p, int* dPerm, rbrp_result* out);
rbrp_status rbrp_id_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda,
                        const rbrp_params* p, int* dPerm, rbrp_result* out);

/* Fixed-skeleton ID (no counterpart in the reference, which always pivots):
 * the given skeleton dS (k distinct device column indices) is taken b columns
 * at a time, in list order, through the same panels, swaps and updates as an
 * adaptive run (no tolerance, every nonzero pivot kept), so perm[:k] holds S
 * (reordered by the panel pivots), perm[k:] the rest, and T = R11^{-1} R12 =
 * A(:, S)^+ A(:, rd) as in an adaptive run (rbrp_copy_T).  The forward of the
 * differentiable fixed-skeleton ID; synchronises the handle's stream. */
rbrp_status rbrp_fixed_id_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda, const int* dS,
                              int k, int b, int* dPerm, rbrp_result* out);
rbrp_status rbrp_fixed_id_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda, const int* dS,
                              int k, int b, int* dPerm, rbrp_result* out);

/* Loss and gradient of the fixed-skeleton ID of the last FP32 run
 * (rbrp_fixed_id_f32 on the same dA): with C = A(:, S), B = A(:, rd),
 * T = C^+ B, w = dW(rd) (dW has n entries, those at S are ignored),
 *   L = ||B - C T||_F^2 + ||T w||^2  -> *loss (host),
 * and, when dG != NULL, dG (m x n, ldg >= m) = scale * dL/dA, written in full.
 * FP32 GEMM kernels (double-float sums and triangular solve); synchronises the
 * handle's stream.  No counterpart in the reference. */
rbrp_status rbrp_fixed_id_adjoint_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda,
                                      const float* dW, float scale, float* dG, int64_t ldg, double* loss);

/* Gaussian sketch for the sketch-based comparison IDs (RandCPQR_OS / RandLUPP_OS,
 * gpu/randCPQR_OS.cu:20-111, whose G is drawn in gpu/random.cu and applied by
 * the cuBLAS GEMM of gpu/gemm.cu:9-15): dY (l x n, ldy >= l) = G A with
 * G (l x m) = scale * N(0, 1) from Philox4x64-10 (key seed) by Box-Muller.
 * The product runs on the tensor cores (tcgen05, 3xTF32: FP32-accurate) when dA
 * and lda are 16-byte aligned; that path waits for its kernels to read their
 * status (a bounded device wait that runs out gives RBRP_ERR_DEVICE_TIMEOUT).
 * Otherwise a CUDA-core FP32 GEMM runs, asynchronously on the handle's stream. */
rbrp_status rbrp_sketch_gaussian_f32(rbrp_handle h, int l, int m, int n, const float* dA, int64_t lda,
                                     uint64_t seed, float scale, float* dY, int64_t ldy);

/* Row pivots of the partial-pivoted LU of W^T, as RandLUPP_OS takes them from
 * cusolverDnDgetrf on the first k rows of its sketch (gpu/randLUPP_OS.cu:48-90)
 * and turns them into a permutation (pivots_to_permutation, gpu/permute.cu:8-23).
 * dW is k x n (ldw >= k, 1 <= k <= n, k <= 25600) FP64; dPerm (n ints) receives
 * the permutation of W's columns (perm[:k] is the skeleton); dIpiv (k ints, may
 * be NULL) receives LAPACK's 1-based pivots.  Ties go to the first current
 * position, as idamax.  RBRP_ERR_NUMERIC for a non-finite W or a zero pivot
 * (the reference asserts info == 0).  One cooperative launch; synchronises the
 * handle's stream. */
rbrp_status rbrp_lupp_pivots_f64(rbrp_handle h, int k, int n, const double* dW, int64_t ldw, int* dPerm,
                                 int* dIpiv);

/* The reference's comparison IDs (gpu/rid.hpp) on this library's kernels.  A is
 * a device FP64 matrix, m x n, ld = m; k is the rank (1 <= k <= min(m, n)); the
 * sketch Y = G A has 2k rows, G ~ N(0, 1/m) from Philox with key `seed` (the
 * reference draws G from a process-wide counter, gpu/random.cu:43).  T is
 * k x (n - k), ld = k, rows in sk order and columns in rd order, allocated here
 * on the device (free with rbrp_free).  Synchronous; own temporary handle.
 *  - RandLUPP_OS (gpu/randLUPP_OS.cu:14-119): sk (k) and rd (n - k) are device
 *    arrays allocated here (free with rbrp_free); skeleton from the LU pivots
 *    of Y(1:k, :)^T.
 *  - RandCPQR_OS (gpu/randCPQR_OS.cu:20-111): h_sk (k) and h_rd (n - k) are
 *    caller-owned host arrays; skeleton from the column-pivoted QR of Y(1:k, :).
 * flops: the reference's operation count where it sets one. */
rbrp_status rbrp_RandLUPP_OS(const double* dA, int m, int n, int k, int** sk, int** rd, double** T,
                             double* flops, uint64_t seed);
rbrp_status rbrp_RandCPQR_OS(const double* dA, int m, int n, int k, int* h_sk, int* h_rd, double** T,
                             double* flops, uint64_t seed);
/* The CPQR baseline (gpu/id_cpqr.hpp, gpu/id_cpqr.cu:30-172): column-pivoted QR
 * of A (device FP64, m x n, ld = m; LAPACK dgeqp3's pivots, greedy b = 1) to the
 * largest of ranks[0..nranks); err[q] receives the squared relative ID error at
 * rank ranks[q], t_ranks[q] (may be NULL) the cumulative seconds to that rank,
 * *t_cpqr the total seconds.  Synchronous; own temporary handle. */
rbrp_status rbrp_CPQR(int m, int n, const double* dA, const int* ranks, int nranks, double* err,
                      double* t_ranks, double* t_cpqr, double* flops);

/* T (k x (n-k), column major) of the last run, into a device buffer with ldt >= k. */
rbrp_status rbrp_copy_T(rbrp_handle h, double* dT, int64_t ldt);
/* The notebook's L of the last run (python/RBRP.ipynb cell 11: L = A^T Q, one
 * row per column of A in its original order, one column per basis vector), into
 * a device buffer (n x k, column major, ldl >= n): L(perm[p], a) = R(a, p), the
 * projection of the column at position p onto basis vector a, for p >= a, and 0
 * for p < a (columns chosen before basis vector a, which the notebook leaves at
 * 0 and which are orthogonal to it).  Each basis vector's sign follows a panel
 * factor with a positive diagonal; LAPACK's QR in the notebook may flip it, which
 * flips that column of L and leaves the interpolation matrix unchanged.
 * Asynchronous on the handle's stream. */
rbrp_status rbrp_copy_L(rbrp_handle h, double* dL, int64_t ldl);
/* Device pointer of T of the last run (ld = k), valid until the next run. */
rbrp_status rbrp_T_device(rbrp_handle h, const double** dT, int* ld);
/* python/RBRP.ipynb cell 2 lines 111-126 (matdivide, A * pinv(B) from the SVD of
 * B, singular values above the absolute cutoff tol kept; TOL_FP = 1e-12, cell 0
 * line 26), which get_rpid_error uses for the interpolation matrix of blocked
 * runs (cell 11 lines 226-232): X (q x nc, ldx >= q) = pinv_tol(B) C for B
 * (p x q, ldb >= p) and C (p x nc, ldc >= p), FP64 device arrays.  The SVD is a
 * one-sided Jacobi iteration in FP64; *rank (may be NULL) receives the number of
 * singular values above tol.  The notebook's matdivide(A2, B2) is X^T for
 * B = B2^T, C = A2^T.  Runs on the handle's stream and returns when done. */
rbrp_status rbrp_matdivide_f64(rbrp_handle h, int p, int q, int nc, const double* dB, int64_t ldb,
                               const double* dC, int64_t ldc, double tol, double* dX, int64_t ldx, int* rank);
/* T of the last run replaced by pinv_tol(R11) R12 (rbrp_matdivide_f64 on the
 * run's factor): the rank-revealing interpolation for a skeleton whose R11 is
 * ill-conditioned or singular (a fixed skeleton given from outside).  Equal to
 * R11^{-1} R12 when every singular value of R11 exceeds tol.  rbrp_copy_T /
 * rbrp_T_device then return it. */
rbrp_status rbrp_T_matdivide(rbrp_handle h, double tol, int* rank);
/* FP64 iterative refinement of the last run's T against the matrix A it was
 * computed from (same m, n; device, column major, lda): each of `steps` steps
 * is T += pinv(A_S) (A(:, rd) - A(:, S) T), in FP64 on the exact values of A
 * (A_S and A(:, rd) gathered through perm, the pseudo-inverse by the Jacobi SVD
 * of rbrp_matdivide_f64 with singular values below max(tol, max(m, k) eps
 * |A_S|_F) dropped).  It recovers the least-squares T of the skeleton where the
 * factor's R11 is ill-conditioned.  *change (may be NULL) receives |dT|_F/|T|_F
 * of the last step.  The precision scheme of the mixed form (FP32 data) with
 * "FP64 iterative refinement of T"; no counterpart in gpu/ (the reference's T
 * is one triangular solve, gpu/id_cpqr.cu:133-136). */
rbrp_status rbrp_refine_T_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda, int steps,
                              double tol, double* change);
rbrp_status rbrp_refine_T_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda, int steps,
                              double tol, double* change);
/* Per-block trace of the last run: cumulative ranks and squared relative
 * residual estimates (gpu/rbrp.cu:467, 473-475) and cumulative device time per
 * block in ms.  Host arrays of capacity cap; *nblocks receives the count. */
rbrp_status rbrp_get_trace(rbrp_handle h, int* ranks, double* errors, double* t_ms,
                           int cap, int* nblocks);

/* Squared relative ID error ||A(:,rd) - A(:,S) T||_F^2 / ||A||_F^2 of the last run,
 * recomputed in FP64 on the device (python/RBRP.ipynb cell 7 lines 40-53).
 * dA must be the matrix of the last run (FP64 or FP32 as that run). */
rbrp_status rbrp_id_error_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda,
                              double* err);
rbrp_status rbrp_id_error_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda,
                              double* err);

/* No counterpart in the reference.  For callers that cannot let a library
 * allocate device memory (a host runtime that owns a fixed device pool, a hard
 * memory budget, work enqueued where an allocation would synchronise): the
 * squared relative ID error ||A(:,rd) - A(:,S) T||_F^2 / normA2 written to
 * *dErr on `stream` (cudaStream_t), computed without a handle and without any
 * allocation.  Inputs: A (m x n, FP64, lda), perm (n ints; S = perm[:k], rd =
 * perm[k:]), T (k x (n-k), ldt >= k); all device pointers in the current
 * context.  k == 0 writes 1.0 and k == n writes 0.0 (A, perm and T may then be
 * NULL), as rbrp_id_error_f64 reports them.  Its scratch is a fixed 2 MiB device
 * array in the library (held by every GPU that loads it until exit), so sizes
 * with ceil((n-k)/32) * ceil(m/64) > 262144 return RBRP_ERR_CAPACITY.  All calls
 * on a device share that array: calls that overlap on the GPU race and must be
 * serialised.  The first call in each CUDA context (primary or caller-created;
 * a context made after cudaDeviceReset is a new one) looks the array up
 * (cudaGetSymbolAddress); make that call before any stream capture. */
rbrp_status rbrp_id_error_f64_noalloc(int m, int n, const double* dA, int64_t lda, const int* dPerm, int k,
                                      const double* dT, int64_t ldt, double normA2, double* dErr, void* stream);

/* Host-buffer convenience: copies hA (host, column major, lda) in, runs, copies
 * perm (n) and, when hT != NULL, T (k x (n-k), ldt >= k) back to host memory. */
rbrp_status rbrp_id_f64_host(rbrp_handle h, int m, int n, const double* hA, int64_t lda,
                             const rbrp_params* p, int* hPerm, double* hT, int64_t ldt,
                             int64_t t_cap, rbrp_result* out);
rbrp_status rbrp_id_f32_host(rbrp_handle h, int m, int n, const float* hA, int64_t lda,
                             const rbrp_params* p, int* hPerm, double* hT, int64_t ldt,
                             int64_t t_cap, rbrp_result* out);

/* ---- batched form: many independent IDs in one persistent launch -------
 *
 * The reference solves one matrix per RBRP() call (gpu/rbrp.cu:333-503,
 * driven per matrix from gpu/driver.cpp:177); it has no batched entry.  Here
 * each problem runs the same adaptive loop as rbrp_id_f32 (FP32 residual form,
 * double-float panel, sums and T solve) inside one CTA of a persistent kernel
 * that pulls problems, largest first, from a device-side work queue.  The
 * launch (queue reset + kernel) is captured once in a CUDA graph and replayed
 * by rbrp_batch_run.  Problem q uses the Philox key seed + q.  Each problem's
 * data is scaled by a power of two at load (exact), so blocks whose entries
 * are far below 1 (off-diagonal kernel blocks) keep full FP32 resolution.
 */
typedef struct {
  int m, n;            /* shape, m, n >= 1 */
  int64_t lda;         /* leading dimension of A, >= m */
  const float* A;      /* device or pinned host memory, column major, FP32 */
  int* perm;           /* device or pinned host, n ints (output): perm[:k] = S, perm[k:] = rd */
  double* T;           /* device or pinned host (output) T = R11^{-1} R12, k x (n-k), column
                          major, ld = k; NULL: not computed */
  int64_t T_cap;       /* doubles available at T (k * (n-k) are written) */
} rbrp_batch_problem;
/* Pinned (page-locked) host buffers are used in place: a host A is read once by
 * the kernel's first pass over its problem and staged in the CTA's workspace,
 * perm and T are written to host memory by the kernel, so host-device traffic
 * overlaps the IDs of other problems.  Pageable host memory is rejected. */

typedef struct {
  int k;               /* rank found */
  int nblocks;         /* blocks that kept at least one column */
  int status;          /* RBRP_OK, RBRP_ERR_NUMERIC (non-finite input / no progress) or
                          RBRP_ERR_CAPACITY (T_cap < k * (n-k): T not written) */
  int attempts;        /* block attempts, including numerically zero panels */
  double res0;         /* ||A||_F^2 */
  double err_est;      /* squared relative residual at the stop */
  uint64_t draws;      /* uniforms consumed from the np-compat stream */
  double alg_bytes;    /* algorithmic HBM bytes: 4 [m n + sum_t m n_t + sum_t m bs_t]
                          (n_t columns left after block t, bs_t columns sampled) */
  double alg_flops;    /* algorithmic flops: 2 m n + sum_t [2 m n_t b_t + 4 m bs_t^2] + k^2 (n-k) */
} rbrp_batch_result;

typedef struct {
  int b;               /* block size in use (the autotuner's choice when params b <= 0) */
  int panel_cols;      /* panel capacity of the kernel variant in use (16 or 32) */
  int ctas;            /* persistent CTAs of the launch */
  int ctas_per_sm;
  double ms_last;      /* device time of the last rbrp_batch_run, ms */
  double ms_autotune;  /* time the autotuner spent in the last plan, ms */
  size_t workspace_bytes;
} rbrp_batch_info;

/* Plans a batch: validates and uploads the problem list (host array), sizes the
 * per-CTA workspace slots and, when p->b <= 0, runs the autotuner, which times
 * the candidate block sizes (b in {8, 16, 24, 32}) and CTAs per SM on this very
 * batch and keeps the fastest (results for a fixed b are deterministic).  The
 * batched kernel takes b <= 32.  Keeps the problems' buffers by pointer until
 * the next plan. */
rbrp_status rbrp_batch_plan(rbrp_handle h, int nprob, const rbrp_batch_problem* problems,
                            const rbrp_params* p);
/* Enqueues the planned batch on the handle's stream as one CUDA graph launch
 * (captured on first use after a plan); does not synchronise. */
rbrp_status rbrp_batch_run(rbrp_handle h);
/* Waits for the last run and copies its per-problem results (host array of
 * cap >= nprob entries, in the caller's problem order). */
rbrp_status rbrp_batch_results(rbrp_handle h, rbrp_batch_result* out, int cap);
rbrp_status rbrp_batch_get_info(rbrp_handle h, rbrp_batch_info* info);
/* Replaces the planned queue order (problem indices in the order the persistent
 * CTAs take them; the plan's default is largest m*n first).  order must list
 * every problem once.  Results do not depend on the order. */
rbrp_status rbrp_batch_set_order(rbrp_handle h, const int* order, int n);
/* In-kernel phase profile of the batched kernel: when on, thread 0 of every CTA
 * adds the SM cycles of each phase (clock64 between the barriers that end the
 * phases) into device counters, accumulated over runs until switched on again.
 * Phases: 0 column norms, 1 sampler, 2 panel gather + Gram, 3 pivoted Cholesky
 * + filter + swap, 4 basis solve + R/column swaps, 5 projection W = Q^T A_res,
 * 6 update A_res -= Q W + norms, 7 residual sums + stop rule, 8 T solve. */
#define RBRP_BATCH_NPHASES 9
rbrp_status rbrp_batch_set_profiling(rbrp_handle h, int on);
rbrp_status rbrp_batch_get_phase_cycles(rbrp_handle h, double* cycles, int cap);
/* plan + run + results in one call. */
rbrp_status rbrp_id_batched_f32(rbrp_handle h, int nprob, const rbrp_batch_problem* problems,
                                const rbrp_params* p, rbrp_batch_result* out);

/* ---- per-phase timing (CUDA events on the handle's stream) ------------- */
enum {
  RBRP_PHASE_NORMS = 0,    /* initial column norms + totals */
  RBRP_PHASE_SAMPLE = 1,   /* block sampler */
  RBRP_PHASE_CGS = 2,      /* Gram-Schmidt coefficients + panel update + Gram */
  RBRP_PHASE_PANEL = 3,    /* pivoted CholQR2 + filter + swap */
  RBRP_PHASE_PROJECT = 4,  /* projection W = Q_blk^T A of the remaining columns (+ downdate, FP64) */
  RBRP_PHASE_FINISH = 5,   /* residual, stop rule, trace */
  RBRP_PHASE_TSOLVE = 6,   /* T = R11^{-1} R12 */
  RBRP_PHASE_UPDATE = 7,   /* residual update A_res -= Q_blk W + exact norms (FP32 form) */
  RBRP_NPHASES = 8
};
typedef struct {
  double ms[RBRP_NPHASES];      /* summed device time */
  double bytes[RBRP_NPHASES];   /* algorithmic HBM bytes (minimum traffic) */
  double flops[RBRP_NPHASES];   /* algorithmic flops */
  int launches[RBRP_NPHASES];   /* kernel launches */
} rbrp_phase_stats;
/* When on, every phase is bracketed by CUDA events and accumulated until reset. */
rbrp_status rbrp_set_profiling(rbrp_handle h, int on);
rbrp_status rbrp_get_phase_stats(rbrp_handle h, rbrp_phase_stats* out);
rbrp_status rbrp_reset_phase_stats(rbrp_handle h);

/* ---- drop-in shims ----------------------------------------------------- */

/* gpu/rbrp.hpp:6-8: RBRP on a device FP64 matrix (ld = m) to rank min(m, n) with
 * block size blk.  ranks/error/t_ranks are host arrays of capacity cap filled
 * with the cumulative per-block rank, squared relative residual and time (s);
 * *nblocks receives their length, *t_rbrp the total time (s), *flops the
 * algorithmic flop count (the reference leaves it unset). */
rbrp_status rbrp_RBRP(int m, int n, double* dA, int blk, int* ranks, double* error,
                      double* t_ranks, int cap, int* nblocks, double* t_rbrp, double* flops);

/* gpu/rid.hpp:5-7 (RandAdapLUPP's argument meaning, RBRP pivoting): adaptive
 * ID to squared relative tolerance tol with block size blk.  *sk (rank ints),
 * *rd (n - rank ints) and *T (rank x (n - rank), ld = rank) are allocated on
 * the device by the callee; release them with rbrp_free. */
rbrp_status rbrp_RandAdapRBRP(const double* dA, int m, int n, int** sk, int** rd,
                              double** T, int* rank, double* flops, double tol, int blk);
rbrp_status rbrp_free(void* dptr);

#ifdef __cplusplus
}
#endif
#endif /* RBRP_GB300_H */

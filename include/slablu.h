/* slablu: GB300-native slab direct-solve path (HBS compression, HBS ULV,
 * block-tridiagonal red-black / Thomas elimination) behind a C ABI.
 *
 * Conventions
 *   - Every entry point returns an int status: 0 = SLU_OK, otherwise one of
 *     the SLU_ERR_* codes below; slu_last_error() returns the message of the
 *     most recent failure on the calling thread.  No C++ exception crosses
 *     this boundary.
 *   - All matrix arguments are DEVICE pointers to row-major float64 (or
 *     float32 where the name says so) arrays with the stated leading
 *     dimension.  HBS levels use the stacked block layout of the upstream
 *     code: a level with Nb blocks of n rows is one (Nb*n) x c array.
 *   - Work is enqueued on the handle's stream and is asynchronous; callers
 *     synchronise with slu_sync() or their own stream events.
 *   - A handle owns factor storage and a grow-only scratch arena; one handle
 *     must not be used from two host threads at once.
 *
 * Each entry point names the upstream Python function it replaces (paths
 * relative to the SslabLU repository).
 */
#ifndef SLABLU_H
#define SLABLU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SLU_OK 0
#define SLU_ERR_ARG 1
#define SLU_ERR_ALLOC 2
#define SLU_ERR_CUDA 3
#define SLU_ERR_NUMERIC 4
#define SLU_ERR_STATE 5
#define SLU_ERR_NOT_CONVERGED 6
#define SLU_ERR_TIMEOUT 7

typedef struct slu_handle_s* slu_handle_t;
typedef struct slu_hbs_s* slu_hbs_t;
typedef struct slu_dense_rb_s* slu_rb_t;
typedef struct slu_solve_plan_s* slu_solve_plan_t;
typedef struct slu_refine_plan_s* slu_refine_plan_t;
typedef struct slu_strong_s* slu_strong_t;

/* ---------------------------------------------------------------- runtime */
int slu_version(void);
/* Kernels launched by this library so far in this process (host-side count,
 * all streams); a diagnostic for benchmarks. */
long long slu_launch_count(void);
/* Host waits made by the calling thread (slu_sync and the library's own
 * waits): 0 spins (the default: lowest latency), 1 sleeps on a blocking-sync
 * event.  For worker threads that run many factorisations at once, whose
 * spinning waits would take the host cores from the threads launching work.
 * Beyond upstream (a host runtime setting of this library). */
void slu_set_blocking_waits(int on);
/* Copies the last error message of this thread into buf (NUL terminated). */
int slu_last_error(char* buf, size_t len);
/* stream: a cudaStream_t (NULL = legacy default stream). */
int slu_create(void* stream, slu_handle_t* out);
int slu_destroy(slu_handle_t h);
int slu_set_stream(slu_handle_t h, void* stream);
/* Synchronises the handle's stream and reports device-side status words
 * (e.g. a Jacobi SVD that did not converge) as SLU_ERR_NOT_CONVERGED. */
int slu_sync(slu_handle_t h);

/* ---------------------------------------------------------------- HBS operator
 * Replaces matAssembly/HBS/HBSnew.py:82-118 (HBSMAT.__init__ with a tree):
 * N points, L tree levels (leaves at level 0), fac = 2 (binary) or 4 (quad),
 * perm_host = tree.perm_leaf (N host int64 entries, NULL = identity). */
int slu_hbs_create(slu_handle_t h, int N, int L, int fac, const int64_t* perm_host,
                   slu_hbs_t* out);
/* Frees the object's device memory stream-ordered (cudaFreeAsync on the
 * stream each buffer was allocated on): work that reads the object on any
 * other stream must have completed first (synchronise those streams). */
int slu_hbs_destroy(slu_hbs_t op);

/* Replaces HBSMAT.constructHBS_ULV (matAssembly/HBS/HBSnew.py:211-295) after
 * the sampling step: Om, Psi are the N x s Gaussian sketches and Y = A Om',
 * Z = A^T Psi' the samples, all in tree order (rows permuted by perm_leaf),
 * leading dimension s.  nleaves = tree.nleaves, rk = target rank.  With
 * compute_ulv = 1 the ULV factorisation is interleaved (construct(rk, True)). */
int slu_hbs_compress(slu_handle_t h, slu_hbs_t op, int nleaves, int rk, int s, const double* Om,
                     const double* Psi, const double* Y, const double* Z, int compute_ulv);

/* Replaces HBSMAT.set_mats (matAssembly/HBS/HBSnew.py:125-133) one level at a
 * time: level 0 = leaves.  U, V: (Nb*n) x k, D: (Nb*n) x n (device); on the
 * root pass k = 0 and U = V = NULL.  Every level must be set before use.
 * V may be NULL for an operator that is only solved with loaded ULV factors
 * (slu_hbs_set_ulv_level); apply and factorisation then report an error. */
int slu_hbs_set_level(slu_handle_t h, slu_hbs_t op, int level, int Nb, int n, int k,
                      const double* U, const double* V, const double* D);

/* Loads given ULV factors of one level (ULVsparse.solve's Qlist[level],
 * Wlist[level], Rlist[level], Uulist[level]; ULVsparse.py:295), after every
 * level was set with slu_hbs_set_level (V may be NULL there for an operator
 * that is only solved).  Q, W: (Nb*n) x n; R: (Nb*(n-k)) x n (root: n x n);
 * Uu: (Nb*(n-k)) x k.  W and Uu are ignored (may be NULL) on the root. */
int slu_hbs_set_ulv_level(slu_handle_t h, slu_hbs_t op, int level, const double* Q,
                          const double* W, const double* R, const double* Uu);

/* Replaces ULVsparse.compute_ULV (matAssembly/HBS/ULVsparse.py:231-293) /
 * HBSMAT.compute_ULV (HBSnew.py:390-391) for loaded factors. */
int slu_ulv_factor(slu_handle_t h, slu_hbs_t op);

/* Replaces HBSMAT.matmat / rmatmat (HBSnew.py:308-350): Y = A X (trans = 0)
 * or A^T X, X and Y N x nrhs in the caller's (unpermuted) ordering. */
int slu_hbs_apply(slu_handle_t h, slu_hbs_t op, int trans, const double* X, int ldx, double* Y,
                  int ldy, int nrhs);

/* Replaces HBSMAT.solve (HBSnew.py:393-416) -> ULVsparse.solve
 * (ULVsparse.py:295-358), in place on B (N x nrhs, unpermuted ordering).
 * trans = 1 reproduces upstream's mode 'T' handling of the permutation. */
int slu_ulv_solve(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs, int trans);

/* Allocation-free variant of slu_ulv_solve (same float64 solve, same result).
 * It has no counterpart in the upstream code.  It exists for callers that
 * cannot let a library allocate device memory while they solve: a serving
 * runtime that owns the GPU's memory under a fixed budget, or a latency-
 * critical loop where cudaMalloc's implicit synchronisation is not
 * acceptable.  Scratch comes from a fixed 16 MiB array compiled into the
 * library (held on every GPU that loads it until the process exits); the
 * call makes no cudaMalloc / cudaFree or other allocation.  Limit: five
 * N x nrhs float64 buffers must fit, i.e. 5 * roundup(8*N*nrhs, 256) <=
 * 16 MiB (N = 4096: up to 102 right-hand sides); larger sizes are rejected
 * with SLU_ERR_ARG.  The first call on a device (with that device current)
 * looks up the array's device address with cudaGetSymbolAddress; make that
 * first call before any stream capture.  All calls on a device share the
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller.  The handle's stream must belong to the current device
 * (SLU_ERR_ARG otherwise).  The operator must already be factored
 * (slu_hbs_compress with compute_ulv or slu_ulv_factor). */
int slu_ulv_solve_noalloc(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs, int trans);

/* Out-of-place solve: Y (N x nrhs, ld ldy) <- A^{-1} X (trans = 0) or
 * A^{-T} X (trans = 1) (ld ldx), X unchanged (X == Y with equal leading
 * dimensions solves in place).  The same arithmetic as slu_ulv_solve with
 * the same trans; the first launch reads X and the last writes Y, so no copy
 * of the right-hand sides is made.  Beyond upstream (HBSMAT.solve returns a
 * new array: this is that solve without the copy). */
int slu_ulv_solve_into(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                       int ldy, int nrhs, int trans);

/* Solve plan: slu_ulv_solve_into for fixed X, Y (device or pinned host
 * pointers), nrhs and trans, captured once as a CUDA graph with its own
 * scratch (and the launch plans tuned for nrhs at creation).  Each
 * slu_ulv_solve_plan_launch then solves whatever X holds into Y with one
 * graph launch on h's stream instead of one kernel launch per tree step;
 * wait != 0 also waits for the result.  A plan refuses to launch
 * (SLU_ERR_STATE) once its operator is refactored or destroyed; destroy
 * plans with slu_ulv_solve_plan_destroy.  Beyond upstream. */
int slu_ulv_solve_plan_create(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                              int ldy, int nrhs, int trans, slu_solve_plan_t* out);
int slu_ulv_solve_plan_launch(slu_handle_t h, slu_solve_plan_t plan, int wait);
/* The grouped refinement of slu_refine_grouped for fixed blocks B[i] -> X[i]
 * (device pointers), made once: buffers and task tables built and uploaded
 * at creation, an iteration replayed as CUDA graphs.  slu_refine_plan_run
 * refines whatever the B[i] hold (same results, iteration count and errors
 * as slu_refine_grouped); a plan refuses to run (SLU_ERR_STATE) once one of
 * its operators is refactored or destroyed.  Beyond upstream. */
int slu_refine_grouped_plan_create(slu_handle_t h, int count, const slu_hbs_t* ops,
                                   const double* const* B, const int* ldb, double* const* X,
                                   const int* ldx, const int* nrhs, slu_refine_plan_t* out);
int slu_refine_plan_run(slu_handle_t h, slu_refine_plan_t plan, double tol, int maxit,
                        int* iters_out, double* relres_out);
int slu_refine_plan_destroy(slu_refine_plan_t plan);
/* The grouped solve of slu_ulv_solve_grouped (B[i] <- A_i^{-1} B[i], mode N)
 * for fixed blocks as a solve plan: the step tables of every member are
 * built and uploaded once and the group's launches captured as one CUDA
 * graph; launch and destroy it like any solve plan. */
int slu_ulv_solve_grouped_plan_create(slu_handle_t h, int count, const slu_hbs_t* ops,
                                      double* const* B, const int* ldb, const int* nrhs,
                                      slu_solve_plan_t* out);
int slu_ulv_solve_plan_destroy(slu_solve_plan_t plan);
/* A fixed program of grouped phases as a solve plan: the phases run in
 * order, each over its own members (count[p] of them; the member arrays are
 * concatenated over the phases).  kind 0: X[i] <- A_i^{-1} X[i] (mode N, in
 * place, the grouped solve); kind 1: Y[i] <- A_i X[i] (the grouped apply);
 * X, Y device float64 blocks of nrhs[i] columns, leading dimension ld[i].
 * Elementwise blocks of n[i] contiguous doubles (ops ignored): kind 2
 * Y = X, 3 Y = 0, 4 Y += X, 5 Y -= X, 6 Y = X - Y.  Every table is built and
 * uploaded once and the program captured as one CUDA graph; launch with
 * slu_ulv_solve_plan_launch.  Used to run the red-black HBS solves of many
 * slab systems together (omsdirectsolveHBS.py:489-558, RedBlackSolverHBS.solve,
 * for a batch).  Beyond upstream. */
int slu_grouped_program_create(slu_handle_t h, int nphase, const int* kind, const int* count,
                               const slu_hbs_t* ops, double* const* X, double* const* Y,
                               const int* ld, const int* nrhs, const long long* n,
                               slu_solve_plan_t* out);

/* Single-precision copy of the ULV factors and a float32 solve with the same
 * sweep; used inside iterative refinement (no upstream counterpart: the
 * mixed-precision path of this library). */
int slu_hbs_prepare_f32(slu_handle_t h, slu_hbs_t op);
int slu_ulv_solve_f32(slu_handle_t h, slu_hbs_t op, float* B, int ldb, int nrhs, int trans);

/* Double-float copy of the ULV factors (each float64 split into a float32
 * pair hi + lo, interleaved) and a mode-N solve with the same fused sweep in
 * double-float arithmetic on the float32 units: B (N x nrhs float64, device)
 * <- A^{-1} B to ~1e-14 relative accuracy (48-bit significands, float32
 * exponent range).  slu_ulv_solve_dfloat prepares the copy on first use;
 * slu_hbs_prepare_dfloat does it ahead.  No upstream counterpart: a solve
 * mode of the mixed-precision path of this library. */
int slu_hbs_prepare_dfloat(slu_handle_t h, slu_hbs_t op);
int slu_ulv_solve_dfloat(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs);

/* Iterative refinement of A x = b with ULV solves on the float32 units and a
 * float64-accurate residual r = b - A x of the stored HBS factors (the
 * operator the upstream solve inverts), evaluated in double-float arithmetic
 * (factors as float32 hi/lo pairs, error-free products and sums: ~1e-14
 * relative).  The inner solve is the double-float sweep (default; one
 * iteration reaches 1e-10 on well-conditioned operators) or the float32
 * sweep, chosen by slu_hbs_set_refine_inner.  X holds the result
 * (N x nrhs); iterations stop when every column reaches ||r||/||b|| <= tol or
 * after maxit corrections.  iters_out / relres_out (host pointers, may be
 * NULL) receive the iteration count and the largest final relative
 * residual. */
int slu_refine(slu_handle_t h, slu_hbs_t op, const double* B, int ldb, double* X, int ldx,
               int nrhs, double tol, int maxit, int* iters_out, double* relres_out);
/* Inner solve of slu_refine for `op`: mode 1 double-float sweep (default),
 * mode 0 float32 sweep, mode 2 the tensor-core sweep of slu_ulv_solve_ozaki
 * with the residual from slu_hbs_apply_ozaki's tensor-core apply. */
int slu_hbs_set_refine_inner(slu_hbs_t op, int mode);

/* Tensor-core (tcgen05) mode-N solve and apply at float64-level accuracy.
 * Every step product of the ULV sweep (ULVsparse.solve,
 * matAssembly/HBS/ULVsparse.py:296-327) and of the HBS apply
 * (HBSnew.HBSMAT.matmat, matAssembly/HBS/HBSnew.py:308-350) runs as bfloat16
 * tensor-core products of error-free base-256 digit splits of both operands
 * (the Ozaki scheme: 7 digits each, the 28 digit pairs of weight >= 2^-64
 * accumulated exactly in float32 per digit diagonal, the diagonals summed in
 * double-float); vectors between steps are float32 pairs, each right-hand-
 * side column normalised on entry by the power of two of its largest entry
 * (any float64 magnitude).  Relative error ~2^-50 of |S||z| per product.
 * Steps must read at most 128 rows per block
 * (SLU_ERR_ARG otherwise).  slu_hbs_prepare_ozaki builds the operator digits
 * (7 bf16 digits + a row scale per operator entry) once after a
 * factorisation; the solve / apply do it on first use.
 * slu_ulv_solve_ozaki: Y <- A^{-1} X, or A^{-T} X with trans (the
 * transposed steps of slu_ulv_solve's mode T); slu_hbs_apply_ozaki: Y <- A X,
 * or A^T X (X, Y N x nrhs float64, device, distinct).  No upstream counterpart: the
 * tensor-core form of the mixed-precision path. */
int slu_hbs_prepare_ozaki(slu_handle_t h, slu_hbs_t op);
int slu_ulv_solve_ozaki(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                        int ldy, int nrhs, int trans);
int slu_hbs_apply_ozaki(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                        int ldy, int nrhs, int trans);

/* Null-space rule of the next slu_hbs_compress of `op`: mode 0 projects each
 * block's sketch on the last n columns of the complete Q of Om_blk^T
 * (HBSnew.compute_UV, matAssembly/HBS/HBSnew.py:20-28; the default), mode 1
 * on every column after the first n (HBStorch.compute_UV,
 * matAssembly/HBS/HBStorch.py:73-82, the rkHBS assembler's engine).  Mode 0
 * spans the null space only when s >= 2n; mode 1 does for every s > n. */
int slu_hbs_set_null_space(slu_hbs_t op, int mode);

/* Grouped solves over `count` operators of any sizes and depths, one kernel
 * launch per tree step for the whole group (the batched form of calling
 * HBSnew.HBSMAT.solve, matAssembly/HBS/HBSnew.py:393-416, once per operator;
 * the reference has no grouped call).  Arrays are host arrays of `count`
 * entries; B[i] / X[i] are device pointers to N_i x nrhs[i] row-major blocks
 * with leading dimensions ldb[i] / ldx[i]; members with nrhs[i] == 0 are
 * skipped.  Each member's result equals its own slu_ulv_solve (mode N) /
 * slu_refine result: every member runs the same per-level arithmetic.
 *   slu_ulv_solve_grouped: B[i] <- A_i^{-1} B[i] in float64.
 *   slu_refine_grouped: X[i] from float32 sweeps refined by double-float
 *     residuals until every column of every member reaches tol; iters_out
 *     (may be NULL) receives the common iteration count and relres_out (may
 *     be NULL, else count entries) each member's worst relative residual. */
int slu_ulv_solve_grouped(slu_handle_t h, int count, const slu_hbs_t* ops, double* const* B,
                          const int* ldb, const int* nrhs);
/* Grouped apply: Y[i] (N_i x nrhs[i], ld ldy[i]) <- A_i X[i] (trans[i] = 0)
 * or A_i^T X[i] (trans[i] = 1), one launch per tree step for the whole group
 * (the batched form of HBSMAT.matmat / rmatmat, matAssembly/HBS/
 * HBSnew.py:308-350); every member's result equals its own slu_hbs_apply
 * bitwise.  Host arrays of count entries; nrhs[i] == 0 skips a member. */
int slu_hbs_apply_grouped(slu_handle_t h, int count, const slu_hbs_t* ops, const int* trans,
                          const double* const* X, const int* ldx, double* const* Y,
                          const int* ldy, const int* nrhs);
int slu_refine_grouped(slu_handle_t h, int count, const slu_hbs_t* ops, const double* const* B,
                       const int* ldb, double* const* X, const int* ldx, const int* nrhs,
                       double tol, int maxit, int* iters_out, double* relres_out);

/* Diagnostics: one float64 mode-N solve (as slu_ulv_solve) with a CUDA event
 * pair around each kernel launch; returns after the solve completes.  The
 * solve is queued behind a ~0.5 ms device-side sleep, so every launch is
 * already queued when the device reaches it and the event pairs measure
 * device time only.
 * ms_out[k] is the device time of launch k (launch order), level_out[k] its
 * tree level and kind_out[k] its sweep (0 forward, 1 root, 2 backward), for
 * k < cap (host arrays, each may be NULL); *nlaunch receives the number of
 * launches.  The reference keeps host-side timers on HBSMAT
 * (matAssembly/HBS/HBSnew.py:108-111, 155-200); this is their device-side
 * counterpart for the solve. */
int slu_ulv_solve_timed(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs,
                        float* ms_out, int* level_out, int* kind_out, int cap, int* nlaunch);

/* Autotuner of the mode-N solve's launch plans for `nrhs` right-hand sides:
 * every launch of the solve is timed under a set of plan caps (CTAs per SM
 * aimed for, the row-slice floor, the widest column chunk), `reps` times
 * each, and the fastest caps are kept on `op` for that right-hand-side count
 * and precision (0 float64 slu_ulv_solve, 2 double-float
 * slu_ulv_solve_dfloat); later solves of that width use them.  Results do
 * not change: the caps move work between CTAs, never the order of terms.
 * knobs_out (host, may be NULL) receives 3 ints per launch (target, row
 * floor, column cap) for up to cap launches; *nlaunch the launch count.
 * The tuning is dropped when the operator is refactored.  No upstream
 * counterpart. */
int slu_ulv_autotune(slu_handle_t h, slu_hbs_t op, int nrhs, int precision, int reps,
                     int* knobs_out, int cap, int* nlaunch);

/* Geometry: L, N and per level (Nb, n, k, nu) into levels[4*L]; NNvec[L+1]
 * (ULVsparse.compute_ULV's NNvec).  Host pointers, any may be NULL. */
int slu_hbs_info(slu_hbs_t op, int* L, int* N, int* levels, long long* NNvec, int* nsamples);

/* Copies one stored factor of one level into dst (device pointer, count
 * doubles available).  what: 0 U, 1 V, 2 D, 3 Q, 4 W, 5 R (Rlist entry),
 * 6 Uu.  *count_out receives the number of doubles of the factor. */
int slu_hbs_export(slu_handle_t h, slu_hbs_t op, int what, int level, double* dst, size_t count,
                   size_t* count_out);
/* Bytes of stored factors: which = 0 HBS (U, V, D; HBSMAT.nbytes,
 * HBSnew.py:296-302), 1 solve factors. */
int slu_hbs_nbytes(slu_hbs_t op, int which, size_t* out);

/* Measured float64 FMA throughput of the current device: a register-only
 * kernel of independent FMA chains, 8 CTAs of 256 threads per SM, `iters`
 * FMAs per chain, timed with CUDA events (best of 3 after a warm-up launch).
 * *tflops_out = 2 * FMAs / time; *ms_out (may be NULL) the launch time.  The
 * ceiling of the roofline of the float64 step kernels.  No upstream
 * counterpart. */
int slu_fp64_peak(slu_handle_t h, int iters, double* tflops_out, double* ms_out);

/* ---------------------------------------------------------------- dense kernels
 * Batched LU with partial pivoting of nb matrices A_b (n x n, row-major, lda,
 * batch stride sA), in place; piv (device int32, n per matrix, stride sP)
 * receives LAPACK-style 0-based pivots.  info (device int32[nb], may be NULL)
 * is set to j+1 for a zero pivot.  Replaces scipy.linalg.lu_factor at
 * direct_solve/omsdirectsolve.py:84,96,211,333. */
int slu_lu_factor(slu_handle_t h, int n, double* A, int lda, long long sA, int* piv,
                  long long sP, int nb, int* info);
/* X_b <- A_b^{-1} X_b (trans = 0) or A_b^{-T} X_b from slu_lu_factor output;
 * X_b n x nrhs (ldx, stride sX).  Replaces scipy.linalg.lu_solve. */
int slu_lu_solve(slu_handle_t h, int trans, int n, const double* LU, int lda, long long sA,
                 const int* piv, long long sP, double* X, int ldx, long long sX, int nrhs, int nb);
/* C_b = alpha op(A_b) op(B_b) + beta C_b, strided batch (row-major). */
int slu_gemm_batched(slu_handle_t h, int transa, int transb, int M, int N, int K, double alpha,
                     const double* A, int lda, long long sA, const double* B, int ldb,
                     long long sB, double beta, double* C, int ldc, long long sC, int nb);

/* C = alpha A B + beta C (A M x K, B K x N, C M x N; row-major float64) on the
 * tcgen05 tensor cores as a split-BF16x3 product with float32 accumulation
 * (relative accuracy of a float32 GEMM).  For the mixed-precision path's
 * dense sampling and Schur products (matAssembly/matAssembler.py:115-116,
 * direct_solve/omsdirectsolve.py:316-324); the float64 path does not use it.
 * A wait timeout inside the kernel is reported by slu_sync as
 * SLU_ERR_TIMEOUT. */
int slu_gemm_split3(slu_handle_t h, int M, int N, int K, double alpha, const double* A, int lda,
                    const double* B, int ldb, double beta, double* C, int ldc);

/* ---------------------------------------------------------------- block tridiagonal
 * Dense red-black cyclic reduction (direct_solve/omsdirectsolve.py:177-333,
 * RedBlackSolver.factorize / solve) of nblk blocks of size m: SiM[i] couples
 * block i to i-1, SiP[i] to i+1, T[i] is the diagonal (all nblk*m*m
 * contiguous, device).  nblk must be a power of two (as upstream); the
 * caller pads.  SiM[0] and SiP[nblk-1] are ignored (treated as zero). */
int slu_rb_factor(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                  const double* T, slu_rb_t* out);
/* B (nblk*m x nrhs, ldb) <- solution, in place. */
int slu_rb_solve(slu_handle_t h, slu_rb_t rb, double* B, int ldb, int nrhs);
/* The red-black solve with its block products on the tcgen05 tensor cores
 * (split-BF16x3 GEMMs, float32-level accuracy; B in place): a fast
 * approximate solve for preconditioning an iterative solve of the exact
 * operator (no upstream counterpart).  Any factorisation of slu_rb_factor*. */
int slu_rb_solve_tc(slu_handle_t h, slu_rb_t rb, double* B, int ldb, int nrhs);
/* Periodic red-black (RedBlackSolver with cyclic=True,
 * direct_solve/omsdirectsolve.py:207-209, 249-250, 269-272, 315-327): as
 * slu_rb_factor, with SiM[0] coupling block 0 to block nblk-1 and
 * SiP[nblk-1] coupling the last block to block 0; nblk a power of two >= 2.
 * Solve with slu_rb_solve (and slu_rb_refine). */
int slu_rb_factor_cyclic(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                         const double* T, slu_rb_t* out);
/* Mixed-precision variant of slu_rb_factor: the Schur-complement products of
 * every level (SiM_i T^{-1} [SiM|SiP], omsdirectsolve.py:316-324) run on the
 * tcgen05 tensor cores (slu_gemm_split3); pivot-block LU factors and solves
 * stay float64.  Use with slu_rb_refine. */
int slu_rb_factor_mixed(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                        const double* T, slu_rb_t* out);
/* Iterative refinement of A x = b with the red-black factors and a float64
 * residual of the stored block-tridiagonal system (no upstream counterpart:
 * the mixed path's outer loop).  X (nblk*m x nrhs) receives the solution;
 * stops when every column has ||b - A x|| / ||b|| <= tol or after maxit
 * solves (then SLU_ERR_NOT_CONVERGED). */
int slu_rb_refine(slu_handle_t h, slu_rb_t rb, const double* B, int ldb, double* X, int ldx,
                  int nrhs, double tol, int maxit, int* iters_out, double* relres_out);
/* Frees the object's device memory stream-ordered (cudaFreeAsync on the
 * stream each buffer was allocated on): work that reads the object on any
 * other stream must have completed first (synchronise those streams). */
int slu_rb_destroy(slu_rb_t rb);

/* Slab source-target maps of the stencil discretisation, applied through
 * solves of the slab interiors (multislab/oms.py:96-125, oms.compute_stmaps:
 * S_J g = (A_ii^{-1} A_ib[:, J] g)[Ic]; the operators rkHBS assembly samples,
 * matAssembly/matAssembler.py:112-117).  nslabs double slabs
 * [x0[s], x0[s] + width] x [0,1] (nz = 0) or x [0,1]^2, each with nx grid
 * points across (odd) and ny (nz) along y (z), stencil of
 * solver/stencil/stencilSolver.py (c11 = c22 = c33 = 1, zeroth-order term
 * kappa^2 c(x); coef 0: c = 1, coef 1: c = 1 + 0.5 sin 2pi x sin 2pi y
 * sin 2pi z).  Interface vectors have m = (ny-2)(nz-2) rows per slab (z
 * fastest; m = ny-2 in 2-D), slab s at rows s*m .. s*m+m-1, ncols columns
 * (leading dimensions ldx / ldy), device float64.
 *   trans = 0: YL_s = S_l(s) XL_s + S_r(s) XR_s (XL or XR may be NULL);
 *   trans = 1: YL_s = S_l(s)^T XL_s, YR_s = S_r(s)^T XL_s (either output NULL).
 * The interior solves are Chebyshev iterations on -A_ii with the step count
 * fixed by its spectral bounds for relative accuracy tol (*steps_out);
 * SLU_ERR_ARG when -A_ii is not definite (slab too wide for kappa). */
int slu_slab_maps_apply(slu_handle_t h, int nx, int ny, int nz, double width, double kappa,
                        int coef, int nslabs, const double* x0, const double* XL,
                        const double* XR, int ldx, double* YL, double* YR, int ldy, int ncols,
                        int trans, double tol, int* steps_out);

/* Dense block Thomas (direct_solve/omsdirectsolve.py:48-141,
 * BlockTridiagonalSolver.factorize_helper / solve_helper) with the same block
 * conventions as slu_rb_factor; nblk >= 1, any count. */
int slu_thomas_factor(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                      const double* T, slu_rb_t* out);
int slu_thomas_solve(slu_handle_t h, slu_rb_t th, double* B, int ldb, int nrhs);

/* ------------------------------------------------ strong admissibility */
/* Strong-admissibility HBS operator (matAssembly/HBS/HBStorch_strong.py,
 * HBSMAT 908-1310): per level A = U B V^T + E with E block sparse on each
 * block's near field (its level adjacency plus itself).  N points in
 * nleaves uniform leaves of a tree with fac children per box (2 or 4);
 * perm_host[i] = caller row of tree position i (the tree's perm_leaf; NULL =
 * identity).  Replaces HBSMAT.__init__ (925-975). */
int slu_strong_create(slu_handle_t h, long long N, int nleaves, int fac,
                      const int64_t* perm_host, slu_strong_t* out);
/* Frees the object's device memory stream-ordered (cudaFreeAsync on the
 * stream each buffer was allocated on): work that reads the object on any
 * other stream must have completed first (synchronise those streams). */
int slu_strong_destroy(slu_strong_t op);
/* Compression from sketches (HBSMAT.construct / constructHBS, 1000-1107):
 * Om, Psi, Y = A Om', Z = A^T Psi' (device, N x s row-major, rows already
 * in tree order), rank rk.  nlev levels carry a far field (leaf first); for
 * level t, nb[t] blocks and the near fields as CSR (host arrays: nf_ptr has
 * nb[t] + 1 entries per level, offsets relative to that level's nf_idx
 * slice; each list holds the block itself and is symmetric).  Above the
 * last one the remaining operator is the dense base B = Y pinv(Om).
 * SLU_ERR_ARG when a near-field stack is rank deficient (min |R_ii| <= 1e-12
 * max |R_ii|) or wider than s, where upstream falls back to a truncated
 * SVD. */
int slu_strong_compress(slu_handle_t h, slu_strong_t op, int rk, int s, const double* Om,
                        const double* Psi, const double* Y, const double* Z, int nlev,
                        const int* nb, const int* nf_ptr, const int* nf_idx);
/* Y <- A X (trans = 0) or A^T X (HBSMAT._sweep / matmat / rmatmat,
 * 1232-1299); X, Y N x nrhs device float64 in the caller's ordering,
 * distinct. */
int slu_strong_apply(slu_handle_t h, slu_strong_t op, int trans, const double* X, int ldx,
                     double* Y, int ldy, int nrhs);
/* Queries: what 0 compressed levels (-1 before compression), 1 blocks,
 * 2 block size, 3 rank, 4 near-field tiles of `level`, 5 rows of the dense
 * base, 6 near-field stacks factored, 7 bytes of U, V, E (tiles and their
 * int64 coordinates) and the base (HBSMAT.nbytes, 993-998). */
int slu_strong_info(slu_strong_t op, int what, int level, long long* out);
/* Copies out a level's factors (host or device dst): what 0 U, 1 V
 * (Nb x b x r), 2 the tiles (nnz x b x b, sorted by (row, col)), 3 the tile
 * coordinates (int32 row, col pairs; host dst), 4 the dense base. */
int slu_strong_export(slu_handle_t h, slu_strong_t op, int what, int level, void* dst);

#ifdef __cplusplus
}
#endif
#endif /* SLABLU_H */

/*
 * lla_gb300.h — C ABI of the GB300 (sm_103a) SPD factor-and-solve library.
 *
 * The first group of entry points replaces, one for one, the trait methods of
 * linfa-linalg 0.2.1 on the SPD path (src/cholesky.rs, src/triangular.rs).
 * Matrices are passed as ndarray-style strided views of HOST memory:
 *     (ptr, rows, cols, row_stride, col_stride)
 * where element (i, j) lives at ptr[i*row_stride + j*col_stride] and the
 * strides are signed element counts, so reversed axes (negative strides) and
 * transposed (column-major) views are accepted exactly like the reference's
 * ArrayBase<S, Ix2> arguments.  Each call copies the view to the GPU,
 * computes there, and writes the result back into the same view.  There is no
 * CPU fallback: without a CUDA device every compute call returns
 * LLA_ERR_NO_DEVICE.
 *
 * Error precedence follows the reference exactly (see each declaration).
 * Every entry point returns the status code and, when `err` is non-NULL,
 * fills it with the variant's fields.
 *
 * The second group (lla_*_device, lla_plan_*, lla_batch_*, lla_serve_*) has no
 * counterpart in the reference: device-resident, mixed-precision, batched and
 * serving entry points built on the same kernels.
 */
#ifndef LLA_GB300_H
#define LLA_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------
 * 0..3 mirror linfa_linalg::LinalgError (src/lib.rs:33-60) for the variants
 * this path can raise; 16.. are device-side conditions the reference cannot
 * have. */
enum lla_status {
    LLA_OK = 0,
    LLA_NOT_SQUARE = 1,            /* LinalgError::NotSquare { rows, cols }      src/lib.rs:38 */
    LLA_NOT_POSITIVE_DEFINITE = 2, /* LinalgError::NotPositiveDefinite           src/lib.rs:44 */
    LLA_WRONG_ROWS = 3,            /* LinalgError::WrongRows { expected, actual } src/lib.rs:56 */
    LLA_ERR_CUDA = 16,             /* a CUDA runtime call failed (cuda_error set) */
    LLA_ERR_NO_MEMORY = 17,        /* device or pinned-host allocation failed */
    LLA_ERR_INVALID_ARG = 18,      /* NULL pointer, negative size, bad option */
    LLA_ERR_TIMEOUT = 19,          /* a bounded device wait gave up */
    LLA_ERR_NO_DEVICE = 20,        /* no CUDA device visible */
    LLA_ERR_NOT_CONVERGED = 21,    /* refinement stalled and fallback was disabled */
    LLA_ERR_BUSY = 22,             /* admission refused (serving loop at its HBM budget) */
    LLA_ERR_TOO_LARGE = 23         /* problem exceeds a fixed-size scratch area */
};

typedef struct lla_error {
    int32_t code;       /* one of lla_status */
    int32_t cuda_error; /* raw cudaError_t when code == LLA_ERR_CUDA */
    int64_t rows;       /* NotSquare.rows */
    int64_t cols;       /* NotSquare.cols */
    int64_t expected;   /* WrongRows.expected */
    int64_t actual;     /* WrongRows.actual */
    int64_t index;      /* NotPositiveDefinite: first row j whose pivot d <= 0 */
} lla_error;

/* UPLO (src/triangular.rs:8-13) */
enum lla_uplo { LLA_UPPER = 0, LLA_LOWER = 1 };

/* Factorisation algorithm used by the host-view entry points.
 *  LLA_ALGO_EXACT : the reference's own operation order (row-oriented
 *                   Cholesky-Banachiewicz sums, column-axpy substitution),
 *                   reorganised into blocked GPU kernels that keep every
 *                   per-element accumulation order; separate multiply and add
 *                   (no FMA), IEEE division and square root.  Results are
 *                   bit-identical to the reference.
 *  LLA_ALGO_FAST  : blocked right-looking FP64/FP32 with fused multiply-add
 *                   (normwise errors within 10*n*eps of the reference).
 *                   NotPositiveDefinite is still decided with the reference's
 *                   arithmetic: a failed or near-singular fast factorisation
 *                   is re-run in EXACT order before an error is returned.
 *  LLA_ALGO_AUTO  : EXACT for n <= 1024, FAST above (the default). */
enum lla_algo { LLA_ALGO_AUTO = 0, LLA_ALGO_EXACT = 1, LLA_ALGO_FAST = 2 };

/* Sets the process-wide algorithm for the host-view entry points; returns the
 * previous value, or -1 for an invalid argument. */
int lla_set_algorithm(int algo);
int lla_get_algorithm(void);

/* Number of CUDA devices (0 when none); never fails. */
int lla_device_count(void);
/* Library version string. */
const char *lla_version(void);
/* Human-readable text for a status code. */
const char *lla_status_string(int code);

/* ---- drop-in entry points (host views) ---------------------------------
 * f64 ("d") and f32 ("s") variants of each trait method.  `dirty` selects
 * cholesky_inplace_dirty (upper triangle left untouched) versus
 * cholesky_inplace (upper triangle zeroed). */

/* CholeskyInplace::cholesky_inplace_dirty / ::cholesky_inplace
 * (src/cholesky.rs:19,33,51-82; also backs cholesky_into[_dirty] :24-43 and
 * Cholesky::cholesky[_dirty] :86-115, whose to_owned() copy the caller makes).
 * Errors: NotSquare{rows,cols} (src/lib.rs:64-71), then NotPositiveDefinite
 * at the first row j with d <= 0 (src/cholesky.rs:69-71).  On
 * NotPositiveDefinite the view holds exactly what the reference leaves: rows
 * < j factored, row j's strict lower part written, the rest untouched. */
int lla_dcholesky_inplace(double *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                          int dirty, lla_error *err);
int lla_scholesky_inplace(float *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                          int dirty, lla_error *err);

/* SolveCInplace::solvec_inplace (src/cholesky.rs:122,136-144; backs
 * solvec_into :127-130 and SolveC::solvec :148-163).  `a` is left holding the
 * dirty factor, `b` holds X.  Errors: NotSquare(a), NotPositiveDefinite, then
 * WrongRows{expected=n, actual=b.rows} -- the row check runs after the
 * factorisation, so a mismatched b still leaves `a` factored, as in the
 * reference. */
int lla_dsolvec_inplace(double *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                        double *b, int64_t brows, int64_t bcols, int64_t brs, int64_t bcs,
                        lla_error *err);
int lla_ssolvec_inplace(float *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                        float *b, int64_t brows, int64_t bcols, int64_t brs, int64_t bcs,
                        lla_error *err);

/* InverseCInplace::invc_inplace (src/cholesky.rs:172,178-181; backs
 * InverseC::invc :186-199).  `out` is an n x n view that receives the
 * inverse; `a` is left holding the dirty factor. */
int lla_dinvc_inplace(double *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                      double *out, int64_t out_rs, int64_t out_cs, lla_error *err);
int lla_sinvc_inplace(float *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                      float *out, int64_t out_rs, int64_t out_cs, lla_error *err);

/* SolveTriangularInplace::solve_triangular_inplace (src/triangular.rs:149,
 * 161-168; backs solve_triangular_into :152-155 and
 * SolveTriangular::solve_triangular :172-187).  Only the `uplo` triangle and
 * the diagonal of `a` are read.  Errors: NotSquare(a), then WrongRows.  A zero
 * diagonal is not an error (inf/NaN, as in the reference). */
int lla_dsolve_triangular_inplace(const double *a, int64_t rows, int64_t cols, int64_t rs,
                                  int64_t cs, double *b, int64_t brows, int64_t bcols,
                                  int64_t brs, int64_t bcs, int uplo, lla_error *err);
int lla_ssolve_triangular_inplace(const float *a, int64_t rows, int64_t cols, int64_t rs,
                                  int64_t cs, float *b, int64_t brows, int64_t bcols,
                                  int64_t brs, int64_t bcs, int uplo, lla_error *err);

/* solve_triangular_system with a caller-supplied diagonal
 * (src/triangular.rs:133-144): the closure `diag_fn(i)` becomes the array
 * diag[0..n).  This is the form QR's solve uses (src/qr.rs:145-150,172-177
 * pass |R[i,i]|). */
int lla_dsolve_triangular_diag(const double *a, int64_t rows, int64_t cols, int64_t rs,
                               int64_t cs, const double *diag, double *b, int64_t brows,
                               int64_t bcols, int64_t brs, int64_t bcs, int uplo,
                               lla_error *err);
int lla_ssolve_triangular_diag(const float *a, int64_t rows, int64_t cols, int64_t rs,
                               int64_t cs, const float *diag, float *b, int64_t brows,
                               int64_t bcols, int64_t brs, int64_t bcs, int uplo,
                               lla_error *err);

/* IntoTriangular::triangular_inplace (src/triangular.rs:19,37-53). */
int lla_dtriangular_inplace(double *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                            int uplo, lla_error *err);
int lla_striangular_inplace(float *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                            int uplo, lla_error *err);

/* Triangular::is_triangular (src/triangular.rs:59,67-90): *result = 1/0.
 * A non-square view gives 0, not an error, as in the reference. */
int lla_dis_triangular(const double *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                       int uplo, int *result, lla_error *err);
int lla_sis_triangular(const float *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                       int uplo, int *result, lla_error *err);

/* ---- LOBPCG's Cholesky-QR (callers of the path) ----
 * lla_?orthonormalize replaces `orthonormalize` (src/lobpcg/algorithm.rs:81-96):
 * G = V^T V (n x k view v, read), L = cholesky_into(G) written to the k x k view
 * l (lower factor, upper part zeroed), U = V L^-T written to the n x k view u
 * (solve_triangular_into(V^T, Lower), transposed back).  Returns
 * LLA_ERR_NOT_POSITIVE_DEFINITE (index = failing row of G, u and l untouched)
 * when G is not positive definite; LLA_ERR_INVALID_ARG for mismatched views.
 * The Cholesky of G and the substitution follow the reference's order (EXACT
 * for k <= 1024 in LLA_ALGO_AUTO); G itself is summed in fixed row chunks.
 * lla_?apply_constraints replaces `apply_constraints` (:63-76): v (n x k) -=
 * y (n x ky) U with lyy U = y^T v (lyy: ky x ky lower factor, e.g. from
 * lla_?cholesky_inplace). */
int lla_dorthonormalize(const double *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, double *u,
                        int64_t urows, int64_t ucols, int64_t urs, int64_t ucs, double *l, int64_t lrows,
                        int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err);
int lla_sorthonormalize(const float *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, float *u,
                        int64_t urows, int64_t ucols, int64_t urs, int64_t ucs, float *l, int64_t lrows,
                        int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err);
int lla_dapply_constraints(double *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, const double *y,
                           int64_t yrows, int64_t ycols, int64_t yrs, int64_t ycs, const double *lyy,
                           int64_t lrows, int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err);
int lla_sapply_constraints(float *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, const float *y,
                           int64_t yrows, int64_t ycols, int64_t yrs, int64_t ycs, const float *lyy,
                           int64_t lrows, int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err);

/* ---- device-resident entry points (no counterpart in the reference) ----
 * Matrices are column-major device arrays with a leading dimension; `stream`
 * is a cudaStream_t (NULL = the legacy default stream).  Calls are
 * asynchronous unless stated; statuses that need device results (pivot
 * failure) are written to device memory `d_info` (int64: -1 = success, else
 * the failing row) so that calls can be captured in CUDA graphs. */

/* In-place Cholesky of the lower triangle of the n x n column-major matrix
 * dA (leading dimension ld >= n).  algo: LLA_ALGO_EXACT or LLA_ALGO_FAST.
 * Uses library-owned device workspace (grown on demand). */
int lla_dpotrf_device(double *dA, int64_t n, int64_t ld, int algo, int64_t *d_info,
                      void *stream, lla_error *err);
int lla_spotrf_device(float *dA, int64_t n, int64_t ld, int algo, int64_t *d_info,
                      void *stream, lla_error *err);

/* Triangular solve with the lower-triangular factor L (column-major, ld):
 * trans = 0 solves L X = B, trans = 1 solves L^T X = B; dB (n x m, ldb) is
 * overwritten with X.  algo as above (EXACT follows the reference's
 * substitution order).  Asynchronous: a bounded device wait that gave up
 * (X then not valid) is recorded in the calling thread's status word, which
 * lla_device_status reports. */
int lla_dtrsm_device(const double *dL, int64_t n, int64_t ld, int trans, double *dB, int64_t m,
                     int64_t ldb, int algo, void *stream, lla_error *err);
int lla_strsm_device(const float *dL, int64_t n, int64_t ld, int trans, float *dB, int64_t m,
                     int64_t ldb, int algo, void *stream, lla_error *err);

/* IntoTriangular::triangular_inplace (src/triangular.rs:37-53) on a
 * device-resident column-major matrix (rows x cols, ld): uplo = LLA_UPPER
 * zeroes the strict lower part, LLA_LOWER the strict upper part.  Errors:
 * NotSquare{rows, cols} (src/lib.rs:64-71).  Asynchronous on `stream`. */
int lla_dtriangular_device(double *dA, int64_t rows, int64_t cols, int64_t ld, int uplo, void *stream,
                           lla_error *err);
int lla_striangular_device(float *dA, int64_t rows, int64_t cols, int64_t ld, int uplo, void *stream,
                           lla_error *err);
/* Triangular::is_triangular (src/triangular.rs:67-90) on a device-resident
 * column-major matrix: *d_result (device int) receives 1 when every entry
 * outside the uplo triangle is zero, else 0; a non-square matrix gives 0 (not
 * an error, as in the reference).  Asynchronous on `stream`. */
int lla_dis_triangular_device(const double *dA, int64_t rows, int64_t cols, int64_t ld, int uplo,
                              int *d_result, void *stream, lla_error *err);
int lla_sis_triangular_device(const float *dA, int64_t rows, int64_t cols, int64_t ld, int uplo,
                              int *d_result, void *stream, lla_error *err);

/* Synchronises `stream` and reports whether a bounded device wait of an
 * asynchronous call made on this host thread (lla_?trsm_device) gave up since
 * the last query: LLA_ERR_TIMEOUT (the X of such a call is not valid) or
 * LLA_OK; the record is cleared.  No counterpart in the reference. */
int lla_device_status(void *stream, lla_error *err);

/* Allocation-free variant of lla_dtrsm_device (same arguments and results).
 * It has no counterpart in the reference.  It exists for callers that must
 * not allocate device memory (inside another allocator's callback, under a
 * host framework that owns all device memory, in loops where an allocation
 * would synchronise): its scratch is a fixed device array inside the library,
 * so it never calls cudaMalloc/cudaFree.  Limit: ceil(n/32) * ceil(m/min(8,m))
 * <= 65536 (e.g. n <= 16384 with m <= 1024); larger problems return
 * LLA_ERR_TOO_LARGE.  The first call on each device looks up the array's
 * device address (make it before any stream capture).  All calls share the
 * array: calls that overlap on the GPU race. */
int lla_dtrsm_device_noalloc(const double *dL, int64_t n, int64_t ld, int trans, double *dB,
                             int64_t m, int64_t ldb, int algo, void *stream, lla_error *err);
/* Synchronises `stream` and reports LLA_ERR_TIMEOUT when a bounded wait of an
 * lla_dtrsm_device_noalloc call on the current device gave up since the last
 * query (that call's X is not valid), else LLA_OK; clears the record.  The
 * record lives in the same fixed array, so it is per device, shared by all
 * host threads; this call allocates nothing either.  No counterpart in the
 * reference. */
int lla_dtrsm_device_noalloc_status(void *stream, lla_error *err);


/* ---- mixed-precision refined solve (no counterpart in the reference) -----
 * Solves A X = B for SPD A (only its lower triangle is read, as in the
 * reference) by a low-precision Cholesky of the symmetrically equilibrated
 * matrix (exact power-of-two scaling), FP64 iterative refinement to a normwise
 * backward error max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf +
 * ||b_j||_inf) <= tol, and a fallback to the plain FP64 factorisation when the
 * low-precision factorisation breaks down or the refinement stalls.  The FP64
 * fallback decides NotPositiveDefinite: a failed or near-singular
 * (pivot / a_kk < 1e-10) FMA-order factorisation is re-run in the reference's
 * own operation order (src/cholesky.rs:51-76), whose verdict and failing row
 * are returned, as the host-view entry points do. */
enum lla_update {
    LLA_UPDATE_FP32 = 0,    /* FP32 SIMT trailing updates */
    LLA_UPDATE_BF16 = 1,    /* tcgen05: one BF16 term per operand, FP32 accumulation */
    LLA_UPDATE_BF16X3 = 3,  /* tcgen05: hi/lo BF16 split, three products */
    LLA_UPDATE_BF16X6 = 6,  /* tcgen05: three-level BF16 split, six products */
    LLA_UPDATE_FP16 = 11,   /* tcgen05: one FP16 term */
    LLA_UPDATE_FP16X3 = 13  /* tcgen05: hi/lo FP16 split, three products */
};

/* How the refinement computes r = b - A x:
 *  LLA_RESIDUAL_FP64          FP64 arithmetic on the FP64 MMA pipe (default);
 *  LLA_RESIDUAL_EXACT_SLICES  the same quantity on the BF16 tensor cores: A and x
 *                             are cut into 8 exact 7-bit integer slices with
 *                             power-of-two row / column scales, the slice
 *                             products are summed exactly (integers below 2^24 in
 *                             FP32, drained into 64-bit integers) and combined in
 *                             FP64 -- an error bound like an FP64 product's. */
enum lla_residual { LLA_RESIDUAL_FP64 = 0, LLA_RESIDUAL_EXACT_SLICES = 1 };

/* The refinement's FP32 triangular solves (with inverted 64 x 64 diagonal blocks):
 *  LLA_SUB_LOOKBACK  one CTA per (block, column chunk), blocks handed from CTA
 *                    to CTA through epoch-tagged words (default);
 *  LLA_SUB_CHAIN     one CTA per column chunk walks every block and keeps the
 *                    two previous blocks on chip; helper CTAs form the coupling
 *                    sums with earlier blocks in groups (measured slower on
 *                    GB300: 10.7 vs 8.2 ms of substitutions per n=16384 solve). */
enum lla_substitution { LLA_SUB_AUTO = 0, LLA_SUB_CHAIN = 1, LLA_SUB_LOOKBACK = 2 };

typedef struct lla_refine_opts {
    int32_t update;      /* lla_update (default LLA_UPDATE_BF16X6) */
    int32_t max_iters;   /* refinement iterations before giving up (default 30) */
    double tol;          /* target normwise backward error (default 1e-13) */
    int32_t equilibrate; /* 1: symmetric power-of-two scaling (default) */
    int32_t fallback;    /* 1: plain FP64 on breakdown or stall (default); 0: LLA_ERR_NOT_CONVERGED */
    int32_t update_epilogue; /* tensor-core update epilogue: 1 register loads and stores, 2 FP32 tile
                                staged through shared memory by TMA (16-byte rows of the matrix
                                needed); 0 default: TMA for the one- and two-term forms */
    int32_t residual;    /* lla_residual (default LLA_RESIDUAL_FP64) */
    int32_t substitution;    /* lla_substitution: form of the FP32 substitutions (0: default) */
    int32_t update_kchunk;   /* K-chunk of the tensor-core update's operand stages: 64 or 32 (0: default) */
} lla_refine_opts;

typedef struct lla_refine_report {
    int32_t update;          /* update form used */
    int32_t iterations;      /* residual evaluations */
    int32_t converged;       /* 1 when the refinement reached tol */
    int32_t fell_back;       /* 1 when the plain FP64 path produced X */
    int32_t factor_failed;   /* 1 when the low-precision factorisation broke down */
    int32_t schedule;        /* schedule used: update K-chunk << 8 | update epilogue << 4 | substitution */
    double backward_error;   /* final normwise backward error (max over columns) */
    double backward_error0;  /* after the first low-precision solve */
    double ms_factor, ms_refine, ms_fallback, ms_total;
} lla_refine_report;

void lla_refine_opts_default(lla_refine_opts *opts);

/* Device-resident form: dA (n x n, column-major, lda), dB (n x m, ldb) are
 * read; dX (n x m, ldx) receives X.  Synchronous on `stream` (the refinement
 * reads the backward error on the host every iteration). */
int lla_dposv_refined_device(const double *dA, int64_t n, int64_t lda, const double *dB, int64_t m,
                             int64_t ldb, double *dX, int64_t ldx, const lla_refine_opts *opts,
                             lla_refine_report *report, void *stream, lla_error *err);

/* Per-shape autotuner of the refined solve's schedule (no counterpart in the
 * reference): times lla_dposv_refined_device on this system for each candidate
 * of the tensor-core update's epilogue and K-chunk (registers / 64, registers /
 * 32, TMA-staged / 32) and of the substitution form (look-back, chain), keeps
 * the fastest that converges without fallback, records it in the autotune
 * cache (LLA_AUTOTUNE_CACHE, default ~/.cache/lla_gb300_autotune.txt) under the
 * shape key (n and m rounded up to powers of two, update form, residual) and
 * writes it into *opts.  Later solves whose opts leave update_kchunk,
 * update_epilogue and substitution at 0 take the cached schedule for their
 * shape (lla_refine_report.schedule says which ran).  dX receives X; errors as
 * lla_dposv_refined_device. */
int lla_refine_autotune(const double *dA, int64_t n, int64_t lda, const double *dB, int64_t m, int64_t ldb,
                        double *dX, int64_t ldx, lla_refine_opts *opts, double *best_ms, void *stream,
                        lla_error *err);

/* R = B - A_sym X (A_sym: the symmetric matrix defined by the lower triangle
 * of dA), column-major device arrays, by the given lla_residual method;
 * synchronous on `stream`. */
int lla_dresidual_device(const double *dA, int64_t n, int64_t lda, const double *dX, int64_t ldx,
                         const double *dB, int64_t ldb, double *dR, int64_t ldr, int64_t m,
                         int method, void *stream, lla_error *err);

/* Host-view form (SolveC-like): `a` is read only; `b` (n x m) is overwritten
 * with X.  Errors: NotSquare(a), WrongRows(b), NotPositiveDefinite (decided by
 * the FP64 fallback). */
int lla_dposv_refined(const double *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,
                      double *b, int64_t brows, int64_t bcols, int64_t brs, int64_t bcs,
                      const lla_refine_opts *opts, lla_refine_report *report, lla_error *err);

/* The low-precision factorisation on its own: in-place Cholesky of the lower
 * triangle of an FP32 SPD matrix (column-major, ld) with FP32 diagonal blocks
 * and panels and the trailing updates in the given lla_update form.  *d_info
 * (device) receives -1, or the first row of the panel where a non-positive
 * pivot appeared.  Synchronises `stream` for the tensor-core forms (their
 * bounded waits report LLA_ERR_TIMEOUT). */
int lla_spotrf_mixed_device(float *dA, int64_t n, int64_t ld, int update, int64_t *d_info,
                            void *stream, lla_error *err);

/* ---- batched solves of many small SPD systems (no counterpart in the
 * reference; one persistent launch for the whole batch) --------------------
 * Systems of order n_i <= 256 with m_i <= 8 right-hand sides.  The plan fixes
 * where each system lives in two device pools the caller fills: A_i
 * (n_i x n_i, column-major, ld = n_i) at A-pool element offset a_off[i], B_i
 * (n_i x m_i, ld = n_i) at b_off[i].  A solve factors every A_i in place (L in
 * the lower triangle) and overwrites every B_i with X_i; d_info[i] (device
 * int32) receives -1 or the first row with a non-positive pivot of system i.
 * Plain FP64 (or FP32) arithmetic with FMA, as the single-matrix FAST path. */
typedef struct lla_batch_plan lla_batch_plan;

/* elem_bytes: 8 (f64) or 4 (f32).  LLA_ERR_TOO_LARGE for n_i > 256 or
 * m_i > 8.  Picks up a cached launch shape for this batch's size histogram
 * when the autotune cache has one. */
int lla_batch_plan_create(int64_t count, const int32_t *n, const int32_t *m, int elem_bytes,
                          lla_batch_plan **plan, lla_error *err);
void lla_batch_plan_destroy(lla_batch_plan *plan);
/* Pool sizes in elements, per-system offsets (arrays of `count`, may be NULL),
 * the launch shape in use and the batch's flop count. */
int lla_batch_plan_info(const lla_batch_plan *plan, int64_t *a_elems, int64_t *b_elems,
                        int64_t *a_off, int64_t *b_off, int *ctas_per_sm, int *threads,
                        double *flops);
/* f64 plans: refined = 1 solves every system through an FP32 factorisation
 * with FP64 iterative refinement inside the same persistent launch (one CTA
 * per system; A_i is then READ ONLY and B_i receives X_i; a system whose FP32
 * factorisation breaks down or whose backward error stays above 10 n eps is
 * solved again by the plain FP64 routine, whose failing row d_info[i]
 * reports); refined = 0 restores the plain FP64 solve (A factored in place).
 * LLA_ERR_INVALID_ARG for f32 plans. */
int lla_batch_set_refined(lla_batch_plan *plan, int refined, lla_error *err);
/* Overrides the launch shape (CTAs per SM 1..8, threads 128 or 256). */
int lla_batch_set_shape(lla_batch_plan *plan, int ctas_per_sm, int threads);
/* One persistent launch on `stream` (asynchronous). */
int lla_dbatch_posv_device(lla_batch_plan *plan, double *dA, double *dB, int32_t *d_info,
                           void *stream, lla_error *err);
int lla_sbatch_posv_device(lla_batch_plan *plan, float *dA, float *dB, int32_t *d_info,
                           void *stream, lla_error *err);
/* The same launch replayed from a CUDA graph instantiated on first use for
 * these pools and stream (either element type). */
int lla_batch_posv_graph(lla_batch_plan *plan, void *dA, void *dB, int32_t *d_info, void *stream,
                         lla_error *err);
/* Times the launch shapes on this batch (restoring the pools between trials),
 * keeps the fastest and records it in the autotune cache file
 * (LLA_AUTOTUNE_CACHE or ~/.cache/lla_gb300_autotune.txt). */
int lla_batch_autotune(lla_batch_plan *plan, void *dA, void *dB, int32_t *d_info, void *stream,
                       double *best_ms, lla_error *err);

/* ---- serving loop (no counterpart in the reference) ----------------------
 * Requests arrive while others run.  Each is admitted against an HBM budget
 * (first come, first served).  Small systems (n <= small_n, <= 8 RHS) go, as
 * soon as they are admitted, to a device-resident loop: persistent CTAs that
 * claim requests from a ring in mapped host memory and solve each one in
 * place (one CTA per request, the batched kernel's arithmetic), so requests
 * that arrive while others are on the GPU join the running loop; its CTAs
 * return after batch_window_us without work and the host relaunches it on the
 * next request.  Large requests run concurrently on `slots` streams
 * (mixed-precision refined solve for f64, FP32 factor + FP64 refinement for
 * f32, plain FP64 factor when the factor is to be kept); factors can stay on
 * the device for repeat right-hand sides; every request records submit /
 * admit / start / done times.  All data is device-resident (column-major); B
 * is overwritten with X. */
enum lla_request_kind {
    LLA_REQ_SOLVE = 0,   /* A X = B for SPD A (lower triangle read) */
    LLA_REQ_RESOLVE = 1, /* repeat right-hand sides on a kept factor (factor_handle) */
    LLA_REQ_TRSM = 2     /* L X = B with the lower-triangular L given in A */
};
enum lla_result_path {
    LLA_PATH_BATCHED = 1, LLA_PATH_MIXED = 2, LLA_PATH_FP64 = 3, LLA_PATH_KEPT_FACTOR = 4,
    LLA_PATH_TRSM = 5
};

typedef struct lla_serve_opts {
    double hbm_budget_bytes; /* admission budget (default 40e9) */
    int32_t slots;           /* concurrent large-request streams (default 6) */
    int32_t small_n;         /* largest order sent to the device-resident loop (default 256) */
    int32_t batch_max;       /* most small requests in flight in the loop's ring (default and limit 1024) */
    int32_t device_ctas;     /* persistent CTAs of the device loop (0: an eighth of the SMs, at least 8) */
    double batch_window_us;  /* idle time after which the loop's CTAs return (default 2000) */
} lla_serve_opts;

typedef struct lla_request {
    int32_t kind;          /* lla_request_kind */
    int32_t dtype;         /* 8: f64, 4: f32 */
    int64_t n, m;
    const void *A;         /* device, n x n, leading dimension lda */
    int64_t lda;
    void *B;               /* device, n x m, leading dimension ldb; receives X */
    int64_t ldb;
    double tol;            /* target backward error (0: 1e-13 for f64, 1e-6 for f32) */
    int64_t factor_handle; /* LLA_REQ_RESOLVE: handle from an earlier result */
    int32_t keep_factor;   /* LLA_REQ_SOLVE (f64): keep the factor, return its handle */
    int32_t reserved;
    uint64_t user_tag;     /* returned in the result */
} lla_request;

typedef struct lla_result {
    uint64_t user_tag;
    int32_t status;        /* lla_status of this request */
    int32_t path;          /* lla_result_path */
    int64_t factor_handle; /* kept factor (keep_factor) */
    double backward_error; /* refined solves: final normwise backward error */
    int32_t iterations;    /* refined solves: residual evaluations */
    int32_t reserved;
    double t_submit_us, t_admit_us, t_start_us, t_done_us; /* since server creation */
} lla_result;

typedef struct lla_server_stats {
    double bytes_in_use, bytes_peak;
    int64_t queued, running, submitted, completed, kept_factors;
    int64_t device_loop_launches; /* launches of the device-resident loop so far */
} lla_server_stats;

typedef struct lla_server lla_server;

void lla_serve_opts_default(lla_serve_opts *opts);
int lla_server_create(const lla_serve_opts *opts, lla_server **server, lla_error *err);
/* Thread-safe; LLA_ERR_BUSY when the request alone exceeds the budget. */
int lla_server_submit(lla_server *server, const lla_request *req, lla_error *err);
/* Non-blocking: copies up to `max` finished results. */
int lla_server_poll(lla_server *server, lla_result *out, int max, int *n_out);
/* Waits until every submitted request has finished (LLA_ERR_TIMEOUT otherwise). */
int lla_server_drain(lla_server *server, double timeout_s);
int lla_server_release_factor(lla_server *server, int64_t handle);
int lla_server_get_stats(lla_server *server, lla_server_stats *out);
void lla_server_destroy(lla_server *server);

/* ---- diagnostics (no counterpart in the reference) ----------------------
 * Launch accounting and per-kernel CUDA-event timing used by the benchmark:
 * while profiling is on, every kernel launch is bracketed by an event pair on
 * its stream; lla_profile_stop() synchronises and sums the durations and the
 * algorithmic work (flops, or bytes for data-movement kernels) per kernel
 * name ("potrf_fast_update", "trsm", ...). */
int64_t lla_kernel_launches(void);
void lla_profile_start(void);
int lla_profile_stop(void);
int lla_profile_query(const char *kernel, double *total_ms, int64_t *launches, double *work);
const char *lla_profile_kernel_name(int index);
/* Measured arithmetic peak in TFLOP/s of this GPU: which = 0 FP64 tensor pipe
 * (mma m16n8k16 .f64), 1 FP64 FMA, 2 FP32 FMA; negative on error. */
double lla_measure_peak_tflops(int which);
/* Failure injection for tests of the timeout reporting: the next
 * triangular-solve launch in this process (lla_?trsm_device,
 * lla_dtrsm_device_noalloc or a host-view solve) loses its first block --
 * never solved, never published -- and its bounded waits give up after
 * `spin_limit` polls (0: the default limit of a few seconds), so the call
 * reports LLA_ERR_TIMEOUT without faulting the device.  One shot. */
int lla_debug_inject_lost_handoff(int64_t spin_limit);

#ifdef __cplusplus
}
#endif

#endif /* LLA_GB300_H */

// lla_mixed.h -- internal declarations of the mixed-precision path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lla_gb300.h"

namespace lla {

struct Ctx;

// Low-precision Cholesky of the equilibrated FP32 matrix L (lower triangle,
// column-major, ld) in place, with the trailing-update form opts.update.
// *info (device) receives the first non-positive pivot's row or stays -1.
int lowp_factor_launch(float *L, int64_t n, int64_t ld, const lla_refine_opts &opts, int64_t *info,
                       float *diag0, double *min_ratio, Ctx *c, cudaStream_t st);

// Power-of-two scaling s, W = fp32(S A S) (lower), the row sums of |A| and
// ||A||_inf in one pass over A; rowmax (may be NULL): the row maxima of |A| too.
// part: sym_part_doubles(n) doubles of per-tile partial sums.
size_t sym_part_doubles(int64_t n);
int equilibrate_launch(const double *A, int64_t lda, int64_t n, bool scale, double *s, float *W,
                       int64_t ldw, double *rowsum, double *anorm, double *rowmax, double *part, int *bad,
                       cudaStream_t st, int64_t *info = nullptr);

// Refinement control (lla_mixed.cu): kernels that take `state` return at once
// when it is non-NULL and nonzero (the refinement has finished or failed).
__device__ __forceinline__ bool refine_done(const int *state) {
    return state != nullptr && *(volatile const int *)state != 0;
}
// Levels of the exact-slice residual of the current refinement iteration.
// The residual only has to resolve the error that is left.  Dropping levels
// d >= S leaves an error of about (S+1) 2^-7S per product relative to the row
// and column scales, ~2^-7S+4 sqrt(n) summed over a row: for S = 6 about
// 2e-10 and for S = 7 about 2e-12 of the scales at n = 16384, one to two
// orders below the backward error they are used at.  So: all eight for the
// first residual (the first solve may already be accurate), six while the
// previous backward error is above 1e-9, seven while it is above 1e-11,
// eight after; the convergence test accepts only a residual formed with all
// eight (refine_check_kernel evaluates the same rule).  Outside a refinement
// (state == nullptr) always eight.  state points at words + 4 of the
// refinement control block: [0] state, [1] iterations done, and the double
// after it is the previous iteration's backward error.
constexpr double kOzEta6 = 1e-9, kOzEta7 = 1e-11;
__device__ __forceinline__ int refine_levels(const int *state) {
    if (state == nullptr) return 8;
    const int done = *(volatile const int *)(state + 1);
    const double eta_prev = *(volatile const double *)((const double *)state + 1);
    if (done == 0 || eta_prev <= kOzEta7) return 8;
    return eta_prev <= kOzEta6 ? 7 : 6;  // (a NaN backward error stops the refinement first)
}
int colmax_launch(const double *M, int64_t ld, int64_t n, int64_t m, double *colmax, cudaStream_t st);
// R = B - A_sym X in FP64; P: workspace of residual_splits(n, m) * n * m
// doubles for the split-K partials (NULL: no split).
int residual_splits(int64_t n, int64_t m);
int residual_launch(const double *A, int64_t lda, int64_t n, const double *X, int64_t ldx,
                    const double *B, int64_t ldb, double *R, int64_t ldr, int64_t m, double *colmax_r,
                    double *P, cudaStream_t st, const int *state = nullptr);

// FP32 substitutions with inverted 64 x 64 diagonal blocks (lla_trsm_inv.cu).
// W: diag_inverse_floats(n) floats (inverses and the four coupling sets);
// stage: trsm_inv_stage_words(n, m) 64-bit words, zeroed when allocated;
// epoch: nonzero and different for every launch on the same stage array.
size_t diag_inverse_floats(int64_t n);
size_t trsm_inv_ws_ints(int64_t n, int64_t m);
size_t trsm_inv_stage_words(int64_t n, int64_t m);
int diag_inverse_launch(const float *L, int64_t ld, int64_t n, float *W, cudaStream_t st);
int trsm_inv_launch(const float *L, int64_t ld, const float *W, int64_t n, float *B, int64_t ldb,
                    int64_t m, int trans, unsigned long long *stage, unsigned epoch, int *ws, int *err_word,
                    cudaStream_t st, const int *state = nullptr);
// The chain form of the same substitutions (one CTA per column chunk walks the
// blocks; helper CTAs form the coupling sums): stage holds
// trsm_chain_stage_words(n, m) 64-bit words, zeroed when allocated.
size_t trsm_chain_stage_words(int64_t n, int64_t m);
int trsm_chain_launch(const float *L, int64_t ld, const float *W, int64_t n, float *B, int64_t ldb,
                      int64_t m, int trans, unsigned long long *stage, unsigned epoch, int *ws, int *err_word,
                      cudaStream_t st, const int *state = nullptr);

// Exact-slice (tensor-core) residual: workspace size, once-per-solve slicing
// of A, and the per-iteration residual (colmax_x: column maxima of |X|).
// rowmax_ready: the row maxima at oz_rowmax(ws, n, m) were already formed
// (equilibrate_launch); otherwise oz_prepare forms them.
size_t oz_workspace_bytes(int64_t n, int64_t m);
double *oz_rowmax(void *ws, int64_t n, int64_t m);
int oz_prepare(const double *A, int64_t lda, int64_t n, int64_t m, void *ws, bool rowmax_ready, cudaStream_t st);
int oz_residual_launch(const double *X, int64_t ldx, const double *B, int64_t ldb, double *R, int64_t ldr,
                       int64_t n, int64_t m, const double *colmax_x, double *colmax_r, void *ws,
                       int *err_word, cudaStream_t st, const int *state = nullptr);

}  // namespace lla

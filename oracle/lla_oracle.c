/*
 * lla_oracle.c — CPU restatement of linfa-linalg 0.2.1's SPD factor-and-solve
 * path.  TEST INFRASTRUCTURE ONLY: the checker that the GPU library is
 * compared against, and the single-threaded CPU baseline timed beside it.
 * Nothing in the shipped library links, loads or calls this file.
 *
 * Parity pin: the reference is Rust and cannot be compiled in this image (no
 * cargo/rustc), so this restatement is pinned against the reference's own
 * known-answer tests and fixtures (src/cholesky.rs:208-277,
 * src/triangular.rs:248-298, tests/cholesky.rs:87-95,
 * tests/triangular.rs:49-180), extracted verbatim into tests/golden/ by
 * tests/golden/make_golden.py, and cross-checked against LAPACK (scipy).
 *
 * Arithmetic faithfulness: every loop nest, bound and operation order below
 * follows the cited Rust lines.  The file must be compiled with
 * -ffp-contract=off (no FMA contraction, which Rust/LLVM never does either)
 * and without -ffast-math, so each `+`, `*`, `/` and sqrt is one IEEE
 * round-to-nearest operation, exactly as in the reference.  Under these
 * conditions the results are bit-identical to the reference's.
 *
 * ndarray 0.16 (Cargo.toml:16, not vendored in the reference tree) supplies
 * the element access and `scaled_add`; its published behaviour is restated
 * here: `y.scaled_add(alpha, x)` performs `y[e] = y[e] + alpha * x[e]`
 * elementwise (one multiply, one add, no reduction), and views are
 * (ptr, shape, signed strides) in elements.
 *
 * Views: element (i, j) of a matrix is p[i*rs + j*cs]; strides are signed.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/lla_gb300.h"

static void set_ok(lla_error *e) {
    if (e) memset(e, 0, sizeof(*e));
}

/* check_square (src/lib.rs:64-71) */
static int check_square(int64_t rows, int64_t cols, lla_error *e) {
    if (rows != cols) {
        if (e) {
            memset(e, 0, sizeof(*e));
            e->code = LLA_NOT_SQUARE;
            e->rows = rows;
            e->cols = cols;
        }
        return LLA_NOT_SQUARE;
    }
    return LLA_OK;
}

#define AT(p, i, j, rs, cs) (p)[(int64_t)(i) * (rs) + (int64_t)(j) * (cs)]

/* One instantiation per element type (f64 "d", f32 "s").  Rust evaluates f32
 * arithmetic in f32 (no promotion); C does too on the targets we build for
 * (FLT_EVAL_METHOD == 0: x86-64 SSE, AArch64). */
#define DEFINE_ORACLE(T, P, SQRT)                                                              \
                                                                                               \
    /* CholeskyInplace::cholesky_inplace_dirty (src/cholesky.rs:51-76) */                      \
    int ora_##P##cholesky_inplace_dirty(T *a, int64_t rows, int64_t cols, int64_t rs,          \
                                        int64_t cs, lla_error *e) {                            \
        set_ok(e);                                                                             \
        if (check_square(rows, cols, e)) return LLA_NOT_SQUARE;                                \
        const int64_t n = rows;                                                                \
        for (int64_t j = 0; j < n; ++j) {                                                      \
            T d = (T)0;                                                                        \
            for (int64_t k = 0; k < j; ++k) {                                                  \
                T s = (T)0;                                                                    \
                for (int64_t i = 0; i < k; ++i) s += AT(a, k, i, rs, cs) * AT(a, j, i, rs, cs); \
                s = (AT(a, j, k, rs, cs) - s) / AT(a, k, k, rs, cs);                           \
                AT(a, j, k, rs, cs) = s;                                                       \
                d += s * s;                                                                    \
            }                                                                                  \
            d = AT(a, j, j, rs, cs) - d;                                                       \
            /* `d <= 0` is false for NaN, so NaN propagates without error (:69) */             \
            if (d <= (T)0) {                                                                   \
                if (e) {                                                                       \
                    e->code = LLA_NOT_POSITIVE_DEFINITE;                                       \
                    e->index = j;                                                              \
                }                                                                              \
                return LLA_NOT_POSITIVE_DEFINITE;                                              \
            }                                                                                  \
            AT(a, j, j, rs, cs) = SQRT(d);                                                     \
        }                                                                                      \
        return LLA_OK;                                                                         \
    }                                                                                          \
                                                                                               \
    /* IntoTriangular::triangular_inplace (src/triangular.rs:37-53) */                         \
    int ora_##P##triangular_inplace(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,  \
                                    int uplo, lla_error *e) {                                  \
        set_ok(e);                                                                             \
        if (check_square(rows, cols, e)) return LLA_NOT_SQUARE;                                \
        const int64_t n = rows;                                                                \
        if (uplo == LLA_UPPER) {                                                               \
            for (int64_t i = 0; i < n; ++i)                                                    \
                for (int64_t j = 0; j < i; ++j) AT(a, i, j, rs, cs) = (T)0;                    \
        } else {                                                                               \
            for (int64_t i = 0; i < n; ++i)                                                    \
                for (int64_t j = i + 1; j < n; ++j) AT(a, i, j, rs, cs) = (T)0;                \
        }                                                                                      \
        return LLA_OK;                                                                         \
    }                                                                                          \
                                                                                               \
    /* Triangular::is_triangular (src/triangular.rs:67-90); non-square -> false */             \
    int ora_##P##is_triangular(const T *a, int64_t rows, int64_t cols, int64_t rs,             \
                               int64_t cs, int uplo) {                                         \
        if (rows != cols) return 0;                                                            \
        const int64_t n = rows;                                                                \
        if (uplo == LLA_UPPER) {                                                               \
            for (int64_t i = 0; i < n; ++i)                                                    \
                for (int64_t j = 0; j < i; ++j)                                                \
                    if (AT(a, i, j, rs, cs) != (T)0) return 0;                                 \
        } else {                                                                               \
            for (int64_t i = 0; i < n; ++i)                                                    \
                for (int64_t j = i + 1; j < n; ++j)                                            \
                    if (AT(a, i, j, rs, cs) != (T)0) return 0;                                 \
        }                                                                                      \
        return 1;                                                                              \
    }                                                                                          \
                                                                                               \
    /* CholeskyInplace::cholesky_inplace (src/cholesky.rs:78-82) */                            \
    int ora_##P##cholesky_inplace(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,    \
                                  lla_error *e) {                                              \
        int st = ora_##P##cholesky_inplace_dirty(a, rows, cols, rs, cs, e);                    \
        if (st) return st;                                                                     \
        return ora_##P##triangular_inplace(a, rows, cols, rs, cs, LLA_LOWER, e);               \
    }                                                                                          \
                                                                                               \
    /* solve_triangular_system_common / solve_triangular_system                                \
     * (src/triangular.rs:95-144).  diag == NULL means diag_fn(i) = a[i,i]                     \
     * (SolveTriangularInplace, :166); otherwise diag_fn(i) = diag[i]. */                      \
    int ora_##P##solve_triangular_system(const T *a, int64_t rows, int64_t cols, int64_t rs,   \
                                         int64_t cs, const T *diag, T *b, int64_t brows,       \
                                         int64_t bcols, int64_t brs, int64_t bcs, int uplo,    \
                                         lla_error *e) {                                       \
        set_ok(e);                                                                             \
        if (check_square(rows, cols, e)) return LLA_NOT_SQUARE;                                \
        const int64_t n = rows;                                                                \
        if (brows != n) {                                                                      \
            if (e) {                                                                           \
                e->code = LLA_WRONG_ROWS;                                                      \
                e->expected = n;                                                               \
                e->actual = brows;                                                             \
            }                                                                                  \
            return LLA_WRONG_ROWS;                                                             \
        }                                                                                      \
        for (int64_t k = 0; k < bcols; ++k) {                                                  \
            for (int64_t t = 0; t < n; ++t) {                                                  \
                /* Upper iterates rows n-1..0, Lower 0..n-1 (:140,:142) */                     \
                const int64_t i = (uplo == LLA_UPPER) ? (n - 1 - t) : t;                       \
                const T dg = diag ? diag[i] : AT(a, i, i, rs, cs);                             \
                const T coeff = AT(b, i, k, brs, bcs) / dg;                                    \
                AT(b, i, k, brs, bcs) = coeff;                                                 \
                const T alpha = -coeff;                                                        \
                /* b.slice_mut(s![..i, k]).scaled_add(-coeff, a.slice(s![..i, i])) (Upper),    \
                 * b.slice_mut(s![i+1.., k]).scaled_add(-coeff, a.slice(s![i+1.., i])) (Lower) \
                 * (:122-123, slices from :140,:142) */                                        \
                if (uplo == LLA_UPPER) {                                                       \
                    for (int64_t r = 0; r < i; ++r)                                            \
                        AT(b, r, k, brs, bcs) = AT(b, r, k, brs, bcs) + alpha * AT(a, r, i, rs, cs); \
                } else {                                                                       \
                    for (int64_t r = i + 1; r < n; ++r)                                        \
                        AT(b, r, k, brs, bcs) = AT(b, r, k, brs, bcs) + alpha * AT(a, r, i, rs, cs); \
                }                                                                              \
            }                                                                                  \
        }                                                                                      \
        return LLA_OK;                                                                         \
    }                                                                                          \
                                                                                               \
    /* SolveTriangularInplace::solve_triangular_inplace (src/triangular.rs:161-168) */         \
    int ora_##P##solve_triangular_inplace(const T *a, int64_t rows, int64_t cols, int64_t rs,  \
                                          int64_t cs, T *b, int64_t brows, int64_t bcols,      \
                                          int64_t brs, int64_t bcs, int uplo, lla_error *e) {  \
        return ora_##P##solve_triangular_system(a, rows, cols, rs, cs, NULL, b, brows, bcols,  \
                                                brs, bcs, uplo, e);                            \
    }                                                                                          \
                                                                                               \
    /* SolveCInplace::solvec_inplace (src/cholesky.rs:136-144): dirty factor,                  \
     * Lower solve with L, Upper solve with the transposed view L.t() */                       \
    int ora_##P##solvec_inplace(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,      \
                                T *b, int64_t brows, int64_t bcols, int64_t brs, int64_t bcs,  \
                                lla_error *e) {                                                \
        int st = ora_##P##cholesky_inplace_dirty(a, rows, cols, rs, cs, e);                    \
        if (st) return st;                                                                     \
        st = ora_##P##solve_triangular_system(a, rows, cols, rs, cs, NULL, b, brows, bcols,    \
                                              brs, bcs, LLA_LOWER, e);                         \
        if (st) return st;                                                                     \
        /* .t() swaps the axes: shape (cols, rows), strides (cs, rs) */                        \
        return ora_##P##solve_triangular_system(a, cols, rows, cs, rs, NULL, b, brows, bcols,  \
                                                brs, bcs, LLA_UPPER, e);                       \
    }                                                                                          \
                                                                                               \
    /* InverseCInplace::invc_inplace (src/cholesky.rs:178-181): out = eye(nrows),              \
     * then solvec_into(out).  `out` must be a rows x rows view. */                            \
    int ora_##P##invc_inplace(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs,        \
                              T *out, int64_t ors, int64_t ocs, lla_error *e) {                \
        for (int64_t i = 0; i < rows; ++i)                                                     \
            for (int64_t j = 0; j < rows; ++j) AT(out, i, j, ors, ocs) = (i == j) ? (T)1 : (T)0; \
        return ora_##P##solvec_inplace(a, rows, cols, rs, cs, out, rows, rows, ors, ocs, e);   \
    }

DEFINE_ORACLE(double, d, sqrt)
DEFINE_ORACLE(float, s, sqrtf)

/* Build identity for the test harness: lets Python confirm the flags. */
const char *ora_build_info(void) {
#if defined(__FP_FAST_FMA) && defined(__FAST_MATH__)
    return "fast-math";
#else
    return "ieee-ffp-contract-off";
#endif
}

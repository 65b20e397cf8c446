// lla_kernels.h -- internal launcher declarations shared by the .cu files and
// the C-ABI layer.  All launchers are asynchronous on `st` and return 0 on a
// successful launch, -1 when a CUDA call failed (cudaGetLastError tells why).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

namespace lla {

// Cholesky, lower triangle of the n x n column-major W (leading dim ld).
// *d_info (device, int64) must hold -1 on entry; it receives the first
// failing row.  EXACT needs S (ld * n) and D (n) scratch.
template <typename T>
int potrf_exact_launch(T *W, T *S, T *D, int64_t n, int64_t ld, int64_t *d_info, cudaStream_t st);
// FAST needs diag0 (n) scratch and min_ratio (device double, preset to a
// large value) for the near-singular guard.
template <typename T>
int potrf_fast_launch(T *W, int64_t n, int64_t ld, int64_t *d_info, T *diag0, double *min_ratio,
                      cudaStream_t st);

// Triangular solve op(T) X = B in place (see lla_trsm.cu).  ws: trsm_ws_ints
// ints of scratch; err_word: device int, 0 on entry; sticky (optional): a
// device status word that also receives LLA_ERR_TIMEOUT and is never cleared
// by the launch (the record that lla_device_status reads).
template <typename T>
int trsm_launch(const T *M, int64_t ld, int64_t n, int lower, int trans, const T *diag, T *B,
                int64_t ldb, int64_t m, bool exact, int *ws, int *err_word, cudaStream_t st,
                int *sticky = nullptr);
size_t trsm_ws_ints(int64_t n, int64_t m);

// One system of a batched solve: order n, m right-hand sides, caller index,
// element offsets of A (n x n) and B (n x m) in the pools (column-major, ld n).
struct BatchItem {
    int32_t n, m, idx, pad;
    int64_t a_off, b_off;
};
constexpr int kBatchMaxN = 256, kBatchMaxRhs = 8;
// The persistent batched factor-and-solve over `count` items already on the
// device (largest first); *d_counter is reset on `st` before the launch.
template <typename T>
int batch_launch_raw(const BatchItem *d_items, int64_t count, T *dA, T *dB, int32_t *d_info,
                     int *d_counter, int ctas_per_sm, int threads, double flops, cudaStream_t st);

// Device-resident serving loop (lla_batch.cu, driven by lla_serve.cpp).
// The request ring lives in pinned host memory mapped into the device's
// address space: the host writes a request into slot t % kServeRing and then
// raises `published` to t + 1 (release); persistent CTAs claim tickets from a
// device counter, solve the request in place (A copied into per-CTA scratch,
// B overwritten with X) and publish status, failing row and done_seq = t + 1
// (system-scope release).  A slot is reused only after its ticket completed.
constexpr int kServeRing = 1024;
struct ServeReq {
    const void *A;
    void *B;
    int64_t lda, ldb;
    int32_t n, m, dtype, pad;
};
struct ServeRing {
    unsigned long long published;  // host: tickets [0, published) are written
    int stop;                      // host: idle CTAs return at once
    int pad;
    ServeReq req[kServeRing];
    int32_t status[kServeRing];         // device: 0 solved, 1 not positive definite
    int64_t fail_row[kServeRing];       // device: first failing row, or -1
    unsigned long long done_seq[kServeRing];  // device: ticket + 1 once finished
};
// Persistent loop of `ctas` CTAs on `st`: each claims tickets (device counter
// *d_next) and solves them; a CTA returns after about idle_us microseconds
// without work, or at once when ring->stop is set.  scratch: ctas x 256^2
// doubles for the working copies of A.
int serve_loop_launch(ServeRing *ring_dev, unsigned long long *d_next, double *scratch, int ctas,
                      double idle_us, cudaStream_t st);
size_t serve_loop_scratch_bytes(int ctas);

// Layout kernels (lla_layout.cu).
enum ExportMode { EXPORT_FULL = 0, EXPORT_LOWER = 1, EXPORT_LOWER_ZERO_UPPER = 2, EXPORT_FAIL = 3 };
// W[i + j*ld] = R[i*rs + j*cs] for i < rows, j < cols.
template <typename T>
int import_launch(const T *R, int64_t rs, int64_t cs, int64_t rows, int64_t cols, T *W, int64_t ld,
                  cudaStream_t st);
// R[i*rs + j*cs] = W[i + j*ld] for the entries selected by mode (fail_row
// for EXPORT_FAIL: rows < f with j <= i, and row f with j < f).
template <typename T>
int export_launch(const T *W, int64_t ld, T *R, int64_t rs, int64_t cs, int64_t rows, int64_t cols,
                  int mode, int64_t fail_row, cudaStream_t st);
// Zero the strict upper (uplo = LOWER) or strict lower (uplo = UPPER) part of R.
template <typename T>
int mask_launch(T *R, int64_t rs, int64_t cs, int64_t n, int uplo, cudaStream_t st);
// *d_flag (device int, 1 on entry) becomes 0 when a non-zero lies outside the uplo triangle.
template <typename T>
int is_triangular_launch(const T *R, int64_t rs, int64_t cs, int64_t n, int uplo, int *d_flag,
                         cudaStream_t st);
// *p = v (one device int).
int fill_int_launch(int *p, int v, cudaStream_t st);
// W = identity (n x n, ld).
template <typename T>
int eye_launch(T *W, int64_t ld, int64_t n, cudaStream_t st);
// W[i + j*ld] = W[j + i*ld] for i < j: the strict upper part from the lower one.
template <typename T>
int symmetrize_launch(T *W, int64_t ld, int64_t n, cudaStream_t st);

// Tall-skinny products of LOBPCG's Cholesky-QR (lla_lobpcg.cu).
// C (ka x kb, ldc) = A^T B for A n x ka, B n x kb (column-major); P: workspace
// of atb_ws_elems(n, ka, kb) elements; symmetric: A == B (only the lower
// tiles are formed, the upper part mirrors them).  Deterministic.
size_t atb_ws_elems(int64_t n, int64_t ka, int64_t kb);
template <typename T>
int atb_launch(const T *A, int64_t lda, const T *B, int64_t ldb, int64_t n, int64_t ka, int64_t kb, T *C,
               int64_t ldc, T *P, int symmetric, cudaStream_t st);
// V (n x k) -= Y (n x ky) U (ky x k).
template <typename T>
int sub_tall_launch(T *V, int64_t ldv, const T *Y, int64_t ldy, const T *U, int64_t ldu, int64_t n, int64_t ky,
                    int64_t k, cudaStream_t st);

}  // namespace lla

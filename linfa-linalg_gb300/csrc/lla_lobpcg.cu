// lla_lobpcg.cu -- tall-skinny products of LOBPCG's Cholesky-QR
// (src/lobpcg/algorithm.rs:63-96): the Gram matrices V^T V and Y^T V, and the
// constraint update V -= Y U.  The Cholesky of the small Gram matrix and the
// triangular solve with it reuse the library's factor and substitution kernels
// (lla_api.cpp).
//
// C = A^T B for tall A (n x ka) and B (n x kb), column-major: the rows are cut
// into fixed chunks; CTA (chunk, I, J) sums the 32 x 32 output tile (I, J) over
// its chunk in FP64/FP32 FMA, and a second kernel adds the chunk partials in
// chunk order, so the result is deterministic (independent of scheduling).
#include <cuda_runtime.h>

#include "lla_common.cuh"
#include "lla_kernels.h"
#include "lla_prof.h"

namespace lla {

constexpr int kAtbTile = 32;
constexpr int64_t kAtbRows = 1024;  // rows per chunk
constexpr int kAtbMaxChunks = 64;

static int64_t atb_chunks(int64_t n) {
    const int64_t c = (n + kAtbRows - 1) / kAtbRows;
    return c < 1 ? 1 : (c > kAtbMaxChunks ? kAtbMaxChunks : c);
}

size_t atb_ws_elems(int64_t n, int64_t ka, int64_t kb) { return (size_t)atb_chunks(n) * ka * kb; }

// Partial P[z] = A[rows of chunk z]^T B[rows of chunk z] for tile (I, J);
// symmetric (A == B): only tiles I >= J.  Thread (tx, ty) owns outputs
// (I*32 + ty + 8u, J*32 + tx), u < 4.
template <typename T>
__global__ void __launch_bounds__(256) atb_partial_kernel(const T *__restrict__ A, int64_t lda,
                                                          const T *__restrict__ B, int64_t ldb, int64_t n,
                                                          int64_t ka, int64_t kb, int64_t rows_per_chunk,
                                                          int symmetric, T *P) {
    const int I = blockIdx.y, J = blockIdx.z;
    if (symmetric && I < J) return;
    __shared__ T sa[kAtbTile][kAtbTile + 1], sb[kAtbTile][kAtbTile + 1];  // [row][column]
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int64_t r_beg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t r_end = r_beg + rows_per_chunk < n ? r_beg + rows_per_chunk : n;
    T acc[4] = {T(0), T(0), T(0), T(0)};
    for (int64_t r0 = r_beg; r0 < r_end; r0 += kAtbTile) {
        // columns are contiguous over rows: lane tx walks the rows (coalesced)
        for (int c = ty; c < kAtbTile; c += 8) {
            const int64_t r = r0 + tx;
            const int64_t ca = (int64_t)I * kAtbTile + c, cb = (int64_t)J * kAtbTile + c;
            sa[tx][c] = (r < r_end && ca < ka) ? A[r + ca * lda] : T(0);
            sb[tx][c] = (r < r_end && cb < kb) ? B[r + cb * ldb] : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < kAtbTile; ++rr) {
            const T b = sb[rr][tx];
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = fma(sa[rr][ty + 8 * u], b, acc[u]);
        }
        __syncthreads();
    }
    T *Pz = P + (int64_t)blockIdx.x * ka * kb;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t i = (int64_t)I * kAtbTile + ty + 8 * u, j = (int64_t)J * kAtbTile + tx;
        if (i < ka && j < kb) Pz[i + j * ka] = acc[u];
    }
}

// C[i, j] = sum over chunks (in order) of P[z][i, j]; symmetric: the upper
// part mirrors the lower.
template <typename T>
__global__ void atb_reduce_kernel(const T *__restrict__ P, int64_t chunks, int64_t ka, int64_t kb,
                                  int symmetric, T *C, int64_t ldc) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ka * kb) return;
    int64_t i = e % ka, j = e / ka;
    const int64_t src = (symmetric && i < j) ? j + i * ka : i + j * ka;
    T s = P[src];
    for (int64_t z = 1; z < chunks; ++z) s += P[z * ka * kb + src];
    C[i + j * ldc] = s;
}

template <typename T>
int atb_launch(const T *A, int64_t lda, const T *B, int64_t ldb, int64_t n, int64_t ka, int64_t kb, T *C,
               int64_t ldc, T *P, int symmetric, cudaStream_t st) {
    if (ka == 0 || kb == 0) return 0;
    if (n == 0) return cudaMemsetAsync(P, 0, sizeof(T) * ka * kb, st) == cudaSuccess &&
                               cudaMemcpy2DAsync(C, sizeof(T) * ldc, P, sizeof(T) * ka, sizeof(T) * ka, kb,
                                                 cudaMemcpyDeviceToDevice, st) == cudaSuccess
                           ? 0
                           : -1;
    const int64_t chunks = atb_chunks(n);
    const int64_t rpc = (n + chunks - 1) / chunks;
    const int64_t ti = (ka + kAtbTile - 1) / kAtbTile, tj = (kb + kAtbTile - 1) / kAtbTile;
    if (ti > 65535 || tj > 65535) return -1;
    {
        LaunchScope ls(K_MISC, st, 2.0 * n * ka * kb);
        atb_partial_kernel<T><<<dim3((unsigned)chunks, (unsigned)ti, (unsigned)tj), 256, 0, st>>>(
            A, lda, B, ldb, n, ka, kb, rpc, symmetric, P);
        if (cudaGetLastError() != cudaSuccess) return -1;
    }
    LaunchScope ls(K_MISC, st, (double)chunks * ka * kb);
    atb_reduce_kernel<T><<<(unsigned)((ka * kb + 255) / 256), 256, 0, st>>>(P, chunks, ka, kb, symmetric, C,
                                                                             ldc);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// V[r, c] -= sum_t Y[r, t] U[t, c]  (V n x k, Y n x ky, U ky x k; column-major)
template <typename T>
__global__ void __launch_bounds__(256) sub_tall_kernel(T *V, int64_t ldv, const T *__restrict__ Y, int64_t ldy,
                                                       const T *__restrict__ U, int64_t ldu, int64_t n,
                                                       int64_t ky) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (r >= n) return;
    T s = T(0);
    for (int64_t t = 0; t < ky; ++t) s = fma(Y[r + t * ldy], U[t + c * ldu], s);
    V[r + c * ldv] -= s;
}

template <typename T>
int sub_tall_launch(T *V, int64_t ldv, const T *Y, int64_t ldy, const T *U, int64_t ldu, int64_t n, int64_t ky,
                    int64_t k, cudaStream_t st) {
    if (n == 0 || k == 0 || ky == 0) return 0;
    if (k > 65535) return -1;
    LaunchScope ls(K_MISC, st, 2.0 * n * ky * k);
    sub_tall_kernel<T><<<dim3((unsigned)((n + 255) / 256), (unsigned)k), 256, 0, st>>>(V, ldv, Y, ldy, U, ldu, n,
                                                                                       ky);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template int atb_launch<double>(const double *, int64_t, const double *, int64_t, int64_t, int64_t, int64_t,
                                double *, int64_t, double *, int, cudaStream_t);
template int atb_launch<float>(const float *, int64_t, const float *, int64_t, int64_t, int64_t, int64_t,
                               float *, int64_t, float *, int, cudaStream_t);
template int sub_tall_launch<double>(double *, int64_t, const double *, int64_t, const double *, int64_t,
                                     int64_t, int64_t, int64_t, cudaStream_t);
template int sub_tall_launch<float>(float *, int64_t, const float *, int64_t, const float *, int64_t, int64_t,
                                    int64_t, int64_t, cudaStream_t);

}  // namespace lla

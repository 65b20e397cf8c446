// lla_trsm_inv.cu -- FP32 triangular solves of the mixed-precision refinement
// with inverted diagonal blocks.
//
// The refinement solves with the same low-precision factor L eight to ten
// times, so the inverses W_r = L_rr^-1 of its 64 x 64 diagonal blocks are
// formed once (one CTA per block) and every substitution becomes a chain of
// small matrix products:
//     forward  L Y = B  : Y_r = W_r (B_r - sum_{q<r} L_rq Y_q)
//     backward L^T X = Y: X_r = W_r^T (Y_r - sum_{q>r} L_qr^T X_q)
// One CTA per (64-row block, 16-column chunk); CTAs take tickets in
// processing order and wait (bounded) for the blocks they need, as in the
// look-back substitution of lla_trsm.cu, but with no sequential step inside a
// block: the critical path per block is two 64 x 64 x 16 products.
#include <cuda_runtime.h>

#include "lla_common.cuh"
#include "lla_mixed.h"
#include "lla_prof.h"

namespace lla {

constexpr int kIvNb = 64, kIvCols = 16;

// W_r = L_rr^-1 (lower, FP32), padded with the identity past n.  One CTA of
// 64 threads per block; thread j computes column j by forward substitution.
__global__ void __launch_bounds__(64) diag_inverse_kernel(const float *__restrict__ L, int64_t ld, int64_t n,
                                                          float *W) {
    __shared__ float sL[kIvNb][kIvNb + 1];
    const int64_t r0 = (int64_t)blockIdx.x * kIvNb;
    const int j = threadIdx.x;
    for (int e = j; e < kIvNb * kIvNb; e += 64) {
        const int i = e % kIvNb, k = e / kIvNb;
        float v = 0.f;
        if (k <= i) {
            if (r0 + i < n)
                v = L[(r0 + i) + (r0 + k) * ld];
            else
                v = (i == k) ? 1.f : 0.f;
        }
        sL[i][k] = v;
    }
    __syncthreads();
    float w[kIvNb];
#pragma unroll
    for (int i = 0; i < kIvNb; ++i) w[i] = 0.f;
    // column j of the inverse: W[i][j] = (delta_ij - sum_{j<=k<i} L[i][k] W[k][j]) / L[i][i]
#pragma unroll
    for (int i = 0; i < kIvNb; ++i) {
        if (i >= j) {
            float s = (i == j) ? 1.f : 0.f;
#pragma unroll
            for (int k = 0; k < kIvNb; ++k)
                if (k >= j && k < i) s = fmaf(-sL[i][k], w[k], s);
            w[i] = s / sL[i][i];
        }
    }
    float *Wr = W + (int64_t)blockIdx.x * kIvNb * kIvNb;  // column-major 64 x 64
#pragma unroll
    for (int i = 0; i < kIvNb; ++i) Wr[i + j * kIvNb] = w[i];
}

__device__ __forceinline__ int iv_ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// trans = 0: L Y = B (blocks ascending); trans = 1: L^T X = B (descending).
__global__ void __launch_bounds__(256) trsm_inv_kernel(const float *__restrict__ L, int64_t ld,
                                                       const float *__restrict__ W, int64_t n,
                                                       float *B, int64_t ldb, int64_t m, int trans,
                                                       int nchunks, int *ws, int *err_word) {
    __shared__ float sL[kIvNb][kIvNb + 1];  // sL[k][i]: coefficient of x_k in row i
    __shared__ float sX[kIvNb][kIvCols];     // solved block / right-hand side
    __shared__ int s_ticket, s_abort;
    const int tid = threadIdx.x;
    int *counter = ws, *flags = ws + 1;
    if (tid == 0) {
        s_ticket = atomicAdd(counter, 1);
        s_abort = 0;
    }
    __syncthreads();
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    const int64_t pb = s_ticket / nchunks;  // position in processing order
    const int cc = s_ticket % nchunks;
    const int64_t rb = trans ? R - 1 - pb : pb;
    const int row = tid % kIvNb, cg = tid / kIvNb;  // 64 rows x 4 column groups of 4
    const int64_t grow = rb * kIvNb + row;
    float acc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t col = (int64_t)cc * kIvCols + cg * 4 + u;
        acc[u] = (grow < n && col < m) ? B[grow + col * ldb] : 0.f;
    }
    for (int64_t pq = 0; pq < pb; ++pq) {
        const int64_t qb = trans ? R - 1 - pq : pq;
        if (tid == 0) {
            const int *f = flags + pq * nchunks + cc;
            long long spins = 0;
            while (iv_ld_acquire(f) == 0) {
                if (*(volatile int *)err_word != 0 || ++spins > kSpinLimit) {
                    atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
                    s_abort = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        __syncthreads();
        if (s_abort) break;
        // coupling tile: forward L[rb rows][qb cols], backward L[qb rows][rb cols]^T
        for (int e = tid; e < kIvNb * kIvNb; e += 256) {
            const int a = e % kIvNb, b = e / kIvNb;  // consecutive e -> consecutive memory
            float v;
            if (!trans) {  // i = a (row of block rb), k = b (row of block qb)
                const int64_t gi = rb * kIvNb + a, gk = qb * kIvNb + b;
                v = (gi < n && gk < n) ? L[gi + gk * ld] : 0.f;
                sL[b][a] = v;
            } else {  // element L[qb*64 + a][rb*64 + b]: k = a, i = b
                const int64_t gk = qb * kIvNb + a, gi = rb * kIvNb + b;
                v = (gi < n && gk < n) ? L[gk + gi * ld] : 0.f;
                sL[a][b] = v;
            }
        }
        for (int e = tid; e < kIvNb * kIvCols; e += 256) {
            const int k = e % kIvNb, c = e / kIvNb;
            const int64_t gk = qb * kIvNb + k, col = (int64_t)cc * kIvCols + c;
            sX[k][c] = (gk < n && col < m) ? __ldcg(&B[gk + col * ldb]) : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < kIvNb; ++k) {
            const float l = sL[k][row];
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = fmaf(-l, sX[k][cg * 4 + u], acc[u]);
        }
        __syncthreads();
    }
    if (!s_abort) {
        // X_rb = W (or W^T) times acc
#pragma unroll
        for (int u = 0; u < 4; ++u) sX[row][cg * 4 + u] = acc[u];
        const float *Wr = W + rb * kIvNb * kIvNb;
        for (int e = tid; e < kIvNb * kIvNb; e += 256) {
            const int a = e % kIvNb, b = e / kIvNb;  // W column-major: Wr[a + 64 b] = W[a][b]
            if (!trans)
                sL[b][a] = Wr[a + b * kIvNb];  // coefficient of acc_b in row a
            else
                sL[a][b] = Wr[a + b * kIvNb];  // W^T[b][a] = W[a][b]: coefficient of acc_a in row b
        }
        __syncthreads();
        float y[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
        for (int k = 0; k < kIvNb; ++k) {
            const float wv = sL[k][row];
#pragma unroll
            for (int u = 0; u < 4; ++u) y[u] = fmaf(wv, sX[k][cg * 4 + u], y[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t col = (int64_t)cc * kIvCols + cg * 4 + u;
            if (grow < n && col < m) B[grow + col * ldb] = y[u];
        }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) asm volatile("st.release.gpu.b32 [%0], %1;" ::"l"(flags + pb * nchunks + cc), "r"(1) : "memory");
}

size_t trsm_inv_ws_ints(int64_t n, int64_t m) {
    return (size_t)(1 + ((n + kIvNb - 1) / kIvNb) * ((m + kIvCols - 1) / kIvCols));
}

size_t diag_inverse_floats(int64_t n) { return (size_t)((n + kIvNb - 1) / kIvNb) * kIvNb * kIvNb; }

int diag_inverse_launch(const float *L, int64_t ld, int64_t n, float *W, cudaStream_t st) {
    if (n == 0) return 0;
    LaunchScope ls(K_MIXED_TRSM, st, (double)n * kIvNb * kIvNb / 3.0);
    diag_inverse_kernel<<<(unsigned)((n + kIvNb - 1) / kIvNb), 64, 0, st>>>(L, ld, n, W);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int trsm_inv_launch(const float *L, int64_t ld, const float *W, int64_t n, float *B, int64_t ldb,
                    int64_t m, int trans, int *ws, int *err_word, cudaStream_t st) {
    if (n == 0 || m == 0) return 0;
    const int nchunks = (int)((m + kIvCols - 1) / kIvCols);
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    if (cudaMemsetAsync(ws, 0, sizeof(int) * (1 + R * nchunks), st) != cudaSuccess) return -1;
    // algorithmic work: n^2 m flops
    LaunchScope ls(K_MIXED_TRSM, st, (double)n * n * m);
    trsm_inv_kernel<<<(unsigned)(R * nchunks), 256, 0, st>>>(L, ld, W, n, B, ldb, m, trans, nchunks, ws,
                                                             err_word);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace lla

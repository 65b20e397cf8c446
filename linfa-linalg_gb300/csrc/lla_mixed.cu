// lla_mixed.cu -- mixed-precision SPD solve with FP64 iterative refinement.
//
//   1. Equilibrate symmetrically with exact powers of two: A^ = S A S,
//      s_i = 2^-floor(log2(a_ii)/2), so diag(A^) lies in [1, 4) and every
//      entry of A^ is exact in FP64.  (Only the lower triangle of A is read,
//      as in the reference; the solved matrix is the symmetric matrix it
//      defines.)
//   2. Factor A^ ~= L L^T in low precision: FP32 diagonal blocks and panels,
//      trailing updates on the tensor cores (BF16 or FP16 operand terms with
//      FP32 accumulation, lla_tc_update.cu) or in FP32 SIMT.
//   3. Refine in FP64: r = b - A x (FP64 tensor pipe), d = S L^-T L^-1 S r in
//      FP32, x += d (FP64), until the normwise backward error
//      max_j ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) <= tol.
//   4. On a low-precision breakdown (non-positive pivot) or a stall, fall back
//      to the plain FP64 factorisation, whose verdict (NotPositiveDefinite)
//      stands.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lla_api_internal.h"
#include "lla_autotune.h"
#include "lla_common.cuh"
#include "lla_f32_bits.h"
#include "lla_kernels.h"
#include "lla_mixed.h"
#include "lla_prof.h"

namespace lla {

__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    // non-negative doubles order like their bit patterns; NaN/inf map to the top
    if (!(v >= 0.0)) v = __longlong_as_double(0x7ff0000000000000ll);  // NaN -> +inf
    atomicMax((unsigned long long *)addr, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// s_i = 2^-floor(log2(a_ii)/2); a non-positive or non-finite diagonal marks
// the matrix as not factorable in low precision (the FP64 path decides).
__global__ void equil_scale_kernel(const double *A, int64_t lda, int64_t n, int scale, double *s,
                                   int *bad, int64_t *info) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = A[i + i * lda];
    if (!(a > 0.0) || !isfinite(a)) {
        s[i] = 1.0;
        atomicExch(bad, 1);
        // the low-precision factorisation is skipped (its kernels return at once
        // once *info >= 0) and the FP64 fallback decides
        if (info) atomicExch((unsigned long long *)info, 0ull);
        return;
    }
    if (!scale) {
        s[i] = 1.0;
        return;
    }
    const int e = ilogb(a);
    s[i] = ldexp(1.0, -(e >= 0 ? e / 2 : -((-e + 1) / 2)));
}

// One pass over the lower triangle of A in 64 x 64 tiles (I, J), I >= J:
// W = fp32(S A S) (lower triangle, column-major), and per tile the partial
// row sums / maxima of |a_ik| over its columns (elements on or below the
// diagonal) and the partial column sums / maxima over its rows (elements
// strictly below the diagonal, which stand for the upper triangle of A_sym).
// No atomics: sym_rows_kernel adds the partials of each row in a fixed order.
// Partials, n_pad = R * 64 apart: P[0][J] row sums, P[1][J] row maxima (tile
// column J), P[2][I] column sums, P[3][I] column maxima (tile row I).
// FP64 arithmetic is scarce on this GPU (about 1/64 of the FP32 rate), so the
// kernel avoids it: the scaling adds e_i + e_k to the exponent field, the
// conversion to FP32 rounds to nearest even on the bit patterns (the
// hardware conversion only for results outside the FP32 normal range), the
// maxima are taken on the bit patterns (non-negative doubles order like
// unsigned integers), and a tile whose nonzero |a| all lie in [2^-100, 2^100]
// sums its 64-term row and column partials in FP32 (relative error below
// 64 u_fp32 = 4e-6, harmless for the norm of the stopping test; the partials
// are then added in FP64); any other tile sums in FP64.
// Thread (r = tid % 64, cg = tid / 64): row r, columns 16 cg .. 16 cg + 15.
constexpr int kSymT = 64;

__device__ __noinline__ long long sym_plain_product(double si, double a, double sk) {
    return __double_as_longlong(si * a * sk);
}

template <bool MAX>
__global__ void __launch_bounds__(256) sym_tile_kernel(const double *__restrict__ A, int64_t lda, int64_t n,
                                                       const double *__restrict__ s, float *W, int64_t ldw,
                                                       double *P) {
    const int64_t I = blockIdx.y, J = blockIdx.x;
    if (J > I) return;
    const int64_t R = gridDim.y, npad = R * kSymT;
    __shared__ double prs[4][kSymT];
    __shared__ unsigned long long prm[4][kSymT];
    __shared__ unsigned long long sv[kSymT][kSymT + 1];  // sv[c][r]: bits of |a| for the column partials
    __shared__ unsigned long long sdg[kSymT];             // |a_rr| of a diagonal tile (FP64 row sums)
    __shared__ double ss[kSymT];                          // the tile's column scales
    const int tid = threadIdx.x, r = tid % kSymT, cg = tid / kSymT;
    if (tid < kSymT) ss[tid] = J * kSymT + tid < n ? s[J * kSymT + tid] : 0.0;
    const int64_t i = I * kSymT + r;
    const double si = i < n ? s[i] : 0.0;
    // s holds powers of two: the scaling adds e_i + e_k to the exponent field
    const int ei = (int)((__double_as_longlong(si) >> 52) & 0x7ff) - 1023;
    // every load of the thread first (16 elements in flight)
    double av[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int c = 16 * cg + u;
        const int64_t k = J * kSymT + c;
        const bool lower = i < n && k < n && (I > J || r >= c);
        av[u] = lower ? A[i + k * lda] : 0.0;
    }
    __syncthreads();  // ss
    unsigned long long v[16];
    bool in_range = true;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int c = 16 * cg + u;
        const int64_t k = J * kSymT + c;
        const bool lower = i < n && k < n && (I > J || r >= c);
        const double a = av[u];
        if (lower) {
            const double sku = ss[c];
            const int es = ei + (int)((__double_as_longlong(sku) >> 52) & 0x7ff) - 1023;
            const long long ab = __double_as_longlong(a);
            const int ex = (int)((ab >> 52) & 0x7ff), ne = ex + es;
            // normal in and out: exact exponent shift; otherwise (zero, subnormal,
            // inf/NaN, out of range) the plain product, in a call so that the
            // compiler cannot evaluate its two FP64 multiplies for every element
            long long asb = ab + ((long long)es << 52);
            if (!(ex != 0 && ex != 0x7ff && ne > 0 && ne < 0x7ff)) asb = sym_plain_product(si, a, sku);
            W[i + k * ldw] = sym_to_f32(asb);
        }
        v[u] = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
        in_range &= sym_f32_range(v[u]);
        sv[c][r] = (I > J || r > c) ? v[u] : 0ull;
        if (I == J && c == r) sdg[r] = v[u];
    }
    const bool f32 = __syncthreads_and(in_range) != 0;  // also orders the shared stores before the sums
    double rs;
    unsigned long long rm = 0ull;
    if (f32) {
        float t = 0.f;
#pragma unroll
        for (int u = 0; u < 16; ++u) t += sym_abs_f32(v[u]);
        rs = (double)t;
    } else {  // FP64 from shared memory, in a loop the compiler keeps as a branch
        rs = 0.0;
#pragma unroll 1
        for (int u = 0; u < 16; ++u) {
            const int c = 16 * cg + u;
            rs += __longlong_as_double((long long)(c == r && I == J ? sdg[r] : sv[c][r]));
        }
    }
    if (MAX) {
#pragma unroll
        for (int u = 0; u < 16; ++u) rm = v[u] > rm ? v[u] : rm;
    }
    prs[cg][r] = rs;
    if (MAX) prm[cg][r] = rm;
    __syncthreads();
    if (tid < kSymT) {  // row partial of row tid
        P[J * npad + I * kSymT + tid] = ((prs[0][tid] + prs[1][tid]) + prs[2][tid]) + prs[3][tid];
        if (MAX) {
            unsigned long long m = prm[0][tid];
#pragma unroll
            for (int g = 1; g < 4; ++g) m = prm[g][tid] > m ? prm[g][tid] : m;
            P[(R + J) * npad + I * kSymT + tid] = __longlong_as_double((long long)m);
        }
    } else if (tid < 2 * kSymT) {  // column partial of column c
        const int c = tid - kSymT;
        double cs;
        unsigned long long cm = 0ull;
        if (f32) {
            float t = 0.f;
#pragma unroll 8
            for (int q = 0; q < kSymT; ++q) {
                const unsigned long long w = sv[c][q];
                t += sym_abs_f32(w);
                if (MAX) cm = w > cm ? w : cm;
            }
            cs = (double)t;
        } else {
            cs = 0.0;
#pragma unroll 1
            for (int q = 0; q < kSymT; ++q) {
                const unsigned long long w = sv[c][q];
                cs += __longlong_as_double((long long)w);
                if (MAX) cm = w > cm ? w : cm;
            }
        }
        P[(2 * R + I) * npad + J * kSymT + c] = cs;
        if (MAX) P[(3 * R + I) * npad + J * kSymT + c] = __longlong_as_double((long long)cm);
    }
}

// rowsum[i] (and rowmax[i]) from the tile partials: tile columns J <= i/64 in
// order, then tile rows I >= i/64 in order (maxima on the bit patterns; a NaN
// maximum reads as +inf).
__global__ void sym_rows_kernel(const double *__restrict__ P, int64_t R, int64_t n, double *rowsum,
                                double *rowmax) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t b = i / kSymT, npad = R * kSymT;
    const unsigned long long *Pb = reinterpret_cast<const unsigned long long *>(P);
    double sum = 0.0;
    unsigned long long mx = 0ull;
#pragma unroll 8
    for (int64_t J = 0; J <= b; ++J) {
        sum += P[J * npad + i];
        if (rowmax) {
            const unsigned long long v = Pb[(R + J) * npad + i];
            mx = v > mx ? v : mx;
        }
    }
#pragma unroll 8
    for (int64_t I = b; I < R; ++I) {
        sum += P[(2 * R + I) * npad + i];
        if (rowmax) {
            const unsigned long long v = Pb[(3 * R + I) * npad + i];
            mx = v > mx ? v : mx;
        }
    }
    rowsum[i] = sum;
    if (rowmax) rowmax[i] = __longlong_as_double((long long)(mx > 0x7ff0000000000000ull ? 0x7ff0000000000000ull : mx));
}

size_t sym_part_doubles(int64_t n) {
    const int64_t R = (n + kSymT - 1) / kSymT;
    return (size_t)4 * R * R * kSymT;
}

__global__ void max_reduce_kernel(const double *v, int64_t n, double *out) {
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(v[i]));
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(out, m);
}

// colmax[j] = max_i |M[i, j]|  (n x m column-major, leading dim ld)
__global__ void colmax_kernel(const double *M, int64_t ld, int64_t n, int64_t m, double *colmax) {
    const int64_t j = blockIdx.y;
    double v = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v = fmax(v, fabs(M[i + j * ld]));
    v = warp_max(v);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&colmax[j], v);
}

// Y = fp32(s .* R)   (n x m, column-major; ld of Y = n)
__global__ void scale_to_f32_kernel(const double *R, int64_t ldr, const double *s, int64_t n,
                                    int64_t m, float *Y, const int *state) {
    if (refine_done(state)) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t j = blockIdx.y;
    if (i < n && j < m) Y[i + j * n] = (float)(s[i] * R[i + j * ldr]);
}

// X += s .* Y (FP64), and colmax_x[j] = max_i |X[i,j]|
__global__ void update_x_kernel(double *X, int64_t ldx, const double *s, const float *Y, int64_t n,
                                int64_t m, double *colmax_x, const int *state) {
    if (refine_done(state)) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t j = blockIdx.y;
    double v = 0.0;
    if (i < n && j < m) {
        const double x = X[i + j * ldx] + s[i] * (double)Y[i + j * n];
        X[i + j * ldx] = x;
        v = fabs(x);
    }
    v = warp_max(v);
    if ((threadIdx.x & 31) == 0 && j < m) atomic_max_nonneg(&colmax_x[j], v);
}

// R = B - A_sym X on the FP64 tensor pipe (mma.sync m16n8k16 .f64).
// CTA tile: 32 rows x 64 RHS columns, K chunks of 32; four warps, each 16 x 32
// (four m16n8 MMAs per k16 step).  A_sym(i,k) reads the lower triangle:
// A[i + k*lda] for k <= i, A[k + i*lda] otherwise.  Also colmax_r.
constexpr int kResRows = 32, kResCols = 64, kResK = 32;

// K is split into `splits` contiguous ranges (blockIdx.z) so that the grid
// covers the SMs in several full waves; with splits > 1 each range writes its
// partial A_sym X into P[z] and residual_combine_kernel forms R = B - sum_z P[z]
// in a fixed order (deterministic, no atomics).
__global__ void __launch_bounds__(128) residual_dmma_kernel(const double *__restrict__ A, int64_t lda,
                                                            int64_t n, const double *__restrict__ X,
                                                            int64_t ldx, const double *__restrict__ B,
                                                            int64_t ldb, double *R, int64_t ldr,
                                                            int64_t m, double *colmax_r, int splits,
                                                            double *P, const int *state) {
    if (refine_done(state)) return;
    __shared__ double As[kResK][kResRows + 4];  // [k][row], stride 36 = 4 (mod 16)
    __shared__ double Xs[kResK][kResCols + 4];  // [k][col], stride 68 = 4 (mod 16)
    const int64_t i0 = (int64_t)blockIdx.x * kResRows;
    const int64_t c0 = (int64_t)blockIdx.y * kResCols;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int wr = (warp & 1) * 16, wc = (warp >> 1) * 32;
    double acc[4][4];
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[ni][q] = 0.0;
    const int64_t kchunks = (n + kResK - 1) / kResK;
    const int64_t kc_per = (kchunks + splits - 1) / splits;
    const int64_t kbeg = (int64_t)blockIdx.z * kc_per * kResK;
    const int64_t kend = min(n, kbeg + kc_per * kResK);
    for (int64_t k0 = kbeg; k0 < kend; k0 += kResK) {
        const bool upper = k0 > i0 + kResRows - 1;  // whole tile above the diagonal
        for (int e = tid; e < kResRows * kResK; e += 128) {
            int r, c;
            if (upper) {
                r = e / kResK;
                c = e % kResK;  // consecutive e -> consecutive k -> A[k + i*lda]
            } else {
                r = e % kResRows;
                c = e / kResRows;  // consecutive e -> consecutive i -> A[i + k*lda]
            }
            const int64_t i = i0 + r, k = k0 + c;
            double v = 0.0;
            if (i < n && k < n) v = (k <= i) ? A[i + k * lda] : A[k + i * lda];
            As[c][r] = v;
        }
        for (int e = tid; e < kResK * kResCols; e += 128) {
            const int kk = e % kResK, cc = e / kResK;  // consecutive e -> consecutive k in column cc
            const int64_t k = k0 + kk, col = c0 + cc;
            Xs[kk][cc] = (k < n && col < m) ? X[k + col * ldx] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kResK; kk += 16) {
            double af[8], bf[4][4];
#pragma unroll
            for (int q = 0; q < 8; ++q) af[q] = As[kk + t + 4 * (q >> 1)][wr + g + 8 * (q & 1)];
#pragma unroll
            for (int ni = 0; ni < 4; ++ni)
#pragma unroll
                for (int q = 0; q < 4; ++q) bf[ni][q] = Xs[kk + t + 4 * q][wc + ni * 8 + g];
#pragma unroll
            for (int ni = 0; ni < 4; ++ni)
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                    "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
                    : "+d"(acc[ni][0]), "+d"(acc[ni][1]), "+d"(acc[ni][2]), "+d"(acc[ni][3])
                    : "d"(af[0]), "d"(af[1]), "d"(af[2]), "d"(af[3]), "d"(af[4]), "d"(af[5]),
                      "d"(af[6]), "d"(af[7]), "d"(bf[ni][0]), "d"(bf[ni][1]), "d"(bf[ni][2]),
                      "d"(bf[ni][3]));
        }
        __syncthreads();
    }
    if (splits > 1) {  // partial product of this K range
        double *Pz = P + (int64_t)blockIdx.z * n * m;
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t i = i0 + wr + g + 8 * (q >> 1);
                const int64_t col = c0 + wc + ni * 8 + 2 * t + (q & 1);
                if (i < n && col < m) Pz[i + col * n] = acc[ni][q];
            }
        return;
    }
    // epilogue: R = B - acc, and column maxima of |R|
#pragma unroll
    for (int ni = 0; ni < 4; ++ni) {
        double cm2[2] = {0.0, 0.0};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int64_t i = i0 + wr + g + 8 * (q >> 1);
            const int64_t col = c0 + wc + ni * 8 + 2 * t + (q & 1);
            if (i < n && col < m) {
                const double r = B[i + col * ldb] - acc[ni][q];
                R[i + col * ldr] = r;
                cm2[q & 1] = fmax(cm2[q & 1], fabs(r));
            }
        }
        // reduce over the 8 row groups g sharing a column (lanes with equal t)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            double v = cm2[h];
            v = fmax(v, __shfl_xor_sync(0xffffffffu, v, 4));
            v = fmax(v, __shfl_xor_sync(0xffffffffu, v, 8));
            v = fmax(v, __shfl_xor_sync(0xffffffffu, v, 16));
            const int64_t col = c0 + wc + ni * 8 + 2 * t + h;
            if (g == 0 && col < m) atomic_max_nonneg(&colmax_r[col], v);
        }
    }
}

// R = B - (P[0] + P[1] + ...), summed in split order; and column maxima of |R|.
__global__ void residual_combine_kernel(const double *__restrict__ P, int splits, const double *B,
                                        int64_t ldb, double *R, int64_t ldr, int64_t n, int64_t m,
                                        double *colmax_r, const int *state) {
    if (refine_done(state)) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t j = blockIdx.y;
    double v = 0.0;
    if (i < n) {
        double s = P[i + j * n];
        for (int z = 1; z < splits; ++z) s += P[(int64_t)z * n * m + i + j * n];
        const double r = B[i + j * ldb] - s;
        R[i + j * ldr] = r;
        v = fabs(r);
    }
    v = warp_max(v);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&colmax_r[j], v);
}

// ---------------------------------------------------------------------------
// launch helpers

static unsigned gx(int64_t n, int b) { return (unsigned)ceil_div(n, b); }

int equilibrate_launch(const double *A, int64_t lda, int64_t n, bool scale, double *s, float *W,
                       int64_t ldw, double *rowsum, double *anorm, double *rowmax, double *part, int *bad,
                       cudaStream_t st, int64_t *info) {
    {
        LaunchScope ls(K_MIXED_CONVERT, st, 8.0 * n);
        equil_scale_kernel<<<gx(n, 256), 256, 0, st>>>(A, lda, n, scale ? 1 : 0, s, bad, info);
    }
    const int64_t R = (n + kSymT - 1) / kSymT;
    if (R > 65535) return -1;
    {
        // algorithmic bytes: the lower triangle of A read, that of W written
        LaunchScope ls(K_MIXED_CONVERT, st, 12.0 * n * (n + 1) / 2);
        if (rowmax)
            sym_tile_kernel<true><<<dim3((unsigned)R, (unsigned)R), 256, 0, st>>>(A, lda, n, s, W, ldw, part);
        else
            sym_tile_kernel<false><<<dim3((unsigned)R, (unsigned)R), 256, 0, st>>>(A, lda, n, s, W, ldw, part);
        if (cudaGetLastError() != cudaSuccess) return -1;
    }
    {
        LaunchScope ls(K_MIXED_CONVERT, st, 8.0 * R * n * (rowmax ? 2 : 1));
        sym_rows_kernel<<<gx(n, 256), 256, 0, st>>>(part, R, n, rowsum, rowmax);
    }
    {
        LaunchScope ls(K_MISC, st);
        max_reduce_kernel<<<std::min<unsigned>(gx(n, 256), 1024), 256, 0, st>>>(rowsum, n, anorm);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int colmax_launch(const double *M, int64_t ld, int64_t n, int64_t m, double *colmax, cudaStream_t st) {
    LaunchScope ls(K_MISC, st);
    colmax_kernel<<<dim3(std::min<unsigned>(gx(n, 256), 64), (unsigned)m), 256, 0, st>>>(M, ld, n, m,
                                                                                        colmax);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int scale_to_f32_launch(const double *R, int64_t ldr, const double *s, int64_t n, int64_t m, float *Y,
                        cudaStream_t st, const int *state) {
    LaunchScope ls(K_REFINE, st, 12.0 * n * m);
    scale_to_f32_kernel<<<dim3(gx(n, 256), (unsigned)m), 256, 0, st>>>(R, ldr, s, n, m, Y, state);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int update_x_launch(double *X, int64_t ldx, const double *s, const float *Y, int64_t n, int64_t m,
                    double *colmax_x, cudaStream_t st, const int *state) {
    LaunchScope ls(K_REFINE, st, 20.0 * n * m);
    update_x_kernel<<<dim3(gx(n, 256), (unsigned)m), 256, 0, st>>>(X, ldx, s, Y, n, m, colmax_x, state);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Refinement control on the device.  Control words (as doubles): [0] ||A||_inf,
// [2] int64 info of the low-precision factor, [4] int state | int iterations,
// [5] eta, [6] eta of the previous iteration, [7] eta after the first solve,
// [8 ..) column maxima of |r|, |x| and |b|.  state: 0 refining, 1 converged,
// 2 stalled or out of iterations, 3 the low-precision factorisation failed.
// Every per-iteration kernel returns at once when state != 0, so the host can
// enqueue several iterations ahead and synchronise once per group.
__global__ void refine_begin_kernel(double *words) {
    int *st = (int *)(words + 4);
    st[0] = (*(const int64_t *)(words + 2) >= 0) ? 3 : 0;
    st[1] = 0;
}

// eta = max_j ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf); converged when
// eta <= tol (from a full-level residual: with the exact-slice residual the
// levels of this iteration follow refine_levels); stalled when eta is not
// finite, or does not halve over an iteration after the second, or max_iters
// ran out.  While refining, the column maxima of |r| and |x| are cleared for
// the next iteration.
__global__ void __launch_bounds__(256) refine_check_kernel(double *words, int64_t m, double tol, int max_iters,
                                                           int slices) {
    int *st = (int *)(words + 4);
    if (*(volatile int *)st != 0) return;
    const bool coarse = slices && refine_levels(st) < 8;  // before this iteration's updates below
    __shared__ double red[8];
    __shared__ int s_go;
    const int tid = threadIdx.x;
    const double an = words[0];
    const double *cr = words + 8, *cx = cr + m, *cb = cx + m;
    double e = 0.0;
    for (int64_t j = tid; j < m; j += blockDim.x) {
        const double den = an * cx[j] + cb[j];
        double ej = den > 0 ? cr[j] / den : (cr[j] > 0 ? INFINITY : 0.0);
        if (ej != ej) ej = INFINITY;
        e = fmax(e, ej);
    }
    e = warp_max(e);
    if ((tid & 31) == 0) red[tid >> 5] = e;
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) e = fmax(e, red[w]);
        const int it = st[1] + 1;
        st[1] = it;
        words[5] = e;
        if (it == 1) words[7] = e;
        int state = 0;
        if (e <= tol && !coarse)
            state = 1;
        else if (!isfinite(e) || (it >= 3 && e > 0.5 * words[6]) || it >= max_iters)
            state = 2;
        if (state == 0) words[6] = e;
        st[0] = state;
        s_go = state == 0;
    }
    __syncthreads();
    if (s_go) {
        double *c = words + 8;
        for (int64_t j = tid; j < 2 * m; j += blockDim.x) c[j] = 0.0;
    }
}

int refine_begin_launch(double *words, cudaStream_t st) {
    LaunchScope ls(K_MISC, st);
    refine_begin_kernel<<<1, 1, 0, st>>>(words);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int refine_check_launch(double *words, int64_t m, double tol, int max_iters, cudaStream_t st, bool slices) {
    LaunchScope ls(K_MISC, st);
    refine_check_kernel<<<1, 256, 0, st>>>(words, m, tol, max_iters, slices ? 1 : 0);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int residual_splits(int64_t n, int64_t m) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const int64_t tiles = (int64_t)gx(n, kResRows) * gx(m, kResCols);
    // smallest split giving at least four waves of CTAs (at most 8)
    int s = 1;
    while (s < 8 && tiles * s < 4 * (int64_t)sms && n / (kResK * (s + 1)) >= 4) ++s;
    return s;
}

int residual_launch(const double *A, int64_t lda, int64_t n, const double *X, int64_t ldx,
                    const double *B, int64_t ldb, double *R, int64_t ldr, int64_t m, double *colmax_r,
                    double *P, cudaStream_t st, const int *state) {
    const int splits = P ? residual_splits(n, m) : 1;
    {
        // algorithmic work: 2 n^2 m flops
        LaunchScope ls(K_RESIDUAL, st, 2.0 * n * n * m);
        residual_dmma_kernel<<<dim3(gx(n, kResRows), gx(m, kResCols), splits), 128, 0, st>>>(
            A, lda, n, X, ldx, B, ldb, R, ldr, m, colmax_r, splits, P, state);
    }
    if (splits > 1) {
        LaunchScope ls(K_REFINE, st, 8.0 * n * m * (splits + 2));
        residual_combine_kernel<<<dim3(gx(n, 256), (unsigned)m), 256, 0, st>>>(P, splits, B, ldb, R, ldr,
                                                                             n, m, colmax_r, state);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace lla

// ---------------------------------------------------------------------------
// host driver

using namespace lla;

namespace {

cudaError_t last_err(int rc) {
    if (rc == 0) return cudaSuccess;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? cudaErrorUnknown : e;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

// Autotune-cache key of the refined solve's schedule for a shape.
static std::string refine_key(int64_t n, int64_t m, const lla_refine_opts &o) {
    auto lg = [](int64_t v) {
        int e = 0;
        while ((int64_t(1) << e) < v) ++e;
        return e;
    };
    char k[96];
    std::snprintf(k, sizeof(k), "r:n%d:m%d:u%d:s%d", lg(n), lg(m), (int)o.update, (int)o.residual);
    return k;
}

// Smallest pivot_k / a_kk that the FMA-order fallback factorisation accepts
// without the exact-order re-run (the host-view entry points use the same guard).
constexpr double kFallbackPivotGuard = 1e-10;
// Refinement iterations enqueued before the first synchronisation (the usual
// count for an FP32-accurate factor at kappa ~ 1e6), and per later group.
constexpr int kRefineGroup = 4, kRefineGroupNext = 2;

extern "C" void lla_refine_opts_default(lla_refine_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->update = LLA_UPDATE_BF16X6;
    o->max_iters = 30;
    o->tol = 1e-13;
    o->equilibrate = 1;
    o->fallback = 1;
    o->update_epilogue = 0;
    o->residual = LLA_RESIDUAL_FP64;
}

#define MX_TRY(expr)                                                \
    do {                                                            \
        cudaError_t e__ = (expr);                                   \
        if (e__ != cudaSuccess) return lla__set_cuda_error(err, e__); \
    } while (0)

extern "C" int lla_dposv_refined_device(const double *dA, int64_t n, int64_t lda, const double *dB,
                                        int64_t m, int64_t ldb, double *dX, int64_t ldx,
                                        const lla_refine_opts *opts_in, lla_refine_report *rep,
                                        void *stream, lla_error *err) {
    auto t_start = std::chrono::steady_clock::now();
    if (n < 0 || m < 0 || lda < std::max<int64_t>(1, n) || ldb < std::max<int64_t>(1, n) ||
        ldx < std::max<int64_t>(1, n) || (n > 0 && (!dA || (m > 0 && (!dB || !dX)))))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla_refine_opts opts;
    if (opts_in)
        opts = *opts_in;
    else
        lla_refine_opts_default(&opts);
    if (opts.max_iters <= 0) opts.max_iters = 30;
    if (!(opts.tol > 0)) opts.tol = 1e-13;
    if (opts.update_kchunk == 0 && opts.update_epilogue == 0 && opts.substitution == 0) {
        int a, b;  // the schedule the autotuner recorded for this shape, if any
        if (autotune_lookup(refine_key(n, m, opts), a, b)) {
            opts.update_kchunk = a >> 4;
            opts.update_epilogue = a & 15;
            opts.substitution = b;
        }
    }
    lla_refine_report r;
    std::memset(&r, 0, sizeof(r));
    r.update = opts.update;
    r.schedule = (opts.update_kchunk << 8) | (opts.update_epilogue << 4) | opts.substitution;
    lla__set_status(err, LLA_OK);
    if (n == 0 || m == 0) {
        r.converged = 1;
        if (rep) *rep = r;
        return LLA_OK;
    }
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    MixedWs &w = c->mixed;
    // workspace
    // FP32 factor, column-major; a leading dimension of whole 16-byte rows lets the
    // tensor-core update stage its output tiles with TMA
    const int64_t ldl = (n + 3) / 4 * 4;
    MX_TRY(w.L.ensure(sizeof(float) * ldl * n));
    MX_TRY(w.s.ensure(sizeof(double) * n));
    MX_TRY(w.rowsum.ensure(sizeof(double) * n));
    MX_TRY(w.R.ensure(sizeof(double) * n * m));
    MX_TRY(w.P.ensure(sizeof(double) * n * m * residual_splits(n, m)));
    MX_TRY(w.Y.ensure(sizeof(float) * n * m));
    MX_TRY(w.diag0.ensure(sizeof(float) * n));
    MX_TRY(w.words.ensure(sizeof(double) * (8 + 3 * m)));
    MX_TRY(c->ws.ensure(sizeof(int) * (std::max(trsm_ws_ints(n, m), trsm_inv_ws_ints(n, m)) + 1)));
    MX_TRY(w.winv.ensure(sizeof(float) * diag_inverse_floats(n)));
    MX_TRY(w.stage.ensure(sizeof(unsigned long long) *
                          std::max(trsm_inv_stage_words(n, m), trsm_chain_stage_words(n, m))));
    if (w.stage.p != w.stage_seen || w.stage.cap != w.stage_seen_cap) {
        MX_TRY(cudaMemsetAsync(w.stage.p, 0, w.stage.cap, st));
        w.stage_seen = w.stage.p;
        w.stage_seen_cap = w.stage.cap;
        w.stage_epoch = 0;
    }
    auto next_epoch = [&]() -> cudaError_t {  // a fresh nonzero tag per substitution launch
        if (++w.stage_epoch == 0) {
            cudaError_t e = cudaMemsetAsync(w.stage.p, 0, w.stage.cap, st);
            if (e != cudaSuccess) return e;
            w.stage_epoch = 1;
        }
        return cudaSuccess;
    };
    unsigned long long *stage = (unsigned long long *)w.stage.p;
    MX_TRY(w.words_host.ensure(sizeof(double) * (8 + 3 * m)));
    float *L = (float *)w.L.p;
    double *s = (double *)w.s.p;
    double *R = (double *)w.R.p;
    float *Y = (float *)w.Y.p;
    // words: [0] anorm, [1] min_ratio, [2] int64 info, [3] int bad | int err_word,
    //        [8 ..) colmax_r[m], colmax_x[m], colmax_b[m]
    double *words = (double *)w.words.p;
    double *anorm = words + 0;
    double *min_ratio = words + 1;
    int64_t *info = (int64_t *)(words + 2);
    int *bad = (int *)(words + 3);
    int *err_word = bad + 1;
    double *colmax_r = words + 8, *colmax_x = colmax_r + m, *colmax_b = colmax_x + m;
    int *tws = (int *)c->ws.p;
    double *hw = (double *)w.words_host.p;

    auto read_words = [&](size_t count) -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(hw, words, sizeof(double) * count, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e;
    };
    {
        double init[8] = {0.0, 1e300, 0.0, 0.0, 0, 0, 0, 0};
        int64_t minus1 = -1;
        std::memcpy(&init[2], &minus1, sizeof(int64_t));
        std::memcpy(hw, init, sizeof(init));
        MX_TRY(cudaMemcpyAsync(words, hw, sizeof(init), cudaMemcpyHostToDevice, st));
        MX_TRY(cudaMemsetAsync(colmax_r, 0, sizeof(double) * 3 * m, st));
    }
    for (auto &e : w.ev)
        if (!e) MX_TRY(cudaEventCreate(&e));
    MX_TRY(cudaEventRecord(w.ev[0], st));
    // 1. equilibrate (and ||A||_inf, ||b_j||_inf); a non-positive diagonal marks
    // the low-precision factorisation as failed on the device (info >= 0)
    auto t0 = std::chrono::steady_clock::now();
    const bool slices = opts.residual == LLA_RESIDUAL_EXACT_SLICES;
    MX_TRY(w.sympart.ensure(sizeof(double) * sym_part_doubles(n)));
    double *oz_rm = nullptr;  // row maxima of |A| for the exact-slice residual, formed in the same pass
    if (slices) {
        MX_TRY(w.oz.ensure(oz_workspace_bytes(n, m)));
        oz_rm = oz_rowmax(w.oz.p, n, m);
    }
    MX_TRY(last_err(equilibrate_launch(dA, lda, n, opts.equilibrate != 0, s, L, ldl,
                                       (double *)w.rowsum.p, anorm, oz_rm, (double *)w.sympart.p, bad, st, info)));
    MX_TRY(last_err(colmax_launch(dB, ldb, n, m, colmax_b, st)));
    // 2. low-precision factorisation (its kernels return at once after a breakdown)
    MX_TRY(last_err(lowp_factor_launch(L, n, ldl, opts, info, (float *)w.diag0.p, min_ratio, c, st)));
    // inverses of the 64 x 64 diagonal blocks, reused by every substitution
    MX_TRY(last_err(diag_inverse_launch(L, ldl, n, (float *)w.winv.p, st)));
    if (slices)  // slices of A, once per solve
        MX_TRY(last_err(oz_prepare(dA, lda, n, m, w.oz.p, true, st)));
    // 3. refinement, controlled on the device: every iteration ends with a check
    // kernel that sets the state word; the host enqueues iterations in groups and
    // synchronises once per group (all kernels of an iteration return at once
    // when the state is no longer "refining")
    MX_TRY(cudaEventRecord(w.ev[1], st));
    int *state = (int *)(words + 4);
    MX_TRY(last_err(refine_begin_launch(words, st)));
    for (int64_t j = 0; j < m; ++j)
        MX_TRY(cudaMemsetAsync(dX + j * ldx, 0, sizeof(double) * n, st));
    MX_TRY(cudaMemsetAsync(err_word, 0, sizeof(int), st));
    const float *Wi = (const float *)w.winv.p;
    const bool chain = opts.substitution == LLA_SUB_CHAIN;
    auto subst = chain ? trsm_chain_launch : trsm_inv_launch;
    double eta = INFINITY;
    bool converged = false, lowp_ok = true;
    int enqueued = 0, group = kRefineGroup;
    for (;;) {
        for (int g = 0; g < group && enqueued < opts.max_iters; ++g, ++enqueued) {
            // correction d = S L^-T L^-1 S r  (FP32), x += d; the first iteration solves with b
            const double *rhs = enqueued == 0 ? dB : R;
            const int64_t ldrhs = enqueued == 0 ? ldb : n;
            MX_TRY(last_err(scale_to_f32_launch(rhs, ldrhs, s, n, m, Y, st, state)));
            MX_TRY(next_epoch());
            MX_TRY(last_err(subst(L, ldl, Wi, n, Y, n, m, 0, stage, w.stage_epoch, tws, err_word, st, state)));
            MX_TRY(next_epoch());
            MX_TRY(last_err(subst(L, ldl, Wi, n, Y, n, m, 1, stage, w.stage_epoch, tws, err_word, st, state)));
            MX_TRY(last_err(update_x_launch(dX, ldx, s, Y, n, m, colmax_x, st, state)));
            // r = b - A x  (FP64 accuracy)
            if (slices)
                MX_TRY(last_err(oz_residual_launch(dX, ldx, dB, ldb, R, n, n, m, colmax_x, colmax_r,
                                                   w.oz.p, err_word, st, state)));
            else
                MX_TRY(last_err(residual_launch(dA, lda, n, dX, ldx, dB, ldb, R, n, m, colmax_r,
                                                (double *)w.P.p, st, state)));
            MX_TRY(last_err(refine_check_launch(words, m, opts.tol, opts.max_iters, st, slices)));
        }
        MX_TRY(cudaEventRecord(w.ev[2], st));
        MX_TRY(read_words(8));
        if (((int *)(hw + 3))[1] != 0) return lla__set_status(err, LLA_ERR_TIMEOUT);
        const int stv = ((int *)(hw + 4))[0];
        if (stv != 0 || enqueued >= opts.max_iters) {
            lowp_ok = stv != 3;
            converged = stv == 1;
            r.iterations = ((int *)(hw + 4))[1];
            eta = lowp_ok ? hw[5] : INFINITY;
            r.backward_error0 = lowp_ok ? hw[7] : 0.0;
            break;
        }
        group = kRefineGroupNext;
    }
    r.factor_failed = lowp_ok ? 0 : 1;
    {
        float f = 0.f, g = 0.f;
        MX_TRY(cudaEventElapsedTime(&f, w.ev[0], w.ev[1]));
        MX_TRY(cudaEventElapsedTime(&g, w.ev[1], w.ev[2]));
        r.ms_factor = f;  // device time: equilibration, factorisation, block inverses, slices of A
        r.ms_refine = g;  // device time of the refinement iterations (including the enqueued extras)
    }
    (void)t0;
    r.backward_error = eta;
    r.converged = converged ? 1 : 0;
    if (!converged) {
        if (!opts.fallback) {
            if (rep) *rep = r;
            return lla__set_status(err, LLA_ERR_NOT_CONVERGED);
        }
        // 4. plain FP64 fallback
        t0 = std::chrono::steady_clock::now();
        r.fell_back = 1;
        MX_TRY(w.F.ensure(sizeof(double) * n * n));
        MX_TRY(w.fdiag.ensure(sizeof(double) * n));
        double *F = (double *)w.F.p;
        MX_TRY(cudaMemcpy2DAsync(F, sizeof(double) * n, dA, sizeof(double) * lda, sizeof(double) * n, n,
                                 cudaMemcpyDeviceToDevice, st));
        const double big = 1e300;
        int64_t minus1 = -1;
        MX_TRY(cudaMemcpyAsync(info, &minus1, sizeof(int64_t), cudaMemcpyHostToDevice, st));
        MX_TRY(cudaMemcpyAsync(min_ratio, &big, sizeof(double), cudaMemcpyHostToDevice, st));
        MX_TRY(last_err(potrf_fast_launch<double>(F, n, n, info, (double *)w.fdiag.p, min_ratio, st)));
        MX_TRY(read_words(4));
        int64_t finfo;
        std::memcpy(&finfo, hw + 2, sizeof(int64_t));
        if (finfo >= 0 || !(hw[1] >= kFallbackPivotGuard)) {
            // A failed or near-singular FMA-order factorisation: the verdict is
            // decided by a factorisation in the reference's own operation order
            // (src/cholesky.rs:51-76), whose first failing row is returned.
            MX_TRY(w.S.ensure(sizeof(double) * n * n));
            MX_TRY(cudaMemcpy2DAsync(F, sizeof(double) * n, dA, sizeof(double) * lda, sizeof(double) * n, n,
                                     cudaMemcpyDeviceToDevice, st));
            MX_TRY(cudaMemcpyAsync(info, &minus1, sizeof(int64_t), cudaMemcpyHostToDevice, st));
            MX_TRY(last_err(potrf_exact_launch<double>(F, (double *)w.S.p, (double *)w.fdiag.p, n, n, info, st)));
            MX_TRY(read_words(4));
            std::memcpy(&finfo, hw + 2, sizeof(int64_t));
        }
        if (finfo >= 0) {
            r.ms_fallback = ms_since(t0);
            if (rep) *rep = r;
            lla__set_status(err, LLA_NOT_POSITIVE_DEFINITE);
            if (err) err->index = finfo;
            return LLA_NOT_POSITIVE_DEFINITE;
        }
        MX_TRY(cudaMemcpy2DAsync(dX, sizeof(double) * ldx, dB, sizeof(double) * ldb, sizeof(double) * n,
                                 m, cudaMemcpyDeviceToDevice, st));
        MX_TRY(cudaMemsetAsync(err_word, 0, sizeof(int), st));
        MX_TRY(last_err(trsm_launch<double>(F, n, n, 1, 0, nullptr, dX, ldx, m, false, tws, err_word, st)));
        MX_TRY(last_err(trsm_launch<double>(F, n, n, 0, 1, nullptr, dX, ldx, m, false, tws, err_word, st)));
        MX_TRY(cudaMemsetAsync(colmax_r, 0, sizeof(double) * 2 * m, st));
        MX_TRY(last_err(colmax_launch(dX, ldx, n, m, colmax_x, st)));
        MX_TRY(last_err(residual_launch(dA, lda, n, dX, ldx, dB, ldb, R, n, m, colmax_r,
                                        (double *)w.P.p, st)));
        MX_TRY(read_words(8 + 3 * m));
        if (((int *)(hw + 3))[1] != 0) {  // a substitution's bounded wait gave up: X is not valid
            r.ms_fallback = ms_since(t0);
            if (rep) *rep = r;
            return lla__set_status(err, LLA_ERR_TIMEOUT);
        }
        double e = 0.0;
        for (int64_t j = 0; j < m; ++j) {
            const double den = hw[0] * hw[8 + m + j] + hw[8 + 2 * m + j];
            e = std::max(e, den > 0 ? hw[8 + j] / den : 0.0);
        }
        r.backward_error = e;
        r.ms_fallback = ms_since(t0);
    }
    r.ms_total = ms_since(t_start);
    if (rep) *rep = r;
    return LLA_OK;
}

extern "C" int lla_refine_autotune(const double *dA, int64_t n, int64_t lda, const double *dB, int64_t m,
                                   int64_t ldb, double *dX, int64_t ldx, lla_refine_opts *opts, double *best_ms,
                                   void *stream, lla_error *err) {
    if (!opts) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    const lla_refine_opts base = *opts;
    struct Cand {
        int kc, epi, sub;
    };
    const Cand cands[] = {{64, 1, LLA_SUB_LOOKBACK}, {32, 1, LLA_SUB_LOOKBACK}, {32, 2, LLA_SUB_LOOKBACK},
                          {64, 1, LLA_SUB_CHAIN},    {32, 2, LLA_SUB_CHAIN}};
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return lla__set_cuda_error(err, ce);
    }
    float best = 1e30f;
    Cand win = cands[0];
    int rc = LLA_OK;
    for (const Cand &c : cands) {
        lla_refine_opts o = base;
        o.update_kchunk = c.kc;
        o.update_epilogue = c.epi;
        o.substitution = c.sub;
        float tmin = 1e30f;
        bool ok = true;
        for (int rep = 0; rep < 2 && rc == LLA_OK; ++rep) {
            lla_refine_report r;
            if ((ce = cudaEventRecord(e0, st)) != cudaSuccess) break;
            rc = lla_dposv_refined_device(dA, n, lda, dB, m, ldb, dX, ldx, &o, &r, stream, err);
            if (rc != LLA_OK) break;
            float ms = 0.f;
            if ((ce = cudaEventRecord(e1, st)) != cudaSuccess || (ce = cudaEventSynchronize(e1)) != cudaSuccess ||
                (ce = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess)
                break;
            ok = ok && r.converged && !r.fell_back;
            tmin = ms < tmin ? ms : tmin;
        }
        if (rc != LLA_OK || ce != cudaSuccess) break;
        if (ok && tmin < best) {
            best = tmin;
            win = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != LLA_OK) return rc;
    if (ce != cudaSuccess) return lla__set_cuda_error(err, ce);
    if (best < 1e30f) {
        autotune_store(refine_key(n, m, base), (win.kc << 4) | win.epi, win.sub);
        opts->update_kchunk = win.kc;
        opts->update_epilogue = win.epi;
        opts->substitution = win.sub;
        if (best_ms) *best_ms = best;
    }
    return LLA_OK;
}

extern "C" int lla_dresidual_device(const double *dA, int64_t n, int64_t lda, const double *dX, int64_t ldx,
                                    const double *dB, int64_t ldb, double *dR, int64_t ldr, int64_t m,
                                    int method, void *stream, lla_error *err) {
    if (n < 0 || m < 0 || lda < std::max<int64_t>(1, n) || ldx < std::max<int64_t>(1, n) ||
        ldb < std::max<int64_t>(1, n) || ldr < std::max<int64_t>(1, n) ||
        (n > 0 && m > 0 && (!dA || !dX || !dB || !dR)) ||
        (method != LLA_RESIDUAL_FP64 && method != LLA_RESIDUAL_EXACT_SLICES))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (n == 0 || m == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    MixedWs &w = c->mixed;
    MX_TRY(w.words.ensure(sizeof(double) * (8 + 3 * m)));
    double *colmax_r = (double *)w.words.p + 8, *colmax_x = colmax_r + m;
    int *err_word = (int *)((double *)w.words.p + 3) + 1;
    MX_TRY(cudaMemsetAsync(w.words.p, 0, sizeof(double) * (8 + 3 * m), st));
    if (method == LLA_RESIDUAL_FP64) {
        MX_TRY(w.P.ensure(sizeof(double) * n * m * residual_splits(n, m)));
        MX_TRY(last_err(residual_launch(dA, lda, n, dX, ldx, dB, ldb, dR, ldr, m, colmax_r,
                                        (double *)w.P.p, st)));
    } else {
        MX_TRY(w.oz.ensure(oz_workspace_bytes(n, m)));
        MX_TRY(last_err(oz_prepare(dA, lda, n, m, w.oz.p, false, st)));
        MX_TRY(last_err(colmax_launch(dX, ldx, n, m, colmax_x, st)));
        MX_TRY(last_err(oz_residual_launch(dX, ldx, dB, ldb, dR, ldr, n, m, colmax_x, colmax_r, w.oz.p,
                                           err_word, st)));
    }
    int flag = 0;
    MX_TRY(cudaMemcpyAsync(&flag, err_word, sizeof(int), cudaMemcpyDeviceToHost, st));
    MX_TRY(cudaStreamSynchronize(st));
    if (flag) return lla__set_status(err, flag);
    return LLA_OK;
}

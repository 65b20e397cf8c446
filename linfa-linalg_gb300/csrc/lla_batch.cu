// lla_batch.cu -- thousands of independent SPD systems of uneven order in one
// persistent launch.
//
// Layout: the caller packs every system's A_i (n_i x n_i, column-major,
// ld = n_i) into one "A pool" and every B_i (n_i x m_i, ld = n_i) into a "B
// pool" at offsets chosen by the plan.  A plan sorts the systems by
// decreasing cost (n^3/3 + 2 n^2 m) into a device work list; a persistent
// kernel of (CTAs per SM) x (#SMs) blocks takes items from an atomic counter
// (largest first, so the tail is short) and, inside one CTA per system:
//   * factors A_i in place, right-looking with 32-column blocks: one warp
//     factors the diagonal block with register shuffles, one thread per row
//     solves the rows below it into a shared-memory panel, all threads update
//     the trailing lower triangle from that panel (L2-resident);
//   * solves L L^T X = B in place, 32-row blocks: one warp per right-hand side
//     solves each diagonal block with shuffles, all threads update the rows
//     below (above) from it.
// A non-positive pivot stops that system only: info[i] = first failing row
// (-1 when the system solved).  The (CTAs per SM, threads) shape is chosen per
// batch by lla_batch_autotune and cached on disk.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/lla_gb300.h"
#include "lla_autotune.h"
#include "lla_common.cuh"
#include "lla_kernels.h"
#include "lla_prof.h"

namespace lla {

constexpr int kBNb = 32;                // block width
constexpr int kBMaxN = kBatchMaxN;      // largest order a batch system may have
constexpr int kBMaxRhs = kBatchMaxRhs;  // right-hand sides per system

template <typename T>
__device__ __forceinline__ T shfl(T v, int src) {
    return __shfl_sync(0xffffffffu, v, src);
}

// One warp: Cholesky of the bs x bs block at sD (row-major [32][33] in shared
// memory); returns the first failing local row or -1.  Lane i holds row i.
template <typename T>
__device__ int warp_potrf32(T *sD, int bs, int lane) {
    T v[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = (lane < bs && c <= lane) ? sD[lane * 33 + c] : T(0);
    int fail = -1;
#pragma unroll
    for (int c = 0; c < 32; ++c) {
        if (c < bs && fail < 0) {
            const T piv = shfl(v[c], c);
            if (!(piv > T(0))) {
                fail = c;  // non-positive pivot (NaN does not fail, as in the reference: `d <= 0`)
                if (piv != piv) fail = -1;
            }
            if (fail < 0) {
                const T lcc = sqrt(piv);
                if (lane == c) v[c] = lcc;
                if (lane > c) v[c] = v[c] / lcc;
#pragma unroll
                for (int c2 = c + 1; c2 < 32; ++c2) {
                    const T t = shfl(v[c], c2);
                    if (c2 < bs && lane >= c2) v[c2] = fma(-v[c], t, v[c2]);
                }
            }
        }
    }
    if (lane < bs) {
#pragma unroll
        for (int c = 0; c < 32; ++c)
            if (c <= lane) sD[lane * 33 + c] = v[c];
    }
    return fail;
}

// Factor-and-solve of one system by the whole CTA: A (n x n, column-major,
// ld = n) is factored in place (L in the lower triangle), B (n x m, leading
// dimension ldb) is overwritten with X.  sD: [32][33], sP: [kBMaxN][33] shared
// scratch.  Returns the first failing row (non-positive pivot) or -1; every
// thread returns the same value.
template <typename T>
__device__ int batch_factor(T *A, int n, T *sD, T *sP, int *s_fail) {
    const int tid = threadIdx.x, nthr = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarps = nthr >> 5;
    if (tid == 0) *s_fail = -1;
    __syncthreads();
    // ---- factor: right-looking, 32-column blocks ----
    for (int kb = 0; kb < n; kb += kBNb) {
        const int bs = min(kBNb, n - kb);
        for (int e = tid; e < 32 * 32; e += nthr) {
            const int r = e % 32, c = e / 32;
            if (r < bs && c <= r) sD[r * 33 + c] = A[(kb + r) + (int64_t)(kb + c) * n];
        }
        __syncthreads();
        if (warp == 0) {
            const int f = warp_potrf32(sD, bs, lane);
            if (lane == 0 && f >= 0) *s_fail = kb + f;
        }
        __syncthreads();
        if (*s_fail >= 0) break;
        for (int e = tid; e < 32 * 32; e += nthr) {
            const int r = e % 32, c = e / 32;
            if (r < bs && c <= r) A[(kb + r) + (int64_t)(kb + c) * n] = sD[r * 33 + c];
        }
        // panel: each row below the block solves against L_kk
        const int q = kb + bs, rows = n - q;
        for (int rr = tid; rr < rows; rr += nthr) {
            const int r = q + rr;
            T v[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) v[c] = (c < bs) ? A[r + (int64_t)(kb + c) * n] : T(0);
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                if (c < bs) {
                    v[c] = v[c] / sD[c * 33 + c];
#pragma unroll
                    for (int c2 = c + 1; c2 < 32; ++c2)
                        if (c2 < bs) v[c2] = fma(-v[c], sD[c2 * 33 + c], v[c2]);
                }
            }
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                if (c < bs) {
                    sP[rr * 33 + c] = v[c];
                    A[r + (int64_t)(kb + c) * n] = v[c];
                }
            }
        }
        __syncthreads();
        // trailing lower triangle, one column per warp, lanes over rows:
        // A[i,j] -= sum_t P[i][t] P[j][t]
        for (int j = warp; j < rows; j += nwarps) {
            for (int i = j + lane; i < rows; i += 32) {
                T acc = A[(q + i) + (int64_t)(q + j) * n];
#pragma unroll 8
                for (int t = 0; t < bs; ++t) acc = fma(-sP[i * 33 + t], sP[j * 33 + t], acc);
                A[(q + i) + (int64_t)(q + j) * n] = acc;
            }
        }
        __syncthreads();
    }
    const int fail = *s_fail;
    __syncthreads();
    return fail;
}

// L L^T X = B in place for the factor in the lower triangle of A (ld = n).
template <typename T>
__device__ void batch_trsolve(const T *A, int n, T *B, int64_t ldb, int m, T *sD, T *sP) {
    const int tid = threadIdx.x, nthr = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarps = nthr >> 5;
    // ---- solve L y = b (forward), then L^T x = y (backward), 32-row blocks ----
    for (int pass = 0; pass < 2; ++pass) {
        const bool fwd = pass == 0;
        const int nblk = (n + kBNb - 1) / kBNb;
        for (int bi = 0; bi < nblk; ++bi) {
            const int kb = (fwd ? bi : nblk - 1 - bi) * kBNb;
            const int bs = min(kBNb, n - kb);
            for (int e = tid; e < 32 * 32; e += nthr) {
                const int r = e % 32, c = e / 32;
                if (r < bs && c <= r) sD[r * 33 + c] = A[(kb + r) + (int64_t)(kb + c) * n];
            }
            __syncthreads();
            // warp k solves right-hand side k on this block (lane = row)
            for (int k = warp; k < m; k += nwarps) {
                T x = (lane < bs) ? B[(kb + lane) + (int64_t)k * ldb] : T(0);
                if (fwd) {
#pragma unroll
                    for (int c = 0; c < 32; ++c) {
                        if (c < bs) {
                            const T xc = shfl(x, c) / sD[c * 33 + c];
                            if (lane == c) x = xc;
                            if (lane > c && lane < bs) x = fma(-xc, sD[lane * 33 + c], x);
                        }
                    }
                } else {
#pragma unroll
                    for (int cc = 31; cc >= 0; --cc) {
                        if (cc < bs) {
                            const T xc = shfl(x, cc) / sD[cc * 33 + cc];
                            if (lane == cc) x = xc;
                            if (lane < cc) x = fma(-xc, sD[cc * 33 + lane], x);
                        }
                    }
                }
                if (lane < bs) B[(kb + lane) + (int64_t)k * ldb] = x;
            }
            // stage the block's coupling to the remaining rows: forward needs
            // L[r][kb+t] for r >= kb+bs, backward L[kb+t][r] for r < kb
            const int q = fwd ? kb + bs : 0, rows = fwd ? n - kb - bs : kb;
            for (int e = tid; e < rows * bs; e += nthr) {
                if (fwd) {
                    const int rr = e % rows, t = e / rows;  // consecutive rr: contiguous column
                    sP[rr * 33 + t] = A[(q + rr) + (int64_t)(kb + t) * n];
                } else {
                    const int t = e % bs, rr = e / bs;  // consecutive t: contiguous column rr
                    sP[rr * 33 + t] = A[(kb + t) + (int64_t)rr * n];
                }
            }
            __syncthreads();
            for (int e = tid; e < rows * m; e += nthr) {
                const int rr = e % rows, k = e / rows;
                T acc = B[(q + rr) + (int64_t)k * ldb];
#pragma unroll 8
                for (int t = 0; t < bs; ++t) acc = fma(-sP[rr * 33 + t], B[(kb + t) + (int64_t)k * ldb], acc);
                B[(q + rr) + (int64_t)k * ldb] = acc;
            }
            __syncthreads();
        }
    }
}

template <typename T>
__device__ int batch_solve_one(T *A, int n, T *B, int64_t ldb, int m, T *sD, T *sP, int *s_fail) {
    const int f = batch_factor<T>(A, n, sD, sP, s_fail);
    if (f >= 0) return f;
    batch_trsolve<T>(A, n, B, ldb, m, sD, sP);
    return -1;
}

template <typename T>
__global__ void __launch_bounds__(256, 2) batch_posv_kernel(const BatchItem *__restrict__ items, int64_t count, T *Apool,
                                  T *Bpool, int32_t *info, int *counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sD = (T *)smem_raw;  // [32][33] diagonal block
    T *sP = sD + 32 * 33;   // [kBMaxN][33] panel / block rows (row r at sP[r * 33])
    __shared__ int s_item, s_fail;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int64_t it = s_item;
        if (it >= count) break;
        const BatchItem w = items[it];
        const int f = batch_solve_one<T>(Apool + w.a_off, w.n, Bpool + w.b_off, w.n, w.m, sD, sP, &s_fail);
        if (tid == 0) info[w.idx] = f;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// f64 systems through an FP32 factorisation with FP64 refinement, per system
//
// One CTA per system, as above: the lower triangle of A (FP64, read only) is
// copied to FP32 scratch and factored there; x = 0, r = b; each iteration
// solves L L^T d = fp32(r) in FP32, adds d to x in FP64 and forms
// r = b - A x in FP64 from the lower triangle of A (one thread per row,
// sym_residual).  It stops when the normwise backward error
// max_j ||r_j|| / (||A|| ||x_j|| + ||b_j||) reaches n eps / 16, or once a
// correction no longer halves it.  A system whose FP32 factorisation breaks down, or that ends
// above 10 n eps, is solved again by the plain FP64 routine (whose verdict
// stands) from a working copy of A.  FP64 arithmetic is the scarce resource
// on this GPU: the factorisation (n^3/3) moves to the FP32 pipe and only
// 2 n^2 m per iteration stays in FP64.
constexpr int kBRefIters = 5;
// Stop at n eps / 16 (about what the plain FP64 batched solve reaches); a
// system left above 10 n eps is re-solved in plain FP64.
constexpr double kBRefTolPerN = 2.220446049250313e-16 / 16.0;
constexpr size_t kBRefScratch = (size_t)kBMaxN * kBMaxN * 8 + (size_t)kBMaxN * kBMaxRhs * (4 + 8);

// Column maxima of |X| and |R| (m <= kBMaxRhs columns each) over the CTA in one
// reduction: vx, vr hold this thread's partial maxima; on return every thread
// holds the CTA's.  red: 8 warps x 2 kBMaxRhs doubles of shared memory.
__device__ __forceinline__ void block_max_cols(double (&vx)[kBMaxRhs], double (&vr)[kBMaxRhs], double *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < kBMaxRhs; ++j)
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            vx[j] = fmax(vx[j], __shfl_xor_sync(0xffffffffu, vx[j], o));
            vr[j] = fmax(vr[j], __shfl_xor_sync(0xffffffffu, vr[j], o));
        }
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < kBMaxRhs; ++j) {
            red[warp * 2 * kBMaxRhs + j] = vx[j];
            red[warp * 2 * kBMaxRhs + kBMaxRhs + j] = vr[j];
        }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kBMaxRhs; ++j) {
        vx[j] = 0.0;
        vr[j] = 0.0;
        for (int w = 0; w < nw; ++w) {
            vx[j] = fmax(vx[j], red[w * 2 * kBMaxRhs + j]);
            vr[j] = fmax(vr[j], red[w * 2 * kBMaxRhs + kBMaxRhs + j]);
        }
    }
}

// r = B - A_sym X for the lower triangle of A (ld n), X in shared memory
// (sX[k * kBMaxRhs + j]), one thread per row: the part k <= i along row i
// (consecutive rows read consecutive addresses), the part k > i down column
// i (each thread streams its own column through L1).  M right-hand sides at
// compile time, so the scarce FP64 pipe spends no issue slot on absent
// columns and no lane waits on a shuffle reduction.
template <int M>
__device__ void sym_residual_m(const double *A, int n, const double *sX, const double *B, double *out) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double acc[M];
#pragma unroll
        for (int j = 0; j < M; ++j) acc[j] = 0.0;
        for (int k = 0; k <= i; ++k) {
            const double a = A[i + (int64_t)k * n];
#pragma unroll
            for (int j = 0; j < M; ++j) acc[j] = fma(a, sX[k * kBMaxRhs + j], acc[j]);
        }
        const double *col = A + (int64_t)i * n;
        for (int k = i + 1; k < n; ++k) {
            const double a = col[k];
#pragma unroll
            for (int j = 0; j < M; ++j) acc[j] = fma(a, sX[k * kBMaxRhs + j], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < M; ++j) out[i + (int64_t)j * n] = B[i + (int64_t)j * n] - acc[j];
    }
    __syncthreads();
}

__device__ void sym_residual(const double *A, int n, const double *sX, int m, const double *B, double *out) {
    switch (m) {
        case 1: sym_residual_m<1>(A, n, sX, B, out); break;
        case 2: sym_residual_m<2>(A, n, sX, B, out); break;
        case 3: sym_residual_m<3>(A, n, sX, B, out); break;
        case 4: sym_residual_m<4>(A, n, sX, B, out); break;
        case 5: sym_residual_m<5>(A, n, sX, B, out); break;
        case 6: sym_residual_m<6>(A, n, sX, B, out); break;
        case 7: sym_residual_m<7>(A, n, sX, B, out); break;
        default: sym_residual_m<8>(A, n, sX, B, out); break;
    }
}

// out[i] = sum_k |A_sym(i, k)| (the same traversal).
__device__ void sym_rowsum(const double *A, int n, double *out) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k <= i; ++k) s += fabs(A[i + (int64_t)k * n]);
        const double *col = A + (int64_t)i * n;
        for (int k = i + 1; k < n; ++k) s += fabs(col[k]);
        out[i] = s;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256, 2) batch_posv_refined_kernel(const BatchItem *__restrict__ items, int64_t count,
                                                                   const double *Apool, double *Bpool,
                                                                   int32_t *info, int *counter, char *scratch) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sDd = (double *)smem_raw;  // FP64 fallback: [32][33] + [kBMaxN][33]
    float *sDf = (float *)smem_raw;    // FP32 factor and solves (same space)
    double *sX = (double *)(smem_raw + sizeof(double) * (32 * 33 + kBMaxN * 33));  // [kBMaxN][kBMaxRhs]
    __shared__ int s_item, s_fail;
    __shared__ double red[8 * 2 * kBMaxRhs];
    __shared__ double s_cb[kBMaxRhs];
    const int tid = threadIdx.x, nthr = blockDim.x;
    char *base = scratch + (size_t)blockIdx.x * kBRefScratch;
    float *W = (float *)base;  // FP32 factor (ld n); the FP64 fallback's working copy uses the same space
    double *Wd = (double *)base;
    float *R32 = (float *)(base + (size_t)kBMaxN * kBMaxN * 8);
    double *R = (double *)(R32 + kBMaxN * kBMaxRhs);
    for (;;) {
        if (tid == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int64_t it = s_item;
        if (it >= count) break;
        const BatchItem w = items[it];
        const int n = w.n, m = w.m;
        const double *A = Apool + w.a_off;
        double *B = Bpool + w.b_off;
        for (int64_t e = tid; e < (int64_t)n * n; e += nthr) {
            const int i = (int)(e % n), k = (int)(e / n);
            if (i >= k) W[e] = (float)A[e];
        }
        // ||A||_inf and ||b_j||_inf
        sym_rowsum(A, n, R);
        double an = 0.0;
        {
            double vb[kBMaxRhs], va[kBMaxRhs];
#pragma unroll
            for (int j = 0; j < kBMaxRhs; ++j) vb[j] = va[j] = 0.0;
            for (int i = tid; i < n; i += nthr) {
                va[0] = fmax(va[0], R[i]);
#pragma unroll
                for (int j = 0; j < kBMaxRhs; ++j)
                    if (j < m) vb[j] = fmax(vb[j], fabs(B[i + (int64_t)j * n]));
            }
            block_max_cols(vb, va, red);
            an = va[0];
#pragma unroll
            for (int j = 0; j < kBMaxRhs; ++j)
                if (tid == j) s_cb[j] = vb[j];
        }
        __syncthreads();
        const double tol = kBRefTolPerN * n;
        int f = batch_factor<float>(W, n, sDf, sDf + 32 * 33, &s_fail);
        bool ok = f < 0;
        if (ok) {
            for (int e = tid; e < n * kBMaxRhs; e += nthr) sX[e] = 0.0;
            for (int64_t e = tid; e < (int64_t)n * m; e += nthr) R[e] = B[e];
            __syncthreads();
            double eta = INFINITY, eta_prev = INFINITY;
            for (int itr = 0; itr < kBRefIters; ++itr) {
                for (int64_t e = tid; e < (int64_t)n * m; e += nthr) R32[e] = (float)R[e];
                __syncthreads();
                batch_trsolve<float>(W, n, R32, n, m, sDf, sDf + 32 * 33);
                for (int64_t e = tid; e < (int64_t)n * m; e += nthr) {
                    const int i = (int)(e % n), j = (int)(e / n);
                    sX[i * kBMaxRhs + j] += (double)R32[e];
                }
                __syncthreads();
                sym_residual(A, n, sX, m, B, R);
                double vx[kBMaxRhs], vr[kBMaxRhs];
#pragma unroll
                for (int j = 0; j < kBMaxRhs; ++j) vx[j] = vr[j] = 0.0;
                for (int i = tid; i < n; i += nthr) {
#pragma unroll
                    for (int j = 0; j < kBMaxRhs; ++j)
                        if (j < m) {
                            vx[j] = fmax(vx[j], fabs(sX[i * kBMaxRhs + j]));
                            vr[j] = fmax(vr[j], fabs(R[i + (int64_t)j * n]));
                        }
                }
                block_max_cols(vx, vr, red);
                double e_max = 0.0;
#pragma unroll
                for (int j = 0; j < kBMaxRhs; ++j) {
                    if (j >= m) continue;
                    const double den = an * vx[j] + s_cb[j];
                    double ej = den > 0 ? vr[j] / den : (vr[j] > 0 ? INFINITY : 0.0);
                    if (ej != ej) ej = INFINITY;
                    e_max = fmax(e_max, ej);
                }
                eta = e_max;  // uniform across the CTA
                // done at the target, or once a correction no longer halves the error
                if (eta <= tol || !(eta < INFINITY) || (itr >= 1 && eta > 0.5 * eta_prev)) break;
                eta_prev = eta;
            }
            ok = eta <= 10.0 * n * 2.220446049250313e-16;
            if (ok) {
                for (int64_t e = tid; e < (int64_t)n * m; e += nthr) {
                    const int i = (int)(e % n), j = (int)(e / n);
                    B[e] = sX[i * kBMaxRhs + j];
                }
            }
        }
        if (!ok) {  // plain FP64 from a working copy of A (B still holds b)
            __syncthreads();
            for (int64_t e = tid; e < (int64_t)n * n; e += nthr) {
                const int i = (int)(e % n), k = (int)(e / n);
                if (i >= k) Wd[e] = A[e];
            }
            __syncthreads();
            f = batch_solve_one<double>(Wd, n, B, n, m, sDd, sDd + 32 * 33, &s_fail);
        } else {
            f = -1;
        }
        if (tid == 0) info[w.idx] = f;
        __syncthreads();
    }
}

size_t batch_refined_smem() { return sizeof(double) * (32 * 33 + kBMaxN * 33 + kBMaxN * kBMaxRhs); }
size_t batch_refined_scratch_bytes(int ctas) { return (size_t)ctas * kBRefScratch; }

// ---------------------------------------------------------------------------
// device-resident serving loop

__device__ __forceinline__ unsigned long long ld_acquire_sys_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Persistent CTAs of 256 threads.  Thread 0 claims the next published ticket
// (compare-and-swap on the device counter, so a ticket is claimed at most once
// and only after the host published it), the CTA copies the lower triangle of
// A into its scratch (ld = n) and solves in place with the batched routine;
// thread 0 then publishes the outcome.  Every wait is bounded: an idle CTA
// returns after idle_ns without work (the host relaunches the loop when new
// requests arrive), at once when ring->stop is set.
__global__ void __launch_bounds__(256) serve_loop_kernel(ServeRing *ring, unsigned long long *next,
                                                        double *scratch, unsigned long long idle_ns) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_ticket;
    __shared__ int s_fail;
    __shared__ ServeReq s_req;
    const int tid = threadIdx.x;
    double *myA = scratch + (size_t)blockIdx.x * kBMaxN * kBMaxN;
    for (;;) {
        if (tid == 0) {
            long long claim = -1;
            const unsigned long long t_idle = globaltimer_ns();
            unsigned sleep_ns = 64;
            for (;;) {
                const unsigned long long cur = atomicAdd(next, 0ull);
                const unsigned long long pub = ld_acquire_sys_u64(&ring->published);
                if (cur < pub) {
                    if (atomicCAS(next, cur, cur + 1) == cur) {
                        claim = (long long)cur;
                        break;
                    }
                    continue;
                }
                if (*(volatile int *)&ring->stop) break;
                if (globaltimer_ns() - t_idle > idle_ns) break;
                __nanosleep(sleep_ns);
                if (sleep_ns < 2048) sleep_ns *= 2;
            }
            s_ticket = claim;
            if (claim >= 0) {
                // the host wrote the slot before it raised `published` (acquired above)
                const ServeReq *q = &ring->req[claim % kServeRing];
                s_req.A = *(void *const volatile *)&q->A;
                s_req.B = *(void *volatile *)&q->B;
                s_req.lda = *(volatile const int64_t *)&q->lda;
                s_req.ldb = *(volatile const int64_t *)&q->ldb;
                s_req.n = *(volatile const int32_t *)&q->n;
                s_req.m = *(volatile const int32_t *)&q->m;
                s_req.dtype = *(volatile const int32_t *)&q->dtype;
            }
        }
        __syncthreads();
        const long long t = s_ticket;
        if (t < 0) break;
        const ServeReq q = s_req;
        const int n = q.n;
        int f;
        if (q.dtype == 8) {
            double *W = myA;
            const double *A = (const double *)q.A;
            for (int64_t e = tid; e < (int64_t)n * n; e += blockDim.x) {
                const int i = (int)(e % n), j = (int)(e / n);
                if (i >= j) W[e] = A[i + (int64_t)j * q.lda];
            }
            __syncthreads();
            double *sD = (double *)smem_raw;
            f = batch_solve_one<double>(W, n, (double *)q.B, q.ldb, q.m, sD, sD + 32 * 33, &s_fail);
        } else {
            float *W = (float *)myA;
            const float *A = (const float *)q.A;
            for (int64_t e = tid; e < (int64_t)n * n; e += blockDim.x) {
                const int i = (int)(e % n), j = (int)(e / n);
                if (i >= j) W[e] = A[i + (int64_t)j * q.lda];
            }
            __syncthreads();
            float *sD = (float *)smem_raw;
            f = batch_solve_one<float>(W, n, (float *)q.B, q.ldb, q.m, sD, sD + 32 * 33, &s_fail);
        }
        __syncthreads();  // every thread's writes of X precede the publication
        if (tid == 0) {
            const int slot = (int)(t % kServeRing);
            __threadfence_system();
            *(volatile int32_t *)&ring->status[slot] = f >= 0 ? 1 : 0;
            *(volatile int64_t *)&ring->fail_row[slot] = f;
            st_release_sys_u64(&ring->done_seq[slot], (unsigned long long)t + 1);
        }
    }
}

size_t serve_loop_scratch_bytes(int ctas) { return (size_t)ctas * kBMaxN * kBMaxN * sizeof(double); }

int serve_loop_launch(ServeRing *ring_dev, unsigned long long *d_next, double *scratch, int ctas,
                      double idle_us, cudaStream_t st) {
    const size_t smem = sizeof(double) * (32 * 33 + kBMaxN * 33);
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(serve_loop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return -1;
        attr = true;
    }
    LaunchScope ls(K_BATCH, st);
    serve_loop_kernel<<<(unsigned)ctas, 256, smem, st>>>(ring_dev, d_next, scratch,
                                                         (unsigned long long)(idle_us * 1e3));
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace lla

// ---------------------------------------------------------------------------
// plan, autotune cache, launch

using namespace lla;

struct lla_batch_plan {
    int64_t count = 0;
    int dtype = 8;
    std::vector<int32_t> n, m;
    std::vector<int64_t> a_off, b_off;
    int64_t a_elems = 0, b_elems = 0;
    double flops = 0.0;
    BatchItem *d_items = nullptr;
    int *d_counter = nullptr;
    int ctas_per_sm = 2, threads = 256;
    bool tuned = false;
    bool refined = false;   // f64 systems through an FP32 factor + FP64 refinement (A read only)
    char *d_scratch = nullptr;  // per-CTA scratch of the refined mode
    std::string key;
    // graph replay cache
    cudaGraphExec_t gexec = nullptr;
    void *g_a = nullptr, *g_b = nullptr, *g_info = nullptr;
    cudaStream_t g_stream = nullptr;
};

static size_t batch_smem(int dtype) { return (size_t)dtype * (32 * 33 + (size_t)kBMaxN * 33); }

static bool cache_lookup(const std::string &key, int &cps, int &thr) { return lla::autotune_lookup(key, cps, thr); }
static void cache_store(const std::string &key, int cps, int thr) { lla::autotune_store(key, cps, thr); }

static int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

namespace lla {

template <typename T>
int batch_launch_raw(const BatchItem *d_items, int64_t count, T *dA, T *dB, int32_t *d_info,
                     int *d_counter, int ctas_per_sm, int threads, double flops, cudaStream_t st) {
    if (count <= 0) return 0;
    if (cudaMemsetAsync(d_counter, 0, sizeof(int), st) != cudaSuccess) return -1;
    static bool attr[2] = {false, false};
    const size_t smem = batch_smem(sizeof(T));
    if (!attr[sizeof(T) == 8]) {
        if (cudaFuncSetAttribute(batch_posv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        attr[sizeof(T) == 8] = true;
    }
    const unsigned grid =
        (unsigned)std::max<int64_t>(1, std::min<int64_t>(count, (int64_t)ctas_per_sm * sm_count()));
    LaunchScope ls(K_BATCH, st, flops);
    batch_posv_kernel<T><<<grid, threads, smem, st>>>(d_items, count, dA, dB, d_info, d_counter);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template int batch_launch_raw<double>(const BatchItem *, int64_t, double *, double *, int32_t *, int *,
                                      int, int, double, cudaStream_t);
template int batch_launch_raw<float>(const BatchItem *, int64_t, float *, float *, int32_t *, int *, int,
                                     int, double, cudaStream_t);

}  // namespace lla

// The refined mode's CTAs per SM are limited by its shared memory (two fit).
static int refined_ctas_per_sm(int cps) { return std::min(cps, 2); }

template <typename T>
static cudaError_t batch_launch(lla_batch_plan *p, T *dA, T *dB, int32_t *d_info, cudaStream_t st) {
    if (p->refined && sizeof(T) == 8) {
        if (cudaMemsetAsync(p->d_counter, 0, sizeof(int), st) != cudaSuccess) return cudaGetLastError();
        const int cps = refined_ctas_per_sm(p->ctas_per_sm);
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(p->count, (int64_t)cps * sm_count()));
        LaunchScope ls(K_BATCH, st, p->flops);
        batch_posv_refined_kernel<<<grid, p->threads, batch_refined_smem(), st>>>(
            p->d_items, p->count, (const double *)dA, (double *)dB, d_info, p->d_counter, p->d_scratch);
        return cudaGetLastError();
    }
    if (batch_launch_raw<T>(p->d_items, p->count, dA, dB, d_info, p->d_counter, p->ctas_per_sm,
                            p->threads, p->flops, st) == 0)
        return cudaSuccess;
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? cudaErrorUnknown : e;
}

extern "C" {

int lla_batch_plan_create(int64_t count, const int32_t *n, const int32_t *m, int elem_bytes,
                          lla_batch_plan **out, lla_error *err) {
    if (!out || count < 0 || (count > 0 && (!n || !m)) || (elem_bytes != 4 && elem_bytes != 8))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    for (int64_t i = 0; i < count; ++i) {
        if (n[i] < 0 || m[i] < 0) return lla__set_status(err, LLA_ERR_INVALID_ARG);
        if (n[i] > kBMaxN || m[i] > kBMaxRhs) return lla__set_status(err, LLA_ERR_TOO_LARGE);
    }
    lla__set_status(err, LLA_OK);
    lla_batch_plan *p = new lla_batch_plan();
    p->count = count;
    p->dtype = elem_bytes;
    p->n.assign(n, n + count);
    p->m.assign(m, m + count);
    p->a_off.resize(count);
    p->b_off.resize(count);
    // pools in submission order, each system 16-byte aligned
    const int64_t align = 16 / elem_bytes;
    int64_t ao = 0, bo = 0;
    int hist[9] = {0};
    int maxm = 0;
    for (int64_t i = 0; i < count; ++i) {
        p->a_off[i] = ao;
        p->b_off[i] = bo;
        ao += ((int64_t)n[i] * n[i] + align - 1) / align * align;
        bo += ((int64_t)n[i] * m[i] + align - 1) / align * align;
        p->flops += (double)n[i] * n[i] * n[i] / 3.0 + 2.0 * n[i] * n[i] * m[i];
        int b = 0;
        while ((32 << b) < n[i] && b < 8) ++b;
        hist[b]++;
        maxm = std::max(maxm, (int)m[i]);
    }
    p->a_elems = ao;
    p->b_elems = bo;
    // work list: largest systems first
    std::vector<BatchItem> items(count);
    for (int64_t i = 0; i < count; ++i)
        items[i] = BatchItem{n[i], m[i], (int32_t)i, 0, p->a_off[i], p->b_off[i]};
    std::stable_sort(items.begin(), items.end(), [](const BatchItem &a, const BatchItem &b) {
        const double ca = (double)a.n * a.n * (a.n + 6.0 * a.m), cb = (double)b.n * b.n * (b.n + 6.0 * b.m);
        return ca > cb;
    });
    // autotune-cache key: element size, count, size-bucket histogram, widest RHS
    char key[256];
    std::snprintf(key, sizeof(key), "b%d:c%lld:h%d-%d-%d-%d-%d-%d-%d-%d-%d:m%d", elem_bytes,
                  (long long)count, hist[0], hist[1], hist[2], hist[3], hist[4], hist[5], hist[6],
                  hist[7], hist[8], maxm);
    p->key = key;
    int cps, thr;
    if (cache_lookup(p->key, cps, thr)) {
        p->ctas_per_sm = cps;
        p->threads = thr;
        p->tuned = true;
    }
    cudaError_t e = cudaMalloc(&p->d_items, sizeof(BatchItem) * std::max<int64_t>(1, count));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_counter, sizeof(int));
    if (e == cudaSuccess && count > 0)
        e = cudaMemcpy(p->d_items, items.data(), sizeof(BatchItem) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const size_t smem = batch_smem(elem_bytes);
        e = elem_bytes == 8 ? cudaFuncSetAttribute(batch_posv_kernel<double>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                            : cudaFuncSetAttribute(batch_posv_kernel<float>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    if (e != cudaSuccess) {
        cudaFree(p->d_items);
        cudaFree(p->d_counter);
        delete p;
        return lla__set_cuda_error(err, e);
    }
    *out = p;
    return LLA_OK;
}

void lla_batch_plan_destroy(lla_batch_plan *p) {
    if (!p) return;
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->d_scratch) cudaFree(p->d_scratch);
    cudaFree(p->d_items);
    cudaFree(p->d_counter);
    delete p;
}

int lla_batch_plan_info(const lla_batch_plan *p, int64_t *a_elems, int64_t *b_elems, int64_t *a_off,
                        int64_t *b_off, int *ctas_per_sm, int *threads, double *flops) {
    if (!p) return LLA_ERR_INVALID_ARG;
    if (a_elems) *a_elems = p->a_elems;
    if (b_elems) *b_elems = p->b_elems;
    if (a_off) std::memcpy(a_off, p->a_off.data(), sizeof(int64_t) * p->count);
    if (b_off) std::memcpy(b_off, p->b_off.data(), sizeof(int64_t) * p->count);
    if (ctas_per_sm) *ctas_per_sm = p->ctas_per_sm;
    if (threads) *threads = p->threads;
    if (flops) *flops = p->flops;
    return LLA_OK;
}

int lla_batch_set_shape(lla_batch_plan *p, int ctas_per_sm, int threads) {
    if (!p || ctas_per_sm < 1 || ctas_per_sm > 8 || (threads != 128 && threads != 256))
        return LLA_ERR_INVALID_ARG;
    if (p->ctas_per_sm != ctas_per_sm || p->threads != threads) {
        p->ctas_per_sm = ctas_per_sm;
        p->threads = threads;
        if (p->gexec) {
            cudaGraphExecDestroy(p->gexec);
            p->gexec = nullptr;
        }
    }
    return LLA_OK;
}

// Switches an f64 plan between the plain FP64 solve (A factored in place) and
// the FP32 factorisation with per-system FP64 refinement (A read only).
int lla_batch_set_refined(lla_batch_plan *p, int refined, lla_error *err) {
    if (!p || (refined && p->dtype != 8)) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    const bool want = refined != 0;
    if (want && !p->d_scratch) {
        static bool attr = false;
        if (!attr) {
            const cudaError_t e = cudaFuncSetAttribute(batch_posv_refined_kernel,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)batch_refined_smem());
            if (e != cudaSuccess) return lla__set_cuda_error(err, e);
            attr = true;
        }
        const cudaError_t e = cudaMalloc(&p->d_scratch, batch_refined_scratch_bytes(2 * sm_count()));
        if (e != cudaSuccess) {
            p->d_scratch = nullptr;
            return lla__set_cuda_error(err, e);
        }
    }
    if (p->refined != want) {
        p->refined = want;
        if (p->gexec) {
            cudaGraphExecDestroy(p->gexec);
            p->gexec = nullptr;
        }
        // the launch shape is cached per mode
        p->key += want ? ":r" : "";
        if (!want && p->key.size() > 2 && p->key.compare(p->key.size() - 2, 2, ":r") == 0)
            p->key.resize(p->key.size() - 2);
        int cps, thr;
        if (cache_lookup(p->key, cps, thr)) {
            p->ctas_per_sm = cps;
            p->threads = thr;
        }
    }
    return LLA_OK;
}

static int batch_posv(lla_batch_plan *p, void *dA, void *dB, int32_t *d_info, void *stream,
                      lla_error *err, int elem_bytes) {
    if (!p || p->dtype != elem_bytes || (p->count > 0 && (!dA || !dB || !d_info)))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (p->count == 0) return LLA_OK;
    cudaError_t e = elem_bytes == 8
                        ? batch_launch<double>(p, (double *)dA, (double *)dB, d_info, (cudaStream_t)stream)
                        : batch_launch<float>(p, (float *)dA, (float *)dB, d_info, (cudaStream_t)stream);
    return e == cudaSuccess ? LLA_OK : lla__set_cuda_error(err, e);
}

int lla_dbatch_posv_device(lla_batch_plan *p, double *dA, double *dB, int32_t *d_info, void *stream,
                           lla_error *err) {
    return batch_posv(p, dA, dB, d_info, stream, err, 8);
}

int lla_sbatch_posv_device(lla_batch_plan *p, float *dA, float *dB, int32_t *d_info, void *stream,
                           lla_error *err) {
    return batch_posv(p, dA, dB, d_info, stream, err, 4);
}

// Same work as lla_?batch_posv_device, replayed from a CUDA graph: the first
// call for a given (pools, info, stream) captures [counter reset, persistent
// kernel] and instantiates it; later calls launch the executable graph.
int lla_batch_posv_graph(lla_batch_plan *p, void *dA, void *dB, int32_t *d_info, void *stream,
                         lla_error *err) {
    if (!p || (p->count > 0 && (!dA || !dB || !d_info))) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (p->count == 0) return LLA_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    if (!p->gexec || p->g_a != dA || p->g_b != dB || p->g_info != d_info || p->g_stream != st) {
        if (p->gexec) {
            cudaGraphExecDestroy(p->gexec);
            p->gexec = nullptr;
        }
        cudaStream_t cap = nullptr;
        if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess)
            return lla__set_cuda_error(err, e);
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            prof_capturing() = true;
            const cudaError_t le = p->dtype == 8
                                       ? batch_launch<double>(p, (double *)dA, (double *)dB, d_info, cap)
                                       : batch_launch<float>(p, (float *)dA, (float *)dB, d_info, cap);
            prof_capturing() = false;
            e = cudaStreamEndCapture(cap, &g);
            if (le != cudaSuccess) e = le;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&p->gexec, g, 0);
        if (g) cudaGraphDestroy(g);
        cudaStreamDestroy(cap);
        if (e != cudaSuccess) return lla__set_cuda_error(err, e);
        p->g_a = dA;
        p->g_b = dB;
        p->g_info = d_info;
        p->g_stream = st;
    }
    {
        // one kernel per replay (plus the counter reset): counted and timed like a launch
        LaunchScope ls(K_BATCH, st, p->flops);
        e = cudaGraphLaunch(p->gexec, st);
    }
    return e == cudaSuccess ? LLA_OK : lla__set_cuda_error(err, e);
}

// Times every (CTAs per SM, threads) candidate on the caller's batch (A and B
// are restored from copies between trials, so the pools keep their inputs),
// keeps the fastest and appends it to the autotune cache file
// (LLA_AUTOTUNE_CACHE, default ~/.cache/lla_gb300_autotune.txt) under the
// batch's shape key.  best_ms (optional) receives the winner's time.
int lla_batch_autotune(lla_batch_plan *p, void *dA, void *dB, int32_t *d_info, void *stream,
                       double *best_ms, lla_error *err) {
    if (!p || (p->count > 0 && (!dA || !dB || !d_info))) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (p->count == 0) return LLA_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t abytes = (size_t)p->a_elems * p->dtype, bbytes = (size_t)p->b_elems * p->dtype;
    void *a0 = nullptr, *b0 = nullptr;
    cudaError_t e = cudaMalloc(&a0, abytes);
    if (e == cudaSuccess) e = cudaMalloc(&b0, bbytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a0, dA, abytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b0, dB, bbytes, cudaMemcpyDeviceToDevice, st);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int cands[][2] = {{1, 256}, {2, 256}, {3, 256}, {2, 128}, {3, 128}, {4, 128}};
    int best_c = p->ctas_per_sm, best_t = p->threads;
    float best = 1e30f;
    const size_t smem = batch_smem(p->dtype);
    for (const auto &c : cands) {
        if (e != cudaSuccess) break;
        if (smem * c[0] > 227 * 1024) continue;  // does not fit on one SM
        if (p->refined && c[0] > 2) continue;      // the refined kernel fits two CTAs per SM
        p->ctas_per_sm = c[0];
        p->threads = c[1];
        float tbest = 1e30f;
        for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
            e = cudaMemcpyAsync(dA, a0, abytes, cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(dB, b0, bbytes, cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaEventRecord(e0, st);
            if (e == cudaSuccess)
                e = p->dtype == 8 ? batch_launch<double>(p, (double *)dA, (double *)dB, d_info, st)
                                  : batch_launch<float>(p, (float *)dA, (float *)dB, d_info, st);
            if (e == cudaSuccess) e = cudaEventRecord(e1, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e == cudaSuccess) tbest = std::min(tbest, ms);
        }
        if (e == cudaSuccess && tbest < best) {
            best = tbest;
            best_c = c[0];
            best_t = c[1];
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(dA, a0, abytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dB, b0, bbytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(a0);
    cudaFree(b0);
    lla_batch_set_shape(p, best_c, best_t);
    if (e != cudaSuccess) return lla__set_cuda_error(err, e);
    p->tuned = true;
    cache_store(p->key, best_c, best_t);
    if (best_ms) *best_ms = best;
    return LLA_OK;
}

}  // extern "C"

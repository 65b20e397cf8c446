// lla_potrf.cu -- blocked Cholesky factorisation kernels (lower triangle,
// column-major device matrices) in two arithmetic modes.
//
// EXACT mode keeps the reference's per-element operation order
// (src/cholesky.rs:54-74): for every pair j > k the sum
//     s_jk = sum_{i<k} L[k,i] * L[j,i]
// is accumulated from zero in ascending i, then
//     L[j,k] = (A[j,k] - s_jk) / L[k,k],      d_j += L[j,k]^2   (ascending k),
//     L[j,j] = sqrt(A[j,j] - d_j)             (error when the pivot is <= 0).
// The reference evaluates these row by row; here the same sums are grown
// right-looking, one panel of columns at a time, in separate accumulator
// arrays S (n x n, lower part used) and D (n).  Every accumulator receives
// exactly the same products in exactly the same order, each multiply and add
// rounded separately, so the factor is bit-identical to the reference's.
//
// FAST mode is LAPACK-style right-looking (A22 -= L21 L21^T in place) with
// fused multiply-add; the FP64 trailing update runs on the FP64 tensor pipe
// (mma.sync m16n8k16 .f64), measured on GB300 at 1.05-1.10 TFLOP/s with
// GEMM-like operand use, about the DFMA rate (1.02 TFLOP/s): FP64 is the
// scarce resource on this GPU either way.
#include "lla_common.cuh"
#include "lla_kernels.h"
#include "lla_prof.h"

namespace lla {

// ---------------------------------------------------------------------------
// EXACT: diagonal block [p, p+b), b <= kNbExact, one CTA of 32 x 32 threads.
constexpr int kNbExact = 32;

template <typename T>
__global__ void __launch_bounds__(1024) potrf_exact_diag(T *W, const T *S, T *D, int64_t ld,
                                                         int64_t p, int b, int64_t *info) {
    using Ar = Arith<T>;
    __shared__ T a[kNbExact][kNbExact + 1];
    __shared__ T s[kNbExact][kNbExact + 1];
    __shared__ T d[kNbExact];
    __shared__ int failed;
    const int tx = threadIdx.x, ty = threadIdx.y;  // tx: column k, ty: row j
    if (*(volatile int64_t *)info >= 0) return;    // an earlier panel failed
    if (ty < b && tx <= ty) {
        a[ty][tx] = cm(W, ld, p + ty, p + tx);
        s[ty][tx] = (tx < ty) ? cm(S, ld, p + ty, p + tx) : T(0);
    }
    if (ty == 0 && tx < b) d[tx] = D[p + tx];
    if (tx == 0 && ty == 0) failed = 0;
    __syncthreads();
    int k = 0;
    for (; k < b; ++k) {
        if (tx == 0 && ty == 0) {
            const T dd = Ar::sub(a[k][k], d[k]);  // d = A[j,j] - d  (:66)
            if (dd <= T(0)) {                     // (:69) false for NaN
                failed = 1;
                *info = p + k;
            } else {
                a[k][k] = Ar::sqrt_(dd);  // (:73)
            }
        }
        __syncthreads();
        if (failed) break;
        const T lkk = a[k][k];
        if (ty == 0 && tx > k && tx < b) {
            const int j = tx;
            const T l = Ar::div(Ar::sub(a[j][k], s[j][k]), lkk);  // (:62)
            a[j][k] = l;
            d[j] = Ar::add(d[j], Ar::mul(l, l));  // (:64)
        }
        __syncthreads();
        // s_{j,k2} += L[k2,k] * L[j,k] for k < k2 < j   (:59-61, term i = k)
        if (ty < b && tx > k && tx < ty) s[ty][tx] = Ar::add(s[ty][tx], Ar::mul(a[tx][k], a[ty][k]));
        __syncthreads();
    }
    // Write back every value computed (on failure the host keeps only rows
    // < info and row info's strict lower part).
    if (ty < b && tx <= ty) cm(W, ld, p + ty, p + tx) = a[ty][tx];
}

// EXACT: rows [q, n) below the diagonal block, q = p + b; one thread per row.
template <typename T>
__global__ void __launch_bounds__(128) potrf_exact_panel(T *W, T *S, T *D, int64_t ld, int64_t n,
                                                         int64_t p, int b, const int64_t *info) {
    using Ar = Arith<T>;
    __shared__ T l11[kNbExact][kNbExact + 1];
    if (*(volatile const int64_t *)info >= 0) return;
    for (int e = threadIdx.x; e < kNbExact * kNbExact; e += blockDim.x) {
        const int r = e % kNbExact, c = e / kNbExact;
        if (r < b && c <= r) l11[r][c] = cm(W, ld, p + r, p + c);
    }
    __syncthreads();
    const int64_t j = p + b + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    T av[kNbExact], sv[kNbExact];
#pragma unroll
    for (int k = 0; k < kNbExact; ++k) {
        if (k < b) {
            av[k] = cm(W, ld, j, p + k);
            sv[k] = cm(S, ld, j, p + k);
        }
    }
    T dj = D[j];
#pragma unroll
    for (int k = 0; k < kNbExact; ++k) {
        if (k < b) {
            const T l = Ar::div(Ar::sub(av[k], sv[k]), l11[k][k]);
            av[k] = l;
            dj = Ar::add(dj, Ar::mul(l, l));
#pragma unroll
            for (int k2 = k + 1; k2 < kNbExact; ++k2)
                if (k2 < b) sv[k2] = Ar::add(sv[k2], Ar::mul(l11[k2][k], l));
        }
    }
#pragma unroll
    for (int k = 0; k < kNbExact; ++k)
        if (k < b) cm(W, ld, j, p + k) = av[k];
    D[j] = dj;
}

// Lower-triangular tile enumeration: t -> (I, J) with J <= I.
__device__ __forceinline__ void tri_tile(int64_t t, int64_t &I, int64_t &J) {
    int64_t i = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    I = i;
    J = t - i * (i + 1) / 2;
}

// SIMT trailing update on 64 x 64 tiles of the lower trailing matrix
// [q, n)^2, panel columns [p, p+b), b <= 64.  256 threads, 4 x 4 per thread.
//  EXACT: S[j,k2] = S[j,k2] + L[k2,k]*L[j,k] for ascending k, strictly lower
//         (j > k2) -- each product and sum rounded separately.
//  FAST : A[j,k2] -= sum_k L[j,k]*L[k2,k] with FMA, lower incl. diagonal.
constexpr int kUpdTile = 64;

template <typename T, bool kExact>
__global__ void __launch_bounds__(256) potrf_update_simt(T *W, T *S, int64_t ld, int64_t n,
                                                         int64_t p, int b, const int64_t *info) {
    using Ar = Arith<T>;
    constexpr int KB = kExact ? kNbExact : 64;  // panel width bound (<= 33 KB of smem)
    __shared__ T lj[KB][kUpdTile + 1];  // [k][row]
    __shared__ T lk[KB][kUpdTile + 1];
    if (*(volatile const int64_t *)info >= 0) return;
    const int64_t q = p + b;
    int64_t I, J;
    tri_tile(blockIdx.x, I, J);
    const int64_t j0 = q + I * kUpdTile, k0 = q + J * kUpdTile;
    const int tid = threadIdx.x;
    for (int e = tid; e < kUpdTile * b; e += 256) {
        const int r = e % kUpdTile, k = e / kUpdTile;
        lj[k][r] = (j0 + r < n) ? cm(W, ld, j0 + r, p + k) : T(0);
        lk[k][r] = (k0 + r < n) ? cm(W, ld, k0 + r, p + k) : T(0);
    }
    __syncthreads();
    const int tr = tid % 16, tc = tid / 16;
    T acc[4][4];
    T *Dst = kExact ? S : W;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t j = j0 + tr + 16 * r, k2 = k0 + tc + 16 * c;
            acc[r][c] = (j < n && k2 < n) ? cm(Dst, ld, j, k2) : T(0);
        }
    for (int k = 0; k < b; ++k) {
        T xr[4], xc[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) xr[r] = lj[k][tr + 16 * r];
#pragma unroll
        for (int c = 0; c < 4; ++c) xc[c] = lk[k][tc + 16 * c];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (kExact)
                    acc[r][c] = Ar::add(acc[r][c], Ar::mul(xc[c], xr[r]));
                else
                    acc[r][c] = Ar::fma_(-xr[r], xc[c], acc[r][c]);
            }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t j = j0 + tr + 16 * r, k2 = k0 + tc + 16 * c;
            const bool inside = kExact ? (k2 < j) : (k2 <= j);
            if (j < n && k2 < n && inside) cm(Dst, ld, j, k2) = acc[r][c];
        }
}

// ---------------------------------------------------------------------------
// FAST diagonal block: [p, p+b), b <= 64, one CTA of 1024 threads, in place.
// Also records min_k (pivot_k / A_orig[k,k]) for the near-singular guard.
constexpr int kNbFast = 64;

__device__ __forceinline__ void atomic_min_pos(double *addr, double v) {
    // non-negative doubles order like their int64 bit patterns
    if (v >= 0.0) atomicMin((unsigned long long *)addr, (unsigned long long)__double_as_longlong(v));
}

template <typename T>
__global__ void __launch_bounds__(1024) potrf_fast_diag(T *W, int64_t ld, int64_t p, int b,
                                                        const T *diag0, int64_t *info,
                                                        double *min_ratio) {
    using Ar = Arith<T>;
    __shared__ T a[kNbFast][kNbFast + 1];
    __shared__ int failed;
    if (*(volatile int64_t *)info >= 0) return;
    const int tid = threadIdx.x;
    for (int e = tid; e < kNbFast * kNbFast; e += 1024) {
        const int r = e % kNbFast, c = e / kNbFast;
        if (r < b && c <= r) a[r][c] = cm(W, ld, p + r, p + c);
    }
    if (tid == 0) failed = 0;
    __syncthreads();
    double ratio = 1.0e300;
    for (int k = 0; k < b; ++k) {
        if (tid == 0) {
            const T dd = a[k][k];
            if (dd <= T(0)) {
                failed = 1;
                *info = p + k;
            } else {
                a[k][k] = Ar::sqrt_(dd);
                const double r0 = (double)dd / (double)diag0[p + k];
                if (r0 < ratio) ratio = r0;
            }
        }
        __syncthreads();
        if (failed) break;
        const T lkk = a[k][k];
        if (tid > k && tid < b) a[tid][k] = Ar::div(a[tid][k], lkk);
        __syncthreads();
        // a[j][k2] -= a[j][k] * a[k2][k] for k < k2 <= j < b
        for (int e = tid; e < kNbFast * kNbFast; e += 1024) {
            const int j = e % kNbFast, k2 = e / kNbFast;
            if (j < b && k2 > k && k2 <= j) a[j][k2] = Ar::fma_(-a[j][k], a[k2][k], a[j][k2]);
        }
        __syncthreads();
    }
    if (tid == 0 && min_ratio) atomic_min_pos(min_ratio, ratio);
    for (int e = tid; e < kNbFast * kNbFast; e += 1024) {
        const int r = e % kNbFast, c = e / kNbFast;
        if (r < b && c <= r) cm(W, ld, p + r, p + c) = a[r][c];
    }
}

// FAST panel: rows [q, n): L21[j,:] = A21[j,:] L11^{-T}, one thread per row.
template <typename T>
__global__ void __launch_bounds__(128) potrf_fast_panel(T *W, int64_t ld, int64_t n, int64_t p,
                                                        int b, const int64_t *info) {
    using Ar = Arith<T>;
    __shared__ T l11[kNbFast][kNbFast + 1];
    if (*(volatile const int64_t *)info >= 0) return;
    for (int e = threadIdx.x; e < kNbFast * kNbFast; e += blockDim.x) {
        const int r = e % kNbFast, c = e / kNbFast;
        if (r < b && c <= r) l11[r][c] = cm(W, ld, p + r, p + c);
    }
    __syncthreads();
    const int64_t j = p + b + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    T av[kNbFast];
#pragma unroll
    for (int k = 0; k < kNbFast; ++k)
        if (k < b) av[k] = cm(W, ld, j, p + k);
#pragma unroll
    for (int k = 0; k < kNbFast; ++k) {
        if (k < b) {
            const T l = Ar::div(av[k], l11[k][k]);
            av[k] = l;
#pragma unroll
            for (int k2 = k + 1; k2 < kNbFast; ++k2)
                if (k2 < b) av[k2] = Ar::fma_(-l, l11[k2][k], av[k2]);
        }
    }
#pragma unroll
    for (int k = 0; k < kNbFast; ++k)
        if (k < b) cm(W, ld, j, p + k) = av[k];
}

// FAST FP64 trailing update on the FP64 tensor pipe: A22 -= L21 L21^T on
// 64 x 64 lower tiles, panel width b <= 64 (zero-padded to a multiple of 16).
// 4 warps in 2 x 2, each a 32 x 32 sub-tile of 2 x 4 m16n8k16 MMAs.
// Fragment layout of mma.m16n8k16.row.col.f64 (g = lane/4, t = lane%4):
//   A (16x16): a[i] = A[g + 8*(i&1)][t + 4*(i>>1)],  i = 0..7
//   B (16x8) : b[i] = B[t + 4*i][g],                 i = 0..3
//   C (16x8) : c[i] = C[g + 8*(i>>1)][2*t + (i&1)],  i = 0..3
constexpr int kDmmaStride = 68;  // 68 = 4 (mod 16): conflict-free fragment reads

__global__ void __launch_bounds__(128) potrf_fast_update_dmma(double *W, int64_t ld, int64_t n,
                                                              int64_t p, int b,
                                                              const int64_t *info) {
    __shared__ double lj[32][kDmmaStride];  // [k][row], one 32-wide slice of the panel
    __shared__ double lk[32][kDmmaStride];
    if (*(volatile const int64_t *)info >= 0) return;
    const int64_t q = p + b;
    int64_t I, J;
    tri_tile(blockIdx.x, I, J);
    const int64_t j0 = q + I * 64, k0 = q + J * 64;
    const int tid = threadIdx.x;
    const int bp = (b + 15) & ~15;
    const int warp = tid / 32, lane = tid % 32;
    const int g = lane >> 2, t = lane & 3;
    const int wr = (warp & 1) * 32, wc = (warp >> 1) * 32;
    double acc[2][4][4];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[mi][ni][i] = 0.0;
    for (int kh = 0; kh < bp; kh += 32) {
      const int kw = min(32, bp - kh);
      __syncthreads();
      for (int e = tid; e < 64 * kw; e += 128) {
          const int r = e % 64, k = e / 64;
          const bool kin = kh + k < b;
          lj[k][r] = (kin && j0 + r < n) ? cm(W, ld, j0 + r, p + kh + k) : 0.0;
          lk[k][r] = (kin && k0 + r < n) ? cm(W, ld, k0 + r, p + kh + k) : 0.0;
      }
      __syncthreads();
      for (int kk = 0; kk < kw; kk += 16) {
        double af[2][8], bf[4][4];
#pragma unroll
        for (int mi = 0; mi < 2; ++mi)
#pragma unroll
            for (int i = 0; i < 8; ++i)
                af[mi][i] = lj[kk + t + 4 * (i >> 1)][wr + mi * 16 + g + 8 * (i & 1)];
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int i = 0; i < 4; ++i) bf[ni][i] = lk[kk + t + 4 * i][wc + ni * 8 + g];
#pragma unroll
        for (int mi = 0; mi < 2; ++mi)
#pragma unroll
            for (int ni = 0; ni < 4; ++ni)
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                    "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
                    : "+d"(acc[mi][ni][0]), "+d"(acc[mi][ni][1]), "+d"(acc[mi][ni][2]),
                      "+d"(acc[mi][ni][3])
                    : "d"(af[mi][0]), "d"(af[mi][1]), "d"(af[mi][2]), "d"(af[mi][3]),
                      "d"(af[mi][4]), "d"(af[mi][5]), "d"(af[mi][6]), "d"(af[mi][7]),
                      "d"(bf[ni][0]), "d"(bf[ni][1]), "d"(bf[ni][2]), "d"(bf[ni][3]));
      }
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int64_t j = j0 + wr + mi * 16 + g + 8 * (i >> 1);
                const int64_t k2 = k0 + wc + ni * 8 + 2 * t + (i & 1);
                if (j < n && k2 <= j) cm(W, ld, j, k2) -= acc[mi][ni][i];
            }
}

// Saves the input diagonal (for the fast path's pivot-ratio guard).
template <typename T>
__global__ void copy_diag(const T *W, int64_t ld, int64_t n, T *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cm(W, ld, i, i);
}

// ---------------------------------------------------------------------------
// Host drivers.

static int64_t tri_tiles(int64_t m, int tile) {
    const int64_t t = ceil_div(m, tile);
    return t * (t + 1) / 2;
}

template <typename T>
int potrf_exact_launch(T *W, T *S, T *D, int64_t n, int64_t ld, int64_t *d_info,
                       cudaStream_t st) {
    // S (n x n, ld) and D (n) start at zero.
    if (cudaMemsetAsync(D, 0, sizeof(T) * n, st) != cudaSuccess) return -1;
    if (cudaMemsetAsync(S, 0, sizeof(T) * ld * n, st) != cudaSuccess) return -1;
    for (int64_t p = 0; p < n; p += kNbExact) {
        const int b = (int)std::min<int64_t>(kNbExact, n - p);
        {
            LaunchScope ls(K_POTRF_EXACT_DIAG, st, (double)b * b * b / 3.0);
            potrf_exact_diag<T><<<1, dim3(32, 32), 0, st>>>(W, S, D, ld, p, b, d_info);
        }
        const int64_t rest = n - p - b;
        if (rest > 0) {
            {
                LaunchScope ls(K_POTRF_EXACT_PANEL, st, (double)rest * b * b);
                potrf_exact_panel<T><<<(unsigned)ceil_div(rest, 128), 128, 0, st>>>(
                    W, S, D, ld, n, p, b, d_info);
            }
            LaunchScope ls(K_POTRF_EXACT_UPDATE, st, (double)rest * (rest - 1) * b);
            potrf_update_simt<T, true><<<(unsigned)tri_tiles(rest, kUpdTile), 256, 0, st>>>(
                W, S, ld, n, p, b, d_info);
        }
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T>
int potrf_fast_launch(T *W, int64_t n, int64_t ld, int64_t *d_info, T *diag0, double *min_ratio,
                      cudaStream_t st) {
    {
        LaunchScope ls(K_MISC, st);
        copy_diag<T><<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(W, ld, n, diag0);
    }
    for (int64_t p = 0; p < n; p += kNbFast) {
        const int b = (int)std::min<int64_t>(kNbFast, n - p);
        {
            LaunchScope ls(K_POTRF_FAST_DIAG, st, (double)b * b * b / 3.0);
            potrf_fast_diag<T><<<1, 1024, 0, st>>>(W, ld, p, b, diag0, d_info, min_ratio);
        }
        const int64_t rest = n - p - b;
        if (rest > 0) {
            {
                LaunchScope ls(K_POTRF_FAST_PANEL, st, (double)rest * b * b);
                potrf_fast_panel<T><<<(unsigned)ceil_div(rest, 128), 128, 0, st>>>(W, ld, n, p, b,
                                                                                d_info);
            }
            // algorithmic work: rest*(rest+1)/2 lower entries x b multiply-adds x 2
            LaunchScope ls(K_POTRF_FAST_UPDATE, st, (double)rest * (rest + 1) * b);
            if constexpr (sizeof(T) == 8)
                potrf_fast_update_dmma<<<(unsigned)tri_tiles(rest, 64), 128, 0, st>>>(
                    (double *)W, ld, n, p, b, d_info);
            else
                potrf_update_simt<T, false><<<(unsigned)tri_tiles(rest, kUpdTile), 256, 0, st>>>(
                    W, nullptr, ld, n, p, b, d_info);
        }
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template int potrf_exact_launch<double>(double *, double *, double *, int64_t, int64_t, int64_t *,
                                        cudaStream_t);
template int potrf_exact_launch<float>(float *, float *, float *, int64_t, int64_t, int64_t *,
                                       cudaStream_t);
template int potrf_fast_launch<double>(double *, int64_t, int64_t, int64_t *, double *, double *,
                                       cudaStream_t);
template int potrf_fast_launch<float>(float *, int64_t, int64_t, int64_t *, float *, double *,
                                      cudaStream_t);

}  // namespace lla

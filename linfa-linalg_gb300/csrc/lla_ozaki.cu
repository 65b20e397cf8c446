// lla_ozaki.cu -- FP64-accurate refinement residual R = B - A_sym X on the
// BF16 tensor cores by exact integer slices (the Ozaki scheme).
//
// Each row of A_sym is scaled by a power of two 2^e_i (e_i above its largest
// magnitude) and cut into S = 8 slices of 7 bits:
//     a_ik = 2^e_i * sum_{p<S} alpha_p[i,k] 2^-7(p+1)  (+ a remainder below 2^-56),
// with integer alpha_p in [-127, 127] (the digits of |a|, carrying a's sign),
// exactly representable in BF16.  Each
// column of X is sliced the same way with its own exponent f_j.  Then
//     (A X)_ij = 2^(e_i + f_j) sum_d 2^-7(d+2) sum_{p+q=d} sum_k alpha_p[i,k] xi_q[j,k]
// and the terms with d = p + q < S are kept (the dropped ones lie below
// 2^-56 of 2^(e_i+f_j) per product).  Every product alpha*xi is an integer of
// at most 14 bits; the tensor core sums them in FP32, which is exact as long
// as a partial sum stays below 2^24: the kernel drains the tensor-memory
// accumulators every two K-chunks of 64 (level d gathers at most
// 2 (d+1) x 64 <= 1024 terms of 2^14) and converts the drained integers exactly.  Levels 0-3 are summed at
// their relative weights 2^(21-7d) in one 64-bit integer and levels 4-7 at
// 2^(49-7d) in another (both stay far below 2^63); the two are combined in
// FP64 at the end.  So the only rounding errors are those of the final FP64
// combination and subtraction, like an FP64 GEMM's epilogue -- the residual is
// as accurate as an FP64 one, computed on the BF16 pipe.
//
// Loop order: K-chunks outermost, then the slices of A, then those of X: each
// A slice tile is loaded once per chunk and meets every X slice it pairs
// with, the eight levels accumulating side by side in tensor memory.
//
// Slices of A are built once per solve (A does not change during the
// refinement); slices of X once per iteration.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "lla_common.cuh"
#include "lla_mixed.h"
#include "lla_oz_digits.h"
#include "lla_prof.h"
#include "lla_tcgen05.cuh"

namespace lla {

constexpr int kOzS = 8;                      // slices
constexpr int kOzM = 128, kOzN = 64, kOzK = 64;
constexpr int kOzAStages = 4;
constexpr int kOzATile = kOzM * kOzK * 2;    // 16 KiB: one slice of a 128 x 64 A tile
constexpr int kOzXTile = kOzN * kOzK * 2;    // 8 KiB: one slice of a 64 x 64 X tile
constexpr int kOzXSet = kOzS * kOzXTile;     // 64 KiB: all slices of one X tile
constexpr int kOzSmem = 1024 + kOzAStages * kOzATile + 2 * kOzXSet + 256;
constexpr int kOzThreads = 320;              // 8 epilogue warps + producer + MMA
constexpr uint32_t kOzCols = kOzS * kOzN;    // one FP32 accumulator of 64 columns per level: 512
constexpr int kOzSplitsMax = 8;

// K-chunks per accumulation window: level 7 gathers 8 pairs x 64 products
// below 2^14 per chunk, so two chunks stay within 2^24 (exact in FP32).
constexpr int kOzWin = 2;

// ---- slicing ---------------------------------------------------------------

__device__ __forceinline__ void atomic_max_bits(double *addr, double v) {
    if (!(v >= 0.0)) v = __longlong_as_double(0x7ff0000000000000ll);  // NaN -> +inf
    atomicMax((unsigned long long *)addr, (unsigned long long)__double_as_longlong(v));
}

// rowmax[i] = max_k |A_sym(i, k)| from the lower triangle (one block per
// 32-column strip, as the symmetric row sums).
__global__ void __launch_bounds__(256) oz_rowmax_kernel(const double *__restrict__ A, int64_t lda,
                                                        int64_t n, double *rowmax) {
    __shared__ double red[8][32];
    const int64_t k0 = (int64_t)blockIdx.x * 32;
    double colp[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) colp[c] = 0.0;
    for (int64_t i = k0 + threadIdx.x; i < n; i += blockDim.x) {
        double racc = 0.0;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
            const int64_t k = k0 + c;
            if (k < n && k <= i) {
                const double v = fabs(A[i + k * lda]);
                racc = fmax(racc, v);
                if (k != i) colp[c] = fmax(colp[c], v);
            }
        }
        atomic_max_bits(&rowmax[i], racc);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < 32; ++c) {
        double v = colp[c];
#pragma unroll
        for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 32 && k0 + threadIdx.x < n) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmax(v, red[w][threadIdx.x]);
        atomic_max_bits(&rowmax[k0 + threadIdx.x], v);
    }
}

// Exponent with |v| < 2^e (0 for v == 0); non-finite -> a flag value.
__device__ __forceinline__ int oz_exponent(double v) { return v > 0.0 ? ilogb(v) + 1 : 0; }

// Digits of a with respect to the scale 2^e (|a| < 2^e): the magnitude
// |a| 2^(56 - e) as a 56-bit integer T (low bits truncated -- below 2^-56 of
// the scale), cut into eight 7-bit digits T = sum_p alpha_p 2^(7 (7 - p)), each
// carrying the sign of a (lla_oz_digits.h: integer and FP32 operations only --
// the FP64 pipe is slow -- four elements at a time, packed BF16 pairs).
static_assert(kOzS == kOzDigits, "one plane per digit");

// Slices of A_sym, planes [p][i][k] (row-major, row stride ldp >= n, zero for
// k >= n).  64 x 64 tiles through shared memory (16 loads in flight per
// thread): lower tiles read column-major A coalesced along i, upper tiles
// (mirrored) along k.  Then thread t writes row t / 16, columns 4 (t % 16) ..
// + 3 and the same for the next three groups of 16 rows: one 8-byte store per
// plane (ldp and the plane stride are multiples of 64).
__global__ void __launch_bounds__(256) oz_slice_a_kernel(const double *__restrict__ A, int64_t lda,
                                                         int64_t n, int64_t ldp,
                                                         const double *__restrict__ rowmax,
                                                         __nv_bfloat16 *planes, int64_t plane_stride) {
    __shared__ double tile[64][65];
    const int64_t i0 = (int64_t)blockIdx.y * 64, k0 = (int64_t)blockIdx.x * 64;
    const bool upper = k0 > i0;  // strictly above the diagonal block: mirror of a lower tile
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int e = threadIdx.x + 256 * u;
        int r, c;
        if (upper) {
            c = e % 64;
            r = e / 64;  // consecutive e -> consecutive k -> A[k + i*lda]
        } else {
            r = e % 64;
            c = e / 64;  // consecutive e -> consecutive i -> A[i + k*lda]
        }
        const int64_t i = i0 + r, k = k0 + c;
        v[u] = 0.0;
        if (i < n && k < n) v[u] = (k <= i) ? A[i + k * lda] : A[k + i * lda];
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int e = threadIdx.x + 256 * u;
        if (upper)
            tile[e / 64][e % 64] = v[u];
        else
            tile[e % 64][e / 64] = v[u];
    }
    __syncthreads();
    const int c4 = (threadIdx.x & 15) * 4;
#pragma unroll 1
    for (int g = 0; g < 4; ++g) {
        const int r = (threadIdx.x >> 4) + 16 * g;
        const int64_t i = i0 + r, k = k0 + c4;
        if (i >= n || k >= ldp) continue;
        const double rm = rowmax[i];
        const bool fin = isfinite(rm);
        int64_t b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) b[u] = fin ? __double_as_longlong(tile[r][c4 + u]) : 0ll;
        uint32_t q[kOzDigits][2];
        oz_digits_packed4(b, oz_exponent(rm), q);
#pragma unroll
        for (int p = 0; p < kOzS; ++p)
            *reinterpret_cast<uint2 *>(planes + p * plane_stride + i * ldp + k) = make_uint2(q[p][0], q[p][1]);
    }
}

// Slices of X^T, planes [q][j][k] (m_pad = 64 rows, zero for j >= m or k >= n):
// thread (k4, j) writes columns 4 k4 .. 4 k4 + 3 of row j, one 8-byte store a plane.
__global__ void oz_slice_x_kernel(const double *__restrict__ X, int64_t ldx, int64_t n, int64_t m,
                                  int64_t ldp, const double *__restrict__ colmax,
                                  __nv_bfloat16 *planes, int64_t plane_stride, const int *state) {
    if (refine_done(state)) return;
    const int64_t k = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
    const int64_t j = blockIdx.y;
    if (k >= ldp) return;
    int64_t b[4] = {0, 0, 0, 0};
    int e = 0;
    if (j < m) {
        const double cm = colmax[j];
        e = oz_exponent(cm);
        if (isfinite(cm)) {
#pragma unroll
            for (int u = 0; u < 4; ++u) b[u] = k + u < n ? __double_as_longlong(X[k + u + j * ldx]) : 0ll;
        }
    }
    uint32_t q[kOzDigits][2];
    oz_digits_packed4(b, e, q);
#pragma unroll
    for (int p = 0; p < kOzS; ++p)
        *reinterpret_cast<uint2 *>(planes + p * plane_stride + j * ldp + k) = make_uint2(q[p][0], q[p][1]);
}

// ---- the tensor-core kernel ------------------------------------------------

// Schedule shared by the three roles.  K-chunks kc of 64 columns; per chunk the
// X slices (all eight, one 64 KiB TMA box) and then the A slices p = 0..7 (a
// 4-deep ring).  Slice p of A meets slices q = 0..7-p of X, and the product
// accumulates at level d = p + q in its own 64 TMEM columns (8 levels = all
// 512).  Slice p of A meets up to four X slices in one MMA (N <= 256): the X
// slices are consecutive 64-row blocks of the operand and the levels they
// feed consecutive accumulators.  Every window of kOzWin chunks the epilogue
// drains levels 0-3, then 4-7; the MMA issuer restarts each half as soon as it
// is read out.
__global__ void __launch_bounds__(kOzThreads, 1) oz_residual_kernel(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmX, int64_t n,
    int64_t m, int kchunks, int splits, double *F, int *err_word, const int *state) {
    // uniform for the CTA: nothing below (barriers, tensor memory) is touched
    if (refine_done(state)) return;
    extern __shared__ uint8_t smem_raw[];
    __shared__ int s_abort, s_levels;
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;                              // kOzAStages x 16 KiB
    uint8_t *sX = smem + kOzAStages * kOzATile;      // 2 x 64 KiB
    uint64_t *bars = (uint64_t *)(sX + 2 * kOzXSet);
    uint32_t *tslot = (uint32_t *)(bars + 2 * kOzAStages + 7);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t fullA0 = smem_u32(bars), emptyA0 = fullA0 + 8 * kOzAStages;
    const uint32_t fullX0 = emptyA0 + 8 * kOzAStages, emptyX0 = fullX0 + 16;
    const uint32_t tfull = emptyX0 + 16, tempty0 = tfull + 8;  // tempty0 + 8 h: levels 4h .. 4h+3 drained
    const int row0 = (int)blockIdx.x * kOzM;
    const int z = blockIdx.y;
    const int cps = (kchunks + splits - 1) / splits;
    const int kc_beg = z * cps, kc_end = min(kchunks, kc_beg + cps);
    if (tid == 0) {
        for (int s = 0; s < kOzAStages; ++s) {
            mbar_init(fullA0 + 8 * s, 1);
            mbar_init(emptyA0 + 8 * s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(fullX0 + 8 * b, 1);
            mbar_init(emptyX0 + 8 * b, 1);
        }
        mbar_init(tfull, 1);
        for (int h = 0; h < 2; ++h) mbar_init(tempty0 + 8 * h, 256);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
        s_levels = refine_levels(state);  // levels kept this iteration (6 or 8), the same in every CTA
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tslot)),
                     "r"(kOzCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    // instruction descriptor without N: D F32, A/B BF16, K-major, M = 128
    const uint32_t idesc0 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kOzM >> 4) << 24);

    if (warp == 8) {
        if (lane == 0) {  // TMA producer
            const int S = s_levels;
            int64_t ga = 0;
            for (int kc = kc_beg, j = 0; kc < kc_end && !*(volatile int *)&s_abort; ++kc, ++j) {
                const int xb = j & 1, use = j >> 1;
                if (use > 0 && !mbar_wait(emptyX0 + 8 * xb, (uint32_t)((use - 1) & 1), err_word)) {
                    s_abort = 1;
                    break;
                }
                mbar_expect_tx(fullX0 + 8 * xb, kOzXSet);
                tma_load_3d(smem_u32(sX + xb * kOzXSet), &tmX, kc * kOzK, 0, 0, fullX0 + 8 * xb);
                for (int p = 0; p < S; ++p, ++ga) {
                    const int s = (int)(ga % kOzAStages);
                    const int64_t round = ga / kOzAStages;
                    if (round > 0 && !mbar_wait(emptyA0 + 8 * s, (uint32_t)((round - 1) & 1), err_word)) {
                        s_abort = 1;
                        break;
                    }
                    mbar_expect_tx(fullA0 + 8 * s, kOzATile);
                    tma_load_3d(smem_u32(sA + s * kOzATile), &tmA, kc * kOzK, row0, p, fullA0 + 8 * s);
                }
            }
        }
    } else if (warp == 9) {
        if (lane == 0) {  // MMA issuer
            const int S = s_levels;
            int64_t ga = 0;
            int win = 0;
            for (int kc = kc_beg, j = 0; kc < kc_end && !*(volatile int *)&s_abort; ++kc, ++j) {
                const int xb = j & 1, use = j >> 1;
                const bool wstart = (j % kOzWin) == 0;
                if (!mbar_wait(fullX0 + 8 * xb, (uint32_t)(use & 1), err_word)) {
                    s_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t x0 = smem_u32(sX + xb * kOzXSet);
                for (int p = 0; p < S; ++p, ++ga) {
                    const int s = (int)(ga % kOzAStages);
                    if (!mbar_wait(fullA0 + 8 * s, (uint32_t)((ga / kOzAStages) & 1), err_word)) {
                        s_abort = 1;
                        break;
                    }
                    tc_fence_after();
                    // A slice p against X slices q0 .. q1-1 in one MMA of N = 64 (q1 - q0):
                    // the X slices are consecutive 64-row blocks of one operand and
                    // the levels p+q0 .. p+q1-1 consecutive 64-column accumulators
                    const uint64_t ad = sw128_desc(smem_u32(sA + s * kOzATile));
                    for (int h = 0; h < 2; ++h) {
                        const int q0 = 4 * h, q1 = min(4 * h + 4, S - p);
                        if (q0 >= q1) break;
                        // first product of a window into these levels: wait until the
                        // epilogue has read them out of the previous window
                        if (wstart && p == 0 && win > 0) {
                            if (!mbar_wait(tempty0 + 8 * h, (uint32_t)((win - 1) & 1), err_word)) {
                                s_abort = 1;
                                break;
                            }
                            tc_fence_after();
                        }
                        const uint32_t dt = tmem + (uint32_t)((p + q0) * kOzN);
                        const uint32_t idesc = idesc0 | ((uint32_t)((kOzN * (q1 - q0)) >> 3) << 17);
                        const uint64_t bd = sw128_desc(x0 + (uint32_t)(q0 * kOzXTile));
#pragma unroll
                        for (int k = 0; k < kOzK / 16; ++k)  // +32 bytes along K per step
                            tc_mma(dt, ad + 2 * k, bd + 2 * k, idesc, (wstart && p == 0 && k == 0) ? 0u : 1u);
                    }
                    if (*(volatile int *)&s_abort) break;
                    tc_commit(emptyA0 + 8 * s);
                }
                if (*(volatile int *)&s_abort) break;
                tc_commit(emptyX0 + 8 * xb);
                if ((j % kOzWin) == kOzWin - 1 || kc == kc_end - 1) {
                    tc_commit(tfull);
                    ++win;
                }
            }
        }
    } else {  // epilogue: warp w drains lane quarter w % 4, columns 32 (w / 4) .. of every level
        const int qw = warp & 3, half = warp >> 2;
        const int r = qw * 32 + lane;
        // exact integer sums: hi = sum_{d<4} I_d 2^(21-7d), lo = sum_{d>=4} I_d 2^(49-7d)
        long long hi[32], lo[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) hi[c] = lo[c] = 0;
        bool ok = true;
        const int nwin = (kc_end - kc_beg + kOzWin - 1) / kOzWin;
        for (int win = 0; win < nwin && ok; ++win) {
            bool w = mbar_wait(tfull, (uint32_t)(win & 1), err_word);
            w = __all_sync(0xffffffffu, w) && !*(volatile int *)&s_abort;
            if (!w) {
                if (lane == 0) s_abort = 1;
                ok = false;
                break;
            }
            tc_fence_after();
#pragma unroll 1
            for (int d = 0; d < kOzS; ++d) {
                uint32_t v[32];
                if (d < *(volatile int *)&s_levels) {  // uniform: the levels formed this iteration
                    tc_ld32(tmem + (uint32_t)(d * kOzN) + ((uint32_t)(qw * 32) << 16) + (uint32_t)(half * 32), v);
                } else {
#pragma unroll
                    for (int c = 0; c < 32; ++c) v[c] = 0u;
                }
                if ((d & 3) == 3) {  // levels d-3 .. d read out
                    tc_fence_before();
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tempty0 + 8 * (d >> 2)) : "memory");
                }
                const long long wd = 1ll << (d < 4 ? 21 - 7 * d : 49 - 7 * d);
                if (d < 4) {
#pragma unroll
                    for (int c = 0; c < 32; ++c) hi[c] += (long long)__float2int_rn(__uint_as_float(v[c])) * wd;
                } else {
#pragma unroll
                    for (int c = 0; c < 32; ++c) lo[c] += (long long)__float2int_rn(__uint_as_float(v[c])) * wd;
                }
            }
        }
        const int64_t i = row0 + r;
        if (ok && i < n) {
            double *Fz = F + (int64_t)z * n * m;
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const int64_t j = half * 32 + c;
                if (j < m) Fz[i + j * n] = ldexp((double)hi[c], -35) + ldexp((double)lo[c], -63);
            }
        }
    }
    __syncwarp();
    __syncthreads();
    if (s_abort && tid == 0) atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOzCols)
                     : "memory");
}

// R = B - 2^(e_i + f_j) (F_0 + F_1 + ...), column maxima of |R|; a non-finite
// row or column scale (non-finite data) yields NaN, which the refinement treats
// as a stall.
__global__ void oz_combine_kernel(const double *__restrict__ F, int splits, const double *B, int64_t ldb,
                                  const double *__restrict__ rowmax, const double *__restrict__ colmax_x,
                                  double *R, int64_t ldr, int64_t n, int64_t m, double *colmax_r,
                                  const int *state) {
    if (refine_done(state)) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t j = blockIdx.y;
    double v = 0.0;
    if (i < n) {
        double s = F[i + j * n];
        for (int zz = 1; zz < splits; ++zz) s += F[(int64_t)zz * n * m + i + j * n];
        const double rm = rowmax[i], cm = colmax_x[j];
        double r;
        if (!isfinite(rm) || !isfinite(cm))
            r = __longlong_as_double(0x7ff8000000000000ll);
        else
            r = B[i + j * ldb] - ldexp(s, oz_exponent(rm) + oz_exponent(cm));
        R[i + j * ldr] = r;
        v = fabs(r);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomic_max_bits(&colmax_r[j], v);
}

// ---- host side -------------------------------------------------------------

static int64_t oz_ldp(int64_t n) { return (n + kOzK - 1) / kOzK * kOzK; }

size_t oz_workspace_bytes(int64_t n, int64_t m) {
    const int64_t ldp = oz_ldp(n);
    return (size_t)kOzS * n * ldp * 2        // A slices
           + (size_t)kOzS * kOzN * ldp * 2   // X slices (one 64-column group)
           + (size_t)n * 8                   // row maxima
           + (size_t)kOzSplitsMax * n * std::min<int64_t>(m, kOzN) * 8 + 4096;  // split partials
}

struct OzState {
    __nv_bfloat16 *A, *X;
    double *rowmax, *F;
    int64_t ldp;
    CUtensorMap tmA, tmX;
    int splits;
};

static int oz_splits(int64_t n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    // fewest splits whose CTAs fill the waves of one CTA per SM to within 5 %,
    // keeping at least 8 K-chunks per split
    const int64_t tiles = (n + kOzM - 1) / kOzM, chunks = oz_ldp(n) / kOzK;
    int best = 1;
    double best_eff = 0.0;
    for (int s = 1; s <= kOzSplitsMax; ++s) {
        if (s > 1 && chunks / s < 8) break;
        const int64_t ctas = tiles * s, waves = (ctas + sms - 1) / sms;
        const double eff = (double)ctas / (double)(waves * sms);
        if (eff > best_eff + 0.05) {
            best = s;
            best_eff = eff;
        }
    }
    return best;
}

static void oz_carve(void *ws, int64_t n, int64_t m, OzState &o) {
    o.ldp = oz_ldp(n);
    char *p = (char *)ws;
    o.A = (__nv_bfloat16 *)p;
    p += (size_t)kOzS * n * o.ldp * 2;
    o.X = (__nv_bfloat16 *)p;
    p += (size_t)kOzS * kOzN * o.ldp * 2;
    o.rowmax = (double *)p;
    p += (size_t)n * 8;
    o.F = (double *)p;
    o.splits = oz_splits(n);
}

double *oz_rowmax(void *ws, int64_t n, int64_t m) {
    OzState o;
    oz_carve(ws, n, m, o);
    return o.rowmax;
}

// Once per solve: row maxima (unless already formed) and slices of A.
int oz_prepare(const double *A, int64_t lda, int64_t n, int64_t m, void *ws, bool rowmax_ready, cudaStream_t st) {
    OzState o;
    oz_carve(ws, n, m, o);
    if (!rowmax_ready) {
        if (cudaMemsetAsync(o.rowmax, 0, sizeof(double) * n, st) != cudaSuccess) return -1;
        LaunchScope ls(K_OZ_SLICE, st, 8.0 * n * n);
        oz_rowmax_kernel<<<(unsigned)((n + 31) / 32), 256, 0, st>>>(A, lda, n, o.rowmax);
    }
    {
        LaunchScope ls(K_OZ_SLICE, st, 8.0 * n * n + 2.0 * kOzS * n * o.ldp);
        oz_slice_a_kernel<<<dim3((unsigned)(o.ldp / 64), (unsigned)((n + 63) / 64)), 256, 0, st>>>(
            A, lda, n, o.ldp, o.rowmax, o.A, n * o.ldp);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Every iteration: R = B - A_sym X for up to 64 columns at a time.
int oz_residual_launch(const double *X, int64_t ldx, const double *B, int64_t ldb, double *R, int64_t ldr,
                       int64_t n, int64_t m, const double *colmax_x, double *colmax_r, void *ws,
                       int *err_word, cudaStream_t st, const int *state) {
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(oz_residual_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kOzSmem) !=
            cudaSuccess)
            return -1;
        attr = true;
    }
    PFN_cuTensorMapEncodeTiled_v12000 enc = tma_encoder();
    if (!enc) return -1;
    OzState o;
    oz_carve(ws, n, m, o);
    const cuuint32_t estr[3] = {1, 1, 1};
    {
        const cuuint64_t dims[3] = {(cuuint64_t)o.ldp, (cuuint64_t)n, (cuuint64_t)kOzS};
        const cuuint64_t strides[2] = {(cuuint64_t)o.ldp * 2, (cuuint64_t)n * o.ldp * 2};
        const cuuint32_t box[3] = {(cuuint32_t)kOzK, (cuuint32_t)kOzM, 1};
        if (enc(&o.tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, o.A, dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return -1;
    }
    {
        const cuuint64_t dims[3] = {(cuuint64_t)o.ldp, (cuuint64_t)kOzN, (cuuint64_t)kOzS};
        const cuuint64_t strides[2] = {(cuuint64_t)o.ldp * 2, (cuuint64_t)kOzN * o.ldp * 2};
        const cuuint32_t box[3] = {(cuuint32_t)kOzK, (cuuint32_t)kOzN, (cuuint32_t)kOzS};  // all slices
        if (enc(&o.tmX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, o.X, dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return -1;
    }
    const int kchunks = (int)(o.ldp / kOzK);
    for (int64_t c0 = 0; c0 < m; c0 += kOzN) {
        const int64_t mc = std::min<int64_t>(kOzN, m - c0);
        {
            LaunchScope ls(K_OZ_SLICE, st, 8.0 * n * mc + 2.0 * kOzS * kOzN * o.ldp);
            oz_slice_x_kernel<<<dim3((unsigned)((o.ldp / 4 + 255) / 256), kOzN), 256, 0, st>>>(
                X + c0 * ldx, ldx, n, mc, o.ldp, colmax_x + c0, o.X, kOzN * o.ldp, state);
        }
        {
            // algorithmic work: 2 n^2 mc flops of the FP64 product it replaces
            LaunchScope ls(K_RESIDUAL, st, 2.0 * n * n * mc);
            oz_residual_kernel<<<dim3((unsigned)((n + kOzM - 1) / kOzM), (unsigned)o.splits), kOzThreads,
                                 kOzSmem, st>>>(o.tmA, o.tmX, n, mc, kchunks, o.splits, o.F, err_word, state);
        }
        {
            LaunchScope ls(K_REFINE, st, 8.0 * n * mc * (o.splits + 2));
            oz_combine_kernel<<<dim3((unsigned)((n + 255) / 256), (unsigned)mc), 256, 0, st>>>(
                o.F, o.splits, B + c0 * ldb, ldb, o.rowmax, colmax_x + c0, R + c0 * ldr, ldr, n, mc,
                colmax_r + c0, state);
        }
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace lla

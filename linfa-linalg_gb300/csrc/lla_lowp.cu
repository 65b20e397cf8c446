// lla_lowp.cu -- low-precision Cholesky of the equilibrated FP32 matrix used
// by the mixed-precision solve (lla_mixed.cu).
//
// Right-looking with panels of nb = 128 columns:
//   diag   : one CTA factors the 128 x 128 diagonal block in FP32 (32-column
//            sub-blocks: an unpredicated one-warp shuffle Cholesky without
//            square roots on its pivot chain, a row-parallel solve of the
//            rows below it, a shared-memory update of the next sub-block's
//            columns first and of the rest while the next pivots run; a
//            short last block is padded with the identity);
//   panel  : L21 = A21 L11^-T in FP32 by 32-column blocks (products with the
//            inverted 32 x 32 diagonal blocks of L11), and the operand
//            planes of L21 for the tensor cores: a one-, two- or three-term
//            split of every FP32 value into BF16 (or FP16) parts
//            x ~= h0 + h1 + h2;
//   update : A22 -= L21 L21^T on the 5th-generation tensor cores
//            (lla_tc_update.cu): the products of the chosen term pairs
//            (h0 h0^T, h0 h1^T + h1 h0^T, ...) accumulate in FP32 in tensor
//            memory and are subtracted from the FP32 trailing matrix.
// With two FP16 terms (11 + 11 significant bits) or three BF16 terms the
// update is as accurate as an FP32 one; one BF16 term (8 bits) is the fastest
// and the least accurate (refinement converges only for modest condition
// numbers and otherwise falls back).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>

#include "lla_api_internal.h"
#include "lla_common.cuh"
#include "lla_kernels.h"
#include "lla_mixed.h"
#include "lla_prof.h"
#include "lla_tc.h"

namespace lla {

constexpr int kLpNb = 128;  // panel width
constexpr int kLpLd = kLpNb + 1;
constexpr int kLpPd = kLpNb + 4;  // row stride of the transposed 32-column panel (16-byte rows)

// asynchronous global -> shared copies (all of a thread's copies in flight at once)
__device__ __forceinline__ void lp_cp4(float *dst, const float *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void lp_cp16(float *dst, const float *src, int bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void lp_cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ---------------------------------------------------------------------------
// diagonal block: b <= 128, one CTA of 512 threads, block in shared memory

constexpr int kDgThreads = 512;
constexpr int kDgLd = kLpNb + 4;  // column stride of the block in shared memory (16-byte columns)
constexpr int kDgLt = 36;         // row stride of a transposed 32 x 32 factor (16-byte rows)
constexpr size_t kDgSmem = sizeof(float) * (kLpNb * kDgLd + 32 * kDgLt + 5 * 32);

__device__ __forceinline__ float dg_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// a(r, c) -= sum_t a(r, k0 + t) a(c, k0 + t) over the 32 solved columns
// k0 .. k0 + 31, for rows r >= r0 and columns c0 <= c < c1, c <= r, in 4 x 4
// register tiles (column-major block, sa[c * kDgLd + r]); thread `thr` of `nthr`.
__device__ __forceinline__ void dg_syrk(float *sa, int k0, int r0, int c0, int c1, int thr, int nthr) {
    const int wr = (kLpNb - r0) / 4, wc = (c1 - c0) / 4;
    for (int e = thr; e < wr * wc; e += nthr) {
        const int rr = r0 + 4 * (e % wr), cc = c0 + 4 * (e / wr);
        if (cc > rr + 3) continue;  // above the diagonal
        float4 acc[4];              // acc[j]: column cc + j, rows rr .. rr + 3
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = *reinterpret_cast<const float4 *>(&sa[(cc + j) * kDgLd + rr]);
#pragma unroll 8
        for (int t = 0; t < 32; ++t) {
            const float4 a4 = *reinterpret_cast<const float4 *>(&sa[(k0 + t) * kDgLd + rr]);
            const float4 b4 = *reinterpret_cast<const float4 *>(&sa[(k0 + t) * kDgLd + cc]);
            const float bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                acc[j].x = fmaf(-a4.x, bv[j], acc[j].x);
                acc[j].y = fmaf(-a4.y, bv[j], acc[j].y);
                acc[j].z = fmaf(-a4.z, bv[j], acc[j].z);
                acc[j].w = fmaf(-a4.w, bv[j], acc[j].w);
            }
        }
        if (cc + 3 <= rr) {
#pragma unroll
            for (int j = 0; j < 4; ++j) *reinterpret_cast<float4 *>(&sa[(cc + j) * kDgLd + rr]) = acc[j];
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float av[4] = {acc[j].x, acc[j].y, acc[j].z, acc[j].w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (cc + j <= rr + i) sa[(cc + j) * kDgLd + rr + i] = av[i];
            }
        }
    }
}

// Right-looking by 32-column blocks J with a look-ahead inside the block:
//   (1) warp 0 factors the 32 x 32 diagonal block (lane i holds row i in
//       registers) without square roots on the pivot chain: with d_c the
//       pivot, a_ij -= (a_ic / d_c) a_jc.  Columns go through shared memory
//       two at a time (one store, four-wide broadcast loads) and every lane
//       forms the second pivot of the pair itself, so one store, barrier and
//       load serve two pivots; the columns are scaled by 1/sqrt(d_c)
//       afterwards.  Meanwhile
//       warps 1-15 subtract the previous block's panel from the columns right
//       of the next block;
//   (2) the rows below solve x L_JJ^T = a, and 32 more threads solve the rows
//       of the identity, giving W_JJ = L_JJ^-1 for the panel kernel (products
//       with a transposed copy of L_JJ, read four entries at a time);
//   (3) the panel is subtracted from the next block's 32 columns only, and
//       the finished column block goes back to HBM.
// The block is column-major in shared memory, copied in 16-byte pieces
// (4-byte pieces for an unaligned matrix or a short last block, which is
// padded with the identity: blockdiag(A11, I) factors as blockdiag(L11, I),
// so every step runs unpredicated on 128 rows).
// The kernel starts on whichever SM frees first, with a cold instruction
// cache, and its unrolled steps are tens of KB of code: a first pass of the
// step loop (J = -1) runs on the uninitialised shared memory, with every
// global store off, while the previous kernel still finishes (before
// pdl_wait), so the real passes run from a warm cache; its phases run side
// by side without barriers (warp 0 the pivots, the others the solves and
// updates), so it takes about as long as its longest phase.
__global__ void __launch_bounds__(kDgThreads) lowp_diag_kernel(float *L, int64_t ld, int64_t p, int b,
                                                               int64_t *info, double *min_ratio, float *Wd) {
    extern __shared__ __align__(16) float sa[];  // sa[c * kDgLd + r] = A11[r][c]
    float *slt = sa + kLpNb * kDgLd;              // slt[c * kDgLt + c2] = L_JJ[c2][c] for c2 > c, else 0
    float *colb = slt + 32 * kDgLt;               // two pairs of column buffers, then 1/sqrt(d)
    __shared__ __align__(16) float rdiag[32];     // 1 / L_JJ[c][c]
    __shared__ int failed, skip;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool v16 = b == kLpNb && ld % 4 == 0 && (reinterpret_cast<uintptr_t>(L) & 15) == 0;
    float ratio = 1e30f;
#pragma unroll 1
    for (int J = -1; J < 4; ++J) {
        const bool dry = J < 0;  // the warm-up pass: step 1's code, nothing stored globally
        if (J == 0) {
            __syncthreads();  // the warm-up pass has left shared memory
            pdl_wait();  // the block comes from the update just before
            pdl_trigger();
            // the lower triangle in two copy groups: columns 0-31 (the first step), then the rest
#pragma unroll
            for (int grp = 0; grp < 2; ++grp) {
                const int ncol = grp == 0 ? 32 : kLpNb - 32, cbase = grp == 0 ? 0 : 32;
                if (v16) {
                    for (int e = tid; e < ncol * (kLpNb / 4); e += kDgThreads) {
                        const int r4 = 4 * (e % (kLpNb / 4)), c = cbase + e / (kLpNb / 4);
                        if (r4 + 3 >= c) lp_cp16(&sa[c * kDgLd + r4], &L[(p + r4) + (p + c) * ld], 16);
                    }
                } else {
                    for (int e = tid; e < ncol * kLpNb; e += kDgThreads) {
                        const int r = e % kLpNb, c = cbase + e / kLpNb;
                        if (c <= r) {
                            if (r < b)
                                lp_cp4(&sa[c * kDgLd + r], &L[(p + r) + (p + c) * ld]);
                            else
                                sa[c * kDgLd + r] = (r == c) ? 1.f : 0.f;
                        }
                    }
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
            }
            if (tid == 0) {
                failed = 0;
                skip = *(volatile int64_t *)info >= 0;
            }
            asm volatile("cp.async.wait_group 1;" ::: "memory");
            __syncthreads();
            if (skip) {
                lp_cp_wait_all();
                return;
            }
            ratio = 1e30f;  // forget the warm-up pass's pivots
        }
        const int kb = dry ? 32 : 32 * J;
        if (warp == 0) {
            // (1) sqrt-free Cholesky of the 32 x 32 block
            float v[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) v[c] = (c <= lane) ? sa[(kb + c) * kDgLd + kb + lane] : 0.f;
            bool bad = false;
            float myd = 1.f;  // this lane's pivot d_lane
            // Two columns per round: both go to shared memory together, every lane
            // forms the 2 x 2 pivot block's recurrence itself (d_{c+1} after column
            // c's update) and the column c + 1 entries it needs, so one store,
            // barrier and load serve two pivots.
#pragma unroll
            for (int c = 0; c < 32; c += 2) {
                float *cb0 = colb + ((c >> 1) & 1) * 64, *cb1 = cb0 + 32;  // two buffer pairs: no reuse hazard
                cb0[lane] = v[c];
                cb1[lane] = v[c + 1];
                __syncwarp();
                const float a00 = cb0[c], a10 = cb0[c + 1], a11 = cb1[c + 1];
                const float r0 = dg_rcp(a00);
                const float d1 = fmaf(-(a10 * r0), a10, a11);  // pivot c + 1 after column c's update
                const float r1 = dg_rcp(d1);
                bad |= !(a00 > 0.f) || !(d1 > 0.f);  // non-positive (or NaN) pivot: breakdown
                myd = (lane == c) ? a00 : ((lane == c + 1) ? d1 : myd);
                const float s0 = v[c] * r0;                // l_{lane,c}
                const float u = fmaf(-s0, a10, v[c + 1]);  // a_{lane,c+1} after column c
                v[c + 1] = u;
                const float s1 = u * r1;  // l_{lane,c+1}
#pragma unroll
                for (int g = (c + 2) / 4; g < 8; ++g) {
                    const float4 t0 = *reinterpret_cast<const float4 *>(&cb0[4 * g]);
                    const float4 t1 = *reinterpret_cast<const float4 *>(&cb1[4 * g]);
                    const float tv0[4] = {t0.x, t0.y, t0.z, t0.w}, tv1[4] = {t1.x, t1.y, t1.z, t1.w};
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int c2 = 4 * g + i;
                        if (c2 > c + 1) {
                            const float w1 = fmaf(-(tv0[i] * r0), a10, tv1[i]);  // a_{c2,c+1} after column c
                            v[c2] = fmaf(-s1, w1, fmaf(-s0, tv0[i], v[c2]));
                        }
                    }
                }
            }
            // L[lane][c] = a_{lane,c} / sqrt(d_c) (c < lane), L[lane][lane] = sqrt(d_lane)
            const float rs_me = rsqrtf(myd);
            colb[128 + lane] = rs_me;
            __syncwarp();
#pragma unroll
            for (int g = 0; g < 8; ++g) {
                const float4 r4 = *reinterpret_cast<const float4 *>(&colb[128 + 4 * g]);
                const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int c = 4 * g + i;
                    v[c] = (c < lane) ? v[c] * rv[i] : (c == lane ? myd * rs_me : 0.f);
                }
            }
            if (kb + lane < b) ratio = fminf(ratio, myd);
            if (lane == 0 && bad && !dry) failed = 1;
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                if (c <= lane) sa[(kb + c) * kDgLd + kb + lane] = v[c];
                slt[c * kDgLt + lane] = (lane > c) ? v[c] : 0.f;
            }
            rdiag[lane] = rs_me;
        } else if (J != 0) {
            // the previous panel's product for the columns right of this block
            dg_syrk(sa, kb - 32, kb + 32, kb + 32, kLpNb, tid - 32, kDgThreads - 32);
        }
        if (J == 0) asm volatile("cp.async.wait_group 0;" ::: "memory");  // this thread's copies, columns 32-127
        if (!dry) __syncthreads();  // (the warm-up pass runs its phases side by side: its data is discarded)
        if (failed && !dry) break;  // (`failed` is set at the first real step)
        const int w = kLpNb - kb - 32;  // rows below the diagonal block
        // (2) rows below: x L_JJ^T = a; rows of the identity: W_JJ
        if (tid < w + 32) {
            const int ie = tid - w;                  // identity row, when >= 0
            const int r = ie < 0 ? kb + 32 + tid : 0;  // (row 0: any in-bounds address)
            float v[32], rd[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) v[c] = (ie < 0) ? sa[(kb + c) * kDgLd + r] : (c == ie ? 1.f : 0.f);
#pragma unroll
            for (int g = 0; g < 8; ++g) {  // the reciprocal diagonal in registers: off the chain
                const float4 r4 = *reinterpret_cast<const float4 *>(&rdiag[4 * g]);
                rd[4 * g] = r4.x, rd[4 * g + 1] = r4.y, rd[4 * g + 2] = r4.z, rd[4 * g + 3] = r4.w;
            }
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                v[c] *= rd[c];
#pragma unroll
                for (int g = (c + 1) / 4; g < 8; ++g) {
                    const float4 l4 = *reinterpret_cast<const float4 *>(&slt[c * kDgLt + 4 * g]);
                    const float lv[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        if (4 * g + i > c) v[4 * g + i] = fmaf(-v[c], lv[i], v[4 * g + i]);
                }
            }
            if (ie < 0) {
#pragma unroll
                for (int c = 0; c < 32; ++c) sa[(kb + c) * kDgLd + r] = v[c];
            } else {
#pragma unroll
                for (int c = 0; c < 32; ++c)
                    if (!dry) Wd[kb * 32 + ie * 32 + c] = v[c];  // W[c][ie] at [J][ie][c]
            }
        }
        if (!dry) __syncthreads();
        // (3) the next block's columns; the finished column block to HBM
        if (tid < 256) {
            if (w > 0) dg_syrk(sa, kb, kb + 32, kb + 32, kb + 64, tid, 256);
        } else {
            for (int e = tid - 256; e < (dry ? 0 : (kLpNb - kb) * 32); e += kDgThreads - 256) {
                const int r = kb + e % (kLpNb - kb), c = kb + e / (kLpNb - kb);
                if (r < b && c <= r) L[(p + r) + (p + c) * ld] = sa[c * kDgLd + r];
            }
        }
        if (!dry) __syncthreads();
    }
    if (failed) {
        if (tid == 0) *info = p;  // the low-precision factorisation broke down in this panel
        return;
    }
    if (warp == 0) {
        // smallest pivot of this block relative to the unit-ish equilibrated diagonal
        float rmin = ratio;
#pragma unroll
        for (int o = 16; o; o >>= 1) rmin = fminf(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
        if (lane == 0 && min_ratio) {
            const double d = (double)rmin;
            if (d >= 0.0)
                atomicMin((unsigned long long *)min_ratio,
                          (unsigned long long)__double_as_longlong(d));
        }
    }
}

// ---------------------------------------------------------------------------
// BF16 / FP16 parts of an FP32 value

template <typename H>
__device__ __forceinline__ H to_half(float x);
template <>
__device__ __forceinline__ __nv_bfloat16 to_half<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <>
__device__ __forceinline__ __half to_half<__half>(float x) { return __float2half_rn(x); }
__device__ __forceinline__ float from_half(__nv_bfloat16 h) { return __bfloat162float(h); }
__device__ __forceinline__ float from_half(__half h) { return __half2float(h); }

// ---------------------------------------------------------------------------
// panel: rows [q, n), q = p + 128.  L21 = A21 L11^-T in FP32 by 32-column
// blocks J, each a pair of small products (no sequential step):
//     Y_J = A_J - sum_{I<J} X_I L_JI^T,   X_J = Y_J W_JJ^T,
// W_JJ = L_JJ^-1 from the diagonal kernel (Wd[J][k][c] = W_JJ[c][k]); only the
// blocks of L11 below its diagonal blocks are read.  Then the operand planes of L21
// for the tensor cores (zero for k >= b).  One CTA of 256 threads per 64 rows;
// for products, thread (rt = tid % 32, ct = tid / 32) owns rows rt, rt + 32 and
// columns 4 ct .. 4 ct + 3 of the current block.
constexpr int kPnRows = 64;
constexpr int kPnXd = kPnRows + 4;  // row stride of sXT (k-major copy of the row tile)
constexpr int kPnLd = kLpNb + 4;    // row stride of sLT (k-major copy of L11, columns k < 96)
constexpr int kPnWd = 32 + 4;       // row stride of sWT (k-major W_JJ)
// 103,936 bytes: two CTAs per SM
constexpr size_t kPnSmem = sizeof(float) * (kLpNb * kPnXd + (kLpNb - 32) * kPnLd + 4 * 32 * kPnWd);

template <typename H>
__global__ void __launch_bounds__(256, 2) lowp_panel_kernel(float *L, int64_t ld, int64_t n, int64_t p,
                                                         const float *__restrict__ Wd, H *planes,
                                                         int64_t plane_stride, int64_t ldp, int koff, int terms,
                                                         const int64_t *info) {
    extern __shared__ __align__(16) float sm[];
    float *sXT = sm;                         // sXT[k * kPnXd + r] = row r, column k of the tile
    float *sLT = sXT + kLpNb * kPnXd;        // sLT[k * kPnLd + c] = L11[c][k]
    float *sWT = sLT + (kLpNb - 32) * kPnLd;  // sWT[(J * 32 + k) * kPnWd + c] = W_JJ[c][k]
    const int tid = threadIdx.x;
    const int64_t q = p + kLpNb;
    const int64_t row0 = q + (int64_t)blockIdx.x * kPnRows;
    // Columns of the row tile and of L11 are contiguous in memory.  With
    // 16-byte aligned columns every input is copied by cp.async, all of a
    // thread's copies in flight at once; otherwise by plain loads.
    const bool al16 = ld % 4 == 0 && (reinterpret_cast<uintptr_t>(L) & 15) == 0;
    if (al16) {
        // row tile: sXT[k][r] = L[row0 + r][p + k], 16 four-row chunks per column.
        // It was written by the update before the diagonal block's kernel, so
        // it is copied before the wait on that kernel.
        for (int e = tid; e < kLpNb * (kPnRows / 4); e += 256) {
            const int k = e / (kPnRows / 4), c4 = e % (kPnRows / 4);
            const int64_t r = row0 + 4 * c4;
            const int valid = n - r >= 4 ? 4 : (n - r > 0 ? (int)(n - r) : 0);
            lp_cp16(&sXT[k * kPnXd + 4 * c4], valid ? L + r + (p + k) * ld : L, 4 * valid);
        }
    }
    pdl_wait();  // L11, W_JJ and the status from the diagonal block's kernel
    pdl_trigger();
    if (*(volatile const int64_t *)info >= 0) {
        lp_cp_wait_all();
        return;
    }
    if (al16) {
        // L11 below its diagonal blocks: column k < 96, rows c in [32 (k/32 + 1), 128)
        for (int e = tid; e < 32 * (24 + 16 + 8); e += 256) {
            const int kb = e < 32 * 24 ? 0 : (e < 32 * 40 ? 1 : 2);
            const int idx = e - (kb == 0 ? 0 : (kb == 1 ? 32 * 24 : 32 * 40)), per = 24 - 8 * kb;
            const int k = 32 * kb + idx / per, c = 32 * (kb + 1) + 4 * (idx % per);
            lp_cp16(&sLT[k * kPnLd + c], L + (p + c) + (p + k) * ld, 16);
        }
        // W_JJ, k-major rows of 32
        for (int e = tid; e < 4 * 32 * 8; e += 256) {
            const int row = e / 8, c4 = e % 8;
            lp_cp16(&sWT[row * kPnWd + 4 * c4], Wd + row * 32 + 4 * c4, 16);
        }
        lp_cp_wait_all();
    } else {
        {
            const int r = tid % kPnRows;
            const bool ok = row0 + r < n;
            const float *src = L + (row0 + r) + p * ld;
#pragma unroll 8
            for (int k = tid / kPnRows; k < kLpNb; k += 256 / kPnRows) sXT[k * kPnXd + r] = ok ? src[k * ld] : 0.f;
        }
        {
            const int c = tid % kLpNb;
            const float *src = L + (p + c) + p * ld;
#pragma unroll 8
            for (int k = tid / kLpNb; k < kLpNb - 32; k += 256 / kLpNb)
                sLT[k * kPnLd + c] = (32 * (k / 32 + 1) <= c) ? src[k * ld] : 0.f;
        }
#pragma unroll
        for (int e = tid; e < 4 * 32 * 32; e += 256) sWT[(e / 32) * kPnWd + e % 32] = Wd[e];
    }
    __syncthreads();
    const int rt = tid % 32, ct = tid / 32;
#pragma unroll 1
    for (int J = 0; J < 4; ++J) {
        const int cj = J * 32 + 4 * ct;  // this thread's first column
        float acc[2][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            acc[0][u] = sXT[(cj + u) * kPnXd + rt];
            acc[1][u] = sXT[(cj + u) * kPnXd + rt + 32];
        }
        // Y_J = A_J - X_{<J} L_J,<J^T, eight k at a time: all their shared loads
        // issue before the products, so the loop is not a chain of load latencies
        for (int k0 = 0; k0 < J * 32; k0 += 8) {
            float x0[8], x1[8];
            float4 l4[8];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                x0[kk] = sXT[(k0 + kk) * kPnXd + rt];
                x1[kk] = sXT[(k0 + kk) * kPnXd + rt + 32];
                l4[kk] = *reinterpret_cast<const float4 *>(&sLT[(k0 + kk) * kPnLd + cj]);
            }
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                const float lv[4] = {l4[kk].x, l4[kk].y, l4[kk].z, l4[kk].w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    acc[0][u] = fmaf(-x0[kk], lv[u], acc[0][u]);
                    acc[1][u] = fmaf(-x1[kk], lv[u], acc[1][u]);
                }
            }
        }
        __syncthreads();  // every thread has read A_J
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            sXT[(cj + u) * kPnXd + rt] = acc[0][u];
            sXT[(cj + u) * kPnXd + rt + 32] = acc[1][u];
        }
        __syncthreads();
        // X_J = Y_J W_JJ^T
        float x[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int k0 = 0; k0 < 32; k0 += 8) {
            float y0[8], y1[8];
            float4 w4[8];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                const int k = J * 32 + k0 + kk;
                y0[kk] = sXT[k * kPnXd + rt];
                y1[kk] = sXT[k * kPnXd + rt + 32];
                w4[kk] = *reinterpret_cast<const float4 *>(&sWT[k * kPnWd + 4 * ct]);
            }
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                const float wv[4] = {w4[kk].x, w4[kk].y, w4[kk].z, w4[kk].w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    x[0][u] = fmaf(y0[kk], wv[u], x[0][u]);
                    x[1][u] = fmaf(y1[kk], wv[u], x[1][u]);
                }
            }
        }
        __syncthreads();  // every thread has read Y_J
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            sXT[(cj + u) * kPnXd + rt] = x[0][u];
            sXT[(cj + u) * kPnXd + rt + 32] = x[1][u];
        }
        __syncthreads();
    }
    // L21 back to the factor (columns contiguous)
    for (int e = tid; e < kLpNb * kPnRows; e += 256) {
        const int r = e % kPnRows, k = e / kPnRows;
        const int64_t j = row0 + r;
        if (j < n) L[j + (p + k) * ld] = sXT[k * kPnXd + r];
    }
    // operand planes (row j at j * ldp, columns koff ..), 16-byte stores of 8
    // halves: thread (row, 8-column group)
    for (int e = tid; e < kPnRows * (kLpNb / 8); e += 256) {
        const int r = e % kPnRows, k0 = (e / kPnRows) * 8;
        const int64_t j = row0 + r;
        if (j >= n) continue;
        H h[3][8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const float xv = (k0 + u < kLpNb) ? sXT[(k0 + u) * kPnXd + r] : 0.f;
            const H a0 = to_half<H>(xv);
            const float r1 = xv - from_half(a0);  // exact in FP32
            const H a1 = to_half<H>(r1);
            const float r2 = r1 - from_half(a1);
            h[0][u] = a0;
            h[1][u] = a1;
            h[2][u] = to_half<H>(r2);
        }
#pragma unroll
        for (int t = 0; t < 3; ++t)
            if (t < terms) *(uint4 *)(planes + t * plane_stride + j * ldp + koff + k0) = *(const uint4 *)h[t];
    }
}

// ---------------------------------------------------------------------------
// host loop

int lowp_factor_launch(float *L, int64_t n, int64_t ld, const lla_refine_opts &opts, int64_t *info,
                       float *diag0, double *min_ratio, Ctx *c, cudaStream_t st) {
    const int upd = opts.update;
    if (upd == LLA_UPDATE_FP32) return potrf_fast_launch<float>(L, n, ld, info, diag0, min_ratio, st);
    const bool fp16 = (upd == LLA_UPDATE_FP16 || upd == LLA_UPDATE_FP16X3);
    const int terms = (upd == LLA_UPDATE_BF16 || upd == LLA_UPDATE_FP16) ? 1
                      : (upd == LLA_UPDATE_BF16X6)                        ? 3
                                                                          : 2;
    TcPairs pairs;
    if (terms == 1) {
        pairs.n = 1;
        pairs.pa[0] = 0; pairs.pb[0] = 0;
    } else if (terms == 2) {  // small products first
        pairs.n = 3;
        const int pa[3] = {0, 1, 0}, pb[3] = {1, 0, 0};
        for (int i = 0; i < 3; ++i) pairs.pa[i] = pa[i], pairs.pb[i] = pb[i];
    } else {
        pairs.n = 6;
        const int pa[6] = {0, 1, 2, 0, 1, 0}, pb[6] = {2, 1, 0, 1, 0, 0};
        for (int i = 0; i < 6; ++i) pairs.pa[i] = pa[i], pairs.pb[i] = pb[i];
    }
    // Operand planes indexed by absolute row (row j at j * ldp): two 128-column
    // halves, one per panel of a pair (see the loop below).
    const int64_t ldp = 2 * kLpNb;
    const int64_t plane_stride = n * ldp;  // elements per plane
    if (c->mixed.opA.ensure(sizeof(uint16_t) * plane_stride * terms) != cudaSuccess) return -1;
    void *planes = c->mixed.opA.p;
    // status word, then the update's tile-claim counter (zeroed here; the
    // launches below advance sched_base in step with it)
    if (c->mixed.tcerr.ensure(4 * sizeof(int)) != cudaSuccess) return -1;
    int *err_word = (int *)c->mixed.tcerr.p;
    unsigned *sched = (unsigned *)c->mixed.tcerr.p + 1;
    unsigned sched_base = 0;
    if (cudaMemsetAsync(err_word, 0, 4 * sizeof(int), st) != cudaSuccess) return -1;
    const size_t smem_l11 = kDgSmem;
    const size_t smem_panel = kPnSmem;
    if (c->mixed.pinv.ensure(sizeof(float) * 4 * 32 * 32) != cudaSuccess) return -1;
    float *Wd = (float *)c->mixed.pinv.p;
    // kernel attributes are per device: set them on every call (cheap)
    if (cudaFuncSetAttribute(lowp_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_l11) !=
            cudaSuccess ||
        cudaFuncSetAttribute(lowp_panel_kernel<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_panel) != cudaSuccess ||
        cudaFuncSetAttribute(lowp_panel_kernel<__half>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_panel) != cudaSuccess ||
        tc_update_prepare() != 0)
        return -1;
    const size_t esz = sizeof(uint16_t);
    // Every launch of the loop below is a programmatic dependent of the one
    // before it (each kernel waits for its predecessor's output after its
    // set-up), so a kernel's launch and prologue overlap the previous tail.
    auto diag = [&](int64_t p, int b) {
        LaunchScope ls(K_MIXED_DIAG, st, (double)b * b * b / 3.0);
        launch_maybe_pdl(true, lowp_diag_kernel, dim3(1), dim3(kDgThreads), smem_l11, st, L, ld, p, b, info,
                         min_ratio, Wd);
    };
    // L21 and its planes for rows [p + 128, n), written to plane half `half`
    auto panel = [&](int64_t p, int half) {
        const int64_t rest = n - p - kLpNb;
        LaunchScope ls(K_MIXED_PANEL, st, (double)rest * kLpNb * kLpNb);
        const dim3 grid((unsigned)ceil_div(rest, kPnRows));
        if (fp16)
            launch_maybe_pdl(true, lowp_panel_kernel<__half>, grid, dim3(256), smem_panel, st, L, ld, n, p,
                             (const float *)Wd, (__half *)planes, plane_stride, ldp, half * kLpNb, terms,
                             (const int64_t *)info);
        else
            launch_maybe_pdl(true, lowp_panel_kernel<__nv_bfloat16>, grid, dim3(256), smem_panel, st, L, ld, n,
                             p, (const float *)Wd, (__nv_bfloat16 *)planes, plane_stride, ldp, half * kLpNb,
                             terms, (const int64_t *)info);
    };
    // A22 -= sum of the products of K columns of the planes, rows [q, n)
    auto update = [&](int64_t q, int kext, bool narrow) -> int {
        const int64_t rows = n - q;
        const int64_t cols = narrow ? std::min<int64_t>(kLpNb, rows) : rows;
        // algorithmic work: the lower trailing entries x kext multiply-adds x 2
        LaunchScope ls(K_MIXED_UPDATE, st,
                       narrow ? (double)rows * cols * kext * 2.0 - (double)cols * (cols - 1) * kext
                              : (double)rows * (rows + 1) * kext);
        return tc_update_launch(L, ld, q, n, (char *)planes + (size_t)q * ldp * esz, plane_stride, ldp, rows,
                                kext, terms, fp16, pairs, info, err_word, sched, &sched_base, narrow, st,
                                opts.update_kchunk, opts.update_epilogue, true);
    };
    // Panels in pairs: after panel p only the next panel's 128 columns are
    // updated (narrow); panel p + 128 is factored, and then both panels'
    // products are subtracted from the rest in one pass with K = 256, so the
    // FP32 trailing matrix is read and written once per pair of panels.
    for (int64_t p = 0; p < n;) {
        const int b = (int)std::min<int64_t>(kLpNb, n - p);
        diag(p, b);
        const int64_t rest = n - p - b;
        if (rest <= 0) break;  // b == 128 whenever rows remain below the block
        panel(p, 0);
        if (rest > kLpNb) {
            if (update(p + kLpNb, kLpNb, true) != 0) return -1;
            diag(p + kLpNb, kLpNb);
            panel(p + kLpNb, 1);
            if (update(p + 2 * kLpNb, 2 * kLpNb, false) != 0) return -1;
            p += 2 * kLpNb;
        } else {
            if (update(p + kLpNb, kLpNb, false) != 0) return -1;
            p += kLpNb;
        }
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace lla

// ---------------------------------------------------------------------------
// C ABI: the low-precision factorisation on its own

extern "C" int lla_spotrf_mixed_device(float *dA, int64_t n, int64_t ld, int update, int64_t *d_info,
                                       void *stream, lla_error *err) {
    using namespace lla;
    if (n < 0 || ld < std::max<int64_t>(1, n) || !d_info || (n > 0 && !dA) ||
        !(update == LLA_UPDATE_FP32 || update == LLA_UPDATE_BF16 || update == LLA_UPDATE_BF16X3 ||
          update == LLA_UPDATE_BF16X6 || update == LLA_UPDATE_FP16 || update == LLA_UPDATE_FP16X3))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(d_info, 0xff, sizeof(int64_t), st);
    if (e != cudaSuccess) return lla__set_cuda_error(err, e);
    if (n == 0) return LLA_OK;
    if ((e = c->mixed.diag0.ensure(sizeof(float) * n)) != cudaSuccess) return lla__set_cuda_error(err, e);
    lla_refine_opts o;
    lla_refine_opts_default(&o);
    o.update = update;
    if (lowp_factor_launch(dA, n, ld, o, d_info, (float *)c->mixed.diag0.p, nullptr, c, st) != 0) {
        e = cudaGetLastError();
        return lla__set_cuda_error(err, e == cudaSuccess ? cudaErrorUnknown : e);
    }
    if (update != LLA_UPDATE_FP32) {
        int flag = 0;
        if ((e = cudaMemcpyAsync(&flag, c->mixed.tcerr.p, sizeof(int), cudaMemcpyDeviceToHost, st)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return lla__set_cuda_error(err, e);
        if (flag) return lla__set_status(err, flag);
    }
    return LLA_OK;
}

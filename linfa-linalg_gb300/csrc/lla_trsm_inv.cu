// lla_trsm_inv.cu -- FP32 triangular solves of the mixed-precision refinement
// with inverted diagonal blocks.
//
// The refinement solves with the same low-precision factor L eight to ten
// times, so five small matrices per 64-row block are formed once per factor:
//     W_r   = L_rr^-1                     (diag_inverse_kernel)
//     F_r^d = W_r L_{r,r-d}               (forward coupling, d = 1, 2; fuse_kernel)
//     G_r^d = W_r^T L_{r+d,r}^T           (backward coupling, d = 1, 2; fuse_kernel)
// and every substitution is a chain of small matrix products:
//     forward  L Y = B  : Y_r = W_r (B_r - sum_{q<r-2} L_rq Y_q) - F_r^2 Y_{r-2} - F_r^1 Y_{r-1}
//     backward L^T X = Y: X_r = W_r^T (Y_r - sum_{q>r+2} L_qr^T X_q) - G_r^2 X_{r+2} - G_r^1 X_{r+1}
// One owner CTA per (64-row block, 16-column chunk); CTAs take tickets in
// processing order.  The sum over blocks solved three or more steps earlier
// and its product with W_r are formed while the two previous blocks are
// still being solved, the second neighbour's term while the first is, so the
// only work on the block-to-block critical path is one 64 x 64 x 16 product.
// An owner sums at most the last kIvOwn of those coupling terms itself; wide
// helper CTAs sum the earlier ones in groups of kIvGroup positions for 64
// columns at a time (lla_trsm_sched.h gives the ticket order).
//
// Hand-off between owners: a solved value is published as one 64-bit word
// (launch epoch << 32 | float bits) in a staging array, so a consumer polls
// the data itself -- one memory round trip per hand-off, no separate flag.
// Wide helpers, which read 64 x 64 tiles of solved values, take them as
// plain floats from B once the owners' (position, chunk) flags (epoch << 32 |
// 1, released after the stores) are set, and publish their partial sums as
// tagged words followed by one flag per slot, on which the owner waits.
// The host gives every launch a fresh nonzero epoch and clears the staging
// array whenever it is (re)allocated, so a word or flag from an earlier
// launch never matches.  Every wait is bounded and reports LLA_ERR_TIMEOUT.
#include <cuda_runtime.h>

#include <algorithm>

#include "lla_common.cuh"
#include "lla_mixed.h"
#include "lla_prof.h"
#include "lla_trsm_sched.h"

namespace lla {

constexpr int kIvNb = 64;
constexpr int kIvTile = kIvNb * kIvNb;

// W_r = L_rr^-1 (lower, FP32), padded with the identity past n.  One CTA of
// 64 threads per block; thread j computes column j by forward substitution.
__global__ void __launch_bounds__(64) diag_inverse_kernel(const float *__restrict__ L, int64_t ld, int64_t n,
                                                          float *W) {
    __shared__ float sL[kIvNb][kIvNb + 1];
    const int64_t r0 = (int64_t)blockIdx.x * kIvNb;
    const int j = threadIdx.x;
    for (int e = j; e < kIvTile; e += 64) {
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
    float *Wr = W + (int64_t)blockIdx.x * kIvTile;  // column-major 64 x 64
#pragma unroll
    for (int i = 0; i < kIvNb; ++i) Wr[i + j * kIvNb] = w[i];
}

// F_r^d = W_r L_{r,r-d} and G_r^d = W_r^T L_{r+d,r}^T for d = blockIdx.y + 1
// (zero where that block does not exist), both column-major 64 x 64, in the
// sets 2d - 1 and 2d after the inverses (set 0).  One CTA of 256 threads per
// (block, d); thread (i, kq) forms F[i][k] and G[i][k] for k = kq + 4u.
__global__ void __launch_bounds__(256) fuse_kernel(const float *__restrict__ L, int64_t ld, int64_t n,
                                                   float *Wall) {
    __shared__ float sW[kIvNb][kIvNb + 1];  // sW[a][b] = W_r[a][b]
    __shared__ float sC[kIvNb][kIvNb + 1];
    const int64_t r = blockIdx.x, R = gridDim.x, d = blockIdx.y + 1;
    const int tid = threadIdx.x, i = tid % kIvNb, kq = tid / kIvNb;
    const float *Wr = Wall + r * kIvTile;
    float *F = Wall + (2 * d - 1) * R * kIvTile, *G = Wall + 2 * d * R * kIvTile;
    for (int e = tid; e < kIvTile; e += 256) sW[e % kIvNb][e / kIvNb] = Wr[e];
    // forward: sC[j][k] = L[r*64 + j][(r-d)*64 + k]
    for (int e = tid; e < kIvTile; e += 256) {
        const int j = e % kIvNb, k = e / kIvNb;
        const int64_t gi = r * kIvNb + j, gk = (r - d) * kIvNb + k;
        sC[j][k] = (r >= d && gi < n) ? L[gi + gk * ld] : 0.f;
    }
    __syncthreads();
    float acc[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[u] = 0.f;
    for (int j = 0; j < kIvNb; ++j) {
        const float wv = sW[i][j];
#pragma unroll
        for (int u = 0; u < 16; ++u) acc[u] = fmaf(wv, sC[j][kq + 4 * u], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) F[r * kIvTile + i + (kq + 4 * u) * kIvNb] = acc[u];
    __syncthreads();
    // backward: sC[k][j] = L[(r+d)*64 + k][r*64 + j]; G[i][k] = sum_j W[j][i] sC[k][j]
    for (int e = tid; e < kIvTile; e += 256) {
        const int k = e % kIvNb, j = e / kIvNb;
        const int64_t gk = (r + d) * kIvNb + k, gj = r * kIvNb + j;
        sC[k][j] = (r + d < R && gk < n) ? L[gk + gj * ld] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[u] = 0.f;
    for (int j = 0; j < kIvNb; ++j) {
        const float wv = sW[j][i];
#pragma unroll
        for (int u = 0; u < 16; ++u) acc[u] = fmaf(wv, sC[kq + 4 * u][j], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) G[r * kIvTile + i + (kq + 4 * u) * kIvNb] = acc[u];
}

__device__ __forceinline__ unsigned long long iv_ld_word(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void iv_st_word(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void iv_cp16(void *dst, const void *src, int bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void iv_cp4(void *dst, const void *src, int bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void iv_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void iv_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Bounded re-read of up to four hand-off words (p[u] == nullptr: none)
// until each carries this launch's tag; the words are re-read together, so a
// hand-off costs one memory round trip however many of them were late.  NAP:
// nanoseconds to sleep after every unsuccessful re-read, for waits off the
// critical path (0: re-read at once, for the block-to-block hand-off), so
// that CTAs waiting far ahead of the chain leave L2 and the SMs to the CTAs
// that compute.
template <int NAP = 0>
__device__ __forceinline__ void iv_settle4(unsigned long long (&w)[4], const unsigned long long *const (&p)[4],
                                           unsigned long long tag, int *err_word, int *abort_flag) {
    long long spins = 0;
    for (;;) {
        bool done = true;
#pragma unroll
        for (int u = 0; u < 4; ++u) done &= (p[u] == nullptr) || ((w[u] & 0xffffffff00000000ull) == tag);
        if (done) return;
        if (NAP > 0 || ((++spins) & 63) == 0) {
            if (NAP > 0) ++spins;
            if (*(volatile int *)err_word != 0 || spins > kSpinLimit) {
                atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
                *abort_flag = 1;
                return;
            }
            __nanosleep(NAP > 0 ? NAP : 32);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (p[u] != nullptr && (w[u] & 0xffffffff00000000ull) != tag) w[u] = iv_ld_word(p[u]);
    }
}

constexpr int kIvCols = 16;   // right-hand-side columns per CTA
constexpr int kIvLd = 68;     // shared row stride of a staged 64 x 64 tile (floats; 16-byte rows)
constexpr int kIvStages = 3;  // coupling tiles in flight per CTA
constexpr int kIvYd = kIvNb + 2;  // words per staged column (padded: 528-byte columns)
constexpr size_t kIvSmem = sizeof(float) * ((size_t)kIvStages * kIvNb * kIvLd + 2ull * kIvStages * kIvCols * kIvYd +
                                            2ull * kIvNb * kIvCols + 2ull * kIvCols * kIvLd);

// t[j] += sign * sum_k A[k][ta] X[k][4 tb + j] over the 64 k of a block: four k
// at a time with all their shared loads issued before the products, and two
// partial sums per output (even and odd k), so the loop is neither a chain of
// load latencies nor one long FMA chain.
template <int SIGN, int XC>
__device__ __forceinline__ void iv_dot64(float (&t)[4], const float (*A)[kIvLd], const float (*X)[XC], int ta,
                                         int tb) {
    float pe[4] = {0.f, 0.f, 0.f, 0.f}, po[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k0 = 0; k0 < kIvNb; k0 += 4) {
        float l[4];
        float4 x[4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            l[kk] = A[k0 + kk][ta];
            x[kk] = *reinterpret_cast<const float4 *>(&X[k0 + kk][tb * 4]);
        }
#pragma unroll
        for (int kk = 0; kk < 4; kk += 2) {
            pe[0] = fmaf(l[kk], x[kk].x, pe[0]);
            pe[1] = fmaf(l[kk], x[kk].y, pe[1]);
            pe[2] = fmaf(l[kk], x[kk].z, pe[2]);
            pe[3] = fmaf(l[kk], x[kk].w, pe[3]);
            po[0] = fmaf(l[kk + 1], x[kk + 1].x, po[0]);
            po[1] = fmaf(l[kk + 1], x[kk + 1].y, po[1]);
            po[2] = fmaf(l[kk + 1], x[kk + 1].z, po[2]);
            po[3] = fmaf(l[kk + 1], x[kk + 1].w, po[3]);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) t[j] = SIGN > 0 ? t[j] + (pe[j] + po[j]) : t[j] - (pe[j] + po[j]);
}

// Wide helpers: shared memory of a coupling-tile ring and a ring of 64-column
// tiles of solved values (64 rows each, k contiguous per column).
constexpr size_t kIvWideSmem = sizeof(float) * 2ull * kIvStages * kIvNb * kIvLd;
constexpr size_t kIvLaunchSmem = kIvWideSmem > kIvSmem ? kIvWideSmem : kIvSmem;

__device__ __forceinline__ unsigned long long iv_ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void iv_st_release(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// One wide helper: the coupling terms of positions [q0, q1) for block rb, all
// 64 columns of column group cgrp at once (four times the work of a 16-column
// stage for the same copies and barriers), published negated as epoch-tagged
// words pw[row + 64 col].  The solved values come as plain floats from B, once
// the owners of (position, chunk) have raised their flags (release after
// their stores; acquire here, all of the group's flags polled at once before
// the first copy: one round trip, not one per position).  Thread (ri = tid % 16,
// ci = tid / 16) owns columns 4 ci .. 4 ci + 3 and rows 4 ri + j (ri + 16 j
// when trans).
template <bool TRANS>
__device__ __forceinline__ void iv_wide_helper(const float *__restrict__ L, int64_t ld, const float *B, int64_t ldb,
                                               int64_t n, int64_t m, int64_t R, int64_t rb, int64_t q0, int64_t q1,
                                               int cgrp, int nch, unsigned long long *pw, unsigned long long *hflag,
                                               const unsigned long long *flags, unsigned long long tag,
                                               int *err_word, int *abort_flag, float *smem, bool al16) {
    constexpr int NS = kIvStages;
    float(*sT)[kIvNb][kIvLd] = reinterpret_cast<float(*)[kIvNb][kIvLd]>(smem);
    float(*sY)[kIvNb][kIvLd] = reinterpret_cast<float(*)[kIvNb][kIvLd]>(smem + NS * kIvNb * kIvLd);
    const int tid = threadIdx.x, ri = tid % 16, ci = tid / 16;
    const int64_t c0 = (int64_t)cgrp * kIvNb;
    const int64_t nst = q1 - q0;
    auto issue = [&](int64_t i, int s) {
        if (i < nst && !*(volatile int *)abort_flag) {
            const int64_t pq = q0 + i;
            const int64_t qb = TRANS ? R - 1 - pq : pq;
            const int64_t rowbase = (TRANS ? qb : rb) * kIvNb, colbase = (TRANS ? rb : qb) * kIvNb;
            if (al16) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int e = tid + 256 * j, a = e >> 4, c4 = e & 15;
                    const int64_t row = rowbase + 4 * c4, col = colbase + a;
                    const bool ok = row < n && col < n;
                    const int bytes = ok ? 4 * (int)(n - row < 4 ? n - row : 4) : 0;
                    iv_cp16(&sT[s][a][4 * c4], ok ? L + row + col * ld : L, bytes);
                }
            } else {
#pragma unroll 4
                for (int j = 0; j < 16; ++j) {
                    const int e = tid + 256 * j, a = e >> 6, b = e & 63;
                    const int64_t row = rowbase + b, col = colbase + a;
                    const bool ok = row < n && col < n;
                    iv_cp4(&sT[s][a][b], ok ? L + row + col * ld : L, ok ? 4 : 0);
                }
            }
            // solved values of block qb, columns c0 + cy: chunk (c0 + cy) / 16 = 4 cgrp + j
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int e = tid + 256 * j, cy = e >> 4, r4 = 4 * (e & 15);
                const int64_t col = c0 + cy, row = qb * kIvNb + r4;
                const bool ok = col < m && row < n;
                if (ok && !(al16 && ldb % 4 == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0)) {
#pragma unroll
                    for (int h = 0; h < 4; ++h)
                        iv_cp4(&sY[s][cy][r4 + h], row + h < n ? B + row + h + col * ldb : B, row + h < n ? 4 : 0);
                } else {
                    const int bytes = ok ? 4 * (int)(n - row < 4 ? n - row : 4) : 0;
                    iv_cp16(&sY[s][cy][r4], ok ? B + row + col * ldb : B, bytes);
                }
            }
        }
        iv_commit();
    };
    {  // every (position, chunk) flag this helper depends on, polled at once: thread 4 i + j
       // waits for position q0 + i, chunk 4 cgrp + j (bounded), then the barrier passes
       // the acquired values on to the whole CTA before the copies
        const int64_t i = tid >> 2;
        const int j = tid & 3;
        if (i < nst && c0 + 16 * j < m) {
            const unsigned long long *f = flags + (q0 + i) * nch + (4 * cgrp + j);
            long long spins = 0;
            while (iv_ld_acquire(f) != (tag | 1ull)) {
                if (*(volatile int *)err_word != 0 || ++spins > kSpinLimit) {
                    atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
                    *abort_flag = 1;
                    break;
                }
                __nanosleep(256);
            }
        }
        __syncthreads();
    }
    float part[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) part[j][jj] = 0.f;
#pragma unroll
    for (int s = 0; s < NS - 1; ++s) issue(s, s);
    for (int64_t pq = 0; pq < nst; ++pq) {
        const int s = (int)(pq % NS);
        iv_wait<NS - 2>();
        __syncthreads();
        if (*(volatile int *)abort_flag) break;
        issue(pq + NS - 1, (int)((pq + NS - 1) % NS));
#pragma unroll 4
        for (int k0 = 0; k0 < kIvNb; k0 += 4) {
            float4 y[4];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) y[jj] = *reinterpret_cast<const float4 *>(&sY[s][4 * ci + jj][k0]);
            if (!TRANS) {  // coefficient of y_k in row i: sT[s][k][i]
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const float4 l4 = *reinterpret_cast<const float4 *>(&sT[s][k0 + kk][4 * ri]);
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        const float yv = kk == 0 ? y[jj].x : kk == 1 ? y[jj].y : kk == 2 ? y[jj].z : y[jj].w;
                        part[0][jj] = fmaf(-l4.x, yv, part[0][jj]);
                        part[1][jj] = fmaf(-l4.y, yv, part[1][jj]);
                        part[2][jj] = fmaf(-l4.z, yv, part[2][jj]);
                        part[3][jj] = fmaf(-l4.w, yv, part[3][jj]);
                    }
                }
            } else {  // coefficient of y_k in row i: sT[s][i][k]
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float4 l4 = *reinterpret_cast<const float4 *>(&sT[s][ri + 16 * j][k0]);
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        float a = part[j][jj];
                        a = fmaf(-l4.x, y[jj].x, a);
                        a = fmaf(-l4.y, y[jj].y, a);
                        a = fmaf(-l4.z, y[jj].z, a);
                        a = fmaf(-l4.w, y[jj].w, a);
                        part[j][jj] = a;
                    }
                }
            }
        }
    }
    iv_wait<0>();
    if (*(volatile int *)abort_flag) return;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int rl = TRANS ? ri + 16 * j : 4 * ri + j;
        if (rb * kIvNb + rl >= n) continue;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int cl = 4 * ci + jj;
            if (c0 + cl < m) iv_st_word(pw + rl + kIvNb * cl, tag | (unsigned long long)__float_as_uint(part[j][jj]));
        }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) iv_st_release(hflag, tag | 1ull);  // one flag for the owners to wait on
}

// TRANS = false: L Y = B (blocks ascending); TRANS = true: L^T X = B (descending).
// 256 threads.  The coupling tiles and the solved words of earlier blocks
// stream through a kIvStages-deep cp.async ring.  Each thread validates the
// words it copied and stores their values into a float copy of the block
// (sYf[c][k], two buffers).  The coupling products are split over K: warp
// pair kg sums k in [16 kg, 16 kg + 16) into a 4 x 4 register tile (columns
// cg + 4 jj; rows 4 rq + j, or rq + 16 j when trans, so that the shared loads
// are free of bank conflicts), and the four partial sums are added in kg
// order at the end, into thread (c = tid % 16, rg = tid / 16)'s column c,
// rows 4 rg .. 4 rg + 3.  For the block's own products (inverse, neighbour)
// thread (ta = tid % 64, tb = tid / 64) owns row ta and columns 4 tb .. 4 tb + 3.
template <bool TRANS>
__global__ void __launch_bounds__(256, 2) trsm_inv_kernel(const float *__restrict__ L, int64_t ld,
                                                          const float *__restrict__ Wall, int64_t n,
                                                          float *B, int64_t ldb, int64_t m, int nchunks,
                                                          unsigned long long *ll, int64_t ldl, unsigned epoch,
                                                          int *counter, int *err_word, int ngrp,
                                                          unsigned long long *pw, unsigned long long *flags,
                                                          const int *state) {
    if (refine_done(state)) return;  // the refinement has finished: nothing to solve
    constexpr int C = kIvCols, LPT = kIvTile / 256, NS = kIvStages;
    constexpr int YCH = kIvNb * C / 2 / 256;  // 16-byte (two-word) copies per thread per stage
    extern __shared__ __align__(16) float iv_smem[];
    // sT[s][a][b]: staged tile; sY[s][c][k]: solved words; sV[2][k][c]: the block's own products
    float(*sT)[kIvNb][kIvLd] = reinterpret_cast<float(*)[kIvNb][kIvLd]>(iv_smem);
    unsigned long long(*sY)[C][kIvYd] =
        reinterpret_cast<unsigned long long(*)[C][kIvYd]>(iv_smem + NS * kIvNb * kIvLd);
    float(*sV)[kIvNb][C] = reinterpret_cast<float(*)[kIvNb][C]>(iv_smem + NS * kIvNb * kIvLd + 2 * NS * C * kIvYd);
    float(*sYf)[C][kIvLd] =
        reinterpret_cast<float(*)[C][kIvLd]>(iv_smem + NS * kIvNb * kIvLd + 2 * NS * C * kIvYd + 2 * kIvNb * C);
    static_assert(NS >= 3, "the partial sums and the second neighbour's coupling matrix reuse stage 2");
    __shared__ int s_ticket, s_abort;
    const int tid = threadIdx.x;
    if (tid == 0) {
        s_ticket = atomicAdd(counter, 1);
        s_abort = 0;
    }
    __syncthreads();
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    bool helper;
    int64_t pb, slot;  // position in processing order; a helper's partial-sum slot
    int grp, cc;
    iv_decode(s_ticket, R, nchunks, ngrp, helper, pb, grp, cc, slot);
    const int64_t rb = TRANS ? R - 1 - pb : pb;
    const unsigned long long tag = (unsigned long long)epoch << 32;
    const bool al16 = (ld % 4 == 0) && ((reinterpret_cast<uintptr_t>(L) & 15) == 0);
    if (helper) {  // a wide helper: coupling terms of positions [grp G, ...) for 64 columns
        const int64_t q0 = (int64_t)grp * kIvGroup, q1 = min(q0 + kIvGroup, iv_qlo(pb));
        iv_wide_helper<TRANS>(L, ld, B, ldb, n, m, R, rb, q0, q1, cc, nchunks, pw + slot * kIvTile,
                              flags + R * nchunks + slot, flags, tag, err_word, &s_abort, iv_smem, al16);
        return;
    }
    const int ta = tid % kIvNb, tb = tid / kIvNb;
    const int64_t grow = rb * kIvNb + ta;
    const int64_t col0 = (int64_t)cc * C;

    const int bc = tid % C, rg = tid / C;  // bulk mapping: column bc, rows 4 rg .. 4 rg + 3
    float acc[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t row = rb * kIvNb + 4 * rg + i, col = col0 + bc;
        acc[i] = (row < n && col < m) ? B[row + col * ldb] : 0.f;
    }
    // this block's inverse and coupling matrix (element (ta, tb + 4u) of each), needed only at the end
    float preW[LPT], preM[LPT];
    {
        const float *Wr = Wall + rb * kIvTile + ta + tb * kIvNb;
        const float *Mr = Wall + ((TRANS ? 2 : 1) * R + rb) * kIvTile + ta + tb * kIvNb;
#pragma unroll
        for (int u = 0; u < LPT; ++u) {
            preW[u] = Wr[u * 4 * kIvNb];
            preM[u] = Mr[u * 4 * kIvNb];
        }
    }
    // the owner's own coupling terms: positions q_lo .. pb-3 (the wide helpers have the earlier ones)
    const int64_t q_lo = iv_qlo(pb);
    const int64_t nbulk = pb > 1 ? pb - 2 - q_lo : 0;

    // Stage s <- coupling tile and solved words of processing position pq.
    // Tile: 64 columns a of 64 contiguous rows b (non-trans: a = k, b = i;
    // trans: a = i, b = k), zero-filled past n.
    auto issue = [&](int64_t pi, int s) {
        if (pi < nbulk) {
            const int64_t pq = q_lo + pi;
            const int64_t qb = TRANS ? R - 1 - pq : pq;
            const int64_t rowbase = (TRANS ? qb : rb) * kIvNb, colbase = (TRANS ? rb : qb) * kIvNb;
            if (al16) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int e = tid + 256 * j, a = e >> 4, c4 = e & 15;
                    const int64_t row = rowbase + 4 * c4, col = colbase + a;
                    const bool ok = row < n && col < n;
                    const int bytes = ok ? 4 * (int)(n - row < 4 ? n - row : 4) : 0;
                    iv_cp16(&sT[s][a][4 * c4], ok ? L + row + col * ld : L, bytes);
                }
            } else {
#pragma unroll 4
                for (int j = 0; j < 16; ++j) {
                    const int e = tid + 256 * j, a = e >> 6, b = e & 63;
                    const int64_t row = rowbase + b, col = colbase + a;
                    const bool ok = row < n && col < n;
                    iv_cp4(&sT[s][a][b], ok ? L + row + col * ld : L, ok ? 4 : 0);
                }
            }
#pragma unroll
            for (int j = 0; j < YCH; ++j) {
                const int e = tid + 256 * j, c = e >> 5, kp = e & 31;
                const int64_t gk = qb * kIvNb + 2 * kp, col = col0 + c;
                const bool ok = col < m;
                iv_cp16(&sY[s][c][2 * kp], ok ? ll + gk + col * ldl : ll, ok ? 16 : 0);
            }
        }
        iv_commit();
    };
    // The words this thread copied into stage s that are not yet published
    // are re-read from global memory until they carry this launch's tag; their
    // values go to sYf[buf] (words past n or m are zero: never written, or
    // zero-filled by the copy).
    static_assert(YCH == 2, "a thread settles the four words of its two copies together");
    auto settle_stage = [&](int64_t pi, int s, int buf) {
        unsigned long long w[4];
        bool tagged = true;  // the usual case: every copied word was already published
#pragma unroll
        for (int j = 0; j < YCH; ++j) {
            const int e = tid + 256 * j, c = e >> 5, kp = e & 31;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                w[2 * j + h] = sY[s][c][2 * kp + h];
                tagged &= (w[2 * j + h] & 0xffffffff00000000ull) == tag;
            }
        }
        if (!tagged) {  // late words (or words past n or m, which are never tagged): poll those
            const int64_t pq = q_lo + pi;
            const int64_t qb = TRANS ? R - 1 - pq : pq;
            const unsigned long long *p[4];
#pragma unroll
            for (int j = 0; j < YCH; ++j) {
                const int e = tid + 256 * j, c = e >> 5, kp = e & 31;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int64_t gk = qb * kIvNb + 2 * kp + h, col = col0 + c;
                    p[2 * j + h] = (gk < n && col < m) ? ll + gk + col * ldl : nullptr;
                }
            }
            iv_settle4<256>(w, p, tag, err_word, &s_abort);  // blocks solved a few steps back
        }
#pragma unroll
        for (int j = 0; j < YCH; ++j) {
            const int e = tid + 256 * j, c = e >> 5, kp = e & 31;
            *reinterpret_cast<float2 *>(&sYf[buf][c][2 * kp]) =
                make_float2(__uint_as_float((unsigned)w[2 * j]), __uint_as_float((unsigned)w[2 * j + 1]));
        }
    };

    // 1. every coupling term but the neighbour's (blocks solved well before this one)
    const int kg = tid >> 6, cg = tid & 3, rq = (tid & 63) >> 2;
    float part[4][4];  // part[j][jj]: row (trans ? rq + 16 j : 4 rq + j), column cg + 4 jj
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) part[j][jj] = 0.f;
#pragma unroll
    for (int s = 0; s < NS - 1; ++s) issue(s, s);
    {  // the wide helpers' partial sums, group by group: read while the first stages copy and
       // long before the neighbours are solved, off the critical path.  One warp waits on the
       // helpers' flags (sleeping between polls), then the barrier passes them on.
        const int cg64 = (int)(col0 / kIvNb), cl = (int)(col0 % kIvNb) + bc;  // column group, column in it
        const int64_t ng = iv_ngroups(pb);
        const int64_t slot0 = (int64_t)ngrp * iv_groups_before(pb) + cg64;  // slot of group 0
        const unsigned long long *pw0 = pw + slot0 * kIvTile;
        if (tid < 32) {
            const unsigned long long *hflags = flags + R * nchunks;
            for (int64_t g = tid; g < ng; g += 32) {
                long long spins = 0;
                while (iv_ld_acquire(hflags + slot0 + g * ngrp) != (tag | 1ull)) {
                    if (*(volatile int *)err_word != 0 || ++spins > kSpinLimit) {
                        atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
                        s_abort = 1;
                        break;
                    }
                    __nanosleep(256);
                }
            }
        }
        __syncthreads();
        for (int64_t g = 0; g < ng; ++g) {
            unsigned long long w[4];
            const unsigned long long *p[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int64_t row = rb * kIvNb + 4 * rg + i;
                p[i] = (row < n && col0 + bc < m) ? pw0 + g * ngrp * kIvTile + (4 * rg + i) + kIvNb * cl : nullptr;
                w[i] = p[i] ? iv_ld_word(p[i]) : 0ull;
            }
            iv_settle4<256>(w, p, tag, err_word, &s_abort);  // published before the flag: no wait
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (p[i]) acc[i] += __uint_as_float((unsigned)(w[i] & 0xffffffffull));
        }
    }  // a timed-out wait is seen after the next barrier (the copies in flight drain first)
    for (int64_t pq = 0; pq < nbulk; ++pq) {
        const int s = (int)(pq % NS), buf = (int)(pq & 1);
        iv_wait<NS - 2>();
        settle_stage(pq, s, buf);
        __syncthreads();
        if (s_abort) break;
        issue(pq + NS - 1, (int)((pq + NS - 1) % NS));
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4) {
            const int k0 = 16 * kg + 4 * k4;
            float4 x[4];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) x[jj] = *reinterpret_cast<const float4 *>(&sYf[buf][cg + 4 * jj][k0]);
            if (!TRANS) {  // coefficient of x_k in row i: sT[s][k][i]
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const float4 l4 = *reinterpret_cast<const float4 *>(&sT[s][k0 + kk][4 * rq]);
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        const float xv = kk == 0 ? x[jj].x : kk == 1 ? x[jj].y : kk == 2 ? x[jj].z : x[jj].w;
                        part[0][jj] = fmaf(-l4.x, xv, part[0][jj]);
                        part[1][jj] = fmaf(-l4.y, xv, part[1][jj]);
                        part[2][jj] = fmaf(-l4.z, xv, part[2][jj]);
                        part[3][jj] = fmaf(-l4.w, xv, part[3][jj]);
                    }
                }
            } else {  // coefficient of x_k in row i: sT[s][i][k]
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float4 l4 = *reinterpret_cast<const float4 *>(&sT[s][rq + 16 * j][k0]);
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        float a = part[j][jj];
                        a = fmaf(-l4.x, x[jj].x, a);
                        a = fmaf(-l4.y, x[jj].y, a);
                        a = fmaf(-l4.z, x[jj].z, a);
                        a = fmaf(-l4.w, x[jj].w, a);
                        part[j][jj] = a;
                    }
                }
            }
        }
    }
    iv_wait<0>();
    __syncthreads();
    {  // add the four K-quarters' partial sums in order (stage 2 is free now)
        float *red = &sT[2][0][0];  // red[kg][row][col], row stride 17
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj)
                red[kg * kIvNb * 17 + (TRANS ? rq + 16 * j : 4 * rq + j) * 17 + cg + 4 * jj] = part[j][jj];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float *r = red + (4 * rg + i) * 17 + bc;
            acc[i] = (((acc[i] + r[0]) + r[kIvNb * 17]) + r[2 * kIvNb * 17]) + r[3 * kIvNb * 17];
        }
    }
    if (s_abort) return;
    // 2. t = W_r acc (W_r^T acc when trans); both neighbours' words and the
    // second neighbour's coupling matrix are read meanwhile
    unsigned long long wy[4], wy2[4];
    float preM2[LPT];
    const int64_t qn = TRANS ? rb + 1 : rb - 1, qn2 = TRANS ? rb + 2 : rb - 2;  // neighbour blocks
    if (pb > 0) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t gk = qn * kIvNb + ta, col = col0 + tb + 4 * u;
            wy[u] = (gk < n && col < m) ? iv_ld_word(ll + gk + col * ldl) : tag;
        }
    }
    if (pb > 1) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t gk = qn2 * kIvNb + ta, col = col0 + tb + 4 * u;
            wy2[u] = (gk < n && col < m) ? iv_ld_word(ll + gk + col * ldl) : tag;
        }
        const float *M2r = Wall + ((TRANS ? 4 : 3) * R + rb) * kIvTile + ta + tb * kIvNb;
#pragma unroll
        for (int u = 0; u < LPT; ++u) preM2[u] = M2r[u * 4 * kIvNb];
    }
    float(*sK)[kIvLd] = sT[0];  // coefficient tile: sK[k][i]
    float(*sX)[C] = sV[0];
#pragma unroll
    for (int i = 0; i < 4; ++i) sX[4 * rg + i][bc] = acc[i];
#pragma unroll
    for (int u = 0; u < LPT; ++u) {  // preW[u] = W[ta][tb + 4u]
        if (!TRANS)
            sK[tb + 4 * u][ta] = preW[u];  // W[i][k]
        else
            sK[ta][tb + 4 * u] = preW[u];  // W[k][i]
    }
    __syncthreads();
    float t[4] = {0.f, 0.f, 0.f, 0.f};
    iv_dot64<1>(t, sK, sX, ta, tb);
    // 3. t -= M2_r x_second_neighbour, then t -= M_r x_neighbour; M_r, M2_r
    // (F_r^1, F_r^2 or G_r^1, G_r^2) stored as plain coefficient matrices
    if (pb > 1) {
        float(*sM)[kIvLd] = sT[2];
        float(*sN)[C] = reinterpret_cast<float(*)[C]>(&sYf[0][0][0]);  // 64 x 16 (free after the bulk)
        const unsigned long long *p[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t gk = qn2 * kIvNb + ta, col = col0 + tb + 4 * u;
            p[u] = (gk < n && col < m) ? ll + gk + col * ldl : nullptr;
        }
#pragma unroll
        for (int u = 0; u < LPT; ++u) sM[tb + 4 * u][ta] = preM2[u];  // before the wait: off the critical path
        iv_settle4(wy2, p, tag, err_word, &s_abort);
#pragma unroll
        for (int u = 0; u < 4; ++u) sN[ta][tb + 4 * u] = p[u] ? __uint_as_float((unsigned)wy2[u]) : 0.f;
        __syncthreads();
        if (s_abort) return;
        iv_dot64<-1>(t, sM, sN, ta, tb);
    }
    if (pb > 0) {
        float(*sM)[kIvLd] = sT[1];
        float(*sN)[C] = sV[1];
        const unsigned long long *p[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t gk = qn * kIvNb + ta, col = col0 + tb + 4 * u;
            p[u] = (gk < n && col < m) ? ll + gk + col * ldl : nullptr;
        }
#pragma unroll
        for (int u = 0; u < LPT; ++u) sM[tb + 4 * u][ta] = preM[u];  // M[i = ta][k = tb + 4u], before the wait
        iv_settle4(wy, p, tag, err_word, &s_abort);
#pragma unroll
        for (int u = 0; u < 4; ++u) sN[ta][tb + 4 * u] = p[u] ? __uint_as_float((unsigned)wy[u]) : 0.f;
        __syncthreads();
        if (s_abort) return;
        iv_dot64<-1>(t, sM, sN, ta, tb);
    }
    // 4. publish: the tagged words for the next blocks' owners, then (off the
    // critical path) the flag that lets wide helpers read the values from B
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t col = col0 + tb * 4 + u;
        if (grow < n && col < m) {
            B[grow + col * ldb] = t[u];
            iv_st_word(ll + grow + col * ldl, tag | (unsigned long long)__float_as_uint(t[u]));
        }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) iv_st_release(flags + pb * nchunks + cc, tag | 1ull);
}

// ---------------------------------------------------------------------------
// Chain form.  One CTA per column chunk (the chain) walks every block of its
// chunk in processing order and keeps the two previously solved blocks in
// shared memory, so the block-to-block critical path has no inter-CTA
// hand-off:
//     y_r = sum_g P_{r,g} - F_r^2 y_{r-2} - F_r^1 y_{r-1}
//     (TRANS: x_r = sum_g P_{r,g} - G_r^2 x_{r+2} - G_r^1 x_{r+1}).
// Helper CTAs form the partial sums P_{r,g} = W_r (b_r [g = 0] - sum_{q in g}
// L_rq y_q) over groups g of S earlier positions (all but the two
// neighbours) with the bulk products above, and publish them as epoch-tagged
// words; the chain reads the next block's words one step ahead.  Ticket
// order (ch_decode): the chains first, then the helpers by position, so every
// wait ends.
template <bool TRANS>
__global__ void __launch_bounds__(256, 2) trsm_chain_kernel(const float *__restrict__ L, int64_t ld,
                                                            const float *__restrict__ Wall, int64_t n,
                                                            float *B, int64_t ldb, int64_t m, int nchunks,
                                                            unsigned long long *yw, int64_t ldy,
                                                            unsigned long long *pw, int64_t S, int64_t Gmax,
                                                            unsigned epoch, int *counter, int *err_word,
                                                            const int *state) {
    if (refine_done(state)) return;  // the refinement has finished: nothing to solve
    constexpr int C = kIvCols, LPT = kIvTile / 256, NS = kIvStages;
    constexpr int YCH = kIvNb * C / 2 / 256;  // 16-byte (two-word) copies per thread per stage
    extern __shared__ __align__(16) float iv_smem[];
    float(*sT)[kIvNb][kIvLd] = reinterpret_cast<float(*)[kIvNb][kIvLd]>(iv_smem);
    unsigned long long(*sY)[C][kIvYd] =
        reinterpret_cast<unsigned long long(*)[C][kIvYd]>(iv_smem + NS * kIvNb * kIvLd);
    float(*sV)[kIvNb][C] = reinterpret_cast<float(*)[kIvNb][C]>(iv_smem + NS * kIvNb * kIvLd + 2 * NS * C * kIvYd);
    float(*sYf)[C][kIvLd] =
        reinterpret_cast<float(*)[C][kIvLd]>(iv_smem + NS * kIvNb * kIvLd + 2 * NS * C * kIvYd + 2 * kIvNb * C);
    __shared__ int s_ticket, s_abort;
    const int tid = threadIdx.x;
    if (tid == 0) {
        s_ticket = atomicAdd(counter, 1);
        s_abort = 0;
    }
    __syncthreads();
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    bool chain;
    int64_t pb;  // position in processing order (helpers)
    int grp, cc;
    ch_decode(s_ticket, R, S, nchunks, chain, pb, grp, cc);
    const int ta = tid % kIvNb, tb = tid / kIvNb;
    const int64_t col0 = (int64_t)cc * C;
    const unsigned long long tag = (unsigned long long)epoch << 32;
    const int64_t ldpw = R * Gmax * kIvNb;  // partial-sum words: (position, group, row) then column

    if (chain) {
        // shared memory of the chain: coupling tiles sM[buf][d - 1][k][i] (element
        // (i, k) of M^d), double-buffered by position; the two previous blocks
        // syv[p & 1][k][c]
        float(*sM)[2][kIvNb][kIvLd] = reinterpret_cast<float(*)[2][kIvNb][kIvLd]>(iv_smem);
        float(*syv)[kIvNb][C] = reinterpret_cast<float(*)[kIvNb][C]>(iv_smem + 4 * kIvNb * kIvLd);
        // coupling tiles of position p into buffer b (column-major 64 x 64: 64 floats a column)
        auto fetch = [&](int64_t p, int b) {
            const int64_t r = TRANS ? R - 1 - p : p;
#pragma unroll
            for (int d = 1; d <= 2; ++d) {
                if (p < d) continue;
                const float *Mr = Wall + ((TRANS ? 2 * d : 2 * d - 1) * R + r) * kIvTile;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int e = tid + 256 * j, k = e >> 4, i4 = (e & 15) * 4;
                    iv_cp16(&sM[b][d - 1][k][i4], Mr + k * kIvNb + i4, 16);
                }
            }
            iv_commit();
        };
        // the partial-sum words of position p, row ta, columns col0 + 4 tb + u
        unsigned long long wn[8][4];
        auto load_words = [&](int64_t p) {
            const int64_t r = TRANS ? R - 1 - p : p;
            const int64_t grow = r * kIvNb + ta;
            const int64_t G = ch_groups(p, S);
#pragma unroll
            for (int g = 0; g < 8; ++g)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t col = col0 + 4 * tb + u;
                    wn[g][u] = (g < G && grow < n && col < m)
                                   ? iv_ld_word(pw + ((p * Gmax + g) * kIvNb + ta) + col * ldpw)
                                   : tag;
                }
        };
        fetch(0, 0);
        load_words(0);
        for (int64_t p = 0; p < R; ++p) {
            const int64_t r = TRANS ? R - 1 - p : p;
            const int64_t grow = r * kIvNb + ta;
            const int buf = (int)(p & 1);
            const int64_t G = ch_groups(p, S);
            unsigned long long(&w)[8][4] = wn;  // this position's words (loaded one step ahead)
            if (p + 1 < R)  // the next position's coupling tiles, one step ahead
                fetch(p + 1, buf ^ 1);
            else
                iv_commit();
            // 1. the helpers' partial sums of this block (bounded wait for late ones)
            {
                long long spins = 0;
                for (;;) {
                    bool done = true;
#pragma unroll
                    for (int g = 0; g < 8; ++g)
#pragma unroll
                        for (int u = 0; u < 4; ++u)
                            done &= (w[g][u] & 0xffffffff00000000ull) == tag;
                    if (done) break;
                    if (((++spins) & 63) == 0) {
                        if (*(volatile int *)err_word != 0 || spins > kSpinLimit) {
                            atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
                            s_abort = 1;
                            break;
                        }
                        __nanosleep(32);
                    }
#pragma unroll
                    for (int g = 0; g < 8; ++g)
#pragma unroll
                        for (int u = 0; u < 4; ++u)
                            if ((w[g][u] & 0xffffffff00000000ull) != tag) {
                                const int64_t col = col0 + 4 * tb + u;
                                w[g][u] = iv_ld_word(pw + ((p * Gmax + g) * kIvNb + ta) + col * ldpw);
                            }
                }
            }
            float t[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t col = col0 + 4 * tb + u;
                float v = 0.f;
                if (grow < n && col < m)
#pragma unroll
                    for (int g = 0; g < 8; ++g)
                        if (g < G) v += __uint_as_float((unsigned)(w[g][u] & 0xffffffffull));
                t[u] = v;
            }
            if (p + 1 < R) load_words(p + 1);  // in flight while the products below run
            iv_wait<1>();  // this position's tiles (fetched one step earlier) have landed
            __syncthreads();
            if (s_abort) return;
            // 2. t -= M^2 y_{p-2}, then t -= M^1 y_{p-1}
#pragma unroll
            for (int d = 2; d >= 1; --d) {
                if (p < d) continue;
                const float(*M)[kIvLd] = sM[buf][d - 1];
                const float(*Y)[C] = syv[(p - d) & 1];
                iv_dot64<-1>(t, M, Y, ta, tb);
            }
            __syncthreads();  // every read of y_{p-2} is done: its buffer takes y_p
            // 3. publish y_p
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t col = col0 + 4 * tb + u;
                const bool in = grow < n && col < m;
                syv[buf][ta][4 * tb + u] = in ? t[u] : 0.f;
                if (in) {
                    B[grow + col * ldb] = t[u];
                    iv_st_word(yw + grow + col * ldy, tag | (unsigned long long)__float_as_uint(t[u]));
                }
            }
        }
        iv_wait<0>();
        return;
    }

    // helper: P_{r,g} for position pb, group grp
    const int64_t rb = TRANS ? R - 1 - pb : pb;
    const bool al16 = (ld % 4 == 0) && ((reinterpret_cast<uintptr_t>(L) & 15) == 0);
    const int bc = tid % C, rg = tid / C;  // bulk mapping: column bc, rows 4 rg .. 4 rg + 3
    float acc[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t row = rb * kIvNb + 4 * rg + i, col = col0 + bc;
        acc[i] = (grp == 0 && row < n && col < m) ? B[row + col * ldb] : 0.f;
    }
    float preW[LPT];
    {
        const float *Wr = Wall + rb * kIvTile + ta + tb * kIvNb;
#pragma unroll
        for (int u = 0; u < LPT; ++u) preW[u] = Wr[u * 4 * kIvNb];
    }
    // coupling terms of this group: positions q_lo .. q_lo + nbulk - 1 (never the two neighbours)
    const int64_t q_lo = (int64_t)grp * S;
    const int64_t q_hi = (q_lo + S < pb - 2) ? q_lo + S : pb - 2;
    const int64_t nbulk = q_hi > q_lo ? q_hi - q_lo : 0;

    // Stage s <- coupling tile and solved words of processing position pq.
    // Tile: 64 columns a of 64 contiguous rows b (non-trans: a = k, b = i;
    // trans: a = i, b = k), zero-filled past n.
    auto issue = [&](int64_t pi, int s) {
        if (pi < nbulk) {
            const int64_t pq = q_lo + pi;
            const int64_t qb = TRANS ? R - 1 - pq : pq;
            const int64_t rowbase = (TRANS ? qb : rb) * kIvNb, colbase = (TRANS ? rb : qb) * kIvNb;
            if (al16) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int e = tid + 256 * j, a = e >> 4, c4 = e & 15;
                    const int64_t row = rowbase + 4 * c4, col = colbase + a;
                    const bool ok = row < n && col < n;
                    const int bytes = ok ? 4 * (int)(n - row < 4 ? n - row : 4) : 0;
                    iv_cp16(&sT[s][a][4 * c4], ok ? L + row + col * ld : L, bytes);
                }
            } else {
#pragma unroll 4
                for (int j = 0; j < 16; ++j) {
                    const int e = tid + 256 * j, a = e >> 6, b = e & 63;
                    const int64_t row = rowbase + b, col = colbase + a;
                    const bool ok = row < n && col < n;
                    iv_cp4(&sT[s][a][b], ok ? L + row + col * ld : L, ok ? 4 : 0);
                }
            }
#pragma unroll
            for (int j = 0; j < YCH; ++j) {
                const int e = tid + 256 * j, c = e >> 5, kp = e & 31;
                const int64_t gk = qb * kIvNb + 2 * kp, col = col0 + c;
                const bool ok = col < m;
                iv_cp16(&sY[s][c][2 * kp], ok ? yw + gk + col * ldy : yw, ok ? 16 : 0);
            }
        }
        iv_commit();
    };
    // The words this thread copied into stage s that are not yet published
    // are re-read from global memory until they carry this launch's tag; their
    // values go to sYf[buf] (words past n or m are zero: never written, or
    // zero-filled by the copy).
    static_assert(YCH == 2, "a thread settles the four words of its two copies together");
    auto settle_stage = [&](int64_t pi, int s, int buf) {
        const int64_t pq = q_lo + pi;
        const int64_t qb = TRANS ? R - 1 - pq : pq;
        unsigned long long w[4];
        const unsigned long long *p[4];
#pragma unroll
        for (int j = 0; j < YCH; ++j) {
            const int e = tid + 256 * j, c = e >> 5, kp = e & 31;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = 2 * kp + h;
                const int64_t gk = qb * kIvNb + k, col = col0 + c;
                w[2 * j + h] = sY[s][c][k];
                p[2 * j + h] = (gk < n && col < m) ? yw + gk + col * ldy : nullptr;
            }
        }
        iv_settle4(w, p, tag, err_word, &s_abort);
#pragma unroll
        for (int j = 0; j < YCH; ++j) {
            const int e = tid + 256 * j, c = e >> 5, kp = e & 31;
            *reinterpret_cast<float2 *>(&sYf[buf][c][2 * kp]) =
                make_float2(__uint_as_float((unsigned)w[2 * j]), __uint_as_float((unsigned)w[2 * j + 1]));
        }
    };

    // 1. every coupling term but the neighbour's (blocks solved well before this one)
    const int kg = tid >> 6, cg = tid & 3, rq = (tid & 63) >> 2;
    float part[4][4];  // part[j][jj]: row (trans ? rq + 16 j : 4 rq + j), column cg + 4 jj
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) part[j][jj] = 0.f;
#pragma unroll
    for (int s = 0; s < NS - 1; ++s) issue(s, s);
    for (int64_t pq = 0; pq < nbulk; ++pq) {
        const int s = (int)(pq % NS), buf = (int)(pq & 1);
        iv_wait<NS - 2>();
        settle_stage(pq, s, buf);
        __syncthreads();
        if (s_abort) break;
        issue(pq + NS - 1, (int)((pq + NS - 1) % NS));
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4) {
            const int k0 = 16 * kg + 4 * k4;
            float4 x[4];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) x[jj] = *reinterpret_cast<const float4 *>(&sYf[buf][cg + 4 * jj][k0]);
            if (!TRANS) {  // coefficient of x_k in row i: sT[s][k][i]
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const float4 l4 = *reinterpret_cast<const float4 *>(&sT[s][k0 + kk][4 * rq]);
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        const float xv = kk == 0 ? x[jj].x : kk == 1 ? x[jj].y : kk == 2 ? x[jj].z : x[jj].w;
                        part[0][jj] = fmaf(-l4.x, xv, part[0][jj]);
                        part[1][jj] = fmaf(-l4.y, xv, part[1][jj]);
                        part[2][jj] = fmaf(-l4.z, xv, part[2][jj]);
                        part[3][jj] = fmaf(-l4.w, xv, part[3][jj]);
                    }
                }
            } else {  // coefficient of x_k in row i: sT[s][i][k]
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float4 l4 = *reinterpret_cast<const float4 *>(&sT[s][rq + 16 * j][k0]);
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        float a = part[j][jj];
                        a = fmaf(-l4.x, x[jj].x, a);
                        a = fmaf(-l4.y, x[jj].y, a);
                        a = fmaf(-l4.z, x[jj].z, a);
                        a = fmaf(-l4.w, x[jj].w, a);
                        part[j][jj] = a;
                    }
                }
            }
        }
    }
    iv_wait<0>();
    __syncthreads();
    {  // add the four K-quarters' partial sums in order (stage 2 is free now)
        float *red = &sT[2][0][0];  // red[kg][row][col], row stride 17
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj)
                red[kg * kIvNb * 17 + (TRANS ? rq + 16 * j : 4 * rq + j) * 17 + cg + 4 * jj] = part[j][jj];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float *r = red + (4 * rg + i) * 17 + bc;
            acc[i] = (((acc[i] + r[0]) + r[kIvNb * 17]) + r[2 * kIvNb * 17]) + r[3 * kIvNb * 17];
        }
    }
    if (s_abort) return;
    // 2. t = W_r acc (W_r^T acc when trans)
    float(*sK)[kIvLd] = sT[0];  // coefficient tile: sK[k][i]
    float(*sX)[C] = sV[0];
#pragma unroll
    for (int i = 0; i < 4; ++i) sX[4 * rg + i][bc] = acc[i];
#pragma unroll
    for (int u = 0; u < LPT; ++u) {  // preW[u] = W[ta][tb + 4u]
        if (!TRANS)
            sK[tb + 4 * u][ta] = preW[u];  // W[i][k]
        else
            sK[ta][tb + 4 * u] = preW[u];  // W[k][i]
    }
    __syncthreads();
    float t[4] = {0.f, 0.f, 0.f, 0.f};
    iv_dot64<1>(t, sK, sX, ta, tb);
    // 3. publish the partial sum for the chain
    {
        const int64_t grow = rb * kIvNb + ta;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t col = col0 + tb * 4 + u;
            if (grow < n && col < m)
                iv_st_word(pw + ((pb * Gmax + grp) * kIvNb + ta) + col * ldpw,
                           tag | (unsigned long long)__float_as_uint(t[u]));
        }
    }
}

size_t trsm_inv_ws_ints(int64_t, int64_t) { return 1; }

// solved words, then the wide helpers' partial sums (64 x 64 words a slot),
// then one flag word per (position, chunk), then one per helper slot
static int iv_ngrp(int64_t m) { return (int)((m + kIvNb - 1) / kIvNb); }
static int iv_nch(int64_t m) { return (int)((m + kIvCols - 1) / kIvCols); }
size_t trsm_inv_stage_words(int64_t n, int64_t m) {
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    return (size_t)R * kIvNb * (size_t)m + (size_t)iv_ngrp(m) * iv_groups_before(R) * (kIvTile + 1) +
           (size_t)R * iv_nch(m);
}

// chain form: the solved words, then the helpers' partial sums (Gmax groups a position)
size_t trsm_chain_stage_words(int64_t n, int64_t m) {
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    const int64_t S = ch_group_size(R), Gmax = ch_groups(R - 1 > 0 ? R - 1 : 0, S);
    return (size_t)(1 + Gmax) * R * kIvNb * (size_t)m;
}

size_t diag_inverse_floats(int64_t n) { return 5 * (size_t)((n + kIvNb - 1) / kIvNb) * kIvTile; }

int diag_inverse_launch(const float *L, int64_t ld, int64_t n, float *W, cudaStream_t st) {
    if (n == 0) return 0;
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    {
        LaunchScope ls(K_MIXED_TRSM, st, (double)n * kIvTile / 3.0);
        diag_inverse_kernel<<<(unsigned)R, 64, 0, st>>>(L, ld, n, W);
        if (cudaGetLastError() != cudaSuccess) return -1;
    }
    LaunchScope ls(K_MIXED_TRSM, st, 8.0 * (double)R * kIvTile * kIvNb);
    fuse_kernel<<<dim3((unsigned)R, 2), 256, 0, st>>>(L, ld, n, W);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int trsm_inv_launch(const float *L, int64_t ld, const float *W, int64_t n, float *B, int64_t ldb,
                    int64_t m, int trans, unsigned long long *stage, unsigned epoch, int *ws, int *err_word,
                    cudaStream_t st, const int *state) {
    if (n == 0 || m == 0) return 0;
    if (epoch == 0) return -1;
    const int nchunks = iv_nch(m), ngrp = iv_ngrp(m);
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    auto kern = trans ? trsm_inv_kernel<true> : trsm_inv_kernel<false>;
    const size_t smem = kIvLaunchSmem;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    if (cudaMemsetAsync(ws, 0, sizeof(int), st) != cudaSuccess) return -1;
    // algorithmic work: n^2 m flops
    LaunchScope ls(K_MIXED_TRSM, st, (double)n * n * m);
    unsigned long long *pw = stage + R * kIvNb * m;
    unsigned long long *flags = pw + (int64_t)ngrp * iv_groups_before(R) * kIvTile;
    const int64_t items = iv_items_before(R, R, nchunks, ngrp);
    kern<<<(unsigned)items, 256, smem, st>>>(L, ld, W, n, B, ldb, m, nchunks, stage, R * kIvNb, epoch, ws,
                                            err_word, ngrp, pw, flags, state);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int trsm_chain_launch(const float *L, int64_t ld, const float *W, int64_t n, float *B, int64_t ldb,
                      int64_t m, int trans, unsigned long long *stage, unsigned epoch, int *ws, int *err_word,
                      cudaStream_t st, const int *state) {
    if (n == 0 || m == 0) return 0;
    if (epoch == 0) return -1;
    const int nchunks = (int)((m + kIvCols - 1) / kIvCols);
    const int64_t R = (n + kIvNb - 1) / kIvNb;
    const int64_t S = ch_group_size(R), Gmax = ch_groups(R - 1, S);
    auto kern = trans ? trsm_chain_kernel<true> : trsm_chain_kernel<false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kIvSmem) != cudaSuccess)
        return -1;
    if (cudaMemsetAsync(ws, 0, sizeof(int), st) != cudaSuccess) return -1;
    // algorithmic work: n^2 m flops
    LaunchScope ls(K_MIXED_TRSM, st, (double)n * n * m);
    const int64_t items = ch_items(R, S, nchunks);
    unsigned long long *yw = stage, *pw = stage + R * kIvNb * m;
    kern<<<(unsigned)items, 256, kIvSmem, st>>>(L, ld, W, n, B, ldb, m, nchunks, yw, R * kIvNb, pw, S, Gmax, epoch,
                                               ws, err_word, state);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace lla

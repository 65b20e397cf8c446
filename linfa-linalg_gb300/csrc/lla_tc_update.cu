// lla_tc_update.cu -- trailing update A22 -= L21 L21^T of the mixed-precision
// Cholesky on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Persistent CTAs (at most one per SM) claim the 128 x 128 lower tiles
// (I >= J) of the trailing matrix one at a time from a global counter, so a
// CTA that starts late -- its SM still busy with another stream's work --
// takes fewer tiles instead of delaying the launch.  The counter is never
// reset between launches: every CTA makes exactly one claim more than the
// tiles it processes, so a launch advances it by tiles + CTAs and the host
// passes each launch the value it starts from:
//   * one thread streams 64-wide K chunks of the two operand row blocks, every
//     term plane of a chunk in one TMA box (cp.async.bulk.tensor, 128-byte
//     swizzle), into a shared-memory ring of 2-6 stages, completion tracked by
//     mbarriers; diagonal tiles load their single row block once;
//   * one thread issues tcgen05.mma (kind::f16, M = 128, N = 128, K = 16, BF16
//     or FP16 operands, FP32 accumulator in tensor memory) for every term pair
//     of every chunk, releasing each stage with tcgen05.commit, alternating
//     between two accumulators;
//   * eight epilogue warps read a finished accumulator from tensor memory
//     (tcgen05.ld 32x32b, two warps per 32-lane quarter) and subtract it from
//     the FP32 tile in HBM (coalesced: a warp covers 32 consecutive rows of a
//     column-major column) while the next tile's MMAs run; diagonal tiles
//     write their lower half only.
// Every wait is bounded: on expiry the CTA records LLA_ERR_TIMEOUT, skips its
// writes, frees its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>

#include "lla_common.cuh"
#include "lla_tc.h"
#include "lla_tcgen05.cuh"

namespace lla {

constexpr int kTcM = 128, kTcN = 128;            // tile
constexpr int kTcMaxStages = 8;
// Shared memory: the operand ring, then (TMA-staged epilogue only) one FP32
// 128 x 128 output tile, then the barriers.
constexpr int kTcTileC = kTcM * kTcN * 4;  // 64 KiB
__host__ __device__ constexpr int tc_ring_bytes(bool epi_tma) { return epi_tma ? 144 * 1024 : 192 * 1024; }
__host__ __device__ constexpr int tc_smem_bytes(bool epi_tma) {
    return 1024 + tc_ring_bytes(epi_tma) + (epi_tma ? kTcTileC : 0) + 256;
}
// K-chunk KC of a stage: 64 (128-byte rows, 128-byte swizzle) or 32 (64-byte
// rows, 64-byte swizzle: twice the stages in the same ring, so more loads are
// in flight ahead of the MMAs).  One term plane of one operand: 128 x KC x 2 B.
template <int KC>
__host__ __device__ constexpr int tc_tile_bytes() { return kTcM * KC * 2; }
// Stages of the ring: a stage holds every term plane of both operands for one
// K-chunk, so each plane is loaded once per chunk and serves all the term
// pairs that use it.
template <int KC>
__host__ __device__ constexpr int tc_stages(int terms, bool epi_tma) {
    return (tc_ring_bytes(epi_tma) / (2 * terms * tc_tile_bytes<KC>())) < kTcMaxStages
               ? tc_ring_bytes(epi_tma) / (2 * terms * tc_tile_bytes<KC>())
               : kTcMaxStages;
}
// Shared-memory descriptor of a K-major tile stored with the KC-wide swizzle:
// 8-row atoms of KC * 2 bytes per row stacked along M.
template <int KC>
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    if (KC == 64) return sw128_desc(saddr);
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}
constexpr uint32_t kTcCols = 128;  // tensor-memory columns of one FP32 128 x 128 accumulator
// Two accumulators per tile: the leading product h0 h0^T, and the sum of the
// small cross-term products (summed among themselves first, as FP32 accuracy
// wants), double-buffered: all 512 columns.
constexpr uint32_t kTcAlloc = 4 * kTcCols;

__device__ __forceinline__ void tc_tri_tile(int64_t t, int64_t &I, int64_t &J);
// Tile t of a launch: the lower tiles (I >= J) in row-major order, or, for a
// narrow update, the tiles (t, 0) of the first tile column only.
__device__ __forceinline__ void tc_tile(int64_t t, int narrow, int64_t &I, int64_t &J) {
    if (narrow) {
        I = t;
        J = 0;
    } else {
        tc_tri_tile(t, I, J);
    }
}
__device__ __forceinline__ void tc_tri_tile(int64_t t, int64_t &I, int64_t &J) {
    int64_t i = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    I = i;
    J = t - i * (i + 1) / 2;
}

// Persistent, warp-specialised: warps 0-7 drain accumulators (epilogue, two
// warps per 32-lane quarter of tensor memory, 64 columns each), warp 8 lane 0
// claims tiles and feeds the shared-memory ring with TMA, warp 9 lane 0
// issues the MMAs.  Two tensor-memory accumulators let the epilogue of one
// tile overlap the MMAs of the next, and the epilogue fetches its FP32 tile
// before the accumulator is ready.  The claimed tile indices reach the MMA and
// epilogue warps through a small shared-memory ring (-1: no tiles left).
constexpr int kTcThreads = 320;  // 8 epilogue warps, 1 producer warp, 1 MMA warp
constexpr int kTcEpiThreads = 256;
constexpr int kTcTileRing = 8;  // claimed tile indices in flight inside a CTA

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Term pairs (a, b) per number of terms, small products first; the last one,
// (0, 0), is the leading product.
__device__ __forceinline__ constexpr int tc_npairs(int terms) { return terms == 1 ? 1 : (terms == 2 ? 3 : 6); }
__device__ __forceinline__ constexpr int tc_pa(int terms, int i) {
    return terms == 1 ? 0 : (terms == 2 ? (i == 1 ? 1 : 0) : (i == 1 || i == 4 ? 1 : (i == 2 ? 2 : 0)));
}
__device__ __forceinline__ constexpr int tc_pb(int terms, int i) {
    return terms == 1 ? 0 : (terms == 2 ? (i == 0 ? 1 : 0) : (i == 0 ? 2 : (i == 1 || i == 3 ? 1 : 0)));
}

// 320 threads are 10 warps, so one SM sub-partition runs 3 of them from its
// 16K registers: at most 170 registers a thread (168 allocated).
//
// EPI_TMA: the epilogue stages the FP32 output tile in shared memory -- one
// elected epilogue thread loads it with a TMA box while the tile's MMAs run
// and stores it back with a TMA box -- so the tile's 64 KiB each way are in
// flight without registers; the threads only read the accumulator, read and
// write shared memory.  Diagonal tiles write back their upper part unchanged.
// Needs a leading dimension that is a multiple of 4 floats (16-byte rows).
template <int TERMS, int KC, bool EPI_TMA>
__global__ void __launch_bounds__(kTcThreads, 1) tc_update_kernel(
    const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap cmap, float *C, int64_t ld,
    int64_t q, int64_t n, int kchunks, uint32_t idesc, int64_t ntiles, int narrow, const int64_t *info,
    int *err_word, unsigned *sched, unsigned sched_base) {
    constexpr int terms = TERMS, NP = tc_npairs(TERMS);
    extern __shared__ uint8_t smem_raw[];
    __shared__ int s_abort, s_skip, s_epi_abort, s_epi_tile;
    __shared__ int s_tile[kTcTileRing];
    __shared__ __align__(8) uint64_t s_tbar[2 * kTcTileRing];  // tile ring: full[R], empty[R]
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int kTile = tc_tile_bytes<KC>();
    const int S = tc_stages<KC>(terms, EPI_TMA);
    const uint32_t opnd = (uint32_t)terms * kTile;  // one operand's planes in a stage
    uint8_t *ring = smem;                                   // stage s: A planes, then B planes
    float *sC = (float *)(smem + tc_ring_bytes(EPI_TMA));  // EPI_TMA: sC[c * 128 + r]
    uint64_t *bars = (uint64_t *)(smem + tc_ring_bytes(EPI_TMA) + (EPI_TMA ? kTcTileC : 0));
    // bars: full[S], empty[S], tmem_full[2], tmem_empty[2], c_full
    uint32_t *tslot = (uint32_t *)(bars + 2 * kTcMaxStages + 5);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + kTcMaxStages);
    const uint32_t tfull0 = smem_u32(bars + 2 * kTcMaxStages), tempty0 = tfull0 + 16;
    const uint32_t cfull = tfull0 + 32;
    const uint32_t rfull0 = smem_u32(s_tbar), rempty0 = rfull0 + 8 * kTcTileRing;  // tile ring
    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull0 + 8 * a, 1);
            mbar_init(tempty0 + 8 * a, kTcEpiThreads);  // every epilogue thread releases
        }
        for (int r = 0; r < kTcTileRing; ++r) {
            mbar_init(rfull0 + 8 * r, 1);
            // readers of a claimed index: the MMA thread and the epilogue (one
            // thread for the staged epilogue, each warp's lane 0 otherwise)
            mbar_init(rempty0 + 8 * r, EPI_TMA ? 2 : 9);
        }
        mbar_init(cfull, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
        s_epi_abort = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tslot)),
                     "r"(kTcAlloc)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    // The set-up above may overlap the previous kernel's tail (programmatic
    // launch); the operand planes and the status words come from it.
    pdl_wait();
    pdl_trigger();
    // one reader decides for the whole CTA (another CTA may set err_word meanwhile)
    if (tid == 0) s_skip = (*(volatile const int64_t *)info >= 0 || *(volatile const int *)err_word != 0);
    __syncthreads();
    if (s_skip) {
        if (warp == 0)
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcAlloc)
                         : "memory");
        return;  // the launch is void (a failed or timed-out factorisation): its claims do not matter
    }

    if (warp == 8) {
        if (lane == 0) {  // tile claims and TMA producer
            int64_t g = 0;
            // one claim ahead: the next tile is claimed while this one's chunks load
            int64_t t_next = (int64_t)(atomicAdd(sched, 1u) - sched_base);
            for (int64_t lt = 0; !*(volatile int *)&s_abort; ++lt) {
                const int slot = (int)(lt % kTcTileRing);
                const int64_t ruse = lt / kTcTileRing;
                if (ruse > 0 && !mbar_wait(rempty0 + 8 * slot, (uint32_t)((ruse - 1) & 1), err_word)) {
                    s_abort = 1;
                    break;
                }
                const int64_t t = t_next;
                s_tile[slot] = t < ntiles ? (int)t : -1;
                mbar_arrive(rfull0 + 8 * slot);  // release: the index is visible to the waiters
                if (t >= ntiles) break;
                t_next = (int64_t)(atomicAdd(sched, 1u) - sched_base);
                int64_t I, J;
                tc_tile(t, narrow, I, J);
                for (int kc = 0; kc < kchunks; ++kc, ++g) {
                    const int s = (int)(g % S);
                    const int64_t round = g / S;
                    if (round > 0 && !mbar_wait(empty0 + 8 * s, (uint32_t)((round - 1) & 1), err_word)) {
                        s_abort = 1;
                        break;
                    }
                    const uint32_t st_a = smem_u32(ring + (size_t)s * 2 * opnd);
                    mbar_expect_tx(full0 + 8 * s, (I == J ? 1u : 2u) * opnd);
                    tma_load_3d(st_a, &tmap, kc * KC, (int)(I * kTcM), 0, full0 + 8 * s);
                    if (I != J) tma_load_3d(st_a + opnd, &tmap, kc * KC, (int)(J * kTcN), 0, full0 + 8 * s);
                }
            }
        }
    } else if (warp == 9) {
        if (lane == 0) {  // MMA issuer
            int64_t g = 0;
            for (int64_t lt = 0; !*(volatile int *)&s_abort; ++lt) {
                const int slot = (int)(lt % kTcTileRing);
                if (!mbar_wait(rfull0 + 8 * slot, (uint32_t)((lt / kTcTileRing) & 1), err_word)) {
                    s_abort = 1;
                    break;
                }
                const int t = s_tile[slot];
                mbar_arrive(rempty0 + 8 * slot);
                if (t < 0) break;
                int64_t I, J;
                tc_tile(t, narrow, I, J);
                const int a = (int)(lt & 1);
                const int64_t use = lt >> 1;
                if (use > 0 && !mbar_wait(tempty0 + 8 * a, (uint32_t)((use - 1) & 1), err_word)) {
                    s_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t dt = tmem + (uint32_t)(a * 2 * kTcCols);  // leading; +kTcCols: cross terms
                for (int kc = 0; kc < kchunks; ++kc, ++g) {
                    const int s = (int)(g % S);
                    if (!mbar_wait(full0 + 8 * s, (uint32_t)((g / S) & 1), err_word)) {
                        s_abort = 1;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t st_a = smem_u32(ring + (size_t)s * 2 * opnd);
                    const uint32_t st_b = (I == J) ? st_a : st_a + opnd;  // a diagonal tile uses its rows twice
                    const uint64_t ad0 = tc_desc<KC>(st_a), bd0 = tc_desc<KC>(st_b);
#pragma unroll
                    for (int pr = 0; pr < NP; ++pr) {
                        const bool lead = pr == NP - 1;  // (0, 0)
                        const uint32_t d = lead ? dt : dt + kTcCols;
                        const bool fresh = kc == 0 && (lead || pr == 0);
                        // descriptors address 16-byte units: a plane is kTile / 16 further
                        const uint64_t ad = ad0 + (uint64_t)(tc_pa(TERMS, pr) * (kTile >> 4));
                        const uint64_t bd = bd0 + (uint64_t)(tc_pb(TERMS, pr) * (kTile >> 4));
#pragma unroll
                        for (int k = 0; k < KC / 16; ++k)  // +32 bytes along K per step
                            tc_mma(d, ad + 2 * k, bd + 2 * k, idesc, (fresh && k == 0) ? 0u : 1u);
                    }
                    tc_commit(empty0 + 8 * s);  // frees the stage once these MMAs are done
                }
                if (s_abort) break;
                tc_commit(tfull0 + 8 * a);  // accumulator a is complete
            }
        }
    } else if (EPI_TMA) {  // warps 0-7: epilogue through the shared-memory tile
        const int qw = warp & 3, half = warp >> 2;
        constexpr bool cross = NP > 1;
        const int r = qw * 32 + lane;
        for (int64_t lt = 0;; ++lt) {
            const int a = (int)(lt & 1);
            const int64_t use = lt >> 1;
            if (tid == 0) {
                // thread 0 reads the claimed index for the eight warps (-2: gave up waiting)
                const int slot = (int)(lt % kTcTileRing);
                int t = -2;
                if (mbar_wait(rfull0 + 8 * slot, (uint32_t)((lt / kTcTileRing) & 1), err_word)) {
                    t = s_tile[slot];
                    mbar_arrive(rempty0 + 8 * slot);
                }
                s_epi_tile = t;
                if (t >= 0) {
                    int64_t I, J;
                    tc_tile(t, narrow, I, J);
                    // the previous tile's store has read the buffer: load this tile into it
                    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                    mbar_expect_tx(cfull, (uint32_t)kTcTileC);
                    tma_load_2d(smem_u32(sC), &cmap, (int)(q + I * kTcM), (int)(q + J * kTcN), cfull);
                }
            }
            asm volatile("bar.sync 1, %0;" ::"n"(kTcEpiThreads) : "memory");
            const int t = *(volatile int *)&s_epi_tile;  // the same for all eight warps
            if (t == -1) break;
            if (t < 0) {
                if (tid == 0) s_abort = 1;
                break;
            }
            int64_t I, J;
            tc_tile(t, narrow, I, J);
            bool okc = mbar_wait(cfull, (uint32_t)(lt & 1), err_word);
            bool ok = mbar_wait(tfull0 + 8 * a, (uint32_t)(use & 1), err_word) && okc;
            ok = __all_sync(0xffffffffu, ok) && !*(volatile int *)&s_abort;
            // one decision for all eight epilogue warps (they meet at named barrier 1)
            if (!ok && lane == 0) s_epi_abort = 1;
            asm volatile("bar.sync 1, %0;" ::"n"(kTcEpiThreads) : "memory");
            if (*(volatile int *)&s_epi_abort) {
                if (tid == 0) {
                    s_abort = 1;
                    // the tile load issued above must land before the CTA leaves (bounded)
                    for (long long i = 0; !okc && i < kTcSpin; ++i) okc = mbar_try_wait(cfull, (uint32_t)(lt & 1));
                }
                break;
            }
            tc_fence_after();
            const uint32_t ta = tmem + (uint32_t)(a * 2 * kTcCols) + ((uint32_t)(qw * 32) << 16);
#pragma unroll
            for (int sb = 0; sb < 4; ++sb) {  // 16 columns: leading and cross-term sums
                uint32_t v[16], w[16];
                const uint32_t col = (uint32_t)(half * 64 + sb * 16);
                tc_ld16_nowait(ta + col, v);
                if (cross) tc_ld16_nowait(ta + kTcCols + col, w);
                tc_wait_ld();
#pragma unroll
                for (int c16 = 0; c16 < 16; ++c16) {
                    const int cc = half * 64 + sb * 16 + c16;
                    const float prod =
                        cross ? __uint_as_float(v[c16]) + __uint_as_float(w[c16]) : __uint_as_float(v[c16]);
                    // a diagonal tile keeps its upper part as loaded
                    if (I != J || cc <= r) sC[cc * kTcM + r] -= prod;
                }
            }
            // the accumulator is read: release it to the MMA warp
            tc_fence_before();
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tempty0 + 8 * a) : "memory");
            // the tile's shared-memory writes, then one thread stores it
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("bar.sync 1, %0;" ::"n"(kTcEpiThreads) : "memory");
            if (tid == 0) {
                tma_store_2d(&cmap, smem_u32(sC), (int)(q + I * kTcM), (int)(q + J * kTcN));
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            }
        }
        if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // stores complete
    } else {  // warps 0-7: epilogue; warp w drains lane quarter w % 4, columns 64 (w / 4) ..
        const int qw = warp & 3, half = warp >> 2;
        constexpr bool cross = NP > 1;  // the cross-term accumulator is in use
        const int r = qw * 32 + lane;
        for (int64_t lt = 0;; ++lt) {
            const int a = (int)(lt & 1);
            const int64_t use = lt >> 1;
            int t = -2;  // the claimed index, read by lane 0 (-2: gave up waiting)
            if (lane == 0) {
                const int slot = (int)(lt % kTcTileRing);
                if (mbar_wait(rfull0 + 8 * slot, (uint32_t)((lt / kTcTileRing) & 1), err_word)) {
                    t = s_tile[slot];
                    mbar_arrive(rempty0 + 8 * slot);
                }
            }
            t = __shfl_sync(0xffffffffu, t, 0);
            if (t == -1) break;
            if (t < 0) {
                if (lane == 0) s_abort = 1;
                break;
            }
            int64_t I, J;
            tc_tile(t, narrow, I, J);
            const int64_t grow = q + I * kTcM + r;
            const int64_t gcol0 = q + J * kTcN + half * 64;
            const int64_t cmax = n - gcol0;  // columns left in the matrix
            // the FP32 tile does not depend on the MMAs: fetch its first 32 columns
            // while they run, the next 32 while the first are written back
            float *base = C + grow + gcol0 * ld;
            const bool row_in = grow < n;
            float cur[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const bool in = row_in && c < cmax && (I != J || half * 64 + c <= r);
                cur[c] = in ? base[c * ld] : 0.f;
            }
            bool ok = mbar_wait(tfull0 + 8 * a, (uint32_t)(use & 1), err_word);
            ok = __all_sync(0xffffffffu, ok) && !*(volatile int *)&s_abort;
            if (!ok) {
                if (lane == 0) s_abort = 1;
                break;
            }
            tc_fence_after();
            const uint32_t ta = tmem + (uint32_t)(a * 2 * kTcCols) + ((uint32_t)(qw * 32) << 16);
#pragma unroll
            for (int cb = 0; cb < 2; ++cb) {
#pragma unroll
                for (int sb = 0; sb < 2; ++sb) {  // 16 columns: leading and cross-term sums
                    uint32_t v[16], w[16];
                    const uint32_t col = (uint32_t)(half * 64 + cb * 32 + sb * 16);
                    tc_ld16_nowait(ta + col, v);
                    if (cross) tc_ld16_nowait(ta + kTcCols + col, w);
                    tc_wait_ld();
#pragma unroll
                    for (int c16 = 0; c16 < 16; ++c16) {
                        const int c = sb * 16 + c16, cc = cb * 32 + c;
                        const bool in = row_in && cc < cmax && (I != J || half * 64 + cc <= r);
                        const float prod =
                            cross ? __uint_as_float(v[c16]) + __uint_as_float(w[c16]) : __uint_as_float(v[c16]);
                        const float x = cur[c] - prod;
                        if (cb == 0) {  // fetch the second half before storing the first
                            const int c2 = 32 + c;
                            const bool in2 = row_in && c2 < cmax && (I != J || half * 64 + c2 <= r);
                            cur[c] = in2 ? base[c2 * ld] : 0.f;
                        }
                        if (in) base[cc * ld] = x;
                    }
                }
            }
            tc_fence_before();
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tempty0 + 8 * a) : "memory");
        }
    }
    __syncwarp();
    __syncthreads();
    if (s_abort && tid == 0) atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcAlloc)
                     : "memory");
}

// ---------------------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
    if (!g_encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult qres;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                             &qres) == cudaSuccess &&
            qres == cudaDriverEntryPointSuccess && fn)
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    return g_encode;
}

template <int KC, bool E>
static bool tc_set_attrs() {
    const int sm = tc_smem_bytes(E);
    return cudaFuncSetAttribute(tc_update_kernel<1, KC, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) ==
               cudaSuccess &&
           cudaFuncSetAttribute(tc_update_kernel<2, KC, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) ==
               cudaSuccess &&
           cudaFuncSetAttribute(tc_update_kernel<3, KC, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) ==
               cudaSuccess;
}

int tc_update_prepare() {
    if (!tma_encoder()) return -1;
    return tc_set_attrs<64, false>() && tc_set_attrs<32, false>() && tc_set_attrs<32, true>() ? 0 : -1;
}

int tc_update_launch(float *C, int64_t ld, int64_t q, int64_t n, void *planes, int64_t plane_stride,
                     int64_t ldp, int64_t rows, int kext, int terms, bool fp16, const TcPairs &pairs,
                     const int64_t *info, int *err_word, unsigned *sched, unsigned *sched_base, bool narrow,
                     cudaStream_t st, int kchunk, int epilogue, bool pdl) {
    // The TMA-staged epilogue needs 16-byte rows of C (and 32-wide K-chunks).  By
    // default it serves the one- and two-term forms (fp16x3 at n = 16384: 7.8 vs
    // 8.8 ms a solve); the six-product form keeps the register epilogue, which
    // measured slightly faster with its 64-wide K-chunks (8.9 vs 9.1 ms).
    const bool want_tma = epilogue == 2 || (epilogue == 0 && terms <= 2);
    const bool epi_tma = want_tma && ld % 4 == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0 &&
                         ld * 4 < (1ll << 40) && n < (1ll << 31);
    const int kc = (epi_tma || kchunk == 32) ? 32 : 64;
    if (!g_encode || !sched || !sched_base || rows <= 0 || kext % kc != 0 || kext > ldp || (ldp * 2) % 16 != 0 || terms < 1 ||
        terms > 3 || (reinterpret_cast<uintptr_t>(planes) & 15) != 0)
        return -1;
    const int64_t tr = (rows + kTcM - 1) / kTcM;
    const int64_t tiles = narrow ? tr : tr * (tr + 1) / 2;
    CUtensorMap map;
    const cuuint64_t dims[3] = {(cuuint64_t)kext, (cuuint64_t)rows, (cuuint64_t)terms};
    const cuuint64_t strides[2] = {(cuuint64_t)ldp * 2, (cuuint64_t)plane_stride * 2};
    const cuuint32_t box[3] = {(cuuint32_t)kc, (cuuint32_t)kTcM, (cuuint32_t)terms};  // every term plane
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r =
        g_encode(&map, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                 planes, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                 kc == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return -1;
    CUtensorMap cmap;  // the FP32 matrix, column-major: rows are the inner dimension
    std::memset(&cmap, 0, sizeof(cmap));
    if (epi_tma) {
        const cuuint64_t cdims[2] = {(cuuint64_t)n, (cuuint64_t)n};
        const cuuint64_t cstrides[1] = {(cuuint64_t)ld * 4};
        const cuuint32_t cbox[2] = {(cuuint32_t)kTcM, (cuuint32_t)kTcN};
        const cuuint32_t cestr[2] = {1, 1};
        if (g_encode(&cmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, cdims, cstrides, cbox, cestr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return -1;
    }
    // instruction descriptor: D = F32 (bits 4-5), A/B = BF16 (1) or F16 (0) (bits 7-9, 10-12),
    // both K-major, N >> 3 at bit 17, M >> 4 at bit 24
    const uint32_t ab = fp16 ? 0u : 1u;
    const uint32_t idesc = (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                           ((uint32_t)(kTcM >> 4) << 24);
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, sms);
    // the pair lists are fixed per number of terms (small products first, (0, 0) last)
    if (pairs.n != (terms == 1 ? 1 : (terms == 2 ? 3 : 6)) || pairs.pa[pairs.n - 1] != 0 ||
        pairs.pb[pairs.n - 1] != 0)
        return -1;
    auto kern = epi_tma ? (terms == 1 ? tc_update_kernel<1, 32, true>
                                      : (terms == 2 ? tc_update_kernel<2, 32, true> : tc_update_kernel<3, 32, true>))
                : kc == 32 ? (terms == 1 ? tc_update_kernel<1, 32, false>
                                         : (terms == 2 ? tc_update_kernel<2, 32, false> : tc_update_kernel<3, 32, false>))
                           : (terms == 1 ? tc_update_kernel<1, 64, false>
                                         : (terms == 2 ? tc_update_kernel<2, 64, false> : tc_update_kernel<3, 64, false>));
    const cudaError_t e = launch_maybe_pdl(pdl, kern, dim3(grid), dim3(kTcThreads), (size_t)tc_smem_bytes(epi_tma),
                                           st, map, cmap, C, ld, q, n, kext / kc, idesc, tiles, narrow ? 1 : 0,
                                           info, err_word, sched, *sched_base);
    *sched_base += (unsigned)(tiles + grid);  // every CTA claims once more than it processes
    return e == cudaSuccess ? 0 : -1;
}

}  // namespace lla

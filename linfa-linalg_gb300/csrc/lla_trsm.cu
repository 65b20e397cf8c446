// lla_trsm.cu -- triangular solve op(T) X = B, in place on B (n x m), for a
// column-major triangular matrix M on the device.
//
// The reference's substitution (src/triangular.rs:113-125) walks the rows in
// "processing order" -- ascending for Lower, descending for Upper -- and, for
// each row i, divides b[i] by the diagonal and subtracts coeff * a[r, i] from
// every later row r.  Seen from one row r, that is
//     b[r] <- b[r] - x[i] * T[r, i]   for every earlier row i, in processing order,
//     x[r]  = b[r] / diag(r).
// This kernel keeps exactly that per-row sequence: row blocks of 32 are
// processed left-looking, each CTA applying the already-solved blocks in
// processing order and then solving its own diagonal block.  In EXACT mode
// every product and difference is rounded separately (b + (-c)*a equals
// b - c*a exactly in IEEE arithmetic), so X is bit-identical to the
// reference's; FAST mode uses FMA.
//
// Scheduling ("look-back"): each CTA takes a ticket from an atomic counter;
// tickets map to (row block, RHS chunk) in processing order, so a CTA only
// waits for row blocks whose CTAs took earlier tickets and are therefore
// already resident -- the wait always ends.  Every wait is bounded: after
// kSpinLimit polls the CTA records LLA_ERR_TIMEOUT in `err_word`, publishes
// its flag and returns, so a fault elsewhere cannot hang the device.
//
// T[r, c] (logical) = trans ? M[c, r] : M[r, c]; `diag` (optional) overrides
// the diagonal as the reference's diag_fn does (src/triangular.rs:133-144).
#include <atomic>

#include "lla_common.cuh"
#include "lla_kernels.h"
#include "lla_prof.h"

namespace lla {

constexpr int kTrsmNb = 32;
constexpr int kTrsmMaxMc = 8;

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T, bool kExact>
__global__ void __launch_bounds__(256) trsm_lookback(const T *__restrict__ M, int64_t ld, int64_t n,
                                                     int lower, int trans,
                                                     const T *__restrict__ diag, T *B, int64_t ldb,
                                                     int64_t m, int mc, int n_chunks, int *ws,
                                                     int *err_word, int *sticky, long long spin_limit,
                                                     int lose_first) {
    using Ar = Arith<T>;
    __shared__ T ts[kTrsmNb][kTrsmNb + 1];
    __shared__ T xs[kTrsmMaxMc][kTrsmNb];
    __shared__ T dg[kTrsmNb];
    __shared__ int s_ticket, s_abort;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * kTrsmNb + tx, nthr = kTrsmNb * blockDim.y;
    int *counter = ws, *flags = ws + 1;
    if (tid == 0) {
        s_ticket = atomicAdd(counter, 1);
        s_abort = 0;
    }
    __syncthreads();
    // failure injection (tests only): the first item is lost -- never solved,
    // never published -- so every wait on it runs out
    if (lose_first && s_ticket == 0) return;
    const int64_t rb = s_ticket / n_chunks;
    const int cc = s_ticket % n_chunks;
    const int64_t col = (int64_t)cc * mc + ty;
    const bool col_ok = ty < mc && col < m;
    auto row_of = [&](int64_t t) -> int64_t { return lower ? t : n - 1 - t; };
    auto tval = [&](int64_t r, int64_t c) -> T { return trans ? M[c + r * ld] : M[r + c * ld]; };
    const int64_t t_own = rb * kTrsmNb + tx;
    const bool row_ok = t_own < n;
    const int64_t r_own = row_ok ? row_of(t_own) : 0;
    T bv = (row_ok && col_ok) ? B[r_own + col * ldb] : T(0);

    for (int64_t q = 0; q < rb; ++q) {
        if (tid == 0) {
            const int *f = flags + q * n_chunks + cc;
            long long spins = 0;
            while (ld_acquire(f) == 0) {
                if (*(volatile int *)err_word != 0) {
                    s_abort = 1;
                    break;
                }
                if (++spins > spin_limit) {
                    atomicCAS(err_word, 0, (int)LLA_ERR_TIMEOUT);
                    if (sticky) atomicCAS(sticky, 0, (int)LLA_ERR_TIMEOUT);
                    s_abort = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        __syncthreads();
        if (s_abort) break;
        // solved block q (always a full block: q < rb) and the tile T[block rb, block q]
        for (int e = tid; e < kTrsmNb * mc; e += nthr) {
            const int x = e % kTrsmNb, y = e / kTrsmNb;
            const int64_t c = (int64_t)cc * mc + y;
            xs[y][x] = (c < m) ? __ldcg(&B[row_of(q * kTrsmNb + x) + c * ldb]) : T(0);
        }
        for (int e = tid; e < kTrsmNb * kTrsmNb; e += nthr) {
            const int x = trans ? e / kTrsmNb : e % kTrsmNb;  // consecutive e -> consecutive memory
            const int y = trans ? e % kTrsmNb : e / kTrsmNb;
            const int64_t tr = rb * kTrsmNb + x;
            ts[x][y] = (tr < n) ? tval(row_of(tr), row_of(q * kTrsmNb + y)) : T(0);
        }
        __syncthreads();
        if (row_ok && col_ok) {
#pragma unroll 8
            for (int y = 0; y < kTrsmNb; ++y) {
                if (kExact)
                    bv = Ar::sub(bv, Ar::mul(xs[ty][y], ts[tx][y]));
                else
                    bv = Ar::fma_(-xs[ty][y], ts[tx][y], bv);
            }
        }
        __syncthreads();
    }

    if (!s_abort) {
        const int64_t left = n - rb * kTrsmNb;
        const int bs = left < kTrsmNb ? (int)left : kTrsmNb;
        for (int e = tid; e < kTrsmNb * kTrsmNb; e += nthr) {
            const int x = trans ? e / kTrsmNb : e % kTrsmNb;
            const int y = trans ? e % kTrsmNb : e / kTrsmNb;
            ts[x][y] = (x < bs && y < bs) ? tval(row_of(rb * kTrsmNb + x), row_of(rb * kTrsmNb + y))
                                          : T(0);
        }
        if (tid < bs) {
            const int64_t r = row_of(rb * kTrsmNb + tid);
            dg[tid] = diag ? diag[r] : M[r + r * ld];
        }
        __syncthreads();
        for (int y = 0; y < bs; ++y) {
            if (tx == y) {
                const T xv = Ar::div(bv, dg[y]);  // coeff = b[i,k] / diag  (:117-119)
                bv = xv;
                xs[ty][y] = xv;
            }
            __syncthreads();
            if (tx > y && tx < bs) {
                if (kExact)
                    bv = Ar::sub(bv, Ar::mul(xs[ty][y], ts[tx][y]));
                else
                    bv = Ar::fma_(-xs[ty][y], ts[tx][y], bv);
            }
        }
    }
    if (row_ok && col_ok) B[r_own + col * ldb] = bv;
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(flags + rb * n_chunks + cc, 1);
}

// One-shot failure injection for the tests of timeout reporting
// (lla_debug_inject_lost_handoff): the next triangular-solve launch loses its
// first item and its waits give up after the armed number of polls.
static std::atomic<long long> g_inject_spin{-1};  // -1: nothing armed

struct TrsmWaitCfg {
    long long spin_limit;
    int lose_first;
};

static TrsmWaitCfg take_wait_cfg() {
    const long long s = g_inject_spin.exchange(-1);
    if (s < 0) return {kSpinLimit, 0};
    return {s > 0 ? s : kSpinLimit, 1};
}

template <typename T>
int trsm_launch(const T *M, int64_t ld, int64_t n, int lower, int trans, const T *diag, T *B,
                int64_t ldb, int64_t m, bool exact, int *ws, int *err_word, cudaStream_t st,
                int *sticky) {
    if (n == 0 || m == 0) return 0;
    const int mc = (int)std::min<int64_t>(kTrsmMaxMc, m);
    const int64_t chunks = ceil_div(m, mc);
    const int64_t R = ceil_div(n, kTrsmNb);
    if (cudaMemsetAsync(ws, 0, sizeof(int) * (1 + R * chunks), st) != cudaSuccess) return -1;
    const dim3 block(kTrsmNb, mc);
    const unsigned grid = (unsigned)(R * chunks);
    const TrsmWaitCfg wc = take_wait_cfg();
    // algorithmic work: n^2 * m flops (n(n-1)/2 multiply-adds and n divisions per column)
    LaunchScope ls(K_TRSM, st, (double)n * n * m);
    if (exact)
        trsm_lookback<T, true><<<grid, block, 0, st>>>(M, ld, n, lower, trans, diag, B, ldb, m, mc,
                                                       (int)chunks, ws, err_word, sticky,
                                                       wc.spin_limit, wc.lose_first);
    else
        trsm_lookback<T, false><<<grid, block, 0, st>>>(M, ld, n, lower, trans, diag, B, ldb, m,
                                                        mc, (int)chunks, ws, err_word, sticky,
                                                        wc.spin_limit, wc.lose_first);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t trsm_ws_ints(int64_t n, int64_t m) {
    if (n == 0 || m == 0) return 1;
    const int mc = (int)std::min<int64_t>(kTrsmMaxMc, m);
    return (size_t)(1 + ceil_div(n, kTrsmNb) * ceil_div(m, mc));
}

template int trsm_launch<double>(const double *, int64_t, int64_t, int, int, const double *,
                                 double *, int64_t, int64_t, bool, int *, int *, cudaStream_t, int *);
template int trsm_launch<float>(const float *, int64_t, int64_t, int, int, const float *, float *,
                                int64_t, int64_t, bool, int *, int *, cudaStream_t, int *);

}  // namespace lla

// ---------------------------------------------------------------------------
// Allocation-free triangular solve (lla_dtrsm_device_noalloc).
//
// Some callers cannot call cudaMalloc: code that runs inside another
// library's memory-pool callback, processes whose device memory is carved up
// once at start-up by a host framework that owns every allocation, or
// latency-critical loops where an allocation would synchronise the device.
// This entry point takes its ticket/flag scratch from a fixed, file-scope
// device array instead of library-owned buffers.  The array is part of the
// module image, so every GPU that loads the library holds it (a little over
// 256 KiB) until the process exits.
//
// Host code cannot use the array's name as a device address (on the host it
// names a stand-in object); the device address is obtained once per device
// with cudaGetSymbolAddress, on the first call made while that device is
// current, and cached.  That first call therefore also does the set-up and
// should come before any stream capture.  The cache is not refreshed after a
// cudaDeviceReset (which unloads the module), so the entry point must not be
// used across a device reset.
//
// All calls share the one array and it keeps the last call's contents: each
// call clears the part it uses before its launch, and calls whose work
// overlaps on the GPU (different streams, or different host threads without
// ordering) race on it.  A bounded wait that gives up is recorded in the
// array's status word, which lla_dtrsm_device_noalloc_status reads and clears.

#include <mutex>

namespace lla {

constexpr int kNoAllocMaxFlags = 1 << 16;  // row blocks x RHS chunks
constexpr int kNoAllocMaxDevices = 64;
// [0] ticket counter, [1 .. kNoAllocMaxFlags] flags, [kNoAllocMaxFlags + 1]
// error word of the current call, [kNoAllocMaxFlags + 2] status word (kept
// until lla_dtrsm_device_noalloc_status clears it)
constexpr int kNoAllocErr = kNoAllocMaxFlags + 1, kNoAllocStatus = kNoAllocMaxFlags + 2;
static __device__ __align__(256) int g_trsm_noalloc_scratch[kNoAllocMaxFlags + 3];

static std::mutex g_noalloc_mu;
static int *g_noalloc_addr[kNoAllocMaxDevices] = {};

static cudaError_t noalloc_scratch(int **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_trsm_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[dev] = (int *)p;
    }
    *out = g_noalloc_addr[dev];
    return cudaSuccess;
}

}  // namespace lla

extern "C" int lla_dtrsm_device_noalloc(const double *dL, int64_t n, int64_t ld, int trans,
                                        double *dB, int64_t m, int64_t ldb, int algo, void *stream,
                                        lla_error *err) {
    using namespace lla;
    if (n < 0 || m < 0 || ld < std::max<int64_t>(1, n) || ldb < std::max<int64_t>(1, n) ||
        (n > 0 && m > 0 && (!dL || !dB)) || (algo != LLA_ALGO_EXACT && algo != LLA_ALGO_FAST))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (n == 0 || m == 0) return LLA_OK;
    const int mc = (int)std::min<int64_t>(kTrsmMaxMc, m);
    const int64_t chunks = ceil_div(m, mc);
    const int64_t R = ceil_div(n, kTrsmNb);
    if (R * chunks > kNoAllocMaxFlags) return lla__set_status(err, LLA_ERR_TOO_LARGE);
    int *scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess) return lla__set_cuda_error(err, e);
    cudaStream_t st = (cudaStream_t)stream;
    int *err_word = scratch + kNoAllocErr;
    e = cudaMemsetAsync(scratch, 0, sizeof(int) * (size_t)(1 + R * chunks), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err_word, 0, sizeof(int), st);
    if (e != cudaSuccess) return lla__set_cuda_error(err, e);
    const dim3 block(kTrsmNb, mc);
    const unsigned grid = (unsigned)(R * chunks);
    // trans = 0: L X = B (lower, ascending); trans = 1: L^T X = B (descending)
    const int lower = trans ? 0 : 1;
    const TrsmWaitCfg wc = take_wait_cfg();
    {
        // counted and timed like the allocating entry point's launches
        LaunchScope ls(K_TRSM, st, (double)n * n * m);
        if (algo == LLA_ALGO_EXACT)
            trsm_lookback<double, true><<<grid, block, 0, st>>>(
                dL, ld, n, lower, trans ? 1 : 0, nullptr, dB, ldb, m, mc, (int)chunks, scratch, err_word,
                scratch + kNoAllocStatus, wc.spin_limit, wc.lose_first);
        else
            trsm_lookback<double, false><<<grid, block, 0, st>>>(
                dL, ld, n, lower, trans ? 1 : 0, nullptr, dB, ldb, m, mc, (int)chunks, scratch, err_word,
                scratch + kNoAllocStatus, wc.spin_limit, wc.lose_first);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return lla__set_cuda_error(err, e);
    return LLA_OK;
}

// Synchronises `stream`, reads the status word that the allocation-free
// solves on the current device share, and clears it.  Allocates nothing.
extern "C" int lla_dtrsm_device_noalloc_status(void *stream, lla_error *err) {
    using namespace lla;
    lla__set_status(err, LLA_OK);
    int *scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess) return lla__set_cuda_error(err, e);
    cudaStream_t st = (cudaStream_t)stream;
    int word = 0;
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&word, scratch + kNoAllocStatus, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && word != 0) e = cudaMemsetAsync(scratch + kNoAllocStatus, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return lla__set_cuda_error(err, e);
    return word ? lla__set_status(err, word) : LLA_OK;
}

// Arms the one-shot failure injection of the next triangular-solve launch
// (tests of timeout reporting only).
extern "C" int lla_debug_inject_lost_handoff(int64_t spin_limit) {
    if (spin_limit < 0) return LLA_ERR_INVALID_ARG;
    lla::g_inject_spin.store((long long)spin_limit);
    return LLA_OK;
}

// lla_serve.cpp -- serving loop: SPD solve requests of different order,
// precision and tolerance arrive while others run; they are admitted against
// an HBM budget, small systems are gathered into batched launches, large ones
// run concurrently on per-slot streams, factors are kept on the device for
// repeat right-hand sides, and every request records its queueing and service
// times (p50/p99 are computed from these by the caller).
//
// Threads (host side; the small requests are served by a device-resident loop):
//   * slot workers (opts.slots of them): each owns a CUDA stream and the
//     library's per-thread workspace, takes the next admitted large request
//     and runs it to completion (mixed-precision refined solve, plain FP64
//     factor-and-solve when the factor is to be kept, FP32 solve with FP64
//     refinement for single-precision requests, triangular solve, or a solve
//     with a kept factor);
//   * a device pump: small requests (n <= opts.small_n) go to a
//     device-resident loop -- persistent CTAs that claim requests from a ring
//     in mapped host memory and solve each in place, one CTA per request --
//     as soon as they are admitted; the pump relaunches the loop when its
//     CTAs have returned after an idle limit, and reaps completions.
// Requests run on independent data with fixed kernels, so a request's result
// does not depend on what it shares the device with.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/lla_gb300.h"
#include "lla_api_internal.h"
#include "lla_common.cuh"
#include "lla_kernels.h"

namespace {

using Clock = std::chrono::steady_clock;

double now_us(Clock::time_point t0) {
    return std::chrono::duration<double, std::micro>(Clock::now() - t0).count();
}

struct Factor {
    double *L = nullptr;  // n x n FP64 factor (lower), ld = n
    int64_t n = 0;
    size_t bytes = 0;
    int uses = 0;          // repeat-RHS requests currently reading it
    bool released = false; // freed by the last reader once released
};

struct Pending {
    lla_request req;
    lla_result res;
    size_t bytes = 0;  // admitted footprint
};

}  // namespace

struct lla_server {
    lla_serve_opts opts;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_queue, cv_big, cv_small, cv_done;
    std::deque<std::unique_ptr<Pending>> queue;      // submitted, not yet admitted
    std::deque<std::unique_ptr<Pending>> big, small;  // admitted
    std::vector<lla_result> done;
    std::map<int64_t, Factor> factors;
    int64_t next_handle = 1;
    size_t in_use = 0, peak = 0;
    int64_t submitted = 0, completed = 0, running = 0, loop_launches = 0;
    bool stop = false;
    std::vector<std::thread> threads;
};

namespace {

size_t footprint(const lla_serve_opts &o, const lla_request &r) {
    const size_t s = r.dtype == 4 ? 4 : 8;
    const size_t n = (size_t)r.n, m = (size_t)std::max<int64_t>(r.m, 1);
    if (r.kind == LLA_REQ_TRSM || r.kind == LLA_REQ_RESOLVE) return 64 * n * m + (1 << 20);
    if (n <= (size_t)o.small_n) return 2 * s * (n * n + n * m) + 4096;
    // working copy of A (FP64), FP32 factor, residual / correction, kept factor
    size_t b = 8 * n * n + 4 * n * n + 32 * n * m + (8u << 20);
    if (r.keep_factor) b += 8 * n * n;
    if (r.dtype == 4) b += 8 * n * n;  // FP64 copy of an FP32 system
    return b;
}

void finish(lla_server *s, Pending *p, int status) {
    p->res.status = status;
    p->res.t_done_us = now_us(s->t0);
    std::lock_guard<std::mutex> lk(s->mu);
    s->in_use -= p->bytes;
    s->done.push_back(p->res);
    s->completed++;
    s->running--;
    s->cv_queue.notify_all();
    s->cv_done.notify_all();
}

// f32 -> f64 and back, column-major with leading dimensions (device).
__global__ void widen_kernel(const float *a, int64_t lda, double *b, int64_t ldb, int64_t rows,
                             int64_t cols) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y)
        if (i < rows) b[i + j * ldb] = (double)a[i + j * lda];
}
__global__ void narrow_kernel(const double *a, int64_t lda, float *b, int64_t ldb, int64_t rows,
                              int64_t cols) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t j = blockIdx.y; j < cols; j += gridDim.y)
        if (i < rows) b[i + j * ldb] = (float)a[i + j * lda];
}

dim3 grid2(int64_t rows, int64_t cols) {
    return dim3((unsigned)((rows + 255) / 256), (unsigned)std::min<int64_t>(std::max<int64_t>(cols, 1), 65535));
}

// Runs one large request synchronously on this thread's stream.
int run_big(lla_server *s, Pending *p, cudaStream_t st, std::vector<void *> &scratch,
            std::vector<size_t> &sizes) {
    lla_request &r = p->req;
    lla_error err;
    const int64_t n = r.n, m = r.m;
    auto dbuf = [&](size_t bytes, int slot) -> void * {  // grow-only, stream-ordered
        if (scratch.size() <= (size_t)slot) scratch.resize(slot + 1, nullptr);
        if (sizes.size() <= (size_t)slot) sizes.resize(slot + 1, 0);
        if (sizes[slot] >= bytes) return scratch[slot];
        if (scratch[slot]) cudaFreeAsync(scratch[slot], st);
        scratch[slot] = nullptr;
        sizes[slot] = 0;
        if (cudaMallocAsync(&scratch[slot], std::max<size_t>(bytes, 256), st) != cudaSuccess) return nullptr;
        sizes[slot] = std::max<size_t>(bytes, 256);
        return scratch[slot];
    };
    if (r.kind == LLA_REQ_TRSM) {  // L X = B with the lower factor given in A
        p->res.path = LLA_PATH_TRSM;
        int rc = r.dtype == 4 ? lla_strsm_device((const float *)r.A, n, r.lda, 0, (float *)r.B, m, r.ldb,
                                                 LLA_ALGO_FAST, st, &err)
                              : lla_dtrsm_device((const double *)r.A, n, r.lda, 0, (double *)r.B, m, r.ldb,
                                                 LLA_ALGO_FAST, st, &err);
        if (rc) return rc;
        return lla_device_status(st, &err);  // synchronises; LLA_ERR_TIMEOUT if a wait gave up
    }
    if (r.kind == LLA_REQ_RESOLVE) {
        Factor f;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->factors.find(r.factor_handle);
            if (it == s->factors.end() || it->second.released || it->second.n != n || r.dtype != 8)
                return LLA_ERR_INVALID_ARG;
            it->second.uses++;
            f = it->second;
        }
        int rc = lla_dtrsm_device(f.L, n, n, 0, (double *)r.B, m, r.ldb, LLA_ALGO_FAST, st, &err);
        if (!rc) rc = lla_dtrsm_device(f.L, n, n, 1, (double *)r.B, m, r.ldb, LLA_ALGO_FAST, st, &err);
        const int sc = lla_device_status(st, &err);  // synchronises the stream
        if (!rc) rc = sc;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->factors.find(r.factor_handle);
            if (it != s->factors.end() && --it->second.uses == 0 && it->second.released) {
                cudaFreeAsync(it->second.L, st);
                s->in_use -= it->second.bytes;
                s->factors.erase(it);
                s->cv_queue.notify_all();
            }
        }
        p->res.path = LLA_PATH_KEPT_FACTOR;
        return rc;
    }
    // SOLVE
    if (r.keep_factor && r.dtype == 8) {  // plain FP64 factor that stays on the device
        double *L = nullptr;  // stream-ordered allocation: no device-wide synchronisation
        if (cudaMallocAsync((void **)&L, sizeof(double) * n * n, st) != cudaSuccess) return LLA_ERR_NO_MEMORY;
        cudaError_t e = cudaMemcpy2DAsync(L, sizeof(double) * n, r.A, sizeof(double) * r.lda,
                                          sizeof(double) * n, n, cudaMemcpyDeviceToDevice, st);
        int64_t *info = (int64_t *)dbuf(sizeof(int64_t), 0);
        if (e != cudaSuccess || !info) {
            cudaFreeAsync(L, st);
            return LLA_ERR_NO_MEMORY;
        }
        int rc = lla_dpotrf_device(L, n, n, LLA_ALGO_FAST, info, st, &err);
        int64_t hinfo = -1;
        if (!rc && (cudaMemcpyAsync(&hinfo, info, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                    cudaStreamSynchronize(st) != cudaSuccess))
            rc = LLA_ERR_CUDA;
        if (!rc && hinfo >= 0) rc = LLA_NOT_POSITIVE_DEFINITE;
        if (!rc) rc = lla_dtrsm_device(L, n, n, 0, (double *)r.B, m, r.ldb, LLA_ALGO_FAST, st, &err);
        if (!rc) rc = lla_dtrsm_device(L, n, n, 1, (double *)r.B, m, r.ldb, LLA_ALGO_FAST, st, &err);
        if (!rc) rc = lla_device_status(st, &err);  // synchronises the stream
        if (rc) {
            cudaFreeAsync(L, st);
            return rc;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        const int64_t h = s->next_handle++;
        s->factors[h] = Factor{L, n, sizeof(double) * n * n};
        p->res.factor_handle = h;
        p->res.path = LLA_PATH_FP64;
        p->bytes -= sizeof(double) * n * n;  // the kept factor stays accounted until released
        return LLA_OK;
    }
    lla_refine_opts o;
    lla_refine_opts_default(&o);
    o.tol = r.tol > 0 ? r.tol : (r.dtype == 4 ? 1e-6 : 1e-13);
    if (r.dtype == 4) o.update = LLA_UPDATE_FP32;  // single-precision requests: FP32 factor
    lla_refine_report rep;
    int rc;
    if (r.dtype == 8) {
        double *X = (double *)dbuf(sizeof(double) * n * m, 1);
        if (!X) return LLA_ERR_NO_MEMORY;
        rc = lla_dposv_refined_device((const double *)r.A, n, r.lda, (const double *)r.B, m, r.ldb, X,
                                      n, &o, &rep, st, &err);
        if (!rc && cudaMemcpy2DAsync(r.B, sizeof(double) * r.ldb, X, sizeof(double) * n,
                                     sizeof(double) * n, m, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            rc = LLA_ERR_CUDA;
    } else {
        double *A64 = (double *)dbuf(sizeof(double) * n * n, 2);
        double *B64 = (double *)dbuf(sizeof(double) * n * m, 3);
        double *X = (double *)dbuf(sizeof(double) * n * m, 1);
        if (!A64 || !B64 || !X) return LLA_ERR_NO_MEMORY;
        widen_kernel<<<grid2(n, n), 256, 0, st>>>((const float *)r.A, r.lda, A64, n, n, n);
        widen_kernel<<<grid2(n, m), 256, 0, st>>>((const float *)r.B, r.ldb, B64, n, n, m);
        rc = lla_dposv_refined_device(A64, n, n, B64, m, n, X, n, &o, &rep, st, &err);
        if (!rc) narrow_kernel<<<grid2(n, m), 256, 0, st>>>(X, n, (float *)r.B, r.ldb, n, m);
    }
    if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = LLA_ERR_CUDA;
    p->res.backward_error = rep.backward_error;
    p->res.iterations = rep.iterations;
    p->res.path = rep.fell_back ? LLA_PATH_FP64 : LLA_PATH_MIXED;
    return rc;
}

void slot_worker(lla_server *s) {
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    std::vector<void *> scratch;
    std::vector<size_t> sizes;
    for (;;) {
        std::unique_ptr<Pending> p;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_big.wait(lk, [&] { return s->stop || !s->big.empty(); });
            if (s->stop && s->big.empty()) break;
            p = std::move(s->big.front());
            s->big.pop_front();
        }
        p->res.t_start_us = now_us(s->t0);
        const int rc = run_big(s, p.get(), st, scratch, sizes);
        finish(s, p.get(), rc);
    }
    for (void *q : scratch)
        if (q) cudaFreeAsync(q, st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
}

// Small requests go to the device-resident loop (serve_loop_kernel): this
// thread publishes each admitted small request into the request ring as soon
// as it is admitted (no batching window: requests that arrive while others are
// on the GPU join the running loop), relaunches the loop when its CTAs have
// returned after their idle limit, and reaps completions in any order.
void device_pump(lla_server *s) {
    using lla::kServeRing;
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    lla::ServeRing *ring = nullptr, *ring_dev = nullptr;
    unsigned long long *d_next = nullptr;
    double *scratch = nullptr;
    const int ctas = s->opts.device_ctas;
    bool ok = cudaHostAlloc((void **)&ring, sizeof(lla::ServeRing), cudaHostAllocMapped) == cudaSuccess;
    if (ok) {
        std::memset((void *)ring, 0, sizeof(lla::ServeRing));
        ok = cudaHostGetDevicePointer((void **)&ring_dev, ring, 0) == cudaSuccess &&
             cudaMalloc((void **)&d_next, sizeof(unsigned long long)) == cudaSuccess &&
             cudaMemset(d_next, 0, sizeof(unsigned long long)) == cudaSuccess &&
             cudaMalloc((void **)&scratch, lla::serve_loop_scratch_bytes(ctas)) == cudaSuccess;
    }
    std::vector<std::unique_ptr<Pending>> owned(kServeRing);
    unsigned long long published = 0, low = 0;  // low: the oldest ticket not yet reaped
    bool launched = false;
    auto reap = [&]() {
        for (unsigned long long t = low; t < published; ++t) {
            const int slot = (int)(t % kServeRing);
            if (!owned[slot] || __atomic_load_n(&ring->done_seq[slot], __ATOMIC_ACQUIRE) != t + 1) continue;
            const int status = __atomic_load_n(&ring->status[slot], __ATOMIC_RELAXED);
            finish(s, owned[slot].get(), status ? LLA_NOT_POSITIVE_DEFINITE : LLA_OK);
            owned[slot].reset();
        }
        while (low < published && !owned[low % kServeRing]) ++low;
    };
    for (;;) {
        std::vector<std::unique_ptr<Pending>> take;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (low == published)  // nothing in flight: sleep until work arrives
                s->cv_small.wait(lk, [&] { return s->stop || !s->small.empty(); });
            if (s->stop && s->small.empty() && low == published) break;
            while (!s->small.empty() && published + take.size() - low < (unsigned long long)s->opts.batch_max) {
                take.push_back(std::move(s->small.front()));
                s->small.pop_front();
            }
        }
        if (!ok) {  // the loop's resources could not be set up: fail these requests
            for (auto &p : take) finish(s, p.get(), LLA_ERR_NO_MEMORY);
            continue;
        }
        for (auto &p : take) {
            const lla_request &r = p->req;
            const int slot = (int)(published % kServeRing);
            lla::ServeReq &q = ring->req[slot];
            q.A = r.A;
            q.B = r.B;
            q.lda = r.lda;
            q.ldb = r.ldb;
            q.n = (int32_t)r.n;
            q.m = (int32_t)r.m;
            q.dtype = r.dtype;
            p->res.path = LLA_PATH_BATCHED;
            p->res.t_start_us = now_us(s->t0);
            owned[slot] = std::move(p);
            ++published;
            __atomic_store_n(&ring->published, published, __ATOMIC_RELEASE);
        }
        reap();
        if (low < published && (!launched || cudaStreamQuery(st) == cudaSuccess)) {
            // the loop's CTAs returned after their idle limit (or were never
            // started): whatever they claimed is finished, the rest waits
            reap();
            if (low < published) {
                if (lla::serve_loop_launch(ring_dev, d_next, scratch, ctas, s->opts.batch_window_us, st) != 0) {
                    for (unsigned long long t = low; t < published; ++t)
                        if (owned[t % kServeRing]) finish(s, owned[t % kServeRing].get(), LLA_ERR_CUDA);
                    for (auto &o : owned) o.reset();
                    low = published;
                } else {
                    launched = true;
                    std::lock_guard<std::mutex> lk(s->mu);
                    s->loop_launches++;
                }
            }
        }
        if (low < published && take.empty()) std::this_thread::sleep_for(std::chrono::microseconds(10));
    }
    if (ring) __atomic_store_n(&ring->stop, 1, __ATOMIC_RELEASE);
    cudaStreamSynchronize(st);
    if (scratch) cudaFree(scratch);
    if (d_next) cudaFree(d_next);
    if (ring) cudaFreeHost(ring);
    cudaStreamDestroy(st);
}

// Admission: moves queued requests to the run queues while they fit in the
// HBM budget (first come, first served; a request never admitted alone is
// rejected at submission).
void admitter(lla_server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_queue.wait(lk, [&] { return s->stop || !s->queue.empty(); });
        if (s->stop && s->queue.empty()) break;
        while (!s->queue.empty()) {
            Pending *p = s->queue.front().get();
            if (s->in_use + p->bytes > (size_t)s->opts.hbm_budget_bytes) break;
            s->in_use += p->bytes;
            s->peak = std::max(s->peak, s->in_use);
            s->running++;
            p->res.t_admit_us = now_us(s->t0);
            const bool small = p->req.kind == LLA_REQ_SOLVE && !p->req.keep_factor &&
                               p->req.n <= s->opts.small_n && p->req.m <= 8;
            (small ? s->small : s->big).push_back(std::move(s->queue.front()));
            s->queue.pop_front();
            (small ? s->cv_small : s->cv_big).notify_one();
        }
        if (!s->queue.empty()) s->cv_queue.wait(lk);  // wait for a completion to free memory
    }
}

}  // namespace

extern "C" {

void lla_serve_opts_default(lla_serve_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->hbm_budget_bytes = 40e9;
    o->slots = 6;
    o->small_n = 256;
    o->batch_max = 1024;
    o->batch_window_us = 2000.0;
    o->device_ctas = 0;
}

int lla_server_create(const lla_serve_opts *opts, lla_server **out, lla_error *err) {
    if (!out) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (lla_device_count() == 0) return lla__set_status(err, LLA_ERR_NO_DEVICE);
    lla_server *s = new lla_server();
    if (opts)
        s->opts = *opts;
    else
        lla_serve_opts_default(&s->opts);
    if (s->opts.slots <= 0) s->opts.slots = 1;
    if (s->opts.batch_max <= 0 || s->opts.batch_max > lla::kServeRing) s->opts.batch_max = lla::kServeRing;
    if (s->opts.small_n > 256) s->opts.small_n = 256;
    if (!(s->opts.batch_window_us > 0)) s->opts.batch_window_us = 2000.0;
    s->t0 = Clock::now();
    int dev = 0;
    cudaGetDevice(&dev);
    if (s->opts.device_ctas <= 0) {  // default: one CTA on every eighth SM (19 on 152 SMs)
        // Small requests take 50-300 us each on one CTA, so 19 CTAs serve tens of
        // thousands a second; a larger loop holds SMs the large requests need.
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        s->opts.device_ctas = std::max(8, sms / 8);
    }
    auto bind = [dev](void (*fn)(lla_server *), lla_server *srv) {
        return std::thread([dev, fn, srv] {
            cudaSetDevice(dev);
            fn(srv);
        });
    };
    s->threads.push_back(bind(admitter, s));
    s->threads.push_back(bind(device_pump, s));
    for (int i = 0; i < s->opts.slots; ++i) s->threads.push_back(bind(slot_worker, s));
    *out = s;
    return lla__set_status(err, LLA_OK);
}

int lla_server_submit(lla_server *s, const lla_request *r, lla_error *err) {
    if (!s || !r || r->n < 0 || r->m < 0 || (r->n > 0 && (!r->A || (r->m > 0 && !r->B))) ||
        r->lda < std::max<int64_t>(1, r->n) || (r->m > 0 && r->ldb < std::max<int64_t>(1, r->n)) ||
        (r->dtype != 4 && r->dtype != 8) || r->kind < LLA_REQ_SOLVE || r->kind > LLA_REQ_TRSM)
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    std::unique_ptr<Pending> p(new Pending());
    p->req = *r;
    p->res = lla_result{};
    p->res.user_tag = r->user_tag;
    p->res.factor_handle = r->factor_handle;
    p->bytes = footprint(s->opts, *r);
    if (p->bytes > (size_t)s->opts.hbm_budget_bytes) return lla__set_status(err, LLA_ERR_BUSY);
    p->res.t_submit_us = now_us(s->t0);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->submitted++;
        s->queue.push_back(std::move(p));
    }
    s->cv_queue.notify_all();
    return lla__set_status(err, LLA_OK);
}

int lla_server_poll(lla_server *s, lla_result *out, int max, int *n_out) {
    if (!s || !n_out || (max > 0 && !out)) return LLA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    const int k = std::min<int>(max, (int)s->done.size());
    for (int i = 0; i < k; ++i) out[i] = s->done[i];
    s->done.erase(s->done.begin(), s->done.begin() + k);
    *n_out = k;
    return LLA_OK;
}

int lla_server_drain(lla_server *s, double timeout_s) {
    if (!s) return LLA_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return s->completed == s->submitted; });
    return ok ? LLA_OK : LLA_ERR_TIMEOUT;
}

int lla_server_release_factor(lla_server *s, int64_t handle) {
    if (!s) return LLA_ERR_INVALID_ARG;
    double *L = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->factors.find(handle);
        if (it == s->factors.end() || it->second.released) return LLA_ERR_INVALID_ARG;
        if (it->second.uses > 0) {  // the last repeat-RHS reader frees it
            it->second.released = true;
            return LLA_OK;
        }
        L = it->second.L;
        s->in_use -= it->second.bytes;
        s->factors.erase(it);
    }
    cudaFree(L);  // no request reads it any more
    s->cv_queue.notify_all();
    return LLA_OK;
}

int lla_server_get_stats(lla_server *s, lla_server_stats *out) {
    if (!s || !out) return LLA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    out->bytes_in_use = (double)s->in_use;
    out->bytes_peak = (double)s->peak;
    out->queued = (int64_t)s->queue.size();
    out->running = s->running;
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->kept_factors = (int64_t)s->factors.size();
    out->device_loop_launches = s->loop_launches;
    return LLA_OK;
}

void lla_server_destroy(lla_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_queue.notify_all();
    s->cv_big.notify_all();
    s->cv_small.notify_all();
    for (auto &t : s->threads) t.join();
    for (auto &kv : s->factors) cudaFree(kv.second.L);
    cudaDeviceSynchronize();
    delete s;
}

}  // extern "C"

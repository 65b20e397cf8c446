// lla_api.cpp -- the C ABI (include/lla_gb300.h): host-view entry points that
// mirror linfa-linalg's SPD trait methods, and the device-resident entry
// points.  Host code only; every computation runs in the CUDA kernels of the
// other translation units.  There is deliberately no CPU fallback: without a
// device every compute entry point returns LLA_ERR_NO_DEVICE.
//
// Data flow of a host-view call: the view is copied to a device "raw" buffer
// (directly when it is contiguous in row- or column-major order, else through
// a pinned staging buffer gathered on the host), an import kernel moves it to
// the column-major working layout, the kernels run, an export kernel writes
// the selected entries back into the raw buffer (which still holds the
// original values everywhere else -- this is how the reference's "dirty" and
// failure semantics are kept), and the raw buffer is copied back.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "../../include/lla_gb300.h"
#include "lla_kernels.h"
#include "lla_api_internal.h"

using namespace lla;

// ---------------------------------------------------------------------------
// status helpers

extern "C" int lla__set_status(lla_error *err, int code) {
    if (err) {
        std::memset(err, 0, sizeof(*err));
        err->code = code;
    }
    return code;
}

extern "C" int lla__set_cuda_error(lla_error *err, cudaError_t e) {
    const int code = (e == cudaErrorMemoryAllocation) ? LLA_ERR_NO_MEMORY
                     : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                         ? LLA_ERR_NO_DEVICE
                         : LLA_ERR_CUDA;
    lla__set_status(err, code);
    if (err) err->cuda_error = (int32_t)e;
    return code;
}

static int not_square(lla_error *err, int64_t rows, int64_t cols) {
    lla__set_status(err, LLA_NOT_SQUARE);
    if (err) {
        err->rows = rows;
        err->cols = cols;
    }
    return LLA_NOT_SQUARE;
}

static int wrong_rows(lla_error *err, int64_t expected, int64_t actual) {
    lla__set_status(err, LLA_WRONG_ROWS);
    if (err) {
        err->expected = expected;
        err->actual = actual;
    }
    return LLA_WRONG_ROWS;
}

static int not_pd(lla_error *err, int64_t index) {
    lla__set_status(err, LLA_NOT_POSITIVE_DEFINITE);
    if (err) err->index = index;
    return LLA_NOT_POSITIVE_DEFINITE;
}

// ---------------------------------------------------------------------------
// options

static std::atomic<int> g_algo{LLA_ALGO_AUTO};
static constexpr int64_t kAutoExactMaxN = 1024;
// FAST factorisations whose smallest relative pivot falls below this are
// re-run in EXACT order so that NotPositiveDefinite is decided by the
// reference's own arithmetic.
static constexpr double kPivotGuard = 1e-10;

extern "C" int lla_set_algorithm(int algo) {
    if (algo < LLA_ALGO_AUTO || algo > LLA_ALGO_FAST) return -1;
    return g_algo.exchange(algo);
}
extern "C" int lla_get_algorithm(void) { return g_algo.load(); }

static bool use_exact(int64_t n) {
    const int a = g_algo.load();
    if (a == LLA_ALGO_EXACT) return true;
    if (a == LLA_ALGO_FAST) return false;
    return n <= kAutoExactMaxN;
}

extern "C" int lla_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

extern "C" const char *lla_version(void) { return "lla-gb300 0.1.0 (sm_103a)"; }

extern "C" const char *lla_status_string(int code) {
    switch (code) {
        case LLA_OK: return "ok";
        case LLA_NOT_SQUARE: return "matrix is not square";
        case LLA_NOT_POSITIVE_DEFINITE: return "matrix is not positive definite";
        case LLA_WRONG_ROWS: return "matrix has the wrong number of rows";
        case LLA_ERR_CUDA: return "CUDA error";
        case LLA_ERR_NO_MEMORY: return "out of memory";
        case LLA_ERR_INVALID_ARG: return "invalid argument";
        case LLA_ERR_TIMEOUT: return "device wait timed out";
        case LLA_ERR_NO_DEVICE: return "no CUDA device";
        case LLA_ERR_NOT_CONVERGED: return "refinement did not converge";
        case LLA_ERR_BUSY: return "admission refused";
        case LLA_ERR_TOO_LARGE: return "problem exceeds the fixed scratch area";
        default: return "unknown status";
    }
}

// ---------------------------------------------------------------------------
// per-thread context: stream, grow-only device buffers, pinned staging

namespace lla {

cudaError_t DevBuf::ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
}
DevBuf::~DevBuf() {
    if (p) cudaFree(p);
}

cudaError_t HostBuf::ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) cap = want;
    return e;
}
HostBuf::~HostBuf() {
    if (p) cudaFreeHost(p);
}

Ctx::~Ctx() {
    for (auto &e : mixed.ev)
        if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
}

static thread_local std::unique_ptr<Ctx> tls_ctx;

// Returns the calling thread's context, creating it on first use (bound to
// the device current at that time); NULL with err set when no device exists.
Ctx *get_ctx(lla_error *err) {
    if (tls_ctx) return tls_ctx.get();
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        lla__set_status(err, LLA_ERR_NO_DEVICE);
        return nullptr;
    }
    std::unique_ptr<Ctx> c(new Ctx());
    cudaGetDevice(&c->device);
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = c->small_dev.ensure(256);
    if (e == cudaSuccess) e = c->small_host.ensure(256);
    if (e != cudaSuccess) {
        lla__set_cuda_error(err, e);
        return nullptr;
    }
    tls_ctx = std::move(c);
    return tls_ctx.get();
}

}  // namespace lla

// ---------------------------------------------------------------------------
// host views

namespace {

struct View {
    char *p;
    int64_t rows, cols, rs, cs;
    size_t esz;
};

bool colmajor_contig(const View &v) {
    return (v.rows <= 1 || v.rs == 1) && (v.cols <= 1 || v.cs == v.rows);
}
bool rowmajor_contig(const View &v) {
    return (v.cols <= 1 || v.cs == 1) && (v.rows <= 1 || v.rs == v.cols);
}

// Host gather/scatter between a strided view and a column-major staging
// buffer; byte copies keep every bit pattern (NaN payloads included).  Large
// views are split across host threads by column.
void gather_scatter(const View &v, char *stage, bool gather) {
    const int64_t total = v.rows * v.cols;
    auto work = [&](int64_t j0, int64_t j1) {
        for (int64_t j = j0; j < j1; ++j)
            for (int64_t i = 0; i < v.rows; ++i) {
                char *h = v.p + (i * v.rs + j * v.cs) * (int64_t)v.esz;
                char *s = stage + (i + j * v.rows) * (int64_t)v.esz;
                if (gather)
                    std::memcpy(s, h, v.esz);
                else
                    std::memcpy(h, s, v.esz);
            }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int64_t nt = std::min<int64_t>({(int64_t)hw, 16, std::max<int64_t>(1, total / (1 << 20))});
    if (nt <= 1) {
        work(0, v.cols);
        return;
    }
    std::vector<std::thread> th;
    const int64_t per = (v.cols + nt - 1) / nt;
    for (int64_t t = 0; t < nt; ++t) {
        const int64_t j0 = t * per, j1 = std::min(v.cols, j0 + per);
        if (j0 < j1) th.emplace_back(work, j0, j1);
    }
    for (auto &t : th) t.join();
}

// Copies a host view into `raw` (device).  On return (drs, dcs) describe the
// raw layout: column-major (1, rows) or row-major (cols, 1).
// The device address of a contiguous view in page-locked host memory that is
// mapped into the device's address space (cudaHostAlloc / pinned tensors), or
// nullptr: kernels can then read the view in place over the host link
// instead of from a staged device copy.
const void *mapped_alias(const View &v) {
    if (!(colmajor_contig(v) || rowmajor_contig(v))) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, v.p) != cudaSuccess) {
        cudaGetLastError();  // not a pointer the runtime knows: clear the error
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

cudaError_t upload(Ctx &c, const View &v, DevBuf &raw, HostBuf &stage, int64_t &drs, int64_t &dcs) {
    const size_t bytes = (size_t)(v.rows * v.cols) * v.esz;
    cudaError_t e = raw.ensure(bytes);
    if (e != cudaSuccess || bytes == 0) {
        drs = 1;
        dcs = v.rows;
        return e;
    }
    if (colmajor_contig(v) || rowmajor_contig(v)) {
        if (colmajor_contig(v)) {
            drs = 1;
            dcs = v.rows;
        } else {
            drs = v.cols;
            dcs = 1;
        }
        return cudaMemcpyAsync(raw.p, v.p, bytes, cudaMemcpyHostToDevice, c.stream);
    }
    if ((e = stage.ensure(bytes)) != cudaSuccess) return e;
    // the previous user of the staging buffer may still be copying from it
    if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return e;
    gather_scatter(v, (char *)stage.p, true);
    drs = 1;
    dcs = v.rows;
    return cudaMemcpyAsync(raw.p, stage.p, bytes, cudaMemcpyHostToDevice, c.stream);
}

// Copies `raw` back into the host view (all entries; entries the export
// kernel did not select still hold the values uploaded from the view).
// Synchronises the stream.
cudaError_t download(Ctx &c, const View &v, DevBuf &raw, HostBuf &stage) {
    const size_t bytes = (size_t)(v.rows * v.cols) * v.esz;
    if (bytes == 0) return cudaStreamSynchronize(c.stream);
    cudaError_t e;
    if (colmajor_contig(v) || rowmajor_contig(v)) {
        if ((e = cudaMemcpyAsync(v.p, raw.p, bytes, cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess)
            return e;
        return cudaStreamSynchronize(c.stream);
    }
    if ((e = stage.ensure(bytes)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(stage.p, raw.p, bytes, cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return e;
    gather_scatter(v, (char *)stage.p, false);
    return cudaSuccess;
}

cudaError_t launch_status(int rc) {
    if (rc == 0) return cudaSuccess;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? cudaErrorUnknown : e;
}

// Small device/host words: [0] int64 info, [1] double min_ratio, [2] int err_word.
struct Words {
    int64_t info;
    double min_ratio;
    int32_t err_word;
    int32_t flag;
};

cudaError_t reset_words(Ctx &c) {
    Words *h = (Words *)c.small_host.p;
    h->info = -1;
    h->min_ratio = 1e300;
    h->err_word = 0;
    h->flag = 1;
    return cudaMemcpyAsync(c.small_dev.p, h, sizeof(Words), cudaMemcpyHostToDevice, c.stream);
}

cudaError_t read_words(Ctx &c, Words &out) {
    cudaError_t e = cudaMemcpyAsync(c.small_host.p, c.small_dev.p, sizeof(Words),
                                    cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) out = *(Words *)c.small_host.p;
    return e;
}

Words *dev_words(Ctx &c) { return (Words *)c.small_dev.p; }

}  // namespace

namespace lla {

// Factor the column-major n x n W in place.  On a FAST failure or a
// near-singular FAST factorisation, W is re-imported from (R, drs, dcs) and
// factored in EXACT order, whose verdict stands.  *fail receives the failing
// row or -1.
template <typename T>
cudaError_t factor_on_device(Ctx &c, T *W, int64_t n, int64_t ld, bool exact, const T *R,
                             int64_t drs, int64_t dcs, int64_t *fail) {
    cudaError_t e;
    Words w;
    if ((e = reset_words(c)) != cudaSuccess) return e;
    if (!exact) {
        if ((e = c.aux_d.ensure(sizeof(T) * n)) != cudaSuccess) return e;
        e = launch_status(potrf_fast_launch<T>(W, n, ld, &dev_words(c)->info, (T *)c.aux_d.p,
                                               &dev_words(c)->min_ratio, c.stream));
        if (e != cudaSuccess) return e;
        if ((e = read_words(c, w)) != cudaSuccess) return e;
        if (w.info < 0 && !(w.min_ratio < kPivotGuard)) {
            *fail = -1;
            return cudaSuccess;
        }
        // decide with the reference's arithmetic
        if ((e = launch_status(import_launch<T>(R, drs, dcs, n, n, W, ld, c.stream))) != cudaSuccess)
            return e;
        if ((e = reset_words(c)) != cudaSuccess) return e;
    }
    if ((e = c.aux_s.ensure(sizeof(T) * ld * n)) != cudaSuccess) return e;
    if ((e = c.aux_d.ensure(sizeof(T) * n)) != cudaSuccess) return e;
    e = launch_status(potrf_exact_launch<T>(W, (T *)c.aux_s.p, (T *)c.aux_d.p, n, ld,
                                            &dev_words(c)->info, c.stream));
    if (e != cudaSuccess) return e;
    if ((e = read_words(c, w)) != cudaSuccess) return e;
    *fail = w.info;
    return cudaSuccess;
}

template <typename T>
cudaError_t trsm_on_device(Ctx &c, const T *M, int64_t ld, int64_t n, int lower, int trans,
                           const T *diag, T *B, int64_t ldb, int64_t m, bool exact, int *timed_out) {
    cudaError_t e;
    if ((e = c.ws.ensure(sizeof(int) * trsm_ws_ints(n, m))) != cudaSuccess) return e;
    if ((e = reset_words(c)) != cudaSuccess) return e;
    e = launch_status(trsm_launch<T>(M, ld, n, lower, trans, diag, B, ldb, m, exact, (int *)c.ws.p,
                                     &dev_words(c)->err_word, c.stream));
    if (e != cudaSuccess) return e;
    Words w;
    if ((e = read_words(c, w)) != cudaSuccess) return e;
    *timed_out = (w.err_word == LLA_ERR_TIMEOUT);
    return cudaSuccess;
}

template cudaError_t factor_on_device<double>(Ctx &, double *, int64_t, int64_t, bool,
                                              const double *, int64_t, int64_t, int64_t *);
template cudaError_t factor_on_device<float>(Ctx &, float *, int64_t, int64_t, bool, const float *,
                                             int64_t, int64_t, int64_t *);
template cudaError_t trsm_on_device<double>(Ctx &, const double *, int64_t, int64_t, int, int,
                                            const double *, double *, int64_t, int64_t, bool, int *);
template cudaError_t trsm_on_device<float>(Ctx &, const float *, int64_t, int64_t, int, int,
                                           const float *, float *, int64_t, int64_t, bool, int *);

}  // namespace lla

// ---------------------------------------------------------------------------
// drop-in entry points

#define LLA_TRY_CUDA(expr)                                       \
    do {                                                         \
        cudaError_t e__ = (expr);                                \
        if (e__ != cudaSuccess) return lla__set_cuda_error(err, e__); \
    } while (0)

namespace {

bool bad_view(const void *p, int64_t rows, int64_t cols) {
    return rows < 0 || cols < 0 || (p == nullptr && rows * cols > 0);
}

template <typename T>
int cholesky_impl(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs, int dirty,
                  lla_error *err) {
    if (bad_view(a, rows, cols)) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (rows != cols) return not_square(err, rows, cols);  // check_square (src/lib.rs:64-71)
    lla__set_status(err, LLA_OK);
    const int64_t n = rows;
    if (n == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    View v{(char *)a, rows, cols, rs, cs, sizeof(T)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, v, c->raw_a, c->stage_a, drs, dcs));
    LLA_TRY_CUDA(c->work_a.ensure(sizeof(T) * n * n));
    T *W = (T *)c->work_a.p;
    const T *R = (const T *)c->raw_a.p;
    LLA_TRY_CUDA(launch_status(import_launch<T>(R, drs, dcs, n, n, W, n, c->stream)));
    int64_t fail = -1;
    LLA_TRY_CUDA(factor_on_device<T>(*c, W, n, n, use_exact(n), R, drs, dcs, &fail));
    const int mode = fail >= 0 ? EXPORT_FAIL : (dirty ? EXPORT_LOWER : EXPORT_LOWER_ZERO_UPPER);
    LLA_TRY_CUDA(launch_status(export_launch<T>(W, n, (T *)c->raw_a.p, drs, dcs, n, n, mode, fail,
                                                c->stream)));
    LLA_TRY_CUDA(download(*c, v, c->raw_a, c->stage_a));
    if (fail >= 0) return not_pd(err, fail);
    return LLA_OK;
}

// Shared by solvec_inplace and invc_inplace: factor `a` (dirty, written back),
// then solve with B held in the working buffer work_b (n x m, ld n).
template <typename T>
int factor_then(Ctx *c, T *a, int64_t n, int64_t rs, int64_t cs, bool &failed, lla_error *err) {
    View v{(char *)a, n, n, rs, cs, sizeof(T)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, v, c->raw_a, c->stage_a, drs, dcs));
    LLA_TRY_CUDA(c->work_a.ensure(sizeof(T) * n * n));
    T *W = (T *)c->work_a.p;
    const T *R = (const T *)c->raw_a.p;
    LLA_TRY_CUDA(launch_status(import_launch<T>(R, drs, dcs, n, n, W, n, c->stream)));
    int64_t fail = -1;
    LLA_TRY_CUDA(factor_on_device<T>(*c, W, n, n, use_exact(n), R, drs, dcs, &fail));
    const int mode = fail >= 0 ? EXPORT_FAIL : EXPORT_LOWER;  // self keeps the dirty factor (:140)
    LLA_TRY_CUDA(launch_status(export_launch<T>(W, n, (T *)c->raw_a.p, drs, dcs, n, n, mode, fail,
                                                c->stream)));
    LLA_TRY_CUDA(download(*c, v, c->raw_a, c->stage_a));
    failed = fail >= 0;
    if (failed) return not_pd(err, fail);
    return LLA_OK;
}

// X = L^{-T} L^{-1} B for the factor in work_a (src/cholesky.rs:141-142).
template <typename T>
int cholesky_solve_work(Ctx *c, int64_t n, T *WB, int64_t m, lla_error *err) {
    const T *L = (const T *)c->work_a.p;
    const bool exact = use_exact(n);
    int to1 = 0, to2 = 0;
    LLA_TRY_CUDA(trsm_on_device<T>(*c, L, n, n, /*lower=*/1, /*trans=*/0, nullptr, WB, n, m, exact,
                                   &to1));
    LLA_TRY_CUDA(trsm_on_device<T>(*c, L, n, n, /*lower=*/0, /*trans=*/1, nullptr, WB, n, m, exact,
                                   &to2));
    if (to1 || to2) return lla__set_status(err, LLA_ERR_TIMEOUT);
    return LLA_OK;
}

template <typename T>
int solvec_impl(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs, T *b, int64_t brows,
                int64_t bcols, int64_t brs, int64_t bcs, lla_error *err) {
    if (bad_view(a, rows, cols) || bad_view(b, brows, bcols))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (rows != cols) return not_square(err, rows, cols);
    lla__set_status(err, LLA_OK);
    const int64_t n = rows;
    if (n == 0) {
        if (brows != 0) return wrong_rows(err, 0, brows);
        return LLA_OK;
    }
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    bool failed = false;
    int st = factor_then<T>(c, a, n, rs, cs, failed, err);
    if (st != LLA_OK) return st;
    if (brows != n) return wrong_rows(err, n, brows);  // src/triangular.rs:103-108, after the factor
    if (bcols == 0) return LLA_OK;
    View vb{(char *)b, brows, bcols, brs, bcs, sizeof(T)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, vb, c->raw_b, c->stage_b, drs, dcs));
    LLA_TRY_CUDA(c->work_b.ensure(sizeof(T) * n * bcols));
    T *WB = (T *)c->work_b.p;
    LLA_TRY_CUDA(launch_status(import_launch<T>((const T *)c->raw_b.p, drs, dcs, n, bcols, WB, n,
                                                c->stream)));
    st = cholesky_solve_work<T>(c, n, WB, bcols, err);
    if (st != LLA_OK) return st;
    LLA_TRY_CUDA(launch_status(export_launch<T>(WB, n, (T *)c->raw_b.p, drs, dcs, n, bcols,
                                                EXPORT_FULL, -1, c->stream)));
    LLA_TRY_CUDA(download(*c, vb, c->raw_b, c->stage_b));
    return LLA_OK;
}

template <typename T>
int invc_impl(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs, T *out, int64_t ors,
              int64_t ocs, lla_error *err) {
    if (bad_view(a, rows, cols) || bad_view(out, rows, rows))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (rows != cols) return not_square(err, rows, cols);
    lla__set_status(err, LLA_OK);
    const int64_t n = rows;
    if (n == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    bool failed = false;
    int st = factor_then<T>(c, a, n, rs, cs, failed, err);
    if (st != LLA_OK) return st;
    // solvec_into(Array2::eye(n)) (src/cholesky.rs:178-181)
    LLA_TRY_CUDA(c->work_b.ensure(sizeof(T) * n * n));
    T *WB = (T *)c->work_b.p;
    LLA_TRY_CUDA(launch_status(eye_launch<T>(WB, n, n, c->stream)));
    if (use_exact(n)) {
        st = cholesky_solve_work<T>(c, n, WB, n, err);
        if (st != LLA_OK) return st;
    } else {
        // POTRI-style: column panel [c0, c0 + w) of L^-1 is zero above row c0, and
        // rows >= c0 of L^-T L^-1 there need only the trailing triangle L[c0:, c0:];
        // the strict upper part is then mirrored from the lower one.  About n^3
        // flops instead of n^3/3 + 2n^3 (the result is symmetric by construction).
        const T *L = (const T *)c->work_a.p;
        constexpr int64_t kPanel = 1024;
        for (int64_t c0 = 0; c0 < n; c0 += kPanel) {
            const int64_t w = std::min<int64_t>(kPanel, n - c0), nt = n - c0;
            const T *Ls = L + c0 + c0 * n;
            T *Bp = WB + c0 + c0 * n;
            int to1 = 0, to2 = 0;
            LLA_TRY_CUDA(trsm_on_device<T>(*c, Ls, n, nt, /*lower=*/1, /*trans=*/0, nullptr, Bp, n, w, false, &to1));
            LLA_TRY_CUDA(trsm_on_device<T>(*c, Ls, n, nt, /*lower=*/0, /*trans=*/1, nullptr, Bp, n, w, false, &to2));
            if (to1 || to2) return lla__set_status(err, LLA_ERR_TIMEOUT);
        }
        LLA_TRY_CUDA(launch_status(symmetrize_launch<T>(WB, n, n, c->stream)));
    }
    View vo{(char *)out, n, n, ors, ocs, sizeof(T)};
    const bool contig = colmajor_contig(vo) || rowmajor_contig(vo);
    const int64_t drs = (contig && !colmajor_contig(vo)) ? n : 1;
    const int64_t dcs = (contig && !colmajor_contig(vo)) ? 1 : n;
    LLA_TRY_CUDA(c->raw_b.ensure(sizeof(T) * n * n));
    LLA_TRY_CUDA(launch_status(
        export_launch<T>(WB, n, (T *)c->raw_b.p, drs, dcs, n, n, EXPORT_FULL, -1, c->stream)));
    LLA_TRY_CUDA(download(*c, vo, c->raw_b, c->stage_b));
    return LLA_OK;
}

template <typename T>
int trsm_impl(const T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs, const T *diag, T *b,
              int64_t brows, int64_t bcols, int64_t brs, int64_t bcs, int uplo, lla_error *err) {
    if (bad_view(a, rows, cols) || bad_view(b, brows, bcols) ||
        (uplo != LLA_UPPER && uplo != LLA_LOWER))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    // solve_triangular_system_common (src/triangular.rs:102-108)
    if (rows != cols) return not_square(err, rows, cols);
    const int64_t n = rows;
    if (brows != n) return wrong_rows(err, n, brows);
    lla__set_status(err, LLA_OK);
    if (n == 0 || bcols == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    View va{(char *)a, rows, cols, rs, cs, sizeof(T)};
    int64_t ars, acs;
    LLA_TRY_CUDA(upload(*c, va, c->raw_a, c->stage_a, ars, acs));
    LLA_TRY_CUDA(c->work_a.ensure(sizeof(T) * n * n));
    T *W = (T *)c->work_a.p;
    LLA_TRY_CUDA(launch_status(import_launch<T>((const T *)c->raw_a.p, ars, acs, n, n, W, n,
                                                c->stream)));
    const T *ddiag = nullptr;
    if (diag) {
        LLA_TRY_CUDA(c->aux_diag.ensure(sizeof(T) * n));
        LLA_TRY_CUDA(cudaMemcpyAsync(c->aux_diag.p, diag, sizeof(T) * n, cudaMemcpyHostToDevice,
                                     c->stream));
        ddiag = (const T *)c->aux_diag.p;
    }
    View vb{(char *)b, brows, bcols, brs, bcs, sizeof(T)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, vb, c->raw_b, c->stage_b, drs, dcs));
    LLA_TRY_CUDA(c->work_b.ensure(sizeof(T) * n * bcols));
    T *WB = (T *)c->work_b.p;
    LLA_TRY_CUDA(launch_status(import_launch<T>((const T *)c->raw_b.p, drs, dcs, n, bcols, WB, n,
                                                c->stream)));
    int to = 0;
    LLA_TRY_CUDA(trsm_on_device<T>(*c, W, n, n, uplo == LLA_LOWER ? 1 : 0, 0, ddiag, WB, n, bcols,
                                   use_exact(n), &to));
    if (to) return lla__set_status(err, LLA_ERR_TIMEOUT);
    LLA_TRY_CUDA(launch_status(export_launch<T>(WB, n, (T *)c->raw_b.p, drs, dcs, n, bcols,
                                                EXPORT_FULL, -1, c->stream)));
    LLA_TRY_CUDA(download(*c, vb, c->raw_b, c->stage_b));
    return LLA_OK;
}

template <typename T>
int triangular_impl(T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs, int uplo,
                    lla_error *err) {
    if (bad_view(a, rows, cols) || (uplo != LLA_UPPER && uplo != LLA_LOWER))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (rows != cols) return not_square(err, rows, cols);
    lla__set_status(err, LLA_OK);
    if (rows == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    View v{(char *)a, rows, cols, rs, cs, sizeof(T)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, v, c->raw_a, c->stage_a, drs, dcs));
    LLA_TRY_CUDA(launch_status(mask_launch<T>((T *)c->raw_a.p, drs, dcs, rows, uplo, c->stream)));
    LLA_TRY_CUDA(download(*c, v, c->raw_a, c->stage_a));
    return LLA_OK;
}

template <typename T>
int is_triangular_impl(const T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs, int uplo,
                       int *result, lla_error *err) {
    if (!result || bad_view(a, rows, cols) || (uplo != LLA_UPPER && uplo != LLA_LOWER))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (rows != cols) {  // check_square fails -> false (src/triangular.rs:87-89)
        *result = 0;
        return LLA_OK;
    }
    if (rows == 0) {
        *result = 1;
        return LLA_OK;
    }
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    View v{(char *)a, rows, cols, rs, cs, sizeof(T)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, v, c->raw_a, c->stage_a, drs, dcs));
    LLA_TRY_CUDA(reset_words(*c));
    LLA_TRY_CUDA(launch_status(is_triangular_launch<T>((const T *)c->raw_a.p, drs, dcs, rows, uplo,
                                                       &dev_words(*c)->flag, c->stream)));
    Words w;
    LLA_TRY_CUDA(read_words(*c, w));
    *result = w.flag;
    return LLA_OK;
}

// Layout of an output view's device copy (nothing uploaded: every entry is
// written before the download): the view's own layout when contiguous, else
// column-major with gather/scatter through the staging buffer at download.
cudaError_t prepare_out(const View &v, DevBuf &raw, int64_t &drs, int64_t &dcs) {
    if (rowmajor_contig(v) && !colmajor_contig(v)) {
        drs = v.cols;
        dcs = 1;
    } else {
        drs = 1;
        dcs = v.rows;
    }
    return raw.ensure((size_t)(v.rows * v.cols) * v.esz);
}

// orthonormalize (src/lobpcg/algorithm.rs:81-96): G = V^T V, L = cholesky_into(G),
// U = (L^-1 V^T)^T.
template <typename T>
int orthonormalize_impl(const T *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, T *u, int64_t urows,
                        int64_t ucols, int64_t urs, int64_t ucs, T *l, int64_t lrows, int64_t lcols, int64_t lrs,
                        int64_t lcs, lla_error *err) {
    if (bad_view(v, rows, cols) || bad_view(u, urows, ucols) || bad_view(l, lrows, lcols) || urows != rows ||
        ucols != cols || lrows != cols || lcols != cols)
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    const int64_t n = rows, k = cols;
    if (k == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    View vv{(char *)v, n, k, rs, cs, sizeof(T)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, vv, c->raw_a, c->stage_a, drs, dcs));
    LLA_TRY_CUDA(c->work_b.ensure(sizeof(T) * (n > 0 ? n : 1) * k));
    LLA_TRY_CUDA(c->work_a.ensure(sizeof(T) * k * k));
    LLA_TRY_CUDA(c->lob_g.ensure(sizeof(T) * k * k));
    LLA_TRY_CUDA(c->lob_p.ensure(sizeof(T) * atb_ws_elems(n, k, k)));
    LLA_TRY_CUDA(c->lob_t.ensure(sizeof(T) * k * (n > 0 ? n : 1)));
    T *WV = (T *)c->work_b.p, *G = (T *)c->work_a.p, *Gc = (T *)c->lob_g.p, *VT = (T *)c->lob_t.p;
    LLA_TRY_CUDA(launch_status(import_launch<T>((const T *)c->raw_a.p, drs, dcs, n, k, WV, n, c->stream)));
    LLA_TRY_CUDA(launch_status(atb_launch<T>(WV, n, WV, n, n, k, k, G, k, (T *)c->lob_p.p, 1, c->stream)));
    LLA_TRY_CUDA(cudaMemcpyAsync(Gc, G, sizeof(T) * k * k, cudaMemcpyDeviceToDevice, c->stream));
    int64_t fail = -1;
    LLA_TRY_CUDA(factor_on_device<T>(*c, G, k, k, use_exact(k), Gc, 1, k, &fail));
    if (fail >= 0) return not_pd(err, fail);
    // L: lower factor, upper part zeroed (cholesky_into)
    View vl{(char *)l, k, k, lrs, lcs, sizeof(T)};
    int64_t lrs_d, lcs_d;
    LLA_TRY_CUDA(prepare_out(vl, c->raw_c, lrs_d, lcs_d));
    LLA_TRY_CUDA(launch_status(export_launch<T>(G, k, (T *)c->raw_c.p, lrs_d, lcs_d, k, k, EXPORT_LOWER_ZERO_UPPER,
                                                -1, c->stream)));
    if (n > 0) {
        // V^T (k x n), L Z = V^T, U = Z^T
        LLA_TRY_CUDA(launch_status(import_launch<T>(WV, n, 1, k, n, VT, k, c->stream)));
        int to = 0;
        LLA_TRY_CUDA(trsm_on_device<T>(*c, G, k, k, /*lower=*/1, /*trans=*/0, nullptr, VT, k, n, use_exact(k), &to));
        if (to) return lla__set_status(err, LLA_ERR_TIMEOUT);
        LLA_TRY_CUDA(launch_status(import_launch<T>(VT, k, 1, n, k, WV, n, c->stream)));
        View vu{(char *)u, n, k, urs, ucs, sizeof(T)};
        int64_t urs_d, ucs_d;
        LLA_TRY_CUDA(prepare_out(vu, c->raw_b, urs_d, ucs_d));
        LLA_TRY_CUDA(launch_status(
            export_launch<T>(WV, n, (T *)c->raw_b.p, urs_d, ucs_d, n, k, EXPORT_FULL, -1, c->stream)));
        LLA_TRY_CUDA(download(*c, vu, c->raw_b, c->stage_b));
    }
    LLA_TRY_CUDA(download(*c, vl, c->raw_c, c->stage_c));
    return LLA_OK;
}

// apply_constraints (src/lobpcg/algorithm.rs:63-76): U from lyy U = y^T v, v -= y U.
template <typename T>
int apply_constraints_impl(T *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, const T *y, int64_t yrows,
                           int64_t ycols, int64_t yrs, int64_t ycs, const T *lyy, int64_t lrows, int64_t lcols,
                           int64_t lrs, int64_t lcs, lla_error *err) {
    if (bad_view(v, rows, cols) || bad_view(y, yrows, ycols) || bad_view(lyy, lrows, lcols) || yrows != rows)
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (lrows != lcols) return not_square(err, lrows, lcols);  // solve_triangular_into's check
    if (lrows != ycols) return wrong_rows(err, lrows, ycols);
    lla__set_status(err, LLA_OK);
    const int64_t n = rows, k = cols, ky = ycols;
    if (n == 0 || k == 0 || ky == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    View vv{(char *)v, n, k, rs, cs, sizeof(T)};
    View vy{(char *)y, n, ky, yrs, ycs, sizeof(T)};
    View vl{(char *)lyy, ky, ky, lrs, lcs, sizeof(T)};
    int64_t vrs, vcs, yrs_d, ycs_d, lrs_d, lcs_d;
    LLA_TRY_CUDA(upload(*c, vv, c->raw_a, c->stage_a, vrs, vcs));
    LLA_TRY_CUDA(upload(*c, vy, c->raw_b, c->stage_b, yrs_d, ycs_d));
    LLA_TRY_CUDA(upload(*c, vl, c->raw_c, c->stage_c, lrs_d, lcs_d));
    LLA_TRY_CUDA(c->work_a.ensure(sizeof(T) * ky * ky));
    LLA_TRY_CUDA(c->work_b.ensure(sizeof(T) * n * k));
    LLA_TRY_CUDA(c->lob_t.ensure(sizeof(T) * n * ky));
    LLA_TRY_CUDA(c->lob_g.ensure(sizeof(T) * ky * k));
    LLA_TRY_CUDA(c->lob_p.ensure(sizeof(T) * atb_ws_elems(n, ky, k)));
    T *WL = (T *)c->work_a.p, *WV = (T *)c->work_b.p, *WY = (T *)c->lob_t.p, *GU = (T *)c->lob_g.p;
    LLA_TRY_CUDA(launch_status(import_launch<T>((const T *)c->raw_a.p, vrs, vcs, n, k, WV, n, c->stream)));
    LLA_TRY_CUDA(launch_status(import_launch<T>((const T *)c->raw_b.p, yrs_d, ycs_d, n, ky, WY, n, c->stream)));
    LLA_TRY_CUDA(launch_status(import_launch<T>((const T *)c->raw_c.p, lrs_d, lcs_d, ky, ky, WL, ky, c->stream)));
    LLA_TRY_CUDA(launch_status(atb_launch<T>(WY, n, WV, n, n, ky, k, GU, ky, (T *)c->lob_p.p, 0, c->stream)));
    int to = 0;
    LLA_TRY_CUDA(trsm_on_device<T>(*c, WL, ky, ky, /*lower=*/1, /*trans=*/0, nullptr, GU, ky, k, use_exact(ky), &to));
    if (to) return lla__set_status(err, LLA_ERR_TIMEOUT);
    LLA_TRY_CUDA(launch_status(sub_tall_launch<T>(WV, n, WY, n, GU, ky, n, ky, k, c->stream)));
    LLA_TRY_CUDA(launch_status(
        export_launch<T>(WV, n, (T *)c->raw_a.p, vrs, vcs, n, k, EXPORT_FULL, -1, c->stream)));
    LLA_TRY_CUDA(download(*c, vv, c->raw_a, c->stage_a));
    return LLA_OK;
}

}  // namespace

// ---- mixed-precision refined solve on host views ---------------------------

int lla_dposv_refined(const double *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs, double *b,
                      int64_t brows, int64_t bcols, int64_t brs, int64_t bcs,
                      const lla_refine_opts *opts, lla_refine_report *report, lla_error *err) {
    if (bad_view(a, rows, cols) || bad_view(b, brows, bcols))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (rows != cols) return not_square(err, rows, cols);
    const int64_t n = rows;
    if (brows != n) return wrong_rows(err, n, brows);
    lla__set_status(err, LLA_OK);
    if (n == 0 || bcols == 0) {
        return lla_dposv_refined_device(nullptr, 0, 1, nullptr, 0, 1, nullptr, 1, opts, report,
                                        nullptr, err);
    }
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    View va{(char *)a, rows, cols, rs, cs, sizeof(double)};
    int64_t ars, acs;
    // A in mapped page-locked memory is read in place by the import kernel (one
    // pass over the host link instead of a staging copy followed by a device pass)
    const double *src = (const double *)mapped_alias(va);
    if (src) {
        ars = colmajor_contig(va) ? 1 : n;
        acs = colmajor_contig(va) ? n : 1;
    } else {
        LLA_TRY_CUDA(upload(*c, va, c->raw_a, c->stage_a, ars, acs));
        src = (const double *)c->raw_a.p;
    }
    LLA_TRY_CUDA(c->work_a.ensure(sizeof(double) * n * n));
    double *W = (double *)c->work_a.p;
    LLA_TRY_CUDA(launch_status(import_launch<double>(src, ars, acs, n, n, W, n, c->stream)));
    View vb{(char *)b, brows, bcols, brs, bcs, sizeof(double)};
    int64_t drs, dcs;
    LLA_TRY_CUDA(upload(*c, vb, c->raw_b, c->stage_b, drs, dcs));
    LLA_TRY_CUDA(c->work_b.ensure(sizeof(double) * n * bcols));
    LLA_TRY_CUDA(c->aux_x.ensure(sizeof(double) * n * bcols));
    double *WB = (double *)c->work_b.p, *X = (double *)c->aux_x.p;
    LLA_TRY_CUDA(launch_status(import_launch<double>((const double *)c->raw_b.p, drs, dcs, n, bcols,
                                                     WB, n, c->stream)));
    const int st = lla_dposv_refined_device(W, n, n, WB, bcols, n, X, n, opts, report, c->stream, err);
    if (st != LLA_OK) return st;
    LLA_TRY_CUDA(launch_status(export_launch<double>(X, n, (double *)c->raw_b.p, drs, dcs, n, bcols,
                                                     EXPORT_FULL, -1, c->stream)));
    LLA_TRY_CUDA(download(*c, vb, c->raw_b, c->stage_b));
    return LLA_OK;
}

// ---- device-resident entry points -----------------------------------------

template <typename T>
static int potrf_device_impl(T *dA, int64_t n, int64_t ld, int algo, int64_t *d_info, void *stream,
                             lla_error *err) {
    if (n < 0 || ld < std::max<int64_t>(1, n) || !d_info || (n > 0 && !dA) ||
        (algo != LLA_ALGO_EXACT && algo != LLA_ALGO_FAST))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    LLA_TRY_CUDA(cudaMemsetAsync(d_info, 0xff, sizeof(int64_t), st));  // -1
    if (n == 0) return LLA_OK;
    if (algo == LLA_ALGO_EXACT) {
        LLA_TRY_CUDA(c->dev_s.ensure(sizeof(T) * ld * n));
        LLA_TRY_CUDA(c->dev_d.ensure(sizeof(T) * n));
        LLA_TRY_CUDA(launch_status(
            potrf_exact_launch<T>(dA, (T *)c->dev_s.p, (T *)c->dev_d.p, n, ld, d_info, st)));
    } else {
        LLA_TRY_CUDA(c->dev_d.ensure(sizeof(T) * n));
        LLA_TRY_CUDA(launch_status(
            potrf_fast_launch<T>(dA, n, ld, d_info, (T *)c->dev_d.p, nullptr, st)));
    }
    return LLA_OK;
}

// The calling thread's device-call status word (allocated and zeroed once;
// the asynchronous device entry points record a timed-out wait there).
static cudaError_t device_status_word(Ctx &c, cudaStream_t st, int **out) {
    cudaError_t e = c.status_dev.ensure(sizeof(int));
    if (e != cudaSuccess) return e;
    if (!c.status_clear) {
        if ((e = cudaMemsetAsync(c.status_dev.p, 0, sizeof(int), st)) != cudaSuccess) return e;
        c.status_clear = true;
    }
    *out = (int *)c.status_dev.p;
    return cudaSuccess;
}

template <typename T>
static int trsm_device_impl(const T *dL, int64_t n, int64_t ld, int trans, T *dB, int64_t m,
                            int64_t ldb, int algo, void *stream, lla_error *err) {
    if (n < 0 || m < 0 || ld < std::max<int64_t>(1, n) || ldb < std::max<int64_t>(1, n) ||
        (n > 0 && m > 0 && (!dL || !dB)) || (algo != LLA_ALGO_EXACT && algo != LLA_ALGO_FAST))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (n == 0 || m == 0) return LLA_OK;
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    LLA_TRY_CUDA(c->dev_ws.ensure(sizeof(int) * (trsm_ws_ints(n, m) + 1)));
    int *ws = (int *)c->dev_ws.p;
    int *err_word = ws + trsm_ws_ints(n, m);
    int *sticky = nullptr;
    LLA_TRY_CUDA(device_status_word(*c, st, &sticky));
    LLA_TRY_CUDA(cudaMemsetAsync(err_word, 0, sizeof(int), st));
    // trans = 0: L X = B (lower, processing ascending); trans = 1: L^T X = B
    LLA_TRY_CUDA(launch_status(trsm_launch<T>(dL, ld, n, trans ? 0 : 1, trans ? 1 : 0, nullptr, dB,
                                              ldb, m, algo == LLA_ALGO_EXACT, ws, err_word, st, sticky)));
    return LLA_OK;
}

// triangular_inplace / is_triangular on device-resident column-major matrices
// (src/triangular.rs:37-53, 67-90): no host round trip, so a factor produced by
// lla_?potrf_device can be masked or tested where it lies.
template <typename T>
static int triangular_device_impl(T *dA, int64_t rows, int64_t cols, int64_t ld, int uplo, void *stream,
                                  lla_error *err) {
    if (rows < 0 || cols < 0 || ld < std::max<int64_t>(1, rows) || (rows * cols > 0 && !dA) ||
        (uplo != LLA_UPPER && uplo != LLA_LOWER))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    if (rows != cols) return not_square(err, rows, cols);  // check_square (src/lib.rs:64-71)
    lla__set_status(err, LLA_OK);
    if (rows == 0) return LLA_OK;
    if (!get_ctx(err)) return err ? err->code : LLA_ERR_NO_DEVICE;
    LLA_TRY_CUDA(launch_status(mask_launch<T>(dA, 1, ld, rows, uplo, (cudaStream_t)stream)));
    return LLA_OK;
}

template <typename T>
static int is_triangular_device_impl(const T *dA, int64_t rows, int64_t cols, int64_t ld, int uplo,
                                     int *d_result, void *stream, lla_error *err) {
    if (rows < 0 || cols < 0 || ld < std::max<int64_t>(1, rows) || (rows * cols > 0 && !dA) || !d_result ||
        (uplo != LLA_UPPER && uplo != LLA_LOWER))
        return lla__set_status(err, LLA_ERR_INVALID_ARG);
    lla__set_status(err, LLA_OK);
    if (!get_ctx(err)) return err ? err->code : LLA_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    // a non-square matrix is not triangular (no error, as in the reference)
    LLA_TRY_CUDA(launch_status(fill_int_launch(d_result, rows == cols ? 1 : 0, st)));
    if (rows == cols && rows > 0)
        LLA_TRY_CUDA(launch_status(is_triangular_launch<T>(dA, 1, ld, rows, uplo, d_result, st)));
    return LLA_OK;
}

#define LLA_VIEW_ARGS(T) T *a, int64_t rows, int64_t cols, int64_t rs, int64_t cs

extern "C" {

int lla_dtriangular_device(double *dA, int64_t rows, int64_t cols, int64_t ld, int uplo, void *stream,
                           lla_error *err) {
    return triangular_device_impl<double>(dA, rows, cols, ld, uplo, stream, err);
}
int lla_striangular_device(float *dA, int64_t rows, int64_t cols, int64_t ld, int uplo, void *stream,
                           lla_error *err) {
    return triangular_device_impl<float>(dA, rows, cols, ld, uplo, stream, err);
}
int lla_dis_triangular_device(const double *dA, int64_t rows, int64_t cols, int64_t ld, int uplo,
                              int *d_result, void *stream, lla_error *err) {
    return is_triangular_device_impl<double>(dA, rows, cols, ld, uplo, d_result, stream, err);
}
int lla_sis_triangular_device(const float *dA, int64_t rows, int64_t cols, int64_t ld, int uplo,
                              int *d_result, void *stream, lla_error *err) {
    return is_triangular_device_impl<float>(dA, rows, cols, ld, uplo, d_result, stream, err);
}

int lla_device_status(void *stream, lla_error *err) {
    lla__set_status(err, LLA_OK);
    Ctx *c = get_ctx(err);
    if (!c) return err ? err->code : LLA_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    LLA_TRY_CUDA(cudaStreamSynchronize(st));
    if (!c->status_dev.p || !c->status_clear) return LLA_OK;  // nothing recorded yet
    int word = 0;
    LLA_TRY_CUDA(cudaMemcpyAsync(&word, c->status_dev.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    LLA_TRY_CUDA(cudaStreamSynchronize(st));
    if (word == 0) return LLA_OK;
    LLA_TRY_CUDA(cudaMemsetAsync(c->status_dev.p, 0, sizeof(int), st));
    LLA_TRY_CUDA(cudaStreamSynchronize(st));
    return lla__set_status(err, word);
}

int lla_dcholesky_inplace(LLA_VIEW_ARGS(double), int dirty, lla_error *err) {
    return cholesky_impl<double>(a, rows, cols, rs, cs, dirty, err);
}
int lla_scholesky_inplace(LLA_VIEW_ARGS(float), int dirty, lla_error *err) {
    return cholesky_impl<float>(a, rows, cols, rs, cs, dirty, err);
}
int lla_dsolvec_inplace(LLA_VIEW_ARGS(double), double *b, int64_t brows, int64_t bcols, int64_t brs,
                        int64_t bcs, lla_error *err) {
    return solvec_impl<double>(a, rows, cols, rs, cs, b, brows, bcols, brs, bcs, err);
}
int lla_ssolvec_inplace(LLA_VIEW_ARGS(float), float *b, int64_t brows, int64_t bcols, int64_t brs,
                        int64_t bcs, lla_error *err) {
    return solvec_impl<float>(a, rows, cols, rs, cs, b, brows, bcols, brs, bcs, err);
}
int lla_dinvc_inplace(LLA_VIEW_ARGS(double), double *out, int64_t out_rs, int64_t out_cs,
                      lla_error *err) {
    return invc_impl<double>(a, rows, cols, rs, cs, out, out_rs, out_cs, err);
}
int lla_sinvc_inplace(LLA_VIEW_ARGS(float), float *out, int64_t out_rs, int64_t out_cs,
                      lla_error *err) {
    return invc_impl<float>(a, rows, cols, rs, cs, out, out_rs, out_cs, err);
}
int lla_dsolve_triangular_inplace(LLA_VIEW_ARGS(const double), double *b, int64_t brows,
                                  int64_t bcols, int64_t brs, int64_t bcs, int uplo, lla_error *err) {
    return trsm_impl<double>(a, rows, cols, rs, cs, nullptr, b, brows, bcols, brs, bcs, uplo, err);
}
int lla_ssolve_triangular_inplace(LLA_VIEW_ARGS(const float), float *b, int64_t brows,
                                  int64_t bcols, int64_t brs, int64_t bcs, int uplo, lla_error *err) {
    return trsm_impl<float>(a, rows, cols, rs, cs, nullptr, b, brows, bcols, brs, bcs, uplo, err);
}
int lla_dsolve_triangular_diag(LLA_VIEW_ARGS(const double), const double *diag, double *b,
                               int64_t brows, int64_t bcols, int64_t brs, int64_t bcs, int uplo,
                               lla_error *err) {
    if (!diag && rows > 0) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    return trsm_impl<double>(a, rows, cols, rs, cs, diag, b, brows, bcols, brs, bcs, uplo, err);
}
int lla_ssolve_triangular_diag(LLA_VIEW_ARGS(const float), const float *diag, float *b,
                               int64_t brows, int64_t bcols, int64_t brs, int64_t bcs, int uplo,
                               lla_error *err) {
    if (!diag && rows > 0) return lla__set_status(err, LLA_ERR_INVALID_ARG);
    return trsm_impl<float>(a, rows, cols, rs, cs, diag, b, brows, bcols, brs, bcs, uplo, err);
}
int lla_dtriangular_inplace(LLA_VIEW_ARGS(double), int uplo, lla_error *err) {
    return triangular_impl<double>(a, rows, cols, rs, cs, uplo, err);
}
int lla_striangular_inplace(LLA_VIEW_ARGS(float), int uplo, lla_error *err) {
    return triangular_impl<float>(a, rows, cols, rs, cs, uplo, err);
}
int lla_dorthonormalize(const double *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, double *u,
                        int64_t urows, int64_t ucols, int64_t urs, int64_t ucs, double *l, int64_t lrows,
                        int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err) {
    return orthonormalize_impl<double>(v, rows, cols, rs, cs, u, urows, ucols, urs, ucs, l, lrows, lcols, lrs, lcs,
                                       err);
}
int lla_sorthonormalize(const float *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, float *u,
                        int64_t urows, int64_t ucols, int64_t urs, int64_t ucs, float *l, int64_t lrows,
                        int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err) {
    return orthonormalize_impl<float>(v, rows, cols, rs, cs, u, urows, ucols, urs, ucs, l, lrows, lcols, lrs, lcs,
                                      err);
}
int lla_dapply_constraints(double *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, const double *y,
                           int64_t yrows, int64_t ycols, int64_t yrs, int64_t ycs, const double *lyy,
                           int64_t lrows, int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err) {
    return apply_constraints_impl<double>(v, rows, cols, rs, cs, y, yrows, ycols, yrs, ycs, lyy, lrows, lcols, lrs,
                                          lcs, err);
}
int lla_sapply_constraints(float *v, int64_t rows, int64_t cols, int64_t rs, int64_t cs, const float *y,
                           int64_t yrows, int64_t ycols, int64_t yrs, int64_t ycs, const float *lyy,
                           int64_t lrows, int64_t lcols, int64_t lrs, int64_t lcs, lla_error *err) {
    return apply_constraints_impl<float>(v, rows, cols, rs, cs, y, yrows, ycols, yrs, ycs, lyy, lrows, lcols, lrs,
                                         lcs, err);
}
int lla_dis_triangular(LLA_VIEW_ARGS(const double), int uplo, int *result, lla_error *err) {
    return is_triangular_impl<double>(a, rows, cols, rs, cs, uplo, result, err);
}
int lla_sis_triangular(LLA_VIEW_ARGS(const float), int uplo, int *result, lla_error *err) {
    return is_triangular_impl<float>(a, rows, cols, rs, cs, uplo, result, err);
}

int lla_dpotrf_device(double *dA, int64_t n, int64_t ld, int algo, int64_t *d_info, void *stream,
                      lla_error *err) {
    return potrf_device_impl<double>(dA, n, ld, algo, d_info, stream, err);
}
int lla_spotrf_device(float *dA, int64_t n, int64_t ld, int algo, int64_t *d_info, void *stream,
                      lla_error *err) {
    return potrf_device_impl<float>(dA, n, ld, algo, d_info, stream, err);
}

int lla_dtrsm_device(const double *dL, int64_t n, int64_t ld, int trans, double *dB, int64_t m,
                     int64_t ldb, int algo, void *stream, lla_error *err) {
    return trsm_device_impl<double>(dL, n, ld, trans, dB, m, ldb, algo, stream, err);
}
int lla_strsm_device(const float *dL, int64_t n, int64_t ld, int trans, float *dB, int64_t m,
                     int64_t ldb, int algo, void *stream, lla_error *err) {
    return trsm_device_impl<float>(dL, n, ld, trans, dB, m, ldb, algo, stream, err);
}

}  // extern "C"

// lla_prof.cpp -- see lla_prof.h.
#include "lla_prof.h"

#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/lla_gb300.h"

namespace lla {

static const char *kNames[K_COUNT] = {
    "potrf_exact_diag", "potrf_exact_panel", "potrf_exact_update", "potrf_fast_diag",
    "potrf_fast_panel", "potrf_fast_update", "trsm",              "layout",
    "mixed_diag",       "mixed_panel",       "mixed_update",      "mixed_convert",
    "residual",         "refine",            "mixed_trsm",        "batch",
    "oz_slice",         "misc"};

const char *kernel_name(int id) { return (id >= 0 && id < K_COUNT) ? kNames[id] : "?"; }

static std::atomic<int64_t> g_launches{0};
static std::atomic<bool> g_on{false};

struct Rec {
    int kid;
    double work;
    cudaEvent_t a, b;
};

static std::mutex g_mu;
static std::vector<Rec> g_recs;
static std::vector<cudaEvent_t> g_pool;
static double g_ms[K_COUNT], g_work[K_COUNT];
static int64_t g_count[K_COUNT];

void prof_note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
bool &prof_capturing() {
    static thread_local bool capturing = false;
    return capturing;
}
bool prof_on() { return g_on.load(std::memory_order_relaxed); }

static cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

int prof_begin(int kid, cudaStream_t st, double work) {
    std::lock_guard<std::mutex> lk(g_mu);
    Rec r{kid, work, take_event(), take_event()};
    if (!r.a || !r.b) return -1;
    cudaEventRecord(r.a, st);
    g_recs.push_back(r);
    return (int)g_recs.size() - 1;
}

void prof_end(int slot, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (slot >= 0 && slot < (int)g_recs.size()) cudaEventRecord(g_recs[slot].b, st);
}

}  // namespace lla

using namespace lla;

extern "C" {

int64_t lla_kernel_launches(void) { return g_launches.load(); }

void lla_profile_start(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto &r : g_recs) {
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_recs.clear();
    std::memset(g_ms, 0, sizeof(g_ms));
    std::memset(g_work, 0, sizeof(g_work));
    std::memset(g_count, 0, sizeof(g_count));
    g_on.store(true);
}

int lla_profile_stop(void) {
    g_on.store(false);
    std::lock_guard<std::mutex> lk(g_mu);
    int rc = 0;
    for (auto &r : g_recs) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.b) != cudaSuccess ||
            cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
            rc = LLA_ERR_CUDA;
            continue;
        }
        g_ms[r.kid] += ms;
        g_work[r.kid] += r.work;
        g_count[r.kid] += 1;
    }
    return rc;
}

int lla_profile_query(const char *kernel, double *total_ms, int64_t *launches, double *work) {
    for (int k = 0; k < K_COUNT; ++k) {
        if (std::strcmp(kernel, kNames[k]) == 0) {
            if (total_ms) *total_ms = g_ms[k];
            if (launches) *launches = g_count[k];
            if (work) *work = g_work[k];
            return LLA_OK;
        }
    }
    return LLA_ERR_INVALID_ARG;
}

const char *lla_profile_kernel_name(int index) {
    return (index >= 0 && index < K_COUNT) ? kNames[index] : nullptr;
}

}  // extern "C"

// lla_api_internal.h -- per-thread execution context of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/lla_gb300.h"

namespace lla {

// Grow-only device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes);
    ~DevBuf();
};

// Grow-only pinned host buffer.
struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes);
    ~HostBuf();
};

// Workspace of the mixed-precision refined solve.
struct MixedWs {
    DevBuf L, s, rowsum, R, Y, diag0, words;  // FP32 factor, scaling, norms, residual, correction
    DevBuf P;                                 // split-K partial products of the residual
    DevBuf sympart;                           // per-tile partial row sums / maxima of |A|
    DevBuf oz;                                // exact-slice residual: slices of A and X
    DevBuf winv;                              // inverted 64 x 64 diagonal blocks of L
    DevBuf stage;                             // epoch-tagged hand-off words of the substitutions
    void *stage_seen = nullptr;               // stage allocation that was last cleared
    size_t stage_seen_cap = 0;
    unsigned stage_epoch = 0;                 // epoch of the last substitution launch
    DevBuf F, fdiag, S;                       // plain FP64 fallback (S: exact-order verdict scratch)
    DevBuf opA, opB;                          // tensor-core operand planes of one panel
    DevBuf tcerr;                             // tensor-core update status word
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // start, factor done, refinement done
    DevBuf pinv;                              // inverted 32 x 32 diagonal blocks of one panel
    HostBuf words_host;
};

// One per calling host thread: its own stream and buffers, so concurrent
// callers never share scratch memory.
struct Ctx {
    MixedWs mixed;
    int device = 0;
    cudaStream_t stream = nullptr;
    DevBuf small_dev;                 // status words
    HostBuf small_host;
    DevBuf raw_a, raw_b;              // host views as uploaded
    DevBuf work_a, work_b;            // column-major working copies
    DevBuf aux_s, aux_d, aux_diag;    // factor scratch (EXACT S/D, FAST diag0), diag override
    DevBuf aux_x;                     // solution of the refined solve
    DevBuf ws;                        // triangular-solve tickets and flags
    DevBuf dev_s, dev_d, dev_ws;      // scratch of the device-resident entry points
    DevBuf status_dev;                // device-call status word (read by lla_device_status)
    bool status_clear = false;        // status_dev has been zeroed since its allocation
    HostBuf stage_a, stage_b;         // pinned staging for strided views
    DevBuf raw_c, lob_g, lob_p, lob_t;  // Cholesky-QR: third view, Gram copy, partials, transposes
    HostBuf stage_c;
    ~Ctx();
};

Ctx *get_ctx(lla_error *err);

template <typename T>
cudaError_t factor_on_device(Ctx &c, T *W, int64_t n, int64_t ld, bool exact, const T *R,
                             int64_t drs, int64_t dcs, int64_t *fail);
template <typename T>
cudaError_t trsm_on_device(Ctx &c, const T *M, int64_t ld, int64_t n, int lower, int trans,
                           const T *diag, T *B, int64_t ldb, int64_t m, bool exact, int *timed_out);

}  // namespace lla

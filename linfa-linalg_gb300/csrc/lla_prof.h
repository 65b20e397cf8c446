// lla_prof.h -- launch accounting and optional per-kernel CUDA-event timing.
//
// Every launcher wraps each kernel launch in a LaunchScope.  The scope always
// bumps the library's launch counter; while profiling is switched on
// (lla_profile_start) it also records a CUDA event pair on the launching
// stream and the launch's algorithmic work (flops or bytes), so that a
// benchmark can report each kernel's average duration and achieved rate from
// events taken inside its own timed region.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lla {

enum KernelId {
    K_POTRF_EXACT_DIAG = 0,
    K_POTRF_EXACT_PANEL,
    K_POTRF_EXACT_UPDATE,
    K_POTRF_FAST_DIAG,
    K_POTRF_FAST_PANEL,
    K_POTRF_FAST_UPDATE,
    K_TRSM,
    K_LAYOUT,
    K_MIXED_DIAG,
    K_MIXED_PANEL,
    K_MIXED_UPDATE,
    K_MIXED_CONVERT,
    K_RESIDUAL,
    K_REFINE,
    K_MIXED_TRSM,
    K_BATCH,
    K_OZ_SLICE,
    K_MISC,
    K_COUNT
};

const char *kernel_name(int id);

void prof_note_launch();
bool prof_on();
// While a thread captures a CUDA graph its launches are not counted or timed
// (the graph's replays are, where they are launched).
bool &prof_capturing();
// Returns a slot index (or -1 when profiling is off) after recording the start event.
int prof_begin(int kid, cudaStream_t st, double work);
void prof_end(int slot, cudaStream_t st);

struct LaunchScope {
    int slot;
    cudaStream_t st;
    LaunchScope(int kid, cudaStream_t s, double work = 0.0) : st(s) {
        if (prof_capturing()) {
            slot = -1;
            return;
        }
        prof_note_launch();
        slot = prof_on() ? prof_begin(kid, s, work) : -1;
    }
    ~LaunchScope() {
        if (slot >= 0) prof_end(slot, st);
    }
};

}  // namespace lla

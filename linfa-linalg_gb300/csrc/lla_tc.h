// lla_tc.h -- tensor-core (tcgen05) trailing update of the mixed-precision
// Cholesky.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lla {

// Term pairs (a, b): the update subtracts sum_pairs P_a[I] P_b[J]^T.
struct TcPairs {
    int n;
    int pa[6];
    int pb[6];
};

// One-time set-up (dynamic shared memory limit, driver entry point for TMA
// descriptors); 0 on success.
int tc_update_prepare();

// C[q + I*128 + r, q + J*128 + c] -= sum over pairs of planes[a][I*128 + r, :kext] .
// planes[b][J*128 + c, :kext] for the lower tiles I >= J of the rows x rows
// trailing matrix (FP32, column-major, leading dimension ld, global order n),
// or, when narrow, for the tiles of its first tile column only (J = 0).
// planes: `terms` planes of rows x ldp BF16 (or FP16) values, plane_stride
// elements apart, row-major, 16-byte aligned; kext (a multiple of 64, <= ldp)
// columns of each row are the K extent.  Skips all work when *info >= 0;
// bounded waits record LLA_ERR_TIMEOUT in *err_word.  sched: the tile-claim
// counter (zeroed with *sched_base before a series of launches on one stream);
// each launch claims from *sched_base on and advances it by tiles + CTAs.  A
// launch that skips (a failed or timed-out factorisation) leaves the counter
// behind, so the series must be abandoned then, as every later launch skips.
// pdl: launched as a programmatic dependent of the stream's previous kernel,
// whose output it waits for after its set-up.
int tc_update_launch(float *C, int64_t ld, int64_t q, int64_t n, void *planes, int64_t plane_stride,
                     int64_t ldp, int64_t rows, int kext, int terms, bool fp16, const TcPairs &pairs,
                     const int64_t *info, int *err_word, unsigned *sched, unsigned *sched_base, bool narrow,
                     cudaStream_t st, int kchunk = 64, int epilogue = 0, bool pdl = false);

}  // namespace lla

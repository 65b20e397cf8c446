// lla_trsm_sched.h -- ticket order of the FP32 substitutions with inverted
// diagonal blocks (lla_trsm_inv.cu).  Host and device code: the kernel decodes
// its ticket with these functions, the launcher sizes its grid with them, and a
// host test checks their invariants (every item once; every wait on an item
// with a smaller ticket, so CTAs that take tickets in order never deadlock).
#pragma once

#include <stdint.h>

#ifndef __CUDACC__  // host-only compilers: the qualifiers vanish
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif

namespace lla {

// Work items in ticket order.  Group g (g = 0 .. R-1) holds the owners of
// processing position g (one per column chunk), then the helpers of positions
// p = 2g+2 and 2g+3 (those with hmin <= p < R): a helper sums the coupling
// terms q < p/2 of position p, which are all solved once position p/2 - 1 is,
// so every item waits only on items with smaller tickets.
__host__ __device__ __forceinline__ int64_t iv_items_before(int64_t g, int64_t R, int64_t hmin, int nch) {
    const int64_t top = (2 * g + 1 < R - 1 ? 2 * g + 1 : R - 1) - hmin + 1;  // helpers p in [hmin, 2g+1]
    return (int64_t)nch * (g + (top > 0 ? top : 0));
}
__host__ __device__ __forceinline__ void iv_decode(int64_t t, int64_t R, int64_t hmin, int nch, bool &helper,
                                          int64_t &pos, int &chunk) {
    int64_t lo = 0, hi = R - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if (iv_items_before(mid, R, hmin, nch) <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    const int64_t idx = t - iv_items_before(lo, R, hmin, nch);
    if (idx < nch) {
        helper = false;
        pos = lo;
        chunk = (int)idx;
        return;
    }
    helper = true;
    const int64_t j = (idx - nch) / nch;
    chunk = (int)((idx - nch) % nch);
    int64_t p = 2 * lo + 2;
    if (p < hmin) p = hmin;  // only 2g+3 can qualify then
    pos = p + j;
}

// Chain form of the substitutions (trsm_chain_kernel): tickets 0 .. nch-1 are
// the chain CTAs (one per column chunk); then, in processing order p, the
// helpers of position p: ch_groups(p) groups per chunk, group g summing the
// coupling terms of positions [g S, min((g+1) S, p-2)).  A helper waits only on
// blocks the chain solves before position p-2; the chain waits at position p
// only on helpers of position p, whose tickets precede those of every helper
// that could hold a slot while they wait -- so CTAs that take tickets in order
// never deadlock.
__host__ __device__ __forceinline__ int64_t ch_groups(int64_t p, int64_t S) {
    const int64_t T = p - 2;  // coupling terms: positions 0 .. p-3
    return T <= 0 ? 1 : (T + S - 1) / S;
}
// sum of ch_groups(p') over p' < p
__host__ __device__ __forceinline__ int64_t ch_groups_before(int64_t p, int64_t S) {
    const int64_t a = p < 3 ? p : 3;  // positions 0, 1, 2: one group each
    const int64_t K = p - 3;          // positions 3 .. p-1: ceil(k / S), k = 1 .. K
    if (K <= 0) return a;
    const int64_t q = K / S, r = K % S;
    return a + S * q * (q + 1) / 2 + r * (q + 1);
}
__host__ __device__ __forceinline__ int64_t ch_items(int64_t R, int64_t S, int nch) {
    return nch + (int64_t)nch * ch_groups_before(R, S);
}
// Group size keeping at most eight groups per position.
__host__ __device__ __forceinline__ int64_t ch_group_size(int64_t R) {
    const int64_t s = (R - 3 + 7) / 8;
    return s > 32 ? s : 32;
}
__host__ __device__ __forceinline__ void ch_decode(int64_t t, int64_t R, int64_t S, int nch, bool &chain,
                                                   int64_t &pos, int &group, int &chunk) {
    if (t < nch) {
        chain = true;
        pos = 0;
        group = 0;
        chunk = (int)t;
        return;
    }
    chain = false;
    const int64_t idx = t - nch;
    int64_t lo = 0, hi = R - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if ((int64_t)nch * ch_groups_before(mid, S) <= idx)
            lo = mid;
        else
            hi = mid - 1;
    }
    const int64_t within = idx - (int64_t)nch * ch_groups_before(lo, S);
    pos = lo;
    group = (int)(within / nch);
    chunk = (int)(within % nch);
}

}  // namespace lla

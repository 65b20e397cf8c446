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

// Look-back form (trsm_inv_kernel).  The coupling terms of processing
// position p are positions 0 .. p-3 (its two neighbours come last).  The owner
// of (p, chunk) sums the last of them itself, positions [iv_qlo(p), p-2), at
// most kIvOwn; wide helpers sum the rest for 64 columns at once, kIvGroup
// positions each: group g of p covers [g G, min(g G + G, iv_qlo(p))).
// Tickets come in rounds T = 0 .. R-1: the owners of position T (one per
// 16-column chunk), then the wide helpers whose round is T.  Helper (p, g) has
// round max(p - kIvAhead, g G + G): it starts kIvAhead rounds before its owners
// (a helper takes many chain steps), but not before the round after the last
// position it sums.  Its waits (owners of positions < g G + G) and the waits of
// the owners of p on it (round <= p - 3) are all on smaller tickets.
constexpr int64_t kIvGroup = 16, kIvOwn = 48, kIvAhead = 32;
__host__ __device__ __forceinline__ int64_t iv_qlo(int64_t p) { return p - 2 - kIvOwn > 0 ? p - 2 - kIvOwn : 0; }
__host__ __device__ __forceinline__ int64_t iv_ngroups(int64_t p) { return (iv_qlo(p) + kIvGroup - 1) / kIvGroup; }
// sum of iv_ngroups(q) over q < p: sum over u = 1 .. p-3-kIvOwn of ceil(u / kIvGroup)
__host__ __device__ __forceinline__ int64_t iv_groups_before(int64_t p) {
    const int64_t U = p - 3 - kIvOwn;
    if (U <= 0) return 0;
    const int64_t a = U / kIvGroup, b = U % kIvGroup;
    return kIvGroup * a * (a + 1) / 2 + (a + 1) * b;
}
// helpers (p, g) whose round is before T: p < T + kIvAhead and g G + G < T,
// i.e. sum over p < min(T + kIvAhead, R) of min(iv_ngroups(p), gm)
__host__ __device__ __forceinline__ int64_t iv_helpers_before(int64_t T, int64_t R) {
    const int64_t gm = T > 0 ? (T - 1) / kIvGroup : 0;      // groups g with g G + G < T
    const int64_t pend = T + kIvAhead < R ? T + kIvAhead : R;
    const int64_t pstar = kIvGroup * gm + kIvOwn + 3;        // first p with iv_ngroups(p) > gm
    const int64_t pm = pstar < pend ? pstar : pend;
    return iv_groups_before(pm) + gm * (pend > pstar ? pend - pstar : 0);
}
// tickets of the rounds before T; nch column chunks, ngrp column groups of 64
__host__ __device__ __forceinline__ int64_t iv_items_before(int64_t T, int64_t R, int nch, int ngrp) {
    return T * (int64_t)nch + (int64_t)ngrp * iv_helpers_before(T, R);
}
// Ticket t -> (position, helper?, group, column group or chunk); slot: the
// helper's partial-sum slot (ngrp times the groups of the positions before p,
// then g, then the column group).  Round T's helpers: first group T/G - 1 of
// positions p in [T - G + kIvOwn + 3, T + kIvAhead) when G divides T, then
// groups 0 .. T/G - 1 of position T + kIvAhead.
__host__ __device__ __forceinline__ void iv_decode(int64_t t, int64_t R, int nch, int ngrp, bool &helper,
                                                   int64_t &pos, int &group, int &sub, int64_t &slot) {
    int64_t lo = 0, hi = R - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if (iv_items_before(mid, R, nch, ngrp) <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    const int64_t T = lo, idx = t - iv_items_before(T, R, nch, ngrp);
    helper = idx >= nch;
    if (!helper) {
        pos = T;
        group = 0;
        sub = (int)idx;
        slot = -1;
        return;
    }
    const int64_t h = idx - nch, pair = h / ngrp;
    sub = (int)(h % ngrp);
    const int64_t pend = T + kIvAhead < R ? T + kIvAhead : R;
    int64_t nb = 0, pblo = 0;
    if (T >= kIvGroup && T % kIvGroup == 0) {
        pblo = T - kIvGroup + kIvOwn + 3;
        nb = pend > pblo ? pend - pblo : 0;
    }
    if (pair < nb) {
        pos = pblo + pair;
        group = (int)(T / kIvGroup - 1);
    } else {
        pos = T + kIvAhead;
        group = (int)(pair - nb);
    }
    slot = (int64_t)ngrp * (iv_groups_before(pos) + group) + sub;
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

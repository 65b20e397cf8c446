"""Ticket order of the FP32 substitutions (csrc/lla_trsm_sched.h), checked on the
host with the kernel's own header: every work item is decoded exactly once, and
every item waits only on items with smaller tickets (owners on the previous
owners of their column chunk, which includes the two neighbours; owners on the
wide helpers of their position; helpers on the owners of the positions they
sum), so CTAs that take tickets in order can never wait on a CTA that has not
been scheduled; the helper groups and the owner's own range cover every
coupling term once."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "linfa-linalg_gb300", "csrc")

HARNESS = r"""
#include <cstdio>
#include <map>
#include <tuple>
#include <vector>
#include "lla_trsm_sched.h"
using namespace lla;
int main() {
    const int64_t Rs[] = {1, 2, 3, 4, 5, 16, 18, 19, 20, 21, 32, 33, 35, 36, 37, 48, 50, 51, 52, 53, 64, 67, 80, 100, 129, 256, 257, 1024};
    const int nchs[] = {1, 2, 3, 4, 5, 7, 8};
    long long checked = 0;
    for (int64_t R : Rs)
        for (int nch : nchs) {
            const int ngrp = (nch + 3) / 4;  // 64-column groups of the 16-column chunks
            const int64_t total = iv_items_before(R, R, nch, ngrp);
            // key: (helper, position, group, chunk or column group)
            std::map<std::tuple<int, int64_t, int, int>, int64_t> seen;
            std::map<int64_t, int> slots;
            for (int64_t t = 0; t < total; ++t) {
                bool helper; int64_t pos, slot; int g, sub;
                iv_decode(t, R, nch, ngrp, helper, pos, g, sub, slot);
                const bool ok = pos >= 0 && pos < R &&
                                (helper ? (g >= 0 && g < iv_ngroups(pos) && sub >= 0 && sub < ngrp && slot >= 0 &&
                                           slot < (int64_t)ngrp * iv_groups_before(R))
                                        : (sub >= 0 && sub < nch));
                if (!ok) { std::printf("bad item R=%lld nch=%d t=%lld\n", (long long)R, nch, (long long)t); return 1; }
                if (!seen.emplace(std::make_tuple((int)helper, pos, g, sub), t).second) {
                    std::printf("duplicate R=%lld t=%lld\n", (long long)R, (long long)t); return 1;
                }
                if (helper && !slots.emplace(slot, 1).second) { std::printf("slot twice\n"); return 1; }
            }
            if ((int64_t)seen.size() != R * nch + (int64_t)ngrp * iv_groups_before(R)) { std::printf("count\n"); return 1; }
            for (const auto &kv : seen) {
                const int helper = std::get<0>(kv.first);
                const int64_t p = std::get<1>(kv.first);
                const int g = std::get<2>(kv.first), sub = std::get<3>(kv.first);
                const int64_t t = kv.second;
                if (helper) {  // waits on the owners of its positions, for the chunks of its column group
                    const int64_t lo = g * kIvGroup, hi = lo + kIvGroup < iv_qlo(p) ? lo + kIvGroup : iv_qlo(p);
                    if (hi <= lo || hi > p - 2) { std::printf("empty or late group\n"); return 1; }
                    for (int64_t q = lo; q < hi; ++q)
                        for (int c = 4 * sub; c < 4 * sub + 4 && c < nch; ++c)
                            if (seen.at(std::make_tuple(0, q, 0, c)) >= t) { std::printf("helper wait\n"); return 1; }
                } else {  // the previous owner of its chunk, and every helper of its position
                    if (p > 0 && seen.at(std::make_tuple(0, p - 1, 0, sub)) >= t) { std::printf("owner wait\n"); return 1; }
                    for (int gg = 0; gg < iv_ngroups(p); ++gg)
                        if (seen.at(std::make_tuple(1, p, gg, sub / 4)) >= t) { std::printf("helper order\n"); return 1; }
                    // the groups and the owner's own range cover positions 0 .. p-3 exactly once
                    int64_t covered = 0;
                    for (int gg = 0; gg < iv_ngroups(p); ++gg) {
                        const int64_t lo = gg * kIvGroup, hi = lo + kIvGroup < iv_qlo(p) ? lo + kIvGroup : iv_qlo(p);
                        covered += hi - lo;
                    }
                    covered += (p - 2 > iv_qlo(p)) ? p - 2 - iv_qlo(p) : 0;
                    if (covered != (p > 2 ? p - 2 : 0)) { std::printf("cover p=%lld\n", (long long)p); return 1; }
                    if (p - 2 - iv_qlo(p) > kIvOwn) { std::printf("owner range\n"); return 1; }
                }
                ++checked;
            }
        }
    std::printf("ok %lld\n", checked);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_ticket_order_has_no_forward_waits():
    d = tempfile.mkdtemp(prefix="lla_sched_")
    src, exe = os.path.join(d, "sched.cpp"), os.path.join(d, "sched")
    with open(src, "w") as f:
        f.write(HARNESS)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", CSRC, src, "-o", exe], check=True, timeout=120)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr


CHAIN_HARNESS = r"""
#include <cstdio>
#include <set>
#include <tuple>
#include "lla_trsm_sched.h"
using namespace lla;
int main() {
    const int64_t Rs[] = {1, 2, 3, 4, 5, 34, 35, 36, 67, 100, 256, 257, 1024, 4096};
    const int nchs[] = {1, 2, 4, 7};
    long long checked = 0;
    for (int64_t R : Rs)
        for (int nch : nchs) {
            const int64_t S = ch_group_size(R), total = ch_items(R, S, nch);
            if (R > 1 && ch_groups(R - 1, S) > 8) { std::printf("too many groups R=%lld\n", (long long)R); return 1; }
            std::set<std::tuple<int64_t, int, int>> seen;
            int64_t last_pos = -1;
            for (int64_t t = 0; t < total; ++t) {
                bool chain; int64_t pos; int g, c;
                ch_decode(t, R, S, nch, chain, pos, g, c);
                if (chain != (t < nch)) { std::printf("chain tickets R=%lld t=%lld\n", (long long)R, (long long)t); return 1; }
                if (chain) { if (c != t) return 1; continue; }
                if (pos < 0 || pos >= R || c < 0 || c >= nch || g < 0 || g >= ch_groups(pos, S)) {
                    std::printf("bad helper R=%lld t=%lld\n", (long long)R, (long long)t); return 1;
                }
                // helpers by position: a helper's ticket precedes every helper of a later position
                if (pos < last_pos) { std::printf("order R=%lld\n", (long long)R); return 1; }
                last_pos = pos;
                if (!seen.insert(std::make_tuple(pos, g, c)).second) { std::printf("duplicate\n"); return 1; }
                ++checked;
            }
            // every position has its groups, and the groups cover positions 0 .. p-3 once
            for (int64_t p = 0; p < R; ++p) {
                int64_t covered = 0;
                for (int64_t g = 0; g < ch_groups(p, S); ++g) {
                    for (int c = 0; c < nch; ++c)
                        if (!seen.count(std::make_tuple(p, (int)g, c))) { std::printf("missing\n"); return 1; }
                    const int64_t lo = g * S, hi = (lo + S < p - 2) ? lo + S : p - 2;
                    covered += hi > lo ? hi - lo : 0;
                }
                if (covered != (p > 2 ? p - 2 : 0)) { std::printf("cover R=%lld p=%lld\n", (long long)R, (long long)p); return 1; }
            }
        }
    std::printf("ok %lld\n", checked);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_chain_schedule_covers_every_term_once():
    """Chain form: the chains take the first tickets, helpers follow by position
    (so the chain at position p waits only on helpers scheduled before any
    helper of a later position), and the groups of a position cover its
    coupling terms 0 .. p-3 exactly once, in at most eight groups."""
    d = tempfile.mkdtemp(prefix="lla_chain_")
    src, exe = os.path.join(d, "chain.cpp"), os.path.join(d, "chain")
    with open(src, "w") as f:
        f.write(CHAIN_HARNESS)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", CSRC, src, "-o", exe], check=True, timeout=120)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr

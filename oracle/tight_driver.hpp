/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Host restatement of the reference's tight-rectangle proof driver, generic
 * over the criteria implementation (adapter C):
 *   - the per-lambda-box nested grid over r1..r4 with the strategy checks at
 *     each level (reference: tight_rectangle/tight_rectangle.cu:169-262, the
 *     body of kernel_find_critical_intervals_in; a CUDA thread grid there,
 *     sequential loops here);
 *   - the merge of the critical leaves of one lambda box by r1
 *     (tight_rectangle.cu:121-159, sort_by_r1 + merge_adjacent_r1);
 *   - the initial lambda split and the refinement generations
 *     (tight_rectangle.cu:303-320, 458-498), with split counts as parameters.
 *
 * Besides the critical boxes it produces a trace of every grid cell visited:
 * per level and outcome a count, and an order-independent digest
 * sum(mix64(task, level, indices, outcome)) mod 2^64, which pins the per-box
 * verdict of every cell without storing it.  The GPU prover computes the same
 * trace.
 *
 * Adapter C provides: type V (interval), make(lo,hi), lo(v), hi(v),
 * sub(a,b), tighten_lb(v,x), intersect(a,b), empty(v), subinterval(v,i,n),
 * required_weight(la), r1_range(la), r1_strategies, r1_r2_strategies,
 * r1_r2_r3_strategies (lambda level), two_by_two, r1_r2_r3_leaf, gaps, and
 * trapped()/clear_trap() (a leaf with a trap is kept as critical and flagged).
 */
#ifndef CC_ORACLE_TIGHT_DRIVER_HPP
#define CC_ORACLE_TIGHT_DRIVER_HPP

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/circlecover_gb300.h"

namespace cc_oracle {

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

/* cell key: same packing as the GPU prover (cc_trace_key in the CUDA code) */
static inline uint64_t trace_key(uint64_t task, int level, int i1, int i2, int i3, int i4, int outcome) {
    uint64_t packed = ((uint64_t)outcome) | ((uint64_t)i4 << 4) | ((uint64_t)i3 << 15) | ((uint64_t)i2 << 26) |
                      ((uint64_t)i1 << 37) | ((uint64_t)level << 48);
    return mix64(packed ^ mix64(task + 0x9e3779b97f4a7c15ULL));
}

struct Trace {
    uint64_t counts[4][8];
    uint64_t digest;
    uint64_t leaf_evals;
    void clear() { std::memset(this, 0, sizeof(*this)); }
    void add(const Trace& o) {
        for (int l = 0; l < 4; ++l)
            for (int k = 0; k < 8; ++k) counts[l][k] += o.counts[l][k];
        digest += o.digest;
        leaf_evals += o.leaf_evals;
    }
};

template <class C>
struct TightDriver {
    using V = typename C::V;
    struct Box {
        V la;
        V r[4];
    };

    static void note(Trace& t, uint64_t task, int level, int i1, int i2, int i3, int i4, int outcome) {
        t.counts[level][outcome] += 1;
        t.digest += trace_key(task, level, i1, i2, i3, i4, outcome);
    }

    /* tight_rectangle.cu:169-262 for one lambda box; leaves appended unmerged */
    static void grid(const Box& in, const int splits[4], uint64_t task, std::vector<Box>& crit, std::vector<uint32_t>& flags,
                     Trace& t) {
        V weight = C::required_weight(in.la);
        V r1r = C::intersect(C::r1_range(in.la), in.r[0]);
        if (C::empty(r1r)) return;
        for (int i1 = 0; i1 < splits[0]; ++i1) {
            V r1 = C::subinterval(r1r, i1, splits[0]);
            V r2r = C::intersect(C::r2_range(weight, r1), in.r[1]);
            if (C::empty(r2r)) { note(t, task, 0, i1, 0, 0, 0, CC_T_L1_EMPTY); continue; }
            if (C::r1_strategies(in.la, r1, C::hi(r2r))) { note(t, task, 0, i1, 0, 0, 0, CC_T_L1_R1); continue; }
            note(t, task, 0, i1, 0, 0, 0, CC_T_L1_SPLIT);
            for (int i2 = 0; i2 < splits[1]; ++i2) {
                V r2 = C::subinterval(r2r, i2, splits[1]);
                if (C::r1_strategies(in.la, r1, C::hi(r2))) { note(t, task, 1, i1, i2, 0, 0, CC_T_L2_R1); continue; }
                V r3r = C::intersect(C::r3_range(weight, r1, r2), in.r[2]);
                if (C::empty(r3r)) { note(t, task, 1, i1, i2, 0, 0, CC_T_L2_EMPTY); continue; }
                if (C::r1_r2_strategies(in.la, r1, r2, C::hi(r3r))) { note(t, task, 1, i1, i2, 0, 0, CC_T_L2_R12); continue; }
                note(t, task, 1, i1, i2, 0, 0, CC_T_L2_SPLIT);
                for (int i3 = 0; i3 < splits[2]; ++i3) {
                    V r3 = C::subinterval(r3r, i3, splits[2]);
                    if (C::r1_r2_strategies(in.la, r1, r2, C::hi(r3))) { note(t, task, 2, i1, i2, i3, 0, CC_T_L3_R12); continue; }
                    V r4r = C::intersect(C::r4_range(weight, r1, r2, r3), in.r[3]);
                    if (C::empty(r4r)) { note(t, task, 2, i1, i2, i3, 0, CC_T_L3_EMPTY); continue; }
                    if (C::r1_r2_r3_strategies(in.la, r1, r2, r3, C::hi(r4r))) { note(t, task, 2, i1, i2, i3, 0, CC_T_L3_R123); continue; }
                    V R4 = C::sub(C::sub(C::sub(weight, r1), r2), r3);
                    C::tighten_lb(R4, 0.0);
                    if (C::empty(R4)) { note(t, task, 2, i1, i2, i3, 0, CC_T_L3_R4EMPTY); continue; }
                    note(t, task, 2, i1, i2, i3, 0, CC_T_L3_SPLIT);
                    for (int i4 = 0; i4 < splits[3]; ++i4) {
                        V r4 = C::subinterval(r4r, i4, splits[3]);
                        t.leaf_evals += 1;
                        C::clear_trap();
                        if (C::r1_r2_r3_strategies(in.la, r1, r2, r3, C::hi(r4))) { note(t, task, 3, i1, i2, i3, i4, CC_T_L4_R123); continue; }
                        Box v{in.la, {r1, r2, r3, r4}};
                        C::tighten_lb(v.r[2], C::lo(v.r[3]));
                        C::tighten_lb(v.r[1], C::lo(v.r[2]));
                        C::tighten_lb(v.r[0], C::lo(v.r[1]));
                        V R = C::sub(C::sub(C::sub(C::sub(weight, v.r[0]), v.r[1]), v.r[2]), v.r[3]);
                        C::tighten_lb(R, 0.0);
                        if (C::empty(R)) { note(t, task, 3, i1, i2, i3, i4, CC_T_L4_REMPTY); continue; }
                        int outcome = CC_T_L4_CRITICAL;
                        if (C::two_by_two(v, R)) outcome = CC_T_L4_2X2;
                        else if (C::r1_r2_r3_leaf(v, R4)) outcome = CC_T_L4_R123LEAF;
                        else if (C::gaps(v, R)) outcome = CC_T_L4_GAPS;
                        uint32_t trapped = C::trapped();
                        if (trapped) outcome = CC_T_L4_TRAPPED;
                        note(t, task, 3, i1, i2, i3, i4, outcome);
                        if (outcome == CC_T_L4_CRITICAL || outcome == CC_T_L4_TRAPPED) {
                            crit.push_back(v);
                            flags.push_back(trapped);
                        }
                    }
                }
            }
        }
    }

    /* tight_rectangle.cu:121-159 */
    static std::vector<Box> merge_by_r1(std::vector<Box>& v) {
        std::vector<Box> out;
        if (v.empty()) return out;
        std::sort(v.begin(), v.end(), [](const Box& a, const Box& b) {
            return C::lo(a.r[0]) < C::lo(b.r[0]) || (C::lo(a.r[0]) == C::lo(b.r[0]) && C::hi(a.r[0]) < C::hi(b.r[0]));
        });
        out.push_back(v.front());
        for (const Box& b : v) {
            Box& p = out.back();
            bool merge;
            if (C::lo(p.r[0]) <= C::lo(b.r[0])) merge = C::hi(p.r[0]) >= C::lo(b.r[0]);
            else merge = C::hi(b.r[0]) >= C::lo(p.r[0]);
            if (merge) {
                for (int k = 0; k < 4; ++k) C::do_join(p.r[k], b.r[k]);
                continue;
            }
            out.push_back(b);
        }
        return out;
    }

    struct Result {
        std::vector<Box> criticals;        // final generation, in the reference's order
        std::vector<uint64_t> gen_sizes;   // critical count after init and after each generation
        Trace trace;
        uint64_t trapped_leaves = 0;
        int generations_run = 0;
    };

    /* one generation: every (box, lambda piece) is a task; results are appended in task order */
    static void generation(const std::vector<Box>& in, int la_splits, const int splits[4], int threads,
                           std::vector<Box>& out, Trace& trace, uint64_t& trapped, uint64_t lo = 0,
                           uint64_t hi = ~0ULL) {
        size_t ntasks = in.size() * (size_t)la_splits;
        std::vector<std::vector<Box>> per_task(ntasks);
        std::vector<Trace> traces(threads > 0 ? threads : 1);
        std::vector<uint64_t> traps(traces.size(), 0);
        std::atomic<size_t> next{0};
        auto work = [&](int tid) {
            traces[tid].clear();
            std::vector<Box> leaves;
            std::vector<uint32_t> flags;
            for (;;) {
                size_t task = next.fetch_add(1);
                if (task >= ntasks) break;
                if (task < lo || task >= hi) continue;  // another shard's task
                const Box& s = in[task / la_splits];
                int k = (int)(task % la_splits);
                Box sub{C::subinterval(s.la, k, la_splits), {s.r[0], s.r[1], s.r[2], s.r[3]}};
                leaves.clear();
                flags.clear();
                grid(sub, splits, task, leaves, flags, traces[tid]);
                for (uint32_t f : flags) traps[tid] += f ? 1 : 0;
                per_task[task] = merge_by_r1(leaves);
            }
        };
        int nt = (int)traces.size();
        if (nt == 1) {
            work(0);
        } else {
            std::vector<std::thread> pool;
            for (int i = 0; i < nt; ++i) pool.emplace_back(work, i);
            for (auto& th : pool) th.join();
        }
        for (auto& tr : traces) trace.add(tr);
        for (auto x : traps) trapped += x;
        for (auto& v : per_task) out.insert(out.end(), v.begin(), v.end());
    }

    /* tight_rectangle.cu:458-498 */
    static Result prove(const Box& root, const cc_tight_grid& g, int threads) {
        Result res;
        res.trace.clear();
        std::vector<Box> cur, next;
        std::vector<Box> roots{root};
        generation(roots, g.la_splits_init, g.r_splits_init, threads, next, res.trace, res.trapped_leaves);
        cur.swap(next);
        res.gen_sizes.push_back(cur.size());
        for (int gen = 1; gen <= g.num_generations; ++gen) {
            if (cur.empty()) break;
            next.clear();
            generation(cur, g.la_splits_gen[gen - 1], g.r_splits_gen, threads, next, res.trace, res.trapped_leaves);
            cur.swap(next);
            res.gen_sizes.push_back(cur.size());
            res.generations_run = gen;
        }
        res.criticals = cur;
        return res;
    }
};

}  // namespace cc_oracle

#endif

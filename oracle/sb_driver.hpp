/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Host restatement of the reference's size-bound proof driver, generic over
 * the criteria implementation (adapter C):
 *   - the (lambda, r1, r2) host loops of find_critical_intervals_in, with the
 *     running r1 tightening and Variables::from_la_r1_r2
 *     (rectangle_size_bound/rectangle_size_bound.cu:276-310);
 *   - the body of kernel_find_critical_intervals_in for one task: the
 *     whole-task shortcuts, the r3 loop with its shortcuts, the r4 x r5 x r6
 *     leaves and the cascade (:161-236; a CUDA thread grid there, sequential
 *     loops here);
 *   - merge_critical_intervals<N> (:103-130) and the generation loop
 *     (:312-370), with split counts as parameters.
 *
 * Trace: per level and outcome a count, and an order-independent digest
 * sum(mix(key)) over every task, r3 cell and leaf visited, as the GPU prover
 * computes it (keys: sb_trace_key).
 *
 * Adapter C provides: Box (la, r[6] of its interval type) with lo/hi access
 * through C::lo/C::hi and C::rad(box, i) for radius i, task_box, task_outcome, r3_piece, cell_outcome,
 * leaf_box, leaf_outcome, do_join.
 */
#ifndef CC_ORACLE_SB_DRIVER_HPP
#define CC_ORACLE_SB_DRIVER_HPP

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/circlecover_gb300.h"

namespace cc_oracle {

static inline uint64_t sb_mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

static inline uint64_t sb_trace_key(int gen, uint64_t task, int level, int i3, int i4, int i5, int i6, int outcome) {
    uint64_t packed = (uint64_t)outcome | ((uint64_t)i6 << 5) | ((uint64_t)i5 << 16) | ((uint64_t)i4 << 27) |
                      ((uint64_t)i3 << 38) | ((uint64_t)level << 49) | ((uint64_t)gen << 51);
    return sb_mix64(packed ^ sb_mix64(task + 0x9e3779b97f4a7c15ULL));
}

struct SbTrace {
    uint64_t task_counts[4];
    uint64_t cell_counts[4];
    uint64_t leaf_counts[CC_SBT_LEAF_OUTCOMES];
    uint64_t digest;
    uint64_t leaf_evals;
    uint64_t trapped_shortcuts;
    void clear() { std::memset(this, 0, sizeof(*this)); }
    void add(const SbTrace& o) {
        for (int k = 0; k < 4; ++k) task_counts[k] += o.task_counts[k], cell_counts[k] += o.cell_counts[k];
        for (int k = 0; k < CC_SBT_LEAF_OUTCOMES; ++k) leaf_counts[k] += o.leaf_counts[k];
        digest += o.digest;
        leaf_evals += o.leaf_evals;
        trapped_shortcuts += o.trapped_shortcuts;
    }
};

template <class C>
struct SbDriver {
    using Box = typename C::Box;
    struct Leaf {
        Box box;
        uint32_t trapped;
    };

    /* kernel_find_critical_intervals_in for one task (rectangle_size_bound.cu:161-236) */
    static void run_task(const Box& parent, int gen, uint64_t task, int la_i, int nla, int r1_i, int n1, int r2_i,
                         int n2, const int* rn, std::vector<Leaf>& crit, SbTrace& t) {
        Box tb = C::task_box(parent, la_i, nla, r1_i, n1, r2_i, n2);
        bool trapped = false;
        int to = C::task_outcome(tb, trapped);
        if (trapped) t.trapped_shortcuts += 1;
        t.task_counts[to] += 1;
        t.digest += sb_trace_key(gen, task, 0, 0, 0, 0, 0, to);
        if (to != CC_SBT_TASK_SPLIT) return;
        for (int i3 = 0; i3 < rn[2]; ++i3) {
            auto r3 = C::r3_piece(tb, i3, rn[2]);
            int co = C::cell_outcome(tb, r3, trapped);
            if (trapped) t.trapped_shortcuts += 1;
            t.cell_counts[co] += 1;
            t.digest += sb_trace_key(gen, task, 1, i3, 0, 0, 0, co);
            if (co != CC_SBT_CELL_SPLIT) continue;
            for (int i4 = 0; i4 < rn[3]; ++i4)
                for (int i5 = 0; i5 < rn[4]; ++i5)
                    for (int i6 = 0; i6 < rn[5]; ++i6) {
                        Box b = C::leaf_box(tb, r3, i4, rn[3], i5, rn[4], i6, rn[5]);
                        int lo = C::leaf_outcome(b);
                        t.leaf_evals += 1;
                        t.leaf_counts[lo] += 1;
                        t.digest += sb_trace_key(gen, task, 2, i3, i4, i5, i6, lo);
                        if (lo == CC_SBT_LEAF_CRITICAL || lo == CC_SBT_LEAF_TRAPPED)
                            crit.push_back(Leaf{b, lo == CC_SBT_LEAF_TRAPPED ? 1u : 0u});
                    }
        }
    }

    /* Variables::operator< (variables.hpp:82-94) with Interval_compare */
    static bool iv_less(double al, double ah, double bl, double bh) { return al < bl || (al == bl && ah < bh); }
    static bool less(const Box& a, const Box& b) {
        if (iv_less(C::lo(a.la), C::hi(a.la), C::lo(b.la), C::hi(b.la))) return true;
        if (iv_less(C::lo(b.la), C::hi(b.la), C::lo(a.la), C::hi(a.la))) return false;
        for (int i = 0; i < 6; ++i) {
            if (iv_less(C::lo(C::rad(a, i)), C::hi(C::rad(a, i)), C::lo(C::rad(b, i)), C::hi(C::rad(b, i)))) return true;
            if (iv_less(C::lo(C::rad(b, i)), C::hi(C::rad(b, i)), C::lo(C::rad(a, i)), C::hi(C::rad(a, i)))) return false;
        }
        return false;
    }

    /* merge_critical_intervals<N> (rectangle_size_bound.cu:103-130): sort,
     * then join radii N..5 of consecutive boxes with equal lambda and equal
     * radii 0..N-1 (N = 0: equal lambda only).  Flags are OR-ed. */
    static std::vector<Leaf> merge(std::vector<Leaf>& v, int n_merged) {
        std::vector<Leaf> out;
        if (v.empty()) return out;
        std::sort(v.begin(), v.end(), [](const Leaf& a, const Leaf& b) { return less(a.box, b.box); });
        out.push_back(v.front());
        for (const Leaf& x : v) {
            Leaf& p = out.back();
            bool same = C::lo(x.box.la) == C::lo(p.box.la) && C::hi(x.box.la) == C::hi(p.box.la);
            for (int i = 0; same && i < n_merged; ++i)
                same = C::lo(C::rad(x.box, i)) == C::lo(C::rad(p.box, i)) && C::hi(C::rad(x.box, i)) == C::hi(C::rad(p.box, i));
            if (same) {
                for (int i = n_merged; i < 6; ++i) C::do_join(C::rad(p.box, i), C::rad(x.box, i));
                p.trapped |= x.trapped;
            } else {
                out.push_back(x);
            }
        }
        return out;
    }

    struct Result {
        std::vector<Leaf> criticals;
        std::vector<uint64_t> gen_sizes;
        SbTrace trace;
        uint64_t trapped_leaves = 0;
        int generations_run = 0;
    };

    /* find_critical_intervals_in over every parent (rectangle_size_bound.cu:276-310, 344-350) */
    /* (restricted to the tasks [lo, hi), in the order of the reference's
     * host loops: parent, lambda piece, r1 piece, r2 piece) */
    static void generation(const std::vector<Box>& parents, int gen, int nla, const int* rn, int threads,
                           std::vector<Leaf>& out, SbTrace& trace, uint64_t lo = 0, uint64_t hi = ~0ULL) {
        const uint64_t per_parent = (uint64_t)nla * rn[0] * rn[1];
        const uint64_t ntasks_all = parents.size() * per_parent;
        const uint64_t ntasks = hi < ntasks_all ? hi : ntasks_all;
        int nt = threads > 0 ? threads : 1;
        std::vector<SbTrace> traces(nt);
        std::vector<std::vector<Leaf>> found(nt);
        std::atomic<uint64_t> next{lo};
        auto work = [&](int tid) {
            traces[tid].clear();
            for (;;) {
                uint64_t task = next.fetch_add(1);
                if (task >= ntasks) break;
                uint64_t p = task / per_parent, rem = task % per_parent;
                int r2_i = (int)(rem % rn[1]);
                int r1_i = (int)((rem / rn[1]) % rn[0]);
                int la_i = (int)(rem / ((uint64_t)rn[1] * rn[0]));
                run_task(parents[p], gen, task, la_i, nla, r1_i, rn[0], r2_i, rn[1], rn, found[tid], traces[tid]);
            }
        };
        if (nt == 1) {
            work(0);
        } else {
            std::vector<std::thread> pool;
            for (int i = 0; i < nt; ++i) pool.emplace_back(work, i);
            for (auto& th : pool) th.join();
        }
        for (int i = 0; i < nt; ++i) {
            trace.add(traces[i]);
            out.insert(out.end(), found[i].begin(), found[i].end());
        }
    }

    /* merge width of generation gen (rectangle_size_bound.cu:351-362) */
    static int merge_width(int gen) { return gen == 0 ? 0 : (gen % 3 == 0 ? 3 : (gen % 3 == 1 ? 2 : 1)); }

    /* one generation over the tasks [lo, hi), merged as generation gen */
    static Result generation_range(const std::vector<Box>& parents, int gen, int nla, const int* rn, int threads,
                                   uint64_t lo, uint64_t hi) {
        Result res;
        res.trace.clear();
        std::vector<Leaf> found;
        generation(parents, gen, nla, rn, threads, found, res.trace, lo, hi);
        for (const Leaf& l : found) res.trapped_leaves += l.trapped;
        res.criticals = merge(found, merge_width(gen));
        res.gen_sizes.push_back(res.criticals.size());
        return res;
    }

    /* find_critical_intervals (rectangle_size_bound.cu:312-370) */
    static Result prove(const Box& root, const cc_sb_grid& g, int threads) {
        Result res;
        res.trace.clear();
        std::vector<Leaf> found;
        std::vector<Box> parents{root};
        generation(parents, 0, g.la_splits_init, g.r_splits_init, threads, found, res.trace);
        for (const Leaf& l : found) res.trapped_leaves += l.trapped;
        std::vector<Leaf> cur = merge(found, 0);
        res.gen_sizes.push_back(cur.size());
        for (int gen = 1; gen <= g.num_generations && !cur.empty(); ++gen) {
            parents.clear();
            for (const Leaf& l : cur) parents.push_back(l.box);
            found.clear();
            generation(parents, gen, g.la_splits_gen, g.r_splits_gen, threads, found, res.trace);
            for (const Leaf& l : found) res.trapped_leaves += l.trapped;
            int n_merged = gen % 3 == 0 ? 3 : (gen % 3 == 1 ? 2 : 1);
            cur = merge(found, n_merged);
            res.gen_sizes.push_back(cur.size());
            res.generations_run = gen;
        }
        res.criticals = cur;
        return res;
    }
};

}  // namespace cc_oracle

#endif

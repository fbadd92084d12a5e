/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The CPU port: the prover's own criteria headers (circlecover_gb300/csrc)
 * compiled for the host with the exact directed-rounding layer of
 * oracle/shim/cc_rounding.h.  It restates the reference algorithm
 * (every function cites the reference file:line it follows) and is pinned
 * bit for bit to the reference's own code (oracle/_ref, built from the
 * reference sources) by the CPU test suite.  Where the reference sources are
 * absent (the GPU machine) it is the CPU checker and the timed CPU baseline.
 */
#include "../shim/cc_rounding.h"

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

CC_HOST_TLS unsigned long long cc_port_op_count = 0;
#ifdef CC_PORT_COUNT
#define CC_PORT_TICK() (++cc_port_op_count)
#else
#define CC_PORT_TICK() ((void)0)
#endif

#define CC_HOST_PORT 1
#include "../../circlecover_gb300/csrc/cc_tight.cuh"
#include "../../circlecover_gb300/csrc/cc_sb_proof.cuh"
#include "../../circlecover_gb300/csrc/cc_tight_summary.cuh"

namespace cc {
CC_HOST_TLS uint32_t cc_port_trap_word = 0;
}

#include "../tight_driver.hpp"
#include "../sb_driver.hpp"

using cc::Iv;
namespace ct = cc::tight;

struct PortCriteria {
    using V = Iv;
    static V make(double l, double u) { return Iv{l, u}; }
    static double lo(const V& v) { return v.lo; }
    static double hi(const V& v) { return v.hi; }
    static V sub(const V& a, const V& b) { return a - b; }
    static void tighten_lb(V& v, double x) { cc::tighten_lb(v, x); }
    static void do_join(V& a, const V& b) { cc::do_join(a, b); }
    static V intersect(const V& a, const V& b) { return cc::intersect(a, b); }
    static bool empty(const V& v) { return cc::empty(v); }
    static V subinterval(const V& v, int i, int n) { return cc::subinterval(v, i, n); }
    static V required_weight(const V& la) { return ct::required_weight_for(la); }
    static V r1_range(const V& la) { return ct::r1_range(la); }
    static V r2_range(const V& w, const V& r1) { return ct::r2_range(w, r1); }
    static V r3_range(const V& w, const V& r1, const V& r2) { return ct::r3_range(w, r1, r2); }
    static V r4_range(const V& w, const V& r1, const V& r2, const V& r3) { return ct::r4_range(w, r1, r2, r3); }
    static bool r1_strategies(const V& la, const V& r1, double ub) { return ct::r1_strategies(la, r1, ub); }
    static bool r1_r2_strategies(const V& la, const V& r1, const V& r2, double ub) { return ct::r1_r2_strategies(la, r1, r2, ub); }
    static bool r1_r2_r3_strategies(const V& la, const V& r1, const V& r2, const V& r3, double ub) {
        return ct::r1_r2_r3_strategies(la, r1, r2, r3, ub);
    }
    template <class B>
    static ct::Box box(const B& b) {
        return ct::Box{b.la, {b.r[0], b.r[1], b.r[2], b.r[3]}};
    }
    template <class B>
    static bool two_by_two(const B& b, const V& R) { return ct::two_by_two_strategies(box(b), R); }
    template <class B>
    static bool r1_r2_r3_leaf(const B& b, const V& R4) { return ct::r1_r2_r3_strategies(box(b), R4); }
    template <class B>
    static bool gaps(const B& b, const V& R) { return ct::r1_r2_large_r3_r4_gaps_strategy(box(b), R); }
    static uint32_t trapped() { return cc::trap_status(); }
    static void clear_trap() { cc::trap_clear(); }
};

using Driver = cc_oracle::TightDriver<PortCriteria>;

namespace csb = cc::sb;

struct PortSbC {
    using Box = csb::Box6;
    static double lo(const Iv& v) { return v.lo; }
    static double hi(const Iv& v) { return v.hi; }
    static void do_join(Iv& a, const Iv& b) { cc::do_join(a, b); }
    static Iv& rad(Box& b, int i) { return b.r[i]; }
    static const Iv& rad(const Box& b, int i) { return b.r[i]; }
    static Box task_box(const Box& p, int la_i, int nla, int r1_i, int n1, int r2_i, int n2) {
        return csb::task_box(p, la_i, nla, r1_i, n1, r2_i, n2);
    }
    static int task_outcome(const Box& t, bool& trapped) { return csb::task_outcome(t, trapped); }
    static Iv r3_piece(const Box& t, int i, int n) { return cc::subinterval(t.r[2], i, n); }
    static int cell_outcome(const Box& t, Iv r3, bool& trapped) { return csb::cell_outcome(t, r3, trapped); }
    static Box leaf_box(const Box& t, Iv r3, int i4, int n4, int i5, int n5, int i6, int n6) {
        return csb::leaf_box(t, r3, i4, n4, i5, n5, i6, n6);
    }
    static int leaf_outcome(const Box& b) { return csb::leaf_outcome(b); }
};

using SbDriver = cc_oracle::SbDriver<PortSbC>;

static Iv to_iv(const cc_iv& x) { return Iv{x.lb, x.ub}; }

static uint32_t eval_one(const cc_tight_box& in) {
    ct::Box b{to_iv(in.la), {to_iv(in.r[0]), to_iv(in.r[1]), to_iv(in.r[2]), to_iv(in.r[3])}};
    return ct::eval_all(b);
}

extern "C" {

int ccport_tight_eval(const cc_tight_box* boxes, size_t n, uint32_t* masks, uint64_t* ops, int threads) {
    auto body = [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            unsigned long long before = cc_port_op_count;
            masks[i] = eval_one(boxes[i]);
            if (ops) ops[i] = cc_port_op_count - before;
        }
    };
    if (threads <= 1 || n < 1024) {
        body(0, n);
        return 0;
    }
    std::vector<std::thread> pool;
    size_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        size_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back(body, b, e);
    }
    for (auto& th : pool) th.join();
    return 0;
}

/* Operation counts of the three evaluation passes (main, strip-width
 * bisection, gap-width bisection) per box: ops3[3*i + k].  Meaningful in the
 * counting build only.  Used to attribute the algorithmic work of a box to
 * the GPU kernel that executes each pass. */
int ccport_tight_eval_passes(const cc_tight_box* boxes, size_t n, uint64_t* ops3) {
    for (size_t i = 0; i < n; ++i) {
        const cc_tight_box& in = boxes[i];
        ct::Box b{to_iv(in.la), {to_iv(in.r[0]), to_iv(in.r[1]), to_iv(in.r[2]), to_iv(in.r[3])}};
        bool need_cover, need_gaps;
        ct::CoverJob cj;
        ct::GapsJob gj;
        unsigned long long c0 = cc_port_op_count;
        ct::eval_main(b, need_cover, cj, need_gaps, gj);
        unsigned long long c1 = cc_port_op_count;
        if (need_cover) ct::cover_pass(cj);
        unsigned long long c2 = cc_port_op_count;
        if (need_gaps) ct::gaps_pass(gj);
        unsigned long long c3 = cc_port_op_count;
        ops3[3 * i] = c1 - c0;
        ops3[3 * i + 1] = c2 - c1;
        ops3[3 * i + 2] = c3 - c2;
    }
    return 0;
}

/* Operation counts of each tight criterion evaluated on its own at the leaf
 * arguments (CC_TV_* order; counting build only): ops7[7*i + k], k = 6 the
 * R4/R emptiness test.  For the cost side of strategy ordering. */
int ccport_tight_criterion_ops(const cc_tight_box* boxes, size_t n, uint64_t* ops7) {
    for (size_t i = 0; i < n; ++i) {
        const cc_tight_box& in = boxes[i];
        const Iv la = to_iv(in.la), r1 = to_iv(in.r[0]), r2 = to_iv(in.r[1]), r3 = to_iv(in.r[2]), r4 = to_iv(in.r[3]);
        unsigned long long c = cc_port_op_count;
        const Iv weight = ct::required_weight_for(la);
        auto tick = [&](int k) {
            ops7[7 * i + k] = cc_port_op_count - c;
            c = cc_port_op_count;
        };
        c = cc_port_op_count;
        ct::r1_strategies(la, weight, r1, r2.hi);
        tick(0);
        ct::r1_r2_strategies(la, weight, r1, r2, r3.hi);
        tick(1);
        ct::r1_r2_r3_strategies(la, weight, r1, r2, r3, r4.hi);
        tick(2);
        Iv R4 = weight - r1 - r2 - r3;
        cc::tighten_lb(R4, 0.0);
        ct::Box v{la, {r1, r2, r3, r4}};
        cc::tighten_lb(v.r[2], v.r[3].lo);
        cc::tighten_lb(v.r[1], v.r[2].lo);
        cc::tighten_lb(v.r[0], v.r[1].lo);
        Iv R = weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
        cc::tighten_lb(R, 0.0);
        tick(6);
        ct::two_by_two_strategies(v, R);
        tick(3);
        ct::r1_r2_r3_strategies(v, R4);
        tick(4);
        ct::r1_r2_large_r3_r4_gaps_strategy(v, R);
        tick(5);
    }
    return 0;
}

int ccport_tight_prove(const cc_tight_box* root, const cc_tight_grid* grid, int threads, cc_tight_box** out, size_t* n_out,
                       cc_prove_stats* stats) {
    Driver::Box r{to_iv(root->la), {to_iv(root->r[0]), to_iv(root->r[1]), to_iv(root->r[2]), to_iv(root->r[3])}};
    Driver::Result res = Driver::prove(r, *grid, threads);
    *n_out = res.criticals.size();
    *out = (cc_tight_box*)std::malloc(sizeof(cc_tight_box) * (res.criticals.size() + 1));
    for (size_t i = 0; i < res.criticals.size(); ++i) {
        (*out)[i].la = cc_iv{res.criticals[i].la.lo, res.criticals[i].la.hi};
        for (int k = 0; k < 4; ++k) (*out)[i].r[k] = cc_iv{res.criticals[i].r[k].lo, res.criticals[i].r[k].hi};
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::memcpy(stats->counts, res.trace.counts, sizeof(stats->counts));
        stats->digest = res.trace.digest;
        stats->leaf_evals = res.trace.leaf_evals;
        stats->trapped_leaves = res.trapped_leaves;
        for (size_t g = 0; g < res.gen_sizes.size() && g <= CC_MAX_GENERATIONS; ++g) stats->gen_sizes[g] = res.gen_sizes[g];
        stats->generations_run = res.generations_run;
    }
    return 0;
}

/* one generation restricted to the tasks [lo, hi) (sharding tests) */
int ccport_tight_generation(const cc_tight_box* parents, size_t n, int la_splits, const int* splits, uint64_t lo,
                            uint64_t hi, int threads, cc_tight_box** out, size_t* n_out, cc_prove_stats* stats) {
    std::vector<Driver::Box> in(n);
    for (size_t i = 0; i < n; ++i)
        in[i] = Driver::Box{to_iv(parents[i].la), {to_iv(parents[i].r[0]), to_iv(parents[i].r[1]), to_iv(parents[i].r[2]),
                                                   to_iv(parents[i].r[3])}};
    std::vector<Driver::Box> res;
    cc_oracle::Trace tr;
    tr.clear();
    uint64_t trapped = 0;
    Driver::generation(in, la_splits, splits, threads, res, tr, trapped, lo, hi);
    *n_out = res.size();
    *out = (cc_tight_box*)std::malloc(sizeof(cc_tight_box) * (res.size() + 1));
    for (size_t i = 0; i < res.size(); ++i) {
        (*out)[i].la = cc_iv{res[i].la.lo, res[i].la.hi};
        for (int k = 0; k < 4; ++k) (*out)[i].r[k] = cc_iv{res[i].r[k].lo, res[i].r[k].hi};
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::memcpy(stats->counts, tr.counts, sizeof(stats->counts));
        stats->digest = tr.digest;
        stats->leaf_evals = tr.leaf_evals;
        stats->trapped_leaves = trapped;
        stats->gen_sizes[0] = res.size();
    }
    return 0;
}

/* Max_distances through the prover's own per-box items and in-order fold */
void ccport_tight_summary(const cc_tight_box* crit, size_t n, cc_tight_summary_t* out) {
    std::vector<cc::summary::Item> items(n);
    std::vector<ct::Box> boxes(n);
    for (size_t i = 0; i < n; ++i) {
        boxes[i] = ct::Box{to_iv(crit[i].la), {to_iv(crit[i].r[0]), to_iv(crit[i].r[1]), to_iv(crit[i].r[2]),
                                                to_iv(crit[i].r[3])}};
        cc::trap_clear();
        items[i] = cc::summary::summary_item(boxes[i]);
    }
    cc::summary::summary_fold(items.data(), boxes.data(), n, out);
}

void ccport_free(void* p) { std::free(p); }

int ccport_sb_eval(const cc_sb_box* boxes, size_t n, uint32_t* masks, uint64_t* ops, int threads) {
    auto body = [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            unsigned long long before = cc_port_op_count;
            cc::sb::Box6 x;
            x.la = to_iv(boxes[i].la);
            for (int k = 0; k < 6; ++k) x.r[k] = to_iv(boxes[i].r[k]);
            masks[i] = cc::sb::sb_eval_all(x);
            if (ops) ops[i] = cc_port_op_count - before;
        }
    };
    if (threads <= 1 || n < 64) {
        body(0, n);
        return 0;
    }
    std::vector<std::thread> pool;
    size_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        size_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back(body, b, e);
    }
    for (auto& th : pool) th.join();
    return 0;
}

static void port_sb_out(const SbDriver::Result& res, cc_sb_box** out, uint32_t** flags, size_t* n_out,
                        cc_sb_prove_stats* stats);

int ccport_sb_generation(const cc_sb_box* parents, size_t n, int gen, int la_splits, const int* r_splits, uint64_t lo,
                         uint64_t hi, int threads, cc_sb_box** out, uint32_t** flags, size_t* n_out,
                         cc_sb_prove_stats* stats) {
    std::vector<csb::Box6> ps(n);
    for (size_t i = 0; i < n; ++i) {
        ps[i].la = to_iv(parents[i].la);
        for (int k = 0; k < 6; ++k) ps[i].r[k] = to_iv(parents[i].r[k]);
    }
    port_sb_out(SbDriver::generation_range(ps, gen, la_splits, r_splits, threads, lo, hi), out, flags, n_out, stats);
    return 0;
}

int ccport_sb_prove(const cc_sb_box* root, const cc_sb_grid* grid, int threads, cc_sb_box** out, uint32_t** flags,
                    size_t* n_out, cc_sb_prove_stats* stats) {
    csb::Box6 r;
    r.la = to_iv(root->la);
    for (int i = 0; i < 6; ++i) r.r[i] = to_iv(root->r[i]);
    port_sb_out(SbDriver::prove(r, *grid, threads), out, flags, n_out, stats);
    return 0;
}

static void port_sb_out(const SbDriver::Result& res, cc_sb_box** out, uint32_t** flags, size_t* n_out,
                        cc_sb_prove_stats* stats) {
    size_t n = res.criticals.size();
    *n_out = n;
    *out = (cc_sb_box*)std::malloc(sizeof(cc_sb_box) * (n + 1));
    *flags = (uint32_t*)std::malloc(sizeof(uint32_t) * (n + 1));
    for (size_t i = 0; i < n; ++i) {
        const csb::Box6& b = res.criticals[i].box;
        (*out)[i].la = cc_iv{b.la.lo, b.la.hi};
        for (int k = 0; k < 6; ++k) (*out)[i].r[k] = cc_iv{b.r[k].lo, b.r[k].hi};
        (*flags)[i] = res.criticals[i].trapped;
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::memcpy(stats->task_counts, res.trace.task_counts, sizeof(stats->task_counts));
        std::memcpy(stats->cell_counts, res.trace.cell_counts, sizeof(stats->cell_counts));
        std::memcpy(stats->leaf_counts, res.trace.leaf_counts, sizeof(stats->leaf_counts));
        stats->digest = res.trace.digest;
        stats->leaf_evals = res.trace.leaf_evals;
        stats->trapped_leaves = res.trapped_leaves;
        stats->trapped_shortcuts = res.trace.trapped_shortcuts;
        for (size_t g = 0; g < res.gen_sizes.size() && g <= CC_MAX_GENERATIONS; ++g) stats->gen_sizes[g] = res.gen_sizes[g];
        stats->generations_run = res.generations_run;
    }
}

/* interval times scalar, for the rounding test */
void ccport_iv_mul_scalar(double lo, double hi, double s, double* out) {
    Iv r = Iv{lo, hi} * s;
    out[0] = r.lo;
    out[1] = r.hi;
}

/* one task box of the size-bound driver */
void ccport_sb_task_box(const cc_sb_box* parent, int la_i, int nla, int r1_i, int n1, int r2_i, int n2, cc_sb_box* out) {
    csb::Box6 p;
    p.la = to_iv(parent->la);
    for (int i = 0; i < 6; ++i) p.r[i] = to_iv(parent->r[i]);
    csb::Box6 t = csb::task_box(p, la_i, nla, r1_i, n1, r2_i, n2);
    out->la = cc_iv{t.la.lo, t.la.hi};
    for (int i = 0; i < 6; ++i) out->r[i] = cc_iv{t.r[i].lo, t.r[i].hi};
}

/* the size-bound proof constants from their formulas, for the constant check */
void ccport_sb_constants(double* out) {
    cc::sb::ValsConstants c = cc::sb::vals_constants_formula();
    out[0] = c.weight_bound_wall_building;
    out[1] = c.width_fraction_incomplete;
    out[2] = c.lb_w_infty_denom;
    out[3] = c.phase_factor.lo;
    out[4] = c.phase_factor.hi;
    out[5] = cc::tight::break_even_lo_formula();
    out[6] = cc::tight::break_even_hi_formula();
}

/* Prepared (hoisted) criteria vs the plain ones: for every box and n_ub upper
 * bounds spread over (and just outside) the next radius' interval, compare
 * r1_check / r12_check / r123_check with r1_strategies / r1_r2_strategies /
 * r1_r2_r3_strategies.  Returns the number of disagreements. */
size_t ccport_prepared_mismatches(const cc_tight_box* boxes, size_t n, int n_ub) {
    size_t bad = 0;
    for (size_t i = 0; i < n; ++i) {
        const cc_tight_box& b = boxes[i];
        Iv la = to_iv(b.la), r1 = to_iv(b.r[0]), r2 = to_iv(b.r[1]), r3 = to_iv(b.r[2]), r4 = to_iv(b.r[3]);
        Iv w = ct::required_weight_for(la);
        ct::R1Prep p1 = ct::r1_prepare(la, w, r1);
        ct::R12Prep p2 = ct::r12_prepare(la, w, r1, r2);
        ct::R123Prep p3 = ct::r123_prepare(la, w, r1, r2, r3);
        const Iv next[3] = {r2, r3, r4};
        for (int k = 0; k < 3; ++k) {
            for (int j = 0; j < n_ub; ++j) {
                double t = n_ub > 1 ? (double)j / (n_ub - 1) : 1.0;
                double ub = next[k].lo + (next[k].hi - next[k].lo) * (1.25 * t - 0.125);
                if (!(ub >= 0)) ub = next[k].hi;
                bool a, c;
                if (k == 0) {
                    a = ct::r1_check(p1, ub);
                    c = ct::r1_strategies(la, w, r1, ub);
                } else if (k == 1) {
                    a = ct::r12_check(p2, ub);
                    c = ct::r1_r2_strategies(la, w, r1, r2, ub);
                } else {
                    a = ct::r123_check(p3, ub);
                    c = ct::r1_r2_r3_strategies(la, w, r1, r2, r3, ub);
                }
                bad += a != c;
            }
        }
    }
    return bad;
}

/* The strip-width bisection stopped after k steps and resumed from its
 * bracket and step count (cover_strip_width_resume, as the evaluation's
 * second strip-width kernel does) vs the bisection run in one go, for every
 * box whose strip enters and k = 0, 1, 2, 5, 20, 40.  Returns the number of
 * disagreements (result bits or trap status). */
size_t ccport_resume_mismatches(const cc_tight_box* boxes, size_t n) {
    size_t bad = 0;
    static const int ks[] = {0, 1, 2, 5, 20, 40};
    for (size_t i = 0; i < n; ++i) {
        const cc_tight_box& b = boxes[i];
        const double la_hi = b.la.ub, r1 = b.r[0].lb, r2 = b.r[1].lb, r3 = b.r[2].lb;
        if (!ct::cover_strip_enters(r1, r2, r3)) continue;
        cc::trap_clear();
        const double whole = ct::cover_strip_width_fp64(la_hi, r1, r2, r3);
        const uint32_t tw = cc::trap_status();
        for (int k : ks) {
            double lo = 0.3, hi = la_hi;
            int it = 0;
            for (; it < k; ++it) {  // the first k steps of the same loop
                const double mid = 0.5 * (lo + hi);
                if (mid <= lo || mid >= hi) break;
                if (ct::strip_width_realizable(r1, r2, r3, mid)) lo = mid;
                else hi = mid;
            }
            cc::trap_clear();
            const double res = ct::cover_strip_width_resume(r1, r2, r3, lo, hi, it);
            const uint32_t tr = cc::trap_status();
            cc::trap_clear();
            bad += (std::memcmp(&res, &whole, sizeof(double)) != 0) || tr != tw;
        }
    }
    return bad;
}

/* The proof's prepared leaf form vs the leaf form itself: for every box (as
 * an r3 cell: r1..r3 tightened against each other, R4 = weight - r1 - r2 -
 * r3 tightened at 0) and n_ub upper bounds of r4 spread over [0, r3.lo] and
 * just outside, compare leaf123_check(leaf123_prepare(...), ub) with
 * r1_r2_r3_strategies(box with r4.hi = ub, R4), result and trap status.
 * Returns the number of disagreements. */
size_t ccport_leafprep_mismatches(const cc_tight_box* boxes, size_t n, int n_ub) {
    size_t bad = 0;
    for (size_t i = 0; i < n; ++i) {
        const cc_tight_box& b = boxes[i];
        Iv la = to_iv(b.la), r1 = to_iv(b.r[0]), r2 = to_iv(b.r[1]), r3 = to_iv(b.r[2]);
        Iv w = ct::required_weight_for(la);
        Iv R4 = w - r1 - r2 - r3;
        cc::tighten_lb(R4, 0.0);
        ct::Box vb{la, {r1, r2, r3, r3}};
        cc::tighten_lb(vb.r[1], vb.r[2].lo);
        cc::tighten_lb(vb.r[0], vb.r[1].lo);
        cc::trap_clear();
        const ct::LeafPrep p = ct::leaf123_prepare(vb, R4);
        for (int j = 0; j < n_ub; ++j) {
            double t = n_ub > 1 ? (double)j / (n_ub - 1) : 1.0;
            double ub = r3.lo * (1.25 * t - 0.125);
            if (!(ub >= 0)) ub = r3.lo;
            cc::trap_clear();
            const bool a = ct::leaf123_check(p, ub);
            const uint32_t ta = cc::trap_status();
            ct::Box v = vb;
            v.r[3] = Iv{0.0, ub};
            cc::trap_clear();
            const bool c = ct::r1_r2_r3_strategies(v, R4);
            const uint32_t tc = cc::trap_status();
            cc::trap_clear();
            bad += (a != c) || (ta != tc);
        }
    }
    return bad;
}

/* the rounding layer itself, for the primitive tests (op: 0 add, 1 mul, 2 div, 3 sqrt, 4 rcp) */
void ccport_round(int op, int up, int exact_fenv, const double* a, const double* b, double* out, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        double x = a[i], y = b ? b[i] : 0.0, r = 0.0;
        if (exact_fenv) {
            switch (op) {
                case 0: r = up ? cc_fe_add_ru(x, y) : cc_fe_add_rd(x, y); break;
                case 1: r = up ? cc_fe_mul_ru(x, y) : cc_fe_mul_rd(x, y); break;
                case 2: r = up ? cc_fe_div_ru(x, y) : cc_fe_div_rd(x, y); break;
                case 3: r = up ? cc_fe_sqrt_ru(x) : cc_fe_sqrt_rd(x); break;
                case 4: r = up ? cc_fe_div_ru(1.0, x) : cc_fe_div_rd(1.0, x); break;
            }
        } else {
            switch (op) {
                case 0: r = up ? cc_sw_add_ru(x, y) : cc_sw_add_rd(x, y); break;
                case 1: r = up ? cc_sw_mul_ru(x, y) : cc_sw_mul_rd(x, y); break;
                case 2: r = up ? cc_sw_div_ru(x, y) : cc_sw_div_rd(x, y); break;
                case 3: r = up ? cc_sw_sqrt_ru(x) : cc_sw_sqrt_rd(x); break;
                case 4: r = up ? cc_sw_rcp_ru(x) : cc_sw_rcp_rd(x); break;
            }
        }
        out[i] = r;
    }
}

/* subinterval (get_subinterval with its FMA), for the split tests */
void ccport_subinterval(double lo, double hi, int i, int n, double* out) {
    Iv r = cc::subinterval(Iv{lo, hi}, i, n);
    out[0] = r.lo;
    out[1] = r.hi;
}

}  // extern "C"

/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Per-box verdict masks of the REFERENCE's size-bound criteria (compiled for
 * the host with ref_shim.h).  For a box (lambda, r1..r6) the leaf of the
 * reference's kernel (rectangle_size_bound/rectangle_size_bound.cu:189-231)
 * tightens it, computes its Intermediate_values and runs the cascade; here
 * every criterion of that cascade and every shortcut of the kernel
 * (:162-177) is evaluated on its own.  A criterion that reaches a trap site
 * counts as not certified and sets bit 31.
 *
 * Bits: CC_SV_* in include/circlecover_gb300.h.
 *
 * ccref_sb_prove runs the host restatement of the proof driver
 * (oracle/sb_driver.hpp) on the reference's own pieces: get_subinterval,
 * Variables::from_la_r1_r2 / tighten / empty, Intermediate_values, the
 * shortcuts and the cascade of kernel_find_critical_intervals_in
 * (rectangle_size_bound.cu:161-236), a trap ending the cascade.
 */
#include <csetjmp>
#include <cstring>
#include <cstdint>
#include <cstdlib>
#include <thread>
#include <vector>

#include "rectangle_size_bound/strategies.cuh"
#include "../../include/circlecover_gb300.h"
#include "../sb_driver.hpp"

using circlecover::IV;
namespace rsb = circlecover::rectangle_size_bound;

extern CC_HOST_TLS unsigned long long cc_shim_op_count;
bool cc_ref_guarded_call(bool (*f)(void*), void* ctx, uint32_t* trapped);

namespace {

struct Ctx {
    const rsb::Variables* vars;
    rsb::Intermediate_values* vals;
    int which;
    IV la, r1, r2, r3;
};

bool run(void* p) {
    Ctx& c = *(Ctx*)p;
    const rsb::Variables& v = *c.vars;
    rsb::Intermediate_values& s = *c.vals;
    switch (c.which) {
        case 0: return rsb::even_split_recursion(v, s);
        case 1: return rsb::uneven_split_recursion(v, s);
        case 2: return rsb::multi_disk_strip_vertical(v, s);
        case 3: return rsb::vertical_wall_building_recursion(v, s);
        case 4: return rsb::r1_in_corner_explicit_recursion(v, s);
        case 5: return rsb::r1_r2_opposite_corners_recursion(v, s);
        case 6: return rsb::r1_r2_vertical_strip(v, s);
        case 7: {
            s.cover_2x2 = rsb::compute_two_by_two_cover(+v.radii);
            if (!(s.cover_2x2.width > 0)) return false;
            return s.cover_2x2.width > v.la.get_ub() || rsb::two_by_two_cover_with_strip_and_recursion(v, s);
        }
        case 8: return rsb::l_shaped_recursion(v, s);
        case 9: return rsb::r1_in_corner_wall_building_recursion(v, s);
        case 10: return rsb::advanced_multi_disk_strip_vertical(v, s);
        case 11: return rsb::five_disk_full_cover(v, s);
        case 12: return rsb::six_disk_full_cover(v, s);
        case 13: return rsb::seven_disk_strategies(v, s);
        case 15: return rsb::shortcut_even_split_recursion(c.la, c.r1, c.r2);
        case 16: return rsb::shortcut_uneven_split_recursion(c.la, c.r1, c.r2);
        case 17: return rsb::shortcut_uneven_split_recursion(c.la, c.r1, c.r2, c.r3);
        case 18: return rsb::shortcut_r1_r2_opposite_corners_recursion(c.la, c.r1, c.r2, c.r3);
        case 19: return rsb::shortcut_r1_r2_vertical_strip(c.la, c.r1, c.r2, c.r3);
    }
    return false;
}

uint32_t eval_one(const cc_sb_box& in) {
    rsb::Variables raw;
    raw.la = IV(in.la.lb, in.la.ub);
    for (int i = 0; i < 6; ++i) raw.radii[i] = IV(in.r[i].lb, in.r[i].ub);
    rsb::Variables vars = raw.tighten();
    uint32_t m = 0, trapped = 0;
    Ctx c{&vars, nullptr, 0, raw.la, raw.radii[0], raw.radii[1], raw.radii[2]};
    // the kernel's shortcuts see the untightened ranges
    for (int k = 15; k <= 19; ++k) {
        c.which = k;
        uint32_t t = 0;
        if (cc_ref_guarded_call(run, &c, &t)) m |= 1u << k;
        trapped |= t;
    }
    rsb::Intermediate_values vals{vars};
    c.vals = &vals;
    if (vars.empty() || vals.R.empty()) m |= 1u << 14;
    for (int k = 0; k <= 13; ++k) {
        c.which = k;
        uint32_t t = 0;
        if (cc_ref_guarded_call(run, &c, &t)) m |= 1u << k;
        trapped |= t;
    }
    if (trapped) m |= 1u << 31;
    return m;
}

}  // namespace


namespace {

bool call_shortcut(int which, const rsb::Variables& t, IV r3, bool& trapped) {
    Ctx c{&t, nullptr, which, t.la, t.radii[0], t.radii[1], r3};
    uint32_t tr = 0;
    bool ok = cc_ref_guarded_call(run, &c, &tr);
    trapped = trapped || tr != 0;
    return ok && !tr;
}

struct LeafCtx {
    const rsb::Variables* vars;
    int outcome;
};

// the kernel's leaf (rectangle_size_bound.cu:194-231), reporting which
// criterion ended the cascade
bool run_leaf(void* p) {
    LeafCtx& c = *(LeafCtx*)p;
    const rsb::Variables& vars = *c.vars;
    rsb::Intermediate_values vals{vars};
    if (vars.empty() || vals.R.empty()) {
        c.outcome = CC_SBT_LEAF_EMPTY;
        return true;
    }
    c.outcome = 0;
    if (rsb::even_split_recursion(vars, vals)) return true;
    c.outcome = 1;
    if (rsb::uneven_split_recursion(vars, vals)) return true;
    c.outcome = 2;
    if (rsb::multi_disk_strip_vertical(vars, vals)) return true;
    c.outcome = 3;
    if (rsb::vertical_wall_building_recursion(vars, vals)) return true;
    c.outcome = 4;
    if (rsb::r1_in_corner_explicit_recursion(vars, vals)) return true;
    c.outcome = 5;
    if (rsb::r1_r2_opposite_corners_recursion(vars, vals)) return true;
    c.outcome = 6;
    if (rsb::r1_r2_vertical_strip(vars, vals)) return true;
    c.outcome = 7;
    vals.cover_2x2 = rsb::compute_two_by_two_cover(+vars.radii);
    if (vals.cover_2x2.width > 0) {
        if (vals.cover_2x2.width > vars.la.get_ub() || rsb::two_by_two_cover_with_strip_and_recursion(vars, vals)) return true;
    }
    c.outcome = 8;
    if (rsb::l_shaped_recursion(vars, vals)) return true;
    c.outcome = 9;
    if (rsb::r1_in_corner_wall_building_recursion(vars, vals)) return true;
    c.outcome = 10;
    if (rsb::advanced_multi_disk_strip_vertical(vars, vals)) return true;
    c.outcome = 11;
    if (rsb::five_disk_full_cover(vars, vals)) return true;
    c.outcome = 12;
    if (rsb::six_disk_full_cover(vars, vals)) return true;
    c.outcome = 13;
    if (rsb::seven_disk_strategies(vars, vals)) return true;
    c.outcome = CC_SBT_LEAF_CRITICAL;
    return true;
}

struct RefSbC {
    using Box = rsb::Variables;
    static double lo(const IV& v) { return v.get_lb(); }
    static double hi(const IV& v) { return v.get_ub(); }
    static void do_join(IV& a, const IV& b) { a.do_join(b); }
    static IV& rad(Box& b, int i) { return b.radii[i]; }
    static const IV& rad(const Box& b, int i) { return b.radii[i]; }

    // find_critical_intervals_in's loop body (rectangle_size_bound.cu:281-291)
    static Box task_box(const Box& p, int la_i, int nla, int r1_i, int n1, int r2_i, int n2) {
        IV la = circlecover::get_subinterval(p.la, la_i, nla);
        IV r1 = circlecover::get_subinterval(p.radii[0], r1_i, n1);
        IV r2;
        for (int j = 0; j <= r2_i; ++j) {
            IV r2_range = p.radii[1];
            r2_range.tighten_ub(r1.get_ub());
            r2 = circlecover::get_subinterval(r2_range, j, n2);
            r1.tighten_lb(r2.get_lb());
        }
        return Box::from_la_r1_r2(p, la, r1, r2);
    }
    static int task_outcome(const Box& t, bool& trapped) {
        trapped = false;
        if (t.empty()) return CC_SBT_TASK_EMPTY;
        if (call_shortcut(15, t, IV(0.0, 0.0), trapped)) return CC_SBT_TASK_EVEN;
        if (call_shortcut(16, t, IV(0.0, 0.0), trapped)) return CC_SBT_TASK_UNEVEN;
        return CC_SBT_TASK_SPLIT;
    }
    static IV r3_piece(const Box& t, int i, int n) { return circlecover::get_subinterval(t.radii[2], i, n); }
    static int cell_outcome(const Box& t, IV r3, bool& trapped) {
        trapped = false;
        if (call_shortcut(17, t, r3, trapped)) return CC_SBT_CELL_UNEVEN;
        if (call_shortcut(18, t, r3, trapped)) return CC_SBT_CELL_OPPOSITE;
        if (call_shortcut(19, t, r3, trapped)) return CC_SBT_CELL_VSTRIP;
        return CC_SBT_CELL_SPLIT;
    }
    static Box leaf_box(const Box& t, IV r3, int i4, int n4, int i5, int n5, int i6, int n6) {
        Box v{t.la, {t.radii[0], t.radii[1], r3, circlecover::get_subinterval(t.radii[3], i4, n4),
                     circlecover::get_subinterval(t.radii[4], i5, n5), circlecover::get_subinterval(t.radii[5], i6, n6)}};
        return v.tighten();
    }
    static int leaf_outcome(const Box& b) {
        LeafCtx c{&b, CC_SBT_LEAF_CRITICAL};
        uint32_t tr = 0;
        cc_ref_guarded_call(run_leaf, &c, &tr);
        return tr ? CC_SBT_LEAF_TRAPPED : c.outcome;
    }
};

}  // namespace

extern "C" int ccref_sb_eval(const cc_sb_box* boxes, size_t n, uint32_t* masks, uint64_t* ops, int threads) {
    auto body = [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            unsigned long long before = cc_shim_op_count;
            masks[i] = eval_one(boxes[i]);
            if (ops) ops[i] = cc_shim_op_count - before;
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

static void sb_result_out(const cc_oracle::SbDriver<RefSbC>::Result& res, cc_sb_box** out, uint32_t** flags,
                          size_t* n_out, cc_sb_prove_stats* stats);

/* one generation over the tasks [lo, hi) of the parents, merged as
 * generation gen (the sampled-range oracle of the full size-bound runs) */
extern "C" int ccref_sb_generation(const cc_sb_box* parents, size_t n, int gen, int la_splits, const int* r_splits,
                                   uint64_t lo, uint64_t hi, int threads, cc_sb_box** out, uint32_t** flags,
                                   size_t* n_out, cc_sb_prove_stats* stats) {
    using Driver = cc_oracle::SbDriver<RefSbC>;
    std::vector<rsb::Variables> ps(n);
    for (size_t i = 0; i < n; ++i) {
        ps[i].la = IV(parents[i].la.lb, parents[i].la.ub);
        for (int k = 0; k < 6; ++k) ps[i].radii[k] = IV(parents[i].r[k].lb, parents[i].r[k].ub);
    }
    sb_result_out(Driver::generation_range(ps, gen, la_splits, r_splits, threads, lo, hi), out, flags, n_out, stats);
    return 0;
}

extern "C" int ccref_sb_prove(const cc_sb_box* root, const cc_sb_grid* grid, int threads, cc_sb_box** out,
                              uint32_t** flags, size_t* n_out, cc_sb_prove_stats* stats) {
    using Driver = cc_oracle::SbDriver<RefSbC>;
    rsb::Variables r;
    r.la = IV(root->la.lb, root->la.ub);
    for (int i = 0; i < 6; ++i) r.radii[i] = IV(root->r[i].lb, root->r[i].ub);
    sb_result_out(Driver::prove(r, *grid, threads), out, flags, n_out, stats);
    return 0;
}

static void sb_result_out(const cc_oracle::SbDriver<RefSbC>::Result& res, cc_sb_box** out, uint32_t** flags,
                          size_t* n_out, cc_sb_prove_stats* stats) {
    size_t n = res.criticals.size();
    *n_out = n;
    *out = (cc_sb_box*)std::malloc(sizeof(cc_sb_box) * (n + 1));
    *flags = (uint32_t*)std::malloc(sizeof(uint32_t) * (n + 1));
    for (size_t i = 0; i < n; ++i) {
        const rsb::Variables& b = res.criticals[i].box;
        (*out)[i].la = cc_iv{b.la.get_lb(), b.la.get_ub()};
        for (int k = 0; k < 6; ++k) (*out)[i].r[k] = cc_iv{b.radii[k].get_lb(), b.radii[k].get_ub()};
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

/* the box of one task of find_critical_intervals_in (r1 tightened across the
 * r2 loop, from_la_r1_r2), for the driver-state test */
extern "C" void ccref_sb_task_box(const cc_sb_box* parent, int la_i, int nla, int r1_i, int n1, int r2_i, int n2,
                                  cc_sb_box* out) {
    rsb::Variables p;
    p.la = IV(parent->la.lb, parent->la.ub);
    for (int i = 0; i < 6; ++i) p.radii[i] = IV(parent->r[i].lb, parent->r[i].ub);
    rsb::Variables t = RefSbC::task_box(p, la_i, nla, r1_i, n1, r2_i, n2);
    out->la = cc_iv{t.la.get_lb(), t.la.get_ub()};
    for (int i = 0; i < 6; ++i) out->r[i] = cc_iv{t.radii[i].get_lb(), t.radii[i].get_ub()};
}

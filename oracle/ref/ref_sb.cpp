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
 */
#include <csetjmp>
#include <cstdint>
#include <cstdlib>
#include <thread>
#include <vector>

#include "rectangle_size_bound/strategies.cuh"
#include "../../include/circlecover_gb300.h"

using circlecover::IV;
namespace rsb = circlecover::rectangle_size_bound;

extern thread_local unsigned long long cc_shim_op_count;
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

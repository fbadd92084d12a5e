// Summary of a critical set against the theoretical worst cases of the tight
// proof (reference: tight_rectangle/tight_rectangle.cu:322-456,
// kernel_compute_distance_from_theoretical_worst_cases; printed at :508-533).
// A critical box with r3^2 < 0.1 is classified as a 2-disk case (worst case
// r1^2 = (lambda^2+1)/4, r2^2 = 1/4), any other as a 3-disk case (worst case
// r^2 = (16 lambda^4 + 40 lambda^2 + 9) / (256 lambda^2)).
//
// The pass is order-dependent by construction: a "dominating critical" is
// the first box that strictly extends the running join, so the result is
// defined by the sequential fold over the boxes in their given order.  The
// reference runs the whole pass in one GPU thread; here every box's
// arithmetic (square roots, divisions, the required weight) runs in
// parallel (summary_item) and one thread folds the precomputed values in
// order (summary_fold), which keeps the result bit for bit.
#pragma once

#include "cc_tight.cuh"

namespace cc {
namespace summary {

using tight::Box;

CC_FN cc_iv civ(Iv x) { return cc_iv{x.lo, x.hi}; }
CC_FN Iv fiv(cc_iv x) { return Iv{x.lb, x.ub}; }
CC_FN cc_tight_box cbox(const Box& b) {
    cc_tight_box o;
    o.la = civ(b.la);
    for (int k = 0; k < 4; ++k) o.r[k] = civ(b.r[k]);
    return o;
}

// track the first boxes that push the running join below / above it
CC_FN void extend(cc_iv& acc, Iv d, cc_tight_box* dominating, const Box& b) {
    if (d.lo < acc.lb) dominating[0] = cbox(b);
    if (d.hi > acc.ub) dominating[1] = cbox(b);
    Iv a = fiv(acc);
    do_join(a, d);
    acc = civ(a);
}

// Per-box quantities of the pass (all of its arithmetic; independent per
// box, computed in parallel), then the order-dependent fold over them.
struct Item {
    int is2d;
    Iv d1, d2, d3;       // distances of r1^2, r2^2 (and r3^2) from the worst case
    double R_ub;         // R3 (2-disk) or R4 (3-disk) upper bound
    double la_by_S1;     // 2-disk only
    double lb_h1;        // 2-disk only
    Iv S1, h2, S3;       // 3-disk only
    double pocket;       // 3-disk only
};

CC_FN_INL Item summary_item(const Box& b) {
    Item it;
    it.is2d = b.r[2].hi < 0.1;
    if (it.is2d) {
        Iv r1_theory = 0.25 * (square(b.la) + 1.0);
        Iv r2_theory = ivp(0.25);
        it.d1 = b.r[0] - r1_theory;
        it.d2 = b.r[1] - r2_theory;
        it.R_ub = (tight::required_weight_for(b.la) - b.r[0] - b.r[1]).hi;
        double lb_S1 = mul_dn(2.0, sqrt_dn(add_dn(b.r[0].lo, -0.25)));
        it.la_by_S1 = div_up(b.la.hi, lb_S1);
        double t = add_up(b.la.hi, -mul_dn(0.5, lb_S1));
        it.lb_h1 = mul_dn(2.0, sqrt_dn(add_dn(b.r[0].lo, -mul_up(t, t))));
    } else {
        Iv la2 = square(b.la);
        Iv la4 = square(la2);
        Iv theory = (16.0 * la4 + 40.0 * la2 + 9.0) / (256.0 * la2);
        it.d1 = b.r[0] - theory;
        it.d2 = b.r[1] - theory;
        it.d3 = b.r[2] - theory;
        it.R_ub = (tight::required_weight_for(b.la) - b.r[0] - b.r[1] - b.r[2]).hi;
        it.S1 = sqrt(4.0 * b.r[0] - 1.0);
        it.h2 = sqrt(4.0 * b.r[1] - square(b.la - it.S1));
        it.S3 = sqrt(4.0 * b.r[2] - square(1.0 - it.h2));
        it.pocket = (b.la - it.S1 - it.S3).hi;
    }
    return it;
}

// the fold of tight_rectangle.cu:343-456 over precomputed items, in order
CC_FN_INL void summary_fold(const Item* items, const Box* crit, size_t n, cc_tight_summary_t* out) {
    cc_tight_summary_t o;
    memset(&o, 0, sizeof(o));
    o.have_range_2d = 0;
    o.have_range_3d = 0;
    o.la_range_3d = cc_iv{1.0, 1.0};
    o.la_range_2d = cc_iv{2.0, 2.0};
    o.dist_r1_2d = o.dist_r2_2d = cc_iv{0.0, 0.0};
    o.ub_R3_2d = o.ub_R4_3d = 0.0;
    o.dist_r1_3d = o.dist_r2_3d = o.dist_r3_3d = cc_iv{0.0, 0.0};
    o.pocket_width_3d = -1.0;
    o.lb_h1_2d = 1.0;
    o.ub_la_by_S1 = 1.0;
    for (size_t i = 0; i < n; ++i) {
        const Box& b = crit[i];
        const Item& it = items[i];
        if (it.is2d) {
            o.have_range_2d = 1;
            Iv lr = fiv(o.la_range_2d);
            do_join(lr, b.la);
            o.la_range_2d = civ(lr);
            extend(o.dist_r1_2d, it.d1, o.dist_r1_2d_criticals, b);
            extend(o.dist_r2_2d, it.d2, o.dist_r2_2d_criticals, b);
            if (it.R_ub > o.ub_R3_2d) o.ub_R3_2d = it.R_ub;
            if (it.la_by_S1 > o.ub_la_by_S1) o.ub_la_by_S1 = it.la_by_S1;
            if (it.lb_h1 < o.lb_h1_2d) o.lb_h1_2d = it.lb_h1;
        } else {
            o.have_range_3d = 1;
            Iv lr = fiv(o.la_range_3d);
            do_join(lr, b.la);
            o.la_range_3d = civ(lr);
            // the reference joins after all three comparisons
            if (it.d1.lo < o.dist_r1_3d.lb) o.dist_r1_3d_criticals[0] = cbox(b);
            if (it.d1.hi > o.dist_r1_3d.ub) o.dist_r1_3d_criticals[1] = cbox(b);
            if (it.d2.lo < o.dist_r2_3d.lb) o.dist_r2_3d_criticals[0] = cbox(b);
            if (it.d2.hi > o.dist_r2_3d.ub) o.dist_r2_3d_criticals[1] = cbox(b);
            if (it.d3.lo < o.dist_r3_3d.lb) o.dist_r3_3d_criticals[0] = cbox(b);
            if (it.d3.hi > o.dist_r3_3d.ub) o.dist_r3_3d_criticals[1] = cbox(b);
            Iv j1 = fiv(o.dist_r1_3d), j2 = fiv(o.dist_r2_3d), j3 = fiv(o.dist_r3_3d);
            do_join(j1, it.d1);
            do_join(j2, it.d2);
            do_join(j3, it.d3);
            o.dist_r1_3d = civ(j1);
            o.dist_r2_3d = civ(j2);
            o.dist_r3_3d = civ(j3);
            if (it.R_ub > o.ub_R4_3d) o.ub_R4_3d = it.R_ub;
            if (it.pocket > o.pocket_width_3d) {
                if (o.pocket_width_3d < 0.0) {
                    o.S1 = civ(it.S1);
                    o.h2 = civ(it.h2);
                    o.S3 = civ(it.S3);
                }
                o.pocket_width_3d = it.pocket;
            }
            Iv a = fiv(o.S1), c = fiv(o.h2), e = fiv(o.S3);
            do_join(a, it.S1);
            do_join(c, it.h2);
            do_join(e, it.S3);
            o.S1 = civ(a);
            o.h2 = civ(c);
            o.S3 = civ(e);
        }
    }
    *out = o;
}

#if CC_DEVICE_BUILD
// one thread per critical box: all of the pass's arithmetic
__global__ void k_summary_items(const Box* __restrict__ crit, size_t n, Item* __restrict__ items) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        trap_clear();
        items[i] = summary_item(crit[i]);
    }
}

// the fold: comparisons and joins only, in the boxes' order
__global__ void k_summary_fold(const Item* __restrict__ items, const Box* __restrict__ crit, size_t n,
                               cc_tight_summary_t* out) {
    summary_fold(items, crit, n, out);
}
#endif

}  // namespace summary
}  // namespace cc

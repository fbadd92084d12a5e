// Summary of a critical set against the theoretical worst cases of the tight
// proof (reference: tight_rectangle/tight_rectangle.cu:322-456,
// kernel_compute_distance_from_theoretical_worst_cases; printed at :508-533).
// A critical box with r3^2 < 0.1 is classified as a 2-disk case (worst case
// r1^2 = (lambda^2+1)/4, r2^2 = 1/4), any other as a 3-disk case (worst case
// r^2 = (16 lambda^4 + 40 lambda^2 + 9) / (256 lambda^2)).
//
// The pass is order-dependent by construction: a "dominating critical" is
// the first box that strictly extends the running join, so the result is
// defined by the sequential fold over the boxes in their given order.
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

#if CC_DEVICE_BUILD
__global__ void k_summary(const Box* __restrict__ crit, size_t n, cc_tight_summary_t* out) {
    trap_clear();
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
        const Box b = crit[i];
        if (b.r[2].hi < 0.1) {
            o.have_range_2d = 1;
            Iv lr = fiv(o.la_range_2d);
            do_join(lr, b.la);
            o.la_range_2d = civ(lr);
            Iv r1_theory = 0.25 * (square(b.la) + 1.0);
            Iv r2_theory = ivp(0.25);
            extend(o.dist_r1_2d, b.r[0] - r1_theory, o.dist_r1_2d_criticals, b);
            extend(o.dist_r2_2d, b.r[1] - r2_theory, o.dist_r2_2d_criticals, b);
            Iv R3 = tight::required_weight_for(b.la) - b.r[0] - b.r[1];
            if (R3.hi > o.ub_R3_2d) o.ub_R3_2d = R3.hi;
            double lb_S1 = mul_dn(2.0, sqrt_dn(add_dn(b.r[0].lo, -0.25)));
            double la_by_S1 = div_up(b.la.hi, lb_S1);
            if (la_by_S1 > o.ub_la_by_S1) o.ub_la_by_S1 = la_by_S1;
            double t = add_up(b.la.hi, -mul_dn(0.5, lb_S1));
            double lb_h1 = mul_dn(2.0, sqrt_dn(add_dn(b.r[0].lo, -mul_up(t, t))));
            if (lb_h1 < o.lb_h1_2d) o.lb_h1_2d = lb_h1;
        } else {
            o.have_range_3d = 1;
            Iv lr = fiv(o.la_range_3d);
            do_join(lr, b.la);
            o.la_range_3d = civ(lr);
            Iv la2 = square(b.la);
            Iv la4 = square(la2);
            Iv theory = (16.0 * la4 + 40.0 * la2 + 9.0) / (256.0 * la2);
            Iv d1 = b.r[0] - theory, d2 = b.r[1] - theory, d3 = b.r[2] - theory;
            // the reference joins after all three comparisons
            if (d1.lo < o.dist_r1_3d.lb) o.dist_r1_3d_criticals[0] = cbox(b);
            if (d1.hi > o.dist_r1_3d.ub) o.dist_r1_3d_criticals[1] = cbox(b);
            if (d2.lo < o.dist_r2_3d.lb) o.dist_r2_3d_criticals[0] = cbox(b);
            if (d2.hi > o.dist_r2_3d.ub) o.dist_r2_3d_criticals[1] = cbox(b);
            if (d3.lo < o.dist_r3_3d.lb) o.dist_r3_3d_criticals[0] = cbox(b);
            if (d3.hi > o.dist_r3_3d.ub) o.dist_r3_3d_criticals[1] = cbox(b);
            Iv j1 = fiv(o.dist_r1_3d), j2 = fiv(o.dist_r2_3d), j3 = fiv(o.dist_r3_3d);
            do_join(j1, d1);
            do_join(j2, d2);
            do_join(j3, d3);
            o.dist_r1_3d = civ(j1);
            o.dist_r2_3d = civ(j2);
            o.dist_r3_3d = civ(j3);
            Iv R4 = tight::required_weight_for(b.la) - b.r[0] - b.r[1] - b.r[2];
            if (R4.hi > o.ub_R4_3d) o.ub_R4_3d = R4.hi;
            Iv S1 = sqrt(4.0 * b.r[0] - 1.0);
            Iv h2 = sqrt(4.0 * b.r[1] - square(b.la - S1));
            Iv S3 = sqrt(4.0 * b.r[2] - square(1.0 - h2));
            double pocket = (b.la - S1 - S3).hi;
            if (pocket > o.pocket_width_3d) {
                if (o.pocket_width_3d < 0.0) {
                    o.S1 = civ(S1);
                    o.h2 = civ(h2);
                    o.S3 = civ(S3);
                }
                o.pocket_width_3d = pocket;
            }
            Iv a = fiv(o.S1), c = fiv(o.h2), e = fiv(o.S3);
            do_join(a, S1);
            do_join(c, h2);
            do_join(e, S3);
            o.S1 = civ(a);
            o.h2 = civ(c);
            o.S3 = civ(e);
        }
    }
    *out = o;
}
#endif

}  // namespace summary
}  // namespace cc

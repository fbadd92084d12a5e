// Constants and the small size-bound helpers that the tight-rectangle proof
// also uses (reference: rectangle_size_bound/values.hpp:28-35,
// disk_satisfies_size_bound.cu:25-37, maximize_covered.cu:82-105).
#pragma once

#include "cc_geom.cuh"

namespace cc {
namespace sb {

// efficiency guaranteed for disks of weight <= 9/64 on a rectangle of
// smaller side 1; the double 0.61 is slightly below the real 0.61
static constexpr double kCriticalRatio = 0.61;
static constexpr double kUbDiskRadius = 3.0 / 8.0;   // exact
static constexpr double kUbDiskWeight = 9.0 / 64.0;  // exact
static constexpr double kLbProofLambda = 1.0;
static constexpr double kUbProofLambda = 2.5;

// does a disk of squared radius <= r_sq_ub satisfy the size bound on a strip
// of height >= height_lb?  (disk_satisfies_size_bound.cu:25-28)
template <class S>
CC_FN bool disk_satisfies_size_bound(S r_sq_ub, S height_lb) {
    S s = rcp_up(height_lb);
    return mul_up(r_sq_ub, mul_up(s, s)) <= kUbDiskWeight;
}

// (disk_satisfies_size_bound.cu:30-32)
template <class S>
CC_FN S bound_required_height(S r_sq_ub) {
    return div_up(sqrt_up(r_sq_ub), kUbDiskRadius);
}

// (disk_satisfies_size_bound.cu:34-37)
CC_FN double bound_allowed_weight(double lb_height) {
    double h2 = mul_dn(lb_height, lb_height);
    return mul_dn(kUbDiskWeight, h2);
}

// Lower bound on the height of a strip of width ub_w that two disks side by
// side can cover (maximize_covered.cu:82-105).
template <class I>
CC_FN typename I::S two_disks_maximize_height_t(I d1, I d2, typename I::S ub_w) {
    using S = typename I::S;
    const S a = d1.lo;
    const S b = d2.lo;
    S w_sq = mul_up(ub_w, ub_w);
    S diff_dn = add_dn(a, -b);
    S diff_up = add_up(a, -b);
    S diff_sq = mul_up(diff_up, diff_up);

    // each disk has to reach its part of the strip
    S part1 = add_up(mul_up(0.5, ub_w), mul_up(div_up(2.0, ub_w), diff_up));
    S part2 = add_up(mul_up(0.5, ub_w), -mul_dn(div_dn(2.0, ub_w), diff_dn));
    part1 = mul_up(part1, part1);
    part2 = mul_up(part2, part2);
    if (a <= mul_up(0.25, part1) || b <= mul_up(0.25, part2)) {
        return S(0.0);
    }

    S h_sq = add_dn(mul_dn(2.0, add_dn(a, b)), -add_up(mul_up(0.25, w_sq), mul_up(4.0, div_up(diff_sq, w_sq))));
    if (h_sq <= 0.0) {
        return S(0.0);
    }
    return sqrt_dn(h_sq);
}
CC_FN double two_disks_maximize_height(Iv d1, Iv d2, double ub_w) {
    return two_disks_maximize_height_t<Iv>(d1, d2, ub_w);
}

}  // namespace sb
}  // namespace cc

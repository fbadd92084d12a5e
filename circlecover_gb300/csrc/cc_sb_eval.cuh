// Per-box verdict mask of the size-bound criteria: every criterion of the
// reference kernel's cascade (rectangle_size_bound/rectangle_size_bound.cu:
// 189-231) and its shortcuts (:162-177) on one box, each on its own.  A
// criterion that reaches a trap site counts as not certified and sets bit 31.
// Bits: CC_SV_* in include/circlecover_gb300.h.
#pragma once

#include "cc_sb_seven.cuh"

namespace cc {
namespace sb {

// the criteria in cascade order (the bit index is the position)
enum SbCriterion : int {
    SB_EVEN_SPLIT = 0,
    SB_UNEVEN_SPLIT,
    SB_MULTI_DISK_STRIP,
    SB_WALL_BUILDING,
    SB_R1_CORNER_EXPLICIT,
    SB_OPPOSITE_CORNERS,
    SB_VERTICAL_STRIP,
    SB_TWO_BY_TWO,
    SB_L_SHAPED,
    SB_R1_CORNER_WALL,
    SB_ADVANCED_STRIP,
    SB_FIVE_DISK,
    SB_SIX_DISK,
    SB_SEVEN_DISK,
    SB_NUM_CRITERIA
};

// 2x2 cover on the left plus the rest (rectangle_size_bound.cu:213-219)
CC_FN_INL bool two_by_two_criterion(const Box6& b, Vals& v) {
    v.cover = compute_two_by_two_cover(b.r);
    if (!(v.cover.width > 0)) return false;
    return v.cover.width > b.la.hi || two_by_two_cover_with_strip_and_recursion(b, v);
}

CC_FN_INL bool sb_criterion(int k, const Box6& b, Vals& v) {
    switch (k) {
        case SB_EVEN_SPLIT: return even_split_recursion(b, v);
        case SB_UNEVEN_SPLIT: return uneven_split_recursion(b, v);
        case SB_MULTI_DISK_STRIP: return multi_disk_strip_vertical(b, v);
        case SB_WALL_BUILDING: return vertical_wall_building_recursion(b, v);
        case SB_R1_CORNER_EXPLICIT: return r1_in_corner_explicit_recursion(b, v);
        case SB_OPPOSITE_CORNERS: return r1_r2_opposite_corners_recursion(b, v);
        case SB_VERTICAL_STRIP: return r1_r2_vertical_strip(b, v);
        case SB_TWO_BY_TWO: return two_by_two_criterion(b, v);
        case SB_L_SHAPED: return l_shaped_recursion(b, v);
        case SB_R1_CORNER_WALL: return r1_in_corner_wall_building_recursion(b, v);
        case SB_ADVANCED_STRIP: return advanced_multi_disk_strip_vertical(b, v);
        case SB_FIVE_DISK: return five_disk_full_cover(b, v);
        case SB_SIX_DISK: return six_disk_full_cover(b, v);
        case SB_SEVEN_DISK: return seven_disk_strategies(b, v);
    }
    return false;
}

CC_FN_INL bool sb_shortcut(int k, Iv la, Iv r1, Iv r2, Iv r3) {
    switch (k) {
        case 15: return shortcut_even_split_recursion(la, r1, r2);
        case 16: return shortcut_uneven_split_recursion(la, r1, r2);
        case 17: return shortcut_uneven_split_recursion(la, r1, r2, r3);
        case 18: return shortcut_r1_r2_opposite_corners_recursion(la, r1, r2, r3);
        case 19: return shortcut_r1_r2_vertical_strip(la, r1, r2, r3);
    }
    return false;
}

// one criterion with its own trap status: certified only without a trap
CC_FN bool trap_free(bool result, bool& any_trap) {
    bool t = trap_status() != TRAP_NONE;
    any_trap = any_trap || t;
    return result && !t;
}

CC_FN_INL uint32_t sb_eval_all(const Box6& raw) {
    uint32_t m = 0;
    bool any_trap = false;
    for (int k = 15; k <= 19; ++k) {
        trap_clear();
        if (trap_free(sb_shortcut(k, raw.la, raw.r[0], raw.r[1], raw.r[2]), any_trap)) m |= 1u << k;
    }
    const Box6 b = tightened(raw);
    Vals v;
    v.R = remaining_weight(b);
    if (box_empty(b) || empty(v.R)) m |= 1u << 14;
    for (int k = 0; k < SB_NUM_CRITERIA; ++k) {
        trap_clear();
        if (trap_free(sb_criterion(k, b, v), any_trap)) m |= 1u << k;
    }
    trap_clear();
    if (any_trap) m |= 1u << 31;
    return m;
}

}  // namespace sb
}  // namespace cc

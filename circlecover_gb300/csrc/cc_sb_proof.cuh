// Building blocks of the size-bound proof (reference:
// rectangle_size_bound/rectangle_size_bound.cu:132-236, 276-310), shared by
// the GPU proof engine and the host restatement of the driver:
//   * the task level: one (lambda, r1, r2) piece of a parent box, with the
//     host loop's running tightening of r1 and Variables::from_la_r1_r2;
//   * the whole-task shortcuts the kernel tests before its loops;
//   * the r3 level and its three shortcuts;
//   * the leaf: the box of one (r3, r4, r5, r6) cell, tightened, with R.
// Trace outcomes per level: CC_SBT_* in include/circlecover_gb300.h.
#pragma once

#include "../../include/circlecover_gb300.h"
#include "cc_sb_eval.cuh"

namespace cc {
namespace sb {

// Variables::from_la_r1_r2 (rectangle_size_bound/variables.hpp:37-51)
CC_FN Box6 from_la_r1_r2(const Box6& v, Iv la, Iv r1, Iv r2) {
    Box6 b;
    b.la = intersect(v.la, la);
    b.r[0] = intersect(v.r[0], r1);
    b.r[1] = intersect(v.r[1], r2);
    for (int i = 2; i < 6; ++i) {
        b.r[i] = v.r[i];
        tighten_ub(b.r[i], r2.hi);
    }
    return tightened(b);
}

// The box of task (la_i, r1_i, r2_i) of parent `p` (rectangle_size_bound.cu:
// 281-291).  The host loop declares r1 once per r1 index and raises its lower
// bound to the lower bound of every r2 piece it visits (:289), so the r1 of
// r2 index i2 carries the tightenings of pieces 0..i2.
CC_FN Box6 task_box(const Box6& p, int la_i, int nla, int r1_i, int n1, int r2_i, int n2) {
    const Iv la = subinterval(p.la, la_i, nla);
    Iv r1 = subinterval(p.r[0], r1_i, n1);
    Iv r2_range = p.r[1];
    tighten_ub(r2_range, r1.hi);
    Iv r2{0.0, 0.0};
    for (int j = 0; j <= r2_i; ++j) {
        r2 = subinterval(r2_range, j, n2);
        tighten_lb(r1, r2.lo);
    }
    return from_la_r1_r2(p, la, r1, r2);
}

// whole-task shortcuts (rectangle_size_bound.cu:161-164); a shortcut that
// reaches a trap site is not taken (`trapped` is set)
CC_FN_INL int task_outcome(const Box6& t, bool& trapped) {
    trapped = false;
    if (box_empty(t)) return CC_SBT_TASK_EMPTY;
    trap_clear();
    bool ok = shortcut_even_split_recursion(t.la, t.r[0], t.r[1]);
    if (trap_status() != TRAP_NONE) trapped = true;
    else if (ok) return CC_SBT_TASK_EVEN;
    trap_clear();
    ok = shortcut_uneven_split_recursion(t.la, t.r[0], t.r[1]);
    if (trap_status() != TRAP_NONE) trapped = true;
    else if (ok) return CC_SBT_TASK_UNEVEN;
    trap_clear();
    return CC_SBT_TASK_SPLIT;
}

// r3 shortcuts (rectangle_size_bound.cu:172-178)
CC_FN_INL int cell_outcome(const Box6& t, Iv r3, bool& trapped) {
    trapped = false;
    trap_clear();
    bool ok = shortcut_uneven_split_recursion(t.la, t.r[0], t.r[1], r3);
    if (trap_status() != TRAP_NONE) trapped = true;
    else if (ok) return CC_SBT_CELL_UNEVEN;
    trap_clear();
    ok = shortcut_r1_r2_opposite_corners_recursion(t.la, t.r[0], t.r[1], r3);
    if (trap_status() != TRAP_NONE) trapped = true;
    else if (ok) return CC_SBT_CELL_OPPOSITE;
    trap_clear();
    ok = shortcut_r1_r2_vertical_strip(t.la, t.r[0], t.r[1], r3);
    if (trap_status() != TRAP_NONE) trapped = true;
    else if (ok) return CC_SBT_CELL_VSTRIP;
    trap_clear();
    return CC_SBT_CELL_SPLIT;
}

// the leaf box (rectangle_size_bound.cu:185-197): r4..r6 pieces of the task
// box's ranges, then Variables::tighten
CC_FN Box6 leaf_box(const Box6& t, Iv r3, int i4, int n4, int i5, int n5, int i6, int n6) {
    Box6 b;
    b.la = t.la;
    b.r[0] = t.r[0];
    b.r[1] = t.r[1];
    b.r[2] = r3;
    b.r[3] = subinterval(t.r[3], i4, n4);
    b.r[4] = subinterval(t.r[4], i5, n5);
    b.r[5] = subinterval(t.r[5], i6, n6);
    return tightened(b);
}

// leaf_box with the steps of the r4, r5, r6 splits precomputed per task
// (subinterval_step): the same box
CC_FN Box6 leaf_box_steps(const Box6& t, const double step[3], Iv r3, int i4, int n4, int i5, int n5, int i6, int n6) {
    Box6 b;
    b.la = t.la;
    b.r[0] = t.r[0];
    b.r[1] = t.r[1];
    b.r[2] = r3;
    b.r[3] = subinterval_with_step(t.r[3], step[0], i4, n4);
    b.r[4] = subinterval_with_step(t.r[4], step[1], i5, n5);
    b.r[5] = subinterval_with_step(t.r[5], step[2], i6, n6);
    return tightened(b);
}

// The cascade on one leaf box in the kernel's order (:189-231); the first
// criterion that certifies decides.  A trap ends the cascade: the reference
// would have aborted the run there, here the leaf is reported (critical,
// flagged).  Returns a leaf outcome (criterion index, EMPTY, CRITICAL or
// TRAPPED).
CC_FN_INL int leaf_outcome(const Box6& b) {
    Vals v;
    v.R = remaining_weight(b);
    if (box_empty(b) || empty(v.R)) return CC_SBT_LEAF_EMPTY;
    for (int k = 0; k < SB_NUM_CRITERIA; ++k) {
        trap_clear();
        bool ok = sb_criterion(k, b, v);
        if (trap_status() != TRAP_NONE) {
            trap_clear();
            return CC_SBT_LEAF_TRAPPED;
        }
        if (ok) return k;
    }
    return CC_SBT_LEAF_CRITICAL;
}

// trace key of one decision: (generation, task, level, i3..i6, outcome)
CC_FN uint64_t sb_mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}
// the key in two parts: the task's share (computed once per task) and the rest
CC_FN uint64_t sb_trace_task_mix(uint64_t task) { return sb_mix64(task + 0x9e3779b97f4a7c15ULL); }
CC_FN uint64_t sb_trace_key_mixed(int gen, uint64_t task_mix, int level, int i3, int i4, int i5, int i6,
                                  int outcome) {
    uint64_t packed = (uint64_t)outcome | ((uint64_t)i6 << 5) | ((uint64_t)i5 << 16) | ((uint64_t)i4 << 27) |
                      ((uint64_t)i3 << 38) | ((uint64_t)level << 49) | ((uint64_t)gen << 51);
    return sb_mix64(packed ^ task_mix);
}
CC_FN uint64_t sb_trace_key(int gen, uint64_t task, int level, int i3, int i4, int i5, int i6, int outcome) {
    return sb_trace_key_mixed(gen, sb_trace_task_mix(task), level, i3, i4, i5, i6, outcome);
}

}  // namespace sb
}  // namespace cc

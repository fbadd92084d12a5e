// Device engine of the size-bound proof (reference:
// rectangle_size_bound/rectangle_size_bound.cu:132-382) and its C ABI entry
// point cc_sb_prove.
//
// The reference enumerates the (lambda, r1, r2) tasks of a parent box on the
// host and launches one kernel per task (about 4.2 million synchronous
// launches for its initial pass), each a (r3, r4)-blocks x (r5, r6)-threads
// grid in which every thread runs the whole criteria cascade on its leaf.
// Here the tasks of a generation go through device stages in stream order:
//
//   tasks   one thread per task: its box (running r1 tightening,
//           from_la_r1_r2), empty check, whole-task shortcuts
//   cells   one thread per (task, r3 piece): the three r3 shortcuts
//   leaves  one thread per (cell, r4, r5, r6 piece): an FP32 emptiness
//           pre-filter; then, on the compacted list of leaves it did not
//           prove empty, leaf box, tighten, R, empty check and the first
//           criterion of the cascade
//   pass K  one thread per leaf still undecided: criterion K (K = 1..12),
//           survivors compacted into the next pass's queue; the r1-in-corner
//           criterion (K = 4) runs one thread per (leaf, placement)
//   seven   the seven-disk strategies, the costliest criterion, in three
//           kernels: one thread per leaf for the r7-range prefix, one thread
//           per (leaf, r7 piece) for the 16 pieces, one thread per leaf to
//           combine the pieces' outcomes as the sequential loop would
//
// so that every kernel runs one criterion on full warps of leaves that need
// it, instead of warps in which one lane runs the seven-disk strategies while
// 31 lanes wait.  Survivors of the last criterion and leaves whose cascade
// reached a trap site are the critical boxes; the host merges them per
// generation exactly as merge_critical_intervals<N> does.  Queues are sized
// so that they cannot overflow: a task chunk bounds the cell count, and a
// leaf slice whose undecided leaves would not fit the pass queues is undone
// (counters restored from a snapshot) and redone in halves.  The slice
// length adapts to the share of leaves that the first criterion leaves
// undecided, so that few slices (and few kernel tails) cover a task chunk.
//
// Every task, r3 cell and leaf visited contributes one count and one mixed
// key to the trace (cc_sb_prove_stats), computed the same way by the oracle.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cc_runtime.cuh"
#include "cc_sb_proof.cuh"

using cc::Iv;
namespace sb = cc::sb;
using sb::Box6;

namespace {

// FP32 bounds of a task's FP64 values for the leaf pre-filter (rounded
// down / up once per task instead of once per leaf)
struct SbTaskF32 {
    float la_lo_dn, la_hi_up;
    float cr_dn, cr_up;                       // the critical ratio 0.61 (a double) rounded down / up
    float r_lo_dn[2], r_hi_up[2];             // r1, r2
    float step_dn[3], step_up[3];             // r4..r6 split steps
    float base_dn[3], base_up[3], top_up[3];  // r4..r6 range lower bounds, upper bounds
};

struct SbTask {  // a task that passed the whole-task shortcuts
    Box6 box;
    uint64_t id;
    uint64_t id_mix;  // sb_trace_task_mix(id)
    double step[3];  // steps of its r4, r5, r6 splits
    SbTaskF32 f;
};

struct SbCell {  // an r3 cell that passed the r3 shortcuts
    Iv r3;
    uint32_t task;
    uint32_t i3;
    float r3_lo_dn, r3_hi_up;
};

struct SbLeaf {  // an undecided or critical leaf
    Box6 box;
    uint64_t id;   // task id
    uint64_t idx;  // i3 | i4 << 11 | i5 << 22 | i6 << 33 | trapped << 63
};
static_assert(sizeof(SbLeaf) == 128, "leaf record");

struct SbCounters {
    unsigned long long n_task, n_cell, n_q[2], n_crit;
    unsigned long long overflow;
    unsigned long long leaf_evals, trapped_shortcuts;
    unsigned long long digest;
    unsigned long long task_counts[4], cell_counts[4], leaf_counts[CC_SBT_LEAF_OUTCOMES];
    unsigned long long fp32_empty;      // leaves the FP32 pre-filter proved empty
    unsigned long long widen_count;     // leaves with an FP64 R of nonzero width
    double widen_sum;                   // sum of FP32 / FP64 width of R over them
    unsigned long long widen_max_bits;  // bits of the largest ratio (positive doubles order as integers)
    unsigned long long n_f32_jobs;      // FP64 jobs of an FP32-first pass
    // FP64 certification of the FP32-decided "true" verdicts of the leaf
    // criteria: certified, and not confirmed (the FP64 verdict was used)
    unsigned long long cert_ok, cert_fail;
    // FP64 certification of the pre-filter's empty leaves (k_sbp_empty_cert):
    // anchors queued, anchors certified, anchors not confirmed (this slice)
    unsigned long long n_anchor, empty_cert_ok, empty_cert_fail;
};

struct SevenJob {  // a leaf whose seven-disk prefix left r7 pieces to check
    sb::SevenPrefix pre;
    uint32_t leaf;  // index in the pass queue
    uint32_t fail_mask, trap_mask, pad;
};

constexpr int kThreads = 128;

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ unsigned long long warp_append(unsigned long long* counter, bool want, unsigned long long cap,
                                                          unsigned long long* overflow) {
    const unsigned lane = threadIdx.x & 31;
    unsigned ballot = __ballot_sync(0xffffffffu, want);
    if (ballot == 0) return ~0ULL;
    unsigned long long base = 0;
    if (lane == (unsigned)(__ffs(ballot) - 1)) base = atomicAdd(counter, (unsigned long long)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, __ffs(ballot) - 1);
    unsigned long long slot = base + __popc(ballot & ((1u << lane) - 1));
    if (!want) return ~0ULL;
    if (slot >= cap) {
        atomicExch(overflow, 1ULL);
        return ~0ULL;
    }
    return slot;
}

// warp-uniform grid-stride loop: all 32 lanes enter every iteration
#define SB_WARP_LOOP(total)                                                                              \
    for (unsigned long long base_ = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); \
         base_ < (total); base_ += (unsigned long long)gridDim.x * blockDim.x)

template <int N>
struct BlockTrace {
    unsigned long long counts[N];
    unsigned long long digest;
    unsigned long long extra;  // leaf evaluations or trapped shortcuts
};

template <int N>
__device__ __forceinline__ void trace_init(BlockTrace<N>& bt) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) bt.counts[i] = 0;
    if (threadIdx.x == 0) bt.digest = 0, bt.extra = 0;
    __syncthreads();
}

// every lane of the warp calls this; lanes with the same outcome are counted
// by one shared-memory atomic (a warp whose leaves are all empty would
// otherwise serialise 32 atomics on one address)
template <int N>
__device__ __forceinline__ void trace_note(BlockTrace<N>& bt, bool valid, uint64_t key, int outcome) {
    uint64_t d = valid ? key : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if ((threadIdx.x & 31) == 0 && d) atomicAdd(&bt.digest, (unsigned long long)d);
    const unsigned same = __match_any_sync(0xffffffffu, valid ? outcome : -1);
    if (valid && (threadIdx.x & 31) == (unsigned)(__ffs(same) - 1))
        atomicAdd(&bt.counts[outcome], (unsigned long long)__popc(same));
}

template <int N>
__device__ __forceinline__ void trace_flush(BlockTrace<N>& bt, unsigned long long* counts, SbCounters* c,
                                            unsigned long long* extra) {
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x)
        if (bt.counts[i]) atomicAdd(&counts[i], bt.counts[i]);
    if (threadIdx.x == 0) {
        if (bt.digest) atomicAdd(&c->digest, bt.digest);
        if (bt.extra && extra) atomicAdd(extra, bt.extra);
    }
}

__device__ __forceinline__ uint64_t pack_idx(int i3, int i4, int i5, int i6) {
    return (uint64_t)i3 | ((uint64_t)i4 << 11) | ((uint64_t)i5 << 22) | ((uint64_t)i6 << 33);
}

__device__ __forceinline__ uint64_t leaf_key(int gen, const SbLeaf& l, int outcome) {
    const uint64_t x = l.idx;
    return sb::sb_trace_key(gen, l.id, 2, (int)(x & 2047), (int)((x >> 11) & 2047), (int)((x >> 22) & 2047),
                            (int)((x >> 33) & 2047), outcome);
}

// ---------------------------------------------------------------- stages
struct TaskGrid {
    int gen, nla, n1, n2, n4, n5, n6;
    unsigned long long per_parent;
};

// tasks [t0, t1) of the generation (rectangle_size_bound.cu:281-296, 161-164)
__global__ void __launch_bounds__(kThreads) k_sbp_tasks(const Box6* __restrict__ parents, unsigned long long t0,
                                                         unsigned long long t1, TaskGrid g, SbTask* __restrict__ out,
                                                         unsigned long long cap, SbCounters* c) {
    __shared__ BlockTrace<4> bt;
    trace_init(bt);
    SB_WARP_LOOP(t1 - t0) {
        const unsigned long long idx = t0 + base_ + (threadIdx.x & 31);
        const bool valid = idx < t1;
        int outcome = CC_SBT_TASK_EMPTY;
        Box6 tb;
        if (valid) {
            const unsigned long long p = idx / g.per_parent, rem = idx % g.per_parent;
            const int r2_i = (int)(rem % g.n2);
            const int r1_i = (int)((rem / g.n2) % g.n1);
            const int la_i = (int)(rem / ((unsigned long long)g.n2 * g.n1));
            tb = sb::task_box(parents[p], la_i, g.nla, r1_i, g.n1, r2_i, g.n2);
            bool trapped = false;
            outcome = sb::task_outcome(tb, trapped);
            if (trapped) atomicAdd(&bt.extra, 1ULL);
        }
        trace_note(bt, valid, sb::sb_trace_key(g.gen, idx, 0, 0, 0, 0, 0, outcome), outcome);
        unsigned long long slot = warp_append(&c->n_task, valid && outcome == CC_SBT_TASK_SPLIT, cap, &c->overflow);
        if (slot != ~0ULL) {
            out[slot].box = tb;
            out[slot].id = idx;
            out[slot].id_mix = sb::sb_trace_task_mix(idx);
            out[slot].step[0] = cc::subinterval_step(tb.r[3], g.n4);
            out[slot].step[1] = cc::subinterval_step(tb.r[4], g.n5);
            out[slot].step[2] = cc::subinterval_step(tb.r[5], g.n6);
            SbTaskF32& f = out[slot].f;
            f.la_lo_dn = __double2float_rd(tb.la.lo);
            f.la_hi_up = __double2float_ru(tb.la.hi);
            f.cr_dn = __double2float_rd(sb::kCriticalRatio);
            f.cr_up = __double2float_ru(sb::kCriticalRatio);
            for (int k = 0; k < 2; ++k) {
                f.r_lo_dn[k] = __double2float_rd(tb.r[k].lo);
                f.r_hi_up[k] = __double2float_ru(tb.r[k].hi);
            }
            for (int k = 0; k < 3; ++k) {
                f.step_dn[k] = __double2float_rd(out[slot].step[k]);
                f.step_up[k] = __double2float_ru(out[slot].step[k]);
                f.base_dn[k] = __double2float_rd(tb.r[3 + k].lo);
                f.base_up[k] = __double2float_ru(tb.r[3 + k].lo);
                f.top_up[k] = __double2float_ru(tb.r[3 + k].hi);
            }
        }
    }
    trace_flush(bt, c->task_counts, c, &c->trapped_shortcuts);
}

// r3 cells of the queued tasks (rectangle_size_bound.cu:171-178)
__global__ void __launch_bounds__(kThreads) k_sbp_cells(const SbTask* __restrict__ tasks, int gen, int n3,
                                                         SbCell* __restrict__ out, unsigned long long cap,
                                                         SbCounters* c) {
    __shared__ BlockTrace<4> bt;
    trace_init(bt);
    const unsigned long long total = c->n_task * (unsigned long long)n3;
    SB_WARP_LOOP(total) {
        const unsigned long long idx = base_ + (threadIdx.x & 31);
        const bool valid = idx < total;
        int outcome = CC_SBT_CELL_SPLIT;
        uint32_t t = 0;
        int i3 = 0;
        Iv r3{0.0, 0.0};
        uint64_t key = 0;
        if (valid) {
            t = (uint32_t)(idx / n3);
            i3 = (int)(idx % n3);
            const Box6 tb = tasks[t].box;
            r3 = cc::subinterval(tb.r[2], i3, n3);
            bool trapped = false;
            outcome = sb::cell_outcome(tb, r3, trapped);
            if (trapped) atomicAdd(&bt.extra, 1ULL);
            key = sb::sb_trace_key(gen, tasks[t].id, 1, i3, 0, 0, 0, outcome);
        }
        trace_note(bt, valid, key, outcome);
        unsigned long long slot = warp_append(&c->n_cell, valid && outcome == CC_SBT_CELL_SPLIT, cap, &c->overflow);
        if (slot != ~0ULL) out[slot] = SbCell{r3, t, (uint32_t)i3, __double2float_rd(r3.lo), __double2float_ru(r3.hi)};
    }
    trace_flush(bt, c->cell_counts, c, &c->trapped_shortcuts);
}

struct LeafGrid {
    int gen, n4, n5, n6;
    uint32_t rem0;             // l0 % (n4 n5 n6), when that product is below 2^31
    unsigned long long cell0;  // l0 / (n4 n5 n6)
};

// ---------------------------------------------------------------- FP32 pre-filter
// The leaf kernel skips a leaf (outcome EMPTY) when its tightened box or its
// remaining weight R is empty (rectangle_size_bound.cu:196-198).  Most leaves
// of a pass are empty, and the FP64 instructions that decide it dominate the
// kernel.  The pre-filter decides the same question with outward-rounded FP32
// bounds on the FP64 quantities themselves, and only where it proves the
// FP64 answer "empty":
//   * every FP64 value v the test reads gets FP32 bounds lo32 <= v <= hi32
//     (a double converted with rounding down/up; an FMA piece bound
//     fma(step, i, lo) from the rounded-down/up step and lo, with FMA rounded
//     down/up: any float below/above the exact value is also below/above its
//     FP64 rounding);
//   * tightened lower bounds are maxima of lower bounds, so their FP32 lower
//     bounds are maxima of FP32 lower bounds;
//   * R's upper bound is a chain of FP64 round-up subtractions from
//     la.hi * 0.61 (rounded down); the same chain in FP32 with round-up
//     operations on upper/lower bounds is never below it.
// So "FP32 says empty" implies "FP64 says empty"; otherwise the FP64 test
// runs as before.  Verdicts and traces are unchanged; the pre-filter only
// removes FP64 work.
// true only if the FP64 leaf test certainly finds the leaf empty; `ub_R`
// receives the FP32 upper bound of R.hi and `lb_R` a lower bound of R.lo
__device__ __forceinline__ bool f32_leaf_empty(const SbTaskF32& t, float r3_lo, float r3_hi, const int idx[3],
                                               const int n[3], float& lb_R, float& ub_R) {
    float lo[6], hi[6];
    lo[0] = t.r_lo_dn[0];
    hi[0] = t.r_hi_up[0];
    lo[1] = t.r_lo_dn[1];
    hi[1] = t.r_hi_up[1];
    lo[2] = r3_lo;
    hi[2] = r3_hi;
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // bounds of fma(step, i, lo) and of the piece's upper bound
        const int i = idx[k];
        lo[3 + k] = __fmaf_rd(t.step_dn[k], (float)i, t.base_dn[k]);  // exact: i < 2^24
        hi[3 + k] = (i + 1 == n[k]) ? t.top_up[k] : __fmaf_ru(t.step_up[k], (float)(i + 1), t.base_up[k]);
    }
    // tightened lower bounds (variables.hpp:53-65): running maximum from r6
    // down to r2, starting at 0; r1 keeps its own
    float m = 0.0f;
    bool empty = lo[0] >= hi[0];
#pragma unroll
    for (int k = 5; k >= 1; --k) {
        m = fmaxf(m, lo[k]);
        lo[k] = m;
        empty = empty || (m >= hi[k]);
    }
    // R = la * 0.61 - r1 - ... - r6 (variables.cuh:32-36)
    float u = __fmul_ru(t.la_hi_up, t.cr_up);
    float l = __fmul_rd(t.la_lo_dn, t.cr_dn);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        u = __fadd_ru(u, -lo[k]);
        l = __fadd_rd(l, -hi[k]);
    }
    ub_R = u;
    lb_R = l;
    return empty || u < 0.0f;
}

// Coordinates of leaf idx in [l0, l1) of the cell grid: r3 cell and r4..r6
// piece indices
struct LeafAt {
    unsigned long long ci;
    int i4, i5, i6;
};
__device__ __forceinline__ LeafAt leaf_at(const LeafGrid& g, unsigned long long l0, unsigned long long l1,
                                          unsigned long long idx) {
    const unsigned long long n456 = (unsigned long long)g.n4 * g.n5 * g.n6;
    LeafAt a;
    if (n456 < (1ULL << 31) && l1 - l0 < (1ULL << 31)) {
        // 32-bit index arithmetic: offsets from the slice's first cell
        const uint32_t off = g.rem0 + (uint32_t)(idx - l0);  // < 2^32
        const uint32_t q = off / (uint32_t)n456;
        const uint32_t rem = off - q * (uint32_t)n456;
        const uint32_t r56 = rem / (uint32_t)g.n6;
        a.ci = g.cell0 + q;
        a.i6 = (int)(rem - r56 * (uint32_t)g.n6);
        a.i4 = (int)(r56 / (uint32_t)g.n5);
        a.i5 = (int)(r56 - (uint32_t)a.i4 * (uint32_t)g.n5);
    } else {
        a.ci = idx / n456;
        const unsigned long long rem = idx % n456;
        a.i6 = (int)(rem % g.n6);
        a.i5 = (int)((rem / g.n6) % g.n5);
        a.i4 = (int)(rem / ((unsigned long long)g.n6 * g.n5));
    }
    return a;
}

// The FP64 part of a leaf (rectangle_size_bound.cu:180-205): box, tighten,
// R and the empty checks, then criterion 0 of the cascade (with F32, first
// on FP32 enclosures of the box and R, in FP64 where they leave it
// undecided).  Returns the leaf outcome (0, EMPTY, TRAPPED, or CRITICAL for
// undecided); fills leaf.box.
template <bool F32>
__device__ __forceinline__ int leaf_fp64(const SbTask& task, const SbCell& cell, const LeafAt& a, const LeafGrid& g,
                                         SbLeaf& leaf, sb::Vals& v) {
    leaf.box = sb::leaf_box_steps(task.box, task.step, cell.r3, a.i4, g.n4, a.i5, g.n5, a.i6, g.n6);
    v.R = sb::remaining_weight(leaf.box);
    if (sb::box_empty(leaf.box) || cc::empty(v.R)) return CC_SBT_LEAF_EMPTY;
    cc::trap_clear();
    if (F32) {
        static_assert(sb::SB_EVEN_SPLIT == 0, "criterion 0");
        const bool ok32 = sb::even_split_t(sb::enclose6(leaf.box), cc::f32::of(v.R));
        const bool decided = cc::trap_status() == cc::TRAP_NONE;
        cc::trap_clear();
        if (decided && !ok32) return CC_SBT_LEAF_CRITICAL;
        // an FP32 "true" is certified by the FP64 criterion below: its
        // verdict (the reference's) is the one used
    }
    const bool ok = sb::sb_criterion(0, leaf.box, v);
    int outcome;
    if (cc::trap_status() != cc::TRAP_NONE) outcome = CC_SBT_LEAF_TRAPPED;
    else outcome = ok ? 0 : CC_SBT_LEAF_CRITICAL;  // CRITICAL here = undecided
    cc::trap_clear();
    return outcome;
}

// Trace, queue and criticals of a warp's leaves after the leaf stage
__device__ __forceinline__ void leaf_emit(BlockTrace<CC_SBT_LEAF_OUTCOMES>& bt, bool valid, int outcome, SbLeaf& leaf,
                                          int gen, SbLeaf* __restrict__ q, unsigned long long* n_q,
                                          unsigned long long q_cap, SbLeaf* __restrict__ crit,
                                          unsigned long long crit_cap, SbCounters* c) {
    const bool undecided = valid && outcome == CC_SBT_LEAF_CRITICAL;
    trace_note(bt, valid && !undecided, valid ? leaf_key(gen, leaf, outcome) : 0, outcome);
    unsigned long long slot = warp_append(n_q, undecided, q_cap, &c->overflow);
    if (slot != ~0ULL) q[slot] = leaf;
    const bool trapped = valid && outcome == CC_SBT_LEAF_TRAPPED;
    slot = warp_append(&c->n_crit, trapped, crit_cap, &c->overflow);
    if (slot != ~0ULL) {
        leaf.idx |= 1ULL << 63;
        crit[slot] = leaf;
    }
}

// Leaves [l0, l1) of the cell grid without the pre-filter: the FP64 leaf
// stage on every leaf.  Undecided leaves go to queue `q`, trapped ones to the
// criticals.
__global__ void __launch_bounds__(kThreads) k_sbp_leaves(const SbTask* __restrict__ tasks,
                                                          const SbCell* __restrict__ cells, unsigned long long l0,
                                                          unsigned long long l1, LeafGrid g, SbLeaf* __restrict__ q,
                                                          unsigned long long* n_q, unsigned long long q_cap,
                                                          SbLeaf* __restrict__ crit, unsigned long long crit_cap,
                                                          SbCounters* c) {
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    SB_WARP_LOOP(l1 - l0) {
        const unsigned long long idx = l0 + base_ + (threadIdx.x & 31);
        const bool valid = idx < l1;
        int outcome = CC_SBT_LEAF_EMPTY;
        SbLeaf leaf;
        if (valid) {
            const LeafAt a = leaf_at(g, l0, l1, idx);
            const SbCell cell = cells[a.ci];
            const SbTask& task = tasks[cell.task];
            leaf.id = task.id;
            leaf.idx = pack_idx((int)cell.i3, a.i4, a.i5, a.i6);
            sb::Vals v;
            outcome = leaf_fp64<false>(task, cell, a, g, leaf, v);
        }
        const unsigned nv = __popc(__ballot_sync(0xffffffffu, valid));
        if ((threadIdx.x & 31) == 0) atomicAdd(&bt.extra, (unsigned long long)nv);
        leaf_emit(bt, valid, outcome, leaf, g.gen, q, n_q, q_cap, crit, crit_cap, c);
    }
    trace_flush(bt, c->leaf_counts, c, &c->leaf_evals);
}

// Leaves [l0, l1) through the FP32 pre-filter: a leaf it proves empty is
// decided (outcome EMPTY); the offsets (idx - l0) of the others go to the
// candidate list for k_sbp_leaf_check, so that the FP64 leaf stage runs on
// full warps of leaves that need it (most warps hold only empty leaves).
//
// Every leaf the pre-filter finds empty is certified in FP64.  For a fixed
// (cell, r4 piece, r5 piece) -- a row -- the FP64 test "la empty, or a
// tightened lower bound of r1..r5 at least its upper bound, or R.hi < 0" is
// monotone in the r6 piece index: the r6 lower bound fma(step, i6, lo) grows
// with i6 (the rounding is monotone), the tightened lower bounds are running
// maxima of it, the upper bounds of r1..r5 do not depend on it, and R.hi is a
// chain of round-up subtractions of those lower bounds.  So in each warp the
// first leaf of every run of FP32-empty leaves of a row (an anchor) goes to
// k_sbp_empty_cert, which runs that test in FP64: passing it there certifies
// the leaf and every later leaf of its row as empty in FP64 (the test is
// part of the reference's own emptiness test; the r6 piece's own width is
// left out, as the only term that is not monotone).
__global__ void __launch_bounds__(kThreads) k_sbp_leaf_filter(const SbTask* __restrict__ tasks,
                                                               const SbCell* __restrict__ cells, unsigned long long l0,
                                                               unsigned long long l1, LeafGrid g,
                                                               uint32_t* __restrict__ cand, unsigned long long* n_cand,
                                                               unsigned long long cand_cap,
                                                               uint32_t* __restrict__ anchors,
                                                               unsigned long long anchor_cap, SbCounters* c) {
    // the trace of the empty leaves, summed per thread and flushed once
    unsigned long long digest = 0;
    unsigned int n_empty = 0, n_valid = 0;
    // nearly every warp step has an anchor: they are staged per warp in
    // shared memory and appended 32 at a time (one global atomic per 32)
    __shared__ uint32_t s_anchor[kThreads / 32][64];
    uint32_t* stage = s_anchor[threadIdx.x >> 5];
    const unsigned lane = threadIdx.x & 31;
    int staged = 0;  // warp-uniform
    auto flush = [&](int k) {  // append the first k staged anchors (k <= 32), every lane calls it
        unsigned long long at = 0;
        if (lane == 0) at = atomicAdd(&c->n_anchor, (unsigned long long)k);
        at = __shfl_sync(0xffffffffu, at, 0);
        if ((int)lane < k) {
            if (at + lane < anchor_cap) anchors[at + lane] = stage[lane];
            else atomicExch(&c->overflow, 1ULL);
        }
        uint32_t rest = 0;  // the anchors left, moved to the front
        if ((int)lane < staged - k) rest = stage[k + lane];
        __syncwarp();
        if ((int)lane < staged - k) stage[lane] = rest;
        __syncwarp();
        staged -= k;
    };
    SB_WARP_LOOP(l1 - l0) {
        const unsigned long long idx = l0 + base_ + (threadIdx.x & 31);
        const bool valid = idx < l1;
        bool empty = false;
        unsigned long long row = ~0ULL;
        if (valid) {
            const LeafAt a = leaf_at(g, l0, l1, idx);
            const SbCell cell = cells[a.ci];
            const SbTask& task = tasks[cell.task];
            float lb_R, ub_R;
            const int pidx[3] = {a.i4, a.i5, a.i6}, pn[3] = {g.n4, g.n5, g.n6};
            empty = f32_leaf_empty(task.f, cell.r3_lo_dn, cell.r3_hi_up, pidx, pn, lb_R, ub_R);
            if (empty) {
                digest += sb::sb_trace_key_mixed(g.gen, task.id_mix, 2, (int)cell.i3, a.i4, a.i5, a.i6,
                                                 CC_SBT_LEAF_EMPTY);
                ++n_empty;
            }
            ++n_valid;
            row = (a.ci * (unsigned long long)g.n4 + (unsigned long long)a.i4) * (unsigned long long)g.n5 +
                  (unsigned long long)a.i5;
        }
        const unsigned long long prev_row = __shfl_up_sync(0xffffffffu, row, 1);
        const int prev_empty = __shfl_up_sync(0xffffffffu, empty ? 1 : 0, 1);
        const bool anchor = valid && empty && ((threadIdx.x & 31) == 0 || prev_row != row || !prev_empty);
        unsigned long long slot = warp_append(n_cand, valid && !empty, cand_cap, &c->overflow);
        if (slot != ~0ULL) cand[slot] = (uint32_t)(idx - l0);
        const unsigned ballot = __ballot_sync(0xffffffffu, anchor);
        if (anchor) stage[staged + __popc(ballot & ((1u << lane) - 1u))] = (uint32_t)(idx - l0);
        staged += __popc(ballot);
        __syncwarp();
        if (staged >= 32) flush(32);
    }
    if (staged > 0) flush(staged);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        digest += __shfl_xor_sync(0xffffffffu, digest, o);
        n_empty += __shfl_xor_sync(0xffffffffu, n_empty, o);
        n_valid += __shfl_xor_sync(0xffffffffu, n_valid, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (digest) atomicAdd(&c->digest, digest);
        if (n_empty) {
            atomicAdd(&c->leaf_counts[CC_SBT_LEAF_EMPTY], (unsigned long long)n_empty);
            atomicAdd(&c->fp32_empty, (unsigned long long)n_empty);
        }
        if (n_valid) atomicAdd(&c->leaf_evals, (unsigned long long)n_valid);
    }
}

// The FP64 certificate of the pre-filter's anchors (see k_sbp_leaf_filter).
__global__ void __launch_bounds__(kThreads) k_sbp_empty_cert(const SbTask* __restrict__ tasks,
                                                              const SbCell* __restrict__ cells, unsigned long long l0,
                                                              unsigned long long l1, LeafGrid g,
                                                              const uint32_t* __restrict__ anchors,
                                                              unsigned long long anchor_cap, SbCounters* c) {
    const unsigned long long n = c->n_anchor < anchor_cap ? c->n_anchor : anchor_cap;
    unsigned ok_n = 0, fail_n = 0;
    SB_WARP_LOOP(n) {
        const unsigned long long k = base_ + (threadIdx.x & 31);
        if (k < n) {
            const unsigned long long idx = l0 + anchors[k];
            const LeafAt a = leaf_at(g, l0, l1, idx);
            const SbCell cell = cells[a.ci];
            const SbTask& task = tasks[cell.task];
            const Box6 b = sb::leaf_box_steps(task.box, task.step, cell.r3, a.i4, g.n4, a.i5, g.n5, a.i6, g.n6);
            bool empty = cc::empty(b.la);
#pragma unroll
            for (int r = 0; r < 5; ++r) empty = empty || b.r[r].lo >= b.r[r].hi;
            empty = empty || sb::remaining_weight(b).hi < 0.0;
            if (empty) ++ok_n;
            else ++fail_n;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ok_n += __shfl_xor_sync(0xffffffffu, ok_n, o);
        fail_n += __shfl_xor_sync(0xffffffffu, fail_n, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (ok_n) atomicAdd(&c->empty_cert_ok, (unsigned long long)ok_n);
        if (fail_n) atomicAdd(&c->empty_cert_fail, (unsigned long long)fail_n);
    }
}

// The FP64 leaf stage on the pre-filter's candidates (offsets into the
// slice [l0, l1)); also the statistics of the pre-filter's widening of R.
__global__ void __launch_bounds__(kThreads) k_sbp_leaf_check(const SbTask* __restrict__ tasks,
                                                              const SbCell* __restrict__ cells, unsigned long long l0,
                                                              unsigned long long l1, LeafGrid g,
                                                              const uint32_t* __restrict__ cand,
                                                              const unsigned long long* n_cand,
                                                              unsigned long long cand_cap, SbLeaf* __restrict__ q,
                                                              unsigned long long* n_q, unsigned long long q_cap,
                                                              SbLeaf* __restrict__ crit, unsigned long long crit_cap,
                                                              SbCounters* c) {
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    __shared__ unsigned long long widen_n_b, widen_max_b;
    __shared__ double widen_sum_b;
    if (threadIdx.x == 0) widen_n_b = 0, widen_sum_b = 0.0, widen_max_b = 0;
    // per-thread statistics, reduced once per block
    unsigned int widen_n = 0;
    double widen_sum = 0.0, widen_max = 0.0;
    trace_init(bt);
    // an overflowed list (the slice is redone) is read no further than its capacity
    const unsigned long long total = *n_cand < cand_cap ? *n_cand : cand_cap;
    SB_WARP_LOOP(total) {
        const unsigned long long k = base_ + (threadIdx.x & 31);
        const bool valid = k < total;
        int outcome = CC_SBT_LEAF_EMPTY;
        SbLeaf leaf;
        if (valid) {
            const unsigned long long idx = l0 + cand[k];
            const LeafAt a = leaf_at(g, l0, l1, idx);
            const SbCell cell = cells[a.ci];
            const SbTask& task = tasks[cell.task];
            leaf.id = task.id;
            leaf.idx = pack_idx((int)cell.i3, a.i4, a.i5, a.i6);
            float lb_R, ub_R;
            const int pidx[3] = {a.i4, a.i5, a.i6}, pn[3] = {g.n4, g.n5, g.n6};
            f32_leaf_empty(task.f, cell.r3_lo_dn, cell.r3_hi_up, pidx, pn, lb_R, ub_R);
            sb::Vals v;
            outcome = leaf_fp64<true>(task, cell, a, g, leaf, v);
            if (v.R.hi > v.R.lo) {  // widening of the FP32 bounds of R over FP64 R
                const double w = ((double)ub_R - (double)(lb_R > 0.0f ? lb_R : 0.0f)) / (v.R.hi - v.R.lo);
                ++widen_n;
                widen_sum += w;
                widen_max = w > widen_max ? w : widen_max;
            }
        }
        leaf_emit(bt, valid, outcome, leaf, g.gen, q, n_q, q_cap, crit, crit_cap, c);
    }
    if (widen_n) {
        atomicAdd(&widen_n_b, (unsigned long long)widen_n);
        atomicAdd(&widen_sum_b, widen_sum);
        atomicMax(&widen_max_b, (unsigned long long)__double_as_longlong(widen_max));
    }
    trace_flush(bt, c->leaf_counts, c, nullptr);
    if (threadIdx.x == 0 && widen_n_b) {
        atomicAdd(&c->widen_count, widen_n_b);
        atomicAdd(&c->widen_sum, widen_sum_b);
        atomicMax(&c->widen_max_bits, widen_max_b);
    }
}

// The plain form: one thread runs a leaf's whole cascade, as the reference's
// kernel does (rectangle_size_bound.cu:180-231); no queues, no pre-filter.
__global__ void __launch_bounds__(kThreads) k_sbp_leaves_plain(const SbTask* __restrict__ tasks,
                                                                const SbCell* __restrict__ cells,
                                                                unsigned long long l0, unsigned long long l1, LeafGrid g,
                                                                SbLeaf* __restrict__ crit, unsigned long long crit_cap,
                                                                SbCounters* c) {
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    const unsigned long long n456 = (unsigned long long)g.n4 * g.n5 * g.n6;
    SB_WARP_LOOP(l1 - l0) {
        const unsigned long long idx = l0 + base_ + (threadIdx.x & 31);
        const bool valid = idx < l1;
        int outcome = CC_SBT_LEAF_EMPTY;
        SbLeaf leaf;
        if (valid) {
            const unsigned long long ci = idx / n456, rem = idx % n456;
            const int i6 = (int)(rem % g.n6);
            const int i5 = (int)((rem / g.n6) % g.n5);
            const int i4 = (int)(rem / ((unsigned long long)g.n6 * g.n5));
            const SbCell cell = cells[ci];
            const SbTask& task = tasks[cell.task];
            leaf.box = sb::leaf_box(task.box, cell.r3, i4, g.n4, i5, g.n5, i6, g.n6);
            leaf.id = task.id;
            leaf.idx = pack_idx((int)cell.i3, i4, i5, i6);
            outcome = sb::leaf_outcome(leaf.box);
        }
        trace_note(bt, valid, valid ? leaf_key(g.gen, leaf, outcome) : 0, outcome);
        const unsigned nv = __popc(__ballot_sync(0xffffffffu, valid));
        if ((threadIdx.x & 31) == 0) atomicAdd(&bt.extra, (unsigned long long)nv);
        const bool to_crit = valid && (outcome == CC_SBT_LEAF_CRITICAL || outcome == CC_SBT_LEAF_TRAPPED);
        unsigned long long slot = warp_append(&c->n_crit, to_crit, crit_cap, &c->overflow);
        if (slot != ~0ULL) {
            if (outcome == CC_SBT_LEAF_TRAPPED) leaf.idx |= 1ULL << 63;
            crit[slot] = leaf;
        }
    }
    trace_flush(bt, c->leaf_counts, c, &c->leaf_evals);
}

// Criterion K on the undecided leaves of `qin` (rectangle_size_bound.cu:
// 199-231).  Undecided leaves go to `qout`, or to the criticals after the
// last criterion; a trap sends the leaf to the criticals, flagged.
template <int K>
__global__ void __launch_bounds__(kThreads) k_sbp_pass(const SbLeaf* __restrict__ qin, const unsigned long long* n_in,
                                                        SbLeaf* __restrict__ qout, unsigned long long* n_out,
                                                        unsigned long long q_cap, SbLeaf* __restrict__ crit,
                                                        unsigned long long crit_cap, int gen, SbCounters* c) {
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    const unsigned long long total = *n_in;
    constexpr bool kLast = K == sb::SB_NUM_CRITERIA - 1;
    SB_WARP_LOOP(total) {
        const unsigned long long idx = base_ + (threadIdx.x & 31);
        const bool valid = idx < total;
        int outcome = CC_SBT_LEAF_CRITICAL;
        SbLeaf leaf;
        if (valid) {
            leaf = qin[idx];
            sb::Vals v;
            v.R = sb::remaining_weight(leaf.box);
            cc::trap_clear();
            const bool ok = sb::sb_criterion(K, leaf.box, v);
            if (cc::trap_status() != cc::TRAP_NONE) outcome = CC_SBT_LEAF_TRAPPED;
            else if (ok) outcome = K;
            cc::trap_clear();
        }
        const bool undecided = valid && outcome == CC_SBT_LEAF_CRITICAL;
        const bool decided = valid && (!undecided || kLast);
        trace_note(bt, decided, decided ? leaf_key(gen, leaf, outcome) : 0, outcome);
        if (!kLast) {
            unsigned long long slot = warp_append(n_out, undecided, q_cap, &c->overflow);
            if (slot != ~0ULL) qout[slot] = leaf;
        }
        const bool to_crit = valid && (outcome == CC_SBT_LEAF_TRAPPED || (kLast && undecided));
        unsigned long long slot = warp_append(&c->n_crit, to_crit, crit_cap, &c->overflow);
        if (slot != ~0ULL) {
            if (outcome == CC_SBT_LEAF_TRAPPED) leaf.idx |= 1ULL << 63;
            crit[slot] = leaf;
        }
    }
    trace_flush(bt, c->leaf_counts, c, nullptr);
}

// FP32-first passes.  A criterion with an FP32 form is a sequence of
// placements tried in order until one works; placements 0..kPlacements-1
// are templates over the interval type and run first on FP32 enclosures of
// the leaf box: the first that works decided, or every one decided not to
// work, is the FP64 outcome up to there (cc_f32.cuh).  A leaf whose
// evaluation met an undecided comparison at placement k, or whose FP32
// placements all failed when FP64-only placements follow (kTail), becomes a
// job -- its queue index, and k (or kPlacements) in bits 28..30 -- for
// k_sbp_fp64<K>, which resumes the FP64 criterion at that placement.
template <int K>
struct F32Pass;
template <>
struct F32Pass<sb::SB_UNEVEN_SPLIT> {  // one placement, the whole criterion
    static constexpr int kPlacements = 1;
    static constexpr bool kTail = false;
    template <class I>
    __device__ static bool placement(const sb::Box6T<I>& b, int) {
        return sb::uneven_split_t(b);
    }
    __device__ static bool fp64_from(const Box6& b, const sb::Vals& v, int) { return sb::uneven_split_recursion(b, v); }
};
template <>
struct F32Pass<sb::SB_MULTI_DISK_STRIP> {  // placements 0..6; three rows in FP64 only
    static constexpr int kPlacements = sb::kStripPlacements - 1;
    static constexpr bool kTail = true;
    template <class I>
    __device__ static bool placement(const sb::Box6T<I>& b, int k) {
        return sb::strip_placement(b, k);
    }
    __device__ static bool fp64_from(const Box6& b, const sb::Vals& v, int from) {
        return sb::multi_disk_strip_from(b, v, from);
    }
};

constexpr uint32_t kF32JobIndexBits = 28;  // queue indices are below 2^26 (the largest slice)
static_assert(F32Pass<sb::SB_MULTI_DISK_STRIP>::kPlacements < 8, "placement index in bits 28..30");

template <int K>
__global__ void __launch_bounds__(kThreads) k_sbp_f32(const SbLeaf* __restrict__ qin, const unsigned long long* n_in,
                                                       uint32_t* __restrict__ jobs, unsigned long long* n_jobs,
                                                       unsigned long long job_cap, SbLeaf* __restrict__ qout,
                                                       unsigned long long* n_out, unsigned long long q_cap, int gen,
                                                       SbCounters* c) {
    using P = F32Pass<K>;
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    const unsigned long long total = *n_in;
    SB_WARP_LOOP(total) {
        const unsigned long long idx = base_ + (threadIdx.x & 31);
        const bool valid = idx < total;
        bool works = false, undecided = false;
        int from = P::kPlacements;
        SbLeaf leaf;
        if (valid) {
            leaf = qin[idx];
            const sb::Box6T<cc::f32::IvF> e = sb::enclose6(leaf.box);
            for (int k = 0; k < P::kPlacements; ++k) {
                cc::trap_clear();
                const bool ok = P::placement(e, k);
                if (cc::trap_status() != cc::TRAP_NONE) {
                    from = k;
                    undecided = true;
                    break;
                }
                if (ok) {
                    works = true;
                    from = k;
                    break;
                }
            }
            cc::trap_clear();
        }
        // a placement that works on the enclosures becomes an FP64
        // certification job at that placement (bit 31): k_sbp_fp64 decides
        // and traces the leaf with the FP64 criterion from there
        const bool job = valid && (works || undecided || P::kTail);
        unsigned long long slot = warp_append(n_jobs, job, job_cap, &c->overflow);
        if (slot != ~0ULL)
            jobs[slot] = (uint32_t)idx | ((uint32_t)from << kF32JobIndexBits) | (works ? (1u << 31) : 0u);
        // decided not to work, nothing after the FP32 placements: next pass
        slot = warp_append(n_out, valid && !works && !job, q_cap, &c->overflow);
        if (slot != ~0ULL) qout[slot] = leaf;
    }
    trace_flush(bt, c->leaf_counts, c, nullptr);
}

template <int K>
__global__ void __launch_bounds__(kThreads) k_sbp_fp64(const SbLeaf* __restrict__ qin,
                                                        const uint32_t* __restrict__ jobs,
                                                        const unsigned long long* n_jobs, unsigned long long job_cap,
                                                        SbLeaf* __restrict__ qout, unsigned long long* n_out,
                                                        unsigned long long q_cap, SbLeaf* __restrict__ crit,
                                                        unsigned long long crit_cap, int gen, SbCounters* c) {
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    const unsigned long long total = *n_jobs < job_cap ? *n_jobs : job_cap;
    unsigned cert_ok = 0, cert_fail = 0;
    SB_WARP_LOOP(total) {
        const unsigned long long k = base_ + (threadIdx.x & 31);
        const bool valid = k < total;
        int outcome = CC_SBT_LEAF_CRITICAL;
        SbLeaf leaf;
        if (valid) {
            const uint32_t job = jobs[k];
            leaf = qin[job & ((1u << kF32JobIndexBits) - 1)];
            sb::Vals v;
            v.R = sb::remaining_weight(leaf.box);
            cc::trap_clear();
            const bool ok = F32Pass<K>::fp64_from(leaf.box, v, (int)((job >> kF32JobIndexBits) & 7));
            if (cc::trap_status() != cc::TRAP_NONE) outcome = CC_SBT_LEAF_TRAPPED;
            else if (ok) outcome = K;
            cc::trap_clear();
            if (job >> 31) {  // a certification: the FP32 placement worked
                if (outcome == K) ++cert_ok;
                else ++cert_fail;
            }
        }
        const bool undecided = valid && outcome == CC_SBT_LEAF_CRITICAL;
        const bool decided = valid && !undecided;
        trace_note(bt, decided, decided ? leaf_key(gen, leaf, outcome) : 0, outcome);
        unsigned long long slot = warp_append(n_out, undecided, q_cap, &c->overflow);
        if (slot != ~0ULL) qout[slot] = leaf;
        const bool to_crit = valid && outcome == CC_SBT_LEAF_TRAPPED;
        slot = warp_append(&c->n_crit, to_crit, crit_cap, &c->overflow);
        if (slot != ~0ULL) {
            leaf.idx |= 1ULL << 63;
            crit[slot] = leaf;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cert_ok += __shfl_xor_sync(0xffffffffu, cert_ok, o);
        cert_fail += __shfl_xor_sync(0xffffffffu, cert_fail, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (cert_ok) atomicAdd(&c->cert_ok, (unsigned long long)cert_ok);
        if (cert_fail) atomicAdd(&c->cert_fail, (unsigned long long)cert_fail);
    }
    trace_flush(bt, c->leaf_counts, c, nullptr);
}

// A criterion made of independent placements tried in order until one
// works (r1 in a corner: nine placements) runs one placement per thread; the
// resolve kernel then combines them as the sequential loop would: the first
// placement that works decides, and only traps in placements up to that one
// count.  masks[2 * leaf] = placements that worked, masks[2 * leaf + 1] =
// placements that reached a trap site.
template <int K>
struct SplitCriterion;
template <>
struct SplitCriterion<sb::SB_R1_CORNER_EXPLICIT> {
    static constexpr int kItems = sb::kR1CornerItems;
    __device__ static bool item(const Box6& b, const sb::Vals& v, int i) { return sb::r1_corner_item(b, v, i); }
};

// r1 in a corner, first half: every (leaf, placement), placement-major.
// Placement 8 runs whole here; placements 0..7 run their start (the weight
// bound and the corner disk) and, where that does not already fail, become
// a job for the backtracking kernel, so that the backtracking (93 % of the
// criterion's operations, reached by about a fifth of the placements) runs
// on full warps.  A job is (leaf << 4) | placement.
// With f32, a placement's start is decided on FP32 enclosures first (the
// FP64 start where they leave it undecided).
__global__ void __launch_bounds__(kThreads) k_sbp_r1c_start(const SbLeaf* __restrict__ qin,
                                                             const unsigned long long* n_in, uint32_t* masks,
                                                             unsigned long long* jobs, unsigned long long* n_jobs,
                                                             unsigned long long job_cap, SbCounters* c, int f32) {
    constexpr int I = sb::kR1CornerItems;
    const unsigned long long nl = *n_in, total = nl * (unsigned long long)I;
    SB_WARP_LOOP(total) {
        const unsigned long long idx = base_ + (threadIdx.x & 31);
        const bool valid = idx < total;
        bool job = false;
        unsigned long long leaf = 0;
        int i = 0;
        if (valid) {
            i = (int)(idx / nl);
            leaf = idx - (unsigned long long)i * nl;
            const Box6 box = qin[leaf].box;
            cc::trap_clear();
            bool ok = false;
            if (i == 8) {
                ok = sb::r1_corner_r34_and_r2(box);
            } else {
                bool decided = false;
                if (f32) {
                    const sb::Box6T<cc::f32::IvF> e = sb::enclose6(box);
                    job = sb::r1_corner_starts_f32(e, sb::remaining_weight(e), i);
                    decided = cc::trap_status() == cc::TRAP_NONE;
                    cc::trap_clear();
                }
                if (!decided) {
                    sb::Vals v;
                    v.R = sb::remaining_weight(box);
                    sb::CornerStart st;
                    job = sb::r1_corner_start(box, v, i, st);
                }
            }
            const bool trapped = cc::trap_status() != cc::TRAP_NONE;
            cc::trap_clear();
            if (ok) atomicOr(&masks[2 * leaf], 1u << i);
            if (trapped) atomicOr(&masks[2 * leaf + 1], 1u << i);
        }
        unsigned long long slot = warp_append(n_jobs, job, job_cap, &c->overflow);
        if (slot != ~0ULL) jobs[slot] = (leaf << 4) | (unsigned long long)i;
    }
}

// r1 in a corner, second half: the backtracking of the jobs (the start is
// recomputed; same operations, same values).  Run FP32-first: the
// backtracking on FP32 enclosures of the group heights
// (corner_groups_reach_t<Fv>, its bisections on FP32 decisions alone); a job
// whose evaluation it leaves undecided, or whose start reached a trap site,
// goes to `jobs64` for k_sbp_r1c_reach64.
__global__ void __launch_bounds__(kThreads) k_sbp_r1c_reach(const SbLeaf* __restrict__ qin,
                                                             const unsigned long long* __restrict__ jobs,
                                                             const unsigned long long* n_jobs,
                                                             unsigned long long job_cap, uint32_t* masks,
                                                             unsigned long long* __restrict__ jobs64,
                                                             unsigned long long* n64, SbCounters* c) {
    const unsigned long long total = *n_jobs < job_cap ? *n_jobs : job_cap;
    SB_WARP_LOOP(total) {
        const unsigned long long k = base_ + (threadIdx.x & 31);
        const bool valid = k < total;
        bool need64 = false;
        unsigned long long job = 0;
        if (valid) {
            job = jobs[k];
            const unsigned long long leaf = job >> 4;
            const int i = (int)(job & 15);
            const Box6 box = qin[leaf].box;
            sb::Vals v;
            v.R = sb::remaining_weight(box);
            cc::trap_clear();
            sb::CornerStart st;
            const bool started = sb::r1_corner_start(box, v, i, st);
            if (cc::trap_status() != cc::TRAP_NONE || !started) {
                need64 = true;
            } else {
                const bool ok = sb::corner_groups_reach_t<cc::f32::Fv>(box, 2 + i / 2, st.cross, st.first, st.limit);
                // undecided, or "works" on the enclosures: the FP64
                // backtracking decides (and so certifies a "works")
                if (cc::trap_status() != cc::TRAP_NONE || ok) need64 = true;
            }
            cc::trap_clear();
        }
        const unsigned long long slot = warp_append(n64, need64, job_cap, &c->overflow);
        if (slot != ~0ULL) jobs64[slot] = job;
    }
}

// the FP64 backtracking of the jobs
__global__ void __launch_bounds__(kThreads) k_sbp_r1c_reach64(const SbLeaf* __restrict__ qin,
                                                               const unsigned long long* __restrict__ jobs,
                                                               const unsigned long long* n_jobs,
                                                               unsigned long long job_cap, uint32_t* masks) {
    const unsigned long long total = *n_jobs < job_cap ? *n_jobs : job_cap;
    for (unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long job = jobs[idx];
        const unsigned long long leaf = job >> 4;
        const int i = (int)(job & 15);
        const Box6 box = qin[leaf].box;
        sb::Vals v;
        v.R = sb::remaining_weight(box);
        cc::trap_clear();
        sb::CornerStart st;
        bool ok = sb::r1_corner_start(box, v, i, st);
        ok = ok && sb::corner_groups_reach(box, 2 + i / 2, st.cross, st.first, st.limit);
        const bool trapped = cc::trap_status() != cc::TRAP_NONE;
        cc::trap_clear();
        if (ok) atomicOr(&masks[2 * leaf], 1u << i);
        if (trapped) atomicOr(&masks[2 * leaf + 1], 1u << i);
    }
}

template <int K>
__global__ void __launch_bounds__(kThreads) k_sbp_split_resolve(const SbLeaf* __restrict__ qin,
                                                                 const unsigned long long* n_in,
                                                                 const uint32_t* __restrict__ masks,
                                                                 SbLeaf* __restrict__ qout, unsigned long long* n_out,
                                                                 unsigned long long q_cap, SbLeaf* __restrict__ crit,
                                                                 unsigned long long crit_cap, int gen, SbCounters* c) {
    constexpr int I = SplitCriterion<K>::kItems;
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    const unsigned long long total = *n_in;
    SB_WARP_LOOP(total) {
        const unsigned long long idx = base_ + (threadIdx.x & 31);
        const bool valid = idx < total;
        int outcome = CC_SBT_LEAF_CRITICAL;  // here: undecided
        SbLeaf leaf;
        if (valid) {
            leaf = qin[idx];
            const uint32_t ok = masks[2 * idx], trapped = masks[2 * idx + 1];
            const uint32_t first = ok ? (uint32_t)(__ffs(ok) - 1) : (uint32_t)(I - 1);
            const uint32_t seen = (2u << first) - 1u;
            if (trapped & seen) outcome = CC_SBT_LEAF_TRAPPED;
            else if (ok) outcome = K;
        }
        const bool undecided = valid && outcome == CC_SBT_LEAF_CRITICAL;
        const bool decided = valid && !undecided;
        trace_note(bt, decided, decided ? leaf_key(gen, leaf, outcome) : 0, outcome);
        unsigned long long slot = warp_append(n_out, undecided, q_cap, &c->overflow);
        if (slot != ~0ULL) qout[slot] = leaf;
        slot = warp_append(&c->n_crit, valid && outcome == CC_SBT_LEAF_TRAPPED, crit_cap, &c->overflow);
        if (slot != ~0ULL) {
            leaf.idx |= 1ULL << 63;
            crit[slot] = leaf;
        }
    }
    trace_flush(bt, c->leaf_counts, c, nullptr);
}

// Seven-disk strategies, prefix (seven_disk_strategies.cu:1397-1432): decided
// leaves are traced here, the others become jobs of 16 r7 pieces.
__global__ void __launch_bounds__(kThreads) k_sbp_seven_prefix(const SbLeaf* __restrict__ qin,
                                                                const unsigned long long* n_in, SevenJob* __restrict__ jobs,
                                                                unsigned long long* n_jobs, unsigned long long job_cap,
                                                                SbLeaf* __restrict__ crit, unsigned long long crit_cap,
                                                                int gen, SbCounters* c) {
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    const unsigned long long total = *n_in;
    SB_WARP_LOOP(total) {
        const unsigned long long idx = base_ + (threadIdx.x & 31);
        const bool valid = idx < total;
        int outcome = CC_SBT_LEAF_CRITICAL;  // here: pieces to check
        SbLeaf leaf;
        sb::SevenPrefix pre;
        if (valid) {
            leaf = qin[idx];
            sb::Vals v;
            v.R = sb::remaining_weight(leaf.box);
            cc::trap_clear();
            const bool ok = sb::seven_disk_prefix(leaf.box, v, pre);
            if (cc::trap_status() != cc::TRAP_NONE) outcome = CC_SBT_LEAF_TRAPPED;
            else if (ok) outcome = sb::SB_SEVEN_DISK;
            cc::trap_clear();
        }
        const bool open = valid && outcome == CC_SBT_LEAF_CRITICAL;
        const bool decided = valid && !open;
        trace_note(bt, decided, decided ? leaf_key(gen, leaf, outcome) : 0, outcome);
        unsigned long long slot = warp_append(n_jobs, open, job_cap, &c->overflow);
        if (slot != ~0ULL) jobs[slot] = SevenJob{pre, (uint32_t)idx, 0u, 0u, 0u};
        slot = warp_append(&c->n_crit, valid && outcome == CC_SBT_LEAF_TRAPPED, crit_cap, &c->overflow);
        if (slot != ~0ULL) {
            leaf.idx |= 1ULL << 63;
            crit[slot] = leaf;
        }
    }
    trace_flush(bt, c->leaf_counts, c, nullptr);
}

// Seven-disk strategies, one r7 piece per thread (:1434-1493)
__global__ void __launch_bounds__(kThreads) k_sbp_seven_pieces(const SbLeaf* __restrict__ qin,
                                                                SevenJob* __restrict__ jobs,
                                                                const unsigned long long* n_jobs) {
    // piece-major order: the lanes of a warp check the same piece of
    // consecutive jobs, so they start on the same code path
    const unsigned long long nj = *n_jobs, total = nj * 16ULL;
    for (unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (unsigned long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx / nj);
        SevenJob& job = jobs[idx - (unsigned long long)k * nj];
        const Box6 box = qin[job.leaf].box;
        sb::Vals v;
        v.R = sb::remaining_weight(box);
        cc::trap_clear();
        const bool ok = sb::seven_disk_piece(box, v, job.pre, k);
        const bool trapped = cc::trap_status() != cc::TRAP_NONE;
        cc::trap_clear();
        if (!ok) atomicOr(&job.fail_mask, 1u << k);
        if (trapped) atomicOr(&job.trap_mask, 1u << k);
    }
}

// Seven-disk strategies, the pieces' outcomes combined as the sequential loop
// would: it stops at the first piece that is not covered, so only traps in
// pieces up to that one count.
__global__ void __launch_bounds__(kThreads) k_sbp_seven_resolve(const SbLeaf* __restrict__ qin,
                                                                 const SevenJob* __restrict__ jobs,
                                                                 const unsigned long long* n_jobs,
                                                                 SbLeaf* __restrict__ crit, unsigned long long crit_cap,
                                                                 int gen, SbCounters* c) {
    __shared__ BlockTrace<CC_SBT_LEAF_OUTCOMES> bt;
    trace_init(bt);
    const unsigned long long total = *n_jobs;
    SB_WARP_LOOP(total) {
        const unsigned long long idx = base_ + (threadIdx.x & 31);
        const bool valid = idx < total;
        int outcome = sb::SB_SEVEN_DISK;
        SbLeaf leaf;
        if (valid) {
            const SevenJob job = jobs[idx];
            leaf = qin[job.leaf];
            const uint32_t first_fail = job.fail_mask ? (uint32_t)(__ffs(job.fail_mask) - 1) : 15u;
            const uint32_t seen = first_fail >= 15u ? 0xffffu : ((2u << first_fail) - 1u);
            if (job.trap_mask & seen) outcome = CC_SBT_LEAF_TRAPPED;
            else if (job.fail_mask) outcome = CC_SBT_LEAF_CRITICAL;
        }
        trace_note(bt, valid, valid ? leaf_key(gen, leaf, outcome) : 0, outcome);
        const bool to_crit = valid && outcome != sb::SB_SEVEN_DISK;
        unsigned long long slot = warp_append(&c->n_crit, to_crit, crit_cap, &c->overflow);
        if (slot != ~0ULL) {
            if (outcome == CC_SBT_LEAF_TRAPPED) leaf.idx |= 1ULL << 63;
            crit[slot] = leaf;
        }
    }
    trace_flush(bt, c->leaf_counts, c, nullptr);
}

// ---------------------------------------------------------------- host side
enum Slot { S_PARENTS = 0, S_TASKS, S_CELLS, S_Q0, S_Q1, S_CRIT, S_COUNTERS, S_JOBS };
constexpr int kSlotBase = 24;  // handle buffer slots 24..31

struct Engine {
    cc_handle* h;
    cudaStream_t s;
    int grid;
    unsigned long long task_chunk, cell_cap, slice, crit_cap;
    unsigned long long range;  // leaves per slice, adapted as the proof runs
    bool plain = false;        // one thread per leaf runs the whole cascade
    bool fp32 = true;          // FP32 emptiness pre-filter in the leaf kernel
    Box6* parents = nullptr;
    SbTask* tasks = nullptr;
    SbCell* cells = nullptr;
    SbLeaf* q[2] = {nullptr, nullptr};
    SbLeaf* crit = nullptr;
    SevenJob* jobs = nullptr;
    SbCounters* dc = nullptr;
    SbCounters* backup = nullptr;  // snapshot of dc taken before each slice
    SbCounters* hc = nullptr;      // pinned
    std::vector<SbLeaf> found;
    uint64_t launches = 0;
    uint64_t empty_anchors = 0;  // anchors of empty leaves certified in FP64
};

// criteria K..12 as passes over the compacted queue, then the seven-disk
// kernels; the undecided leaves of one pass are the next one's input
template <int K>
int launch_passes(Engine& e, int gen, int src) {
    if constexpr (K == sb::SB_R1_CORNER_EXPLICIT) {
        const int dst = src ^ 1;
        uint32_t* masks = reinterpret_cast<uint32_t*>(e.jobs);  // free until the seven-disk kernels
        // the jobs live in the output queue's memory until the resolve kernel
        // writes the queue; n_q[dst] counts them until then
        unsigned long long* r1c_jobs = reinterpret_cast<unsigned long long*>(e.q[dst]);
        static_assert(sizeof(SbLeaf) >= 16 * sizeof(unsigned long long), "16 jobs per queue record");
        CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_q[dst], 0, sizeof(unsigned long long), e.s));
        CC_CUDA(e.h, cudaMemsetAsync(masks, 0, e.slice * 2 * sizeof(uint32_t), e.s));
        k_sbp_r1c_start<<<e.grid, kThreads, 0, e.s>>>(e.q[src], &e.dc->n_q[src], masks, r1c_jobs, &e.dc->n_q[dst],
                                                       e.slice * 8, e.dc, e.fp32 ? 1 : 0);
        CC_LAUNCHED(e.h);
        const unsigned long long job_cap = e.slice * 8;
        if (e.fp32) {  // FP32-first; the FP64 jobs in the queue memory's second half
            unsigned long long* jobs64 = r1c_jobs + job_cap;
            CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_f32_jobs, 0, sizeof(unsigned long long), e.s));
            k_sbp_r1c_reach<<<e.grid, kThreads, 0, e.s>>>(e.q[src], r1c_jobs, &e.dc->n_q[dst], job_cap, masks, jobs64,
                                                           &e.dc->n_f32_jobs, e.dc);
            CC_LAUNCHED(e.h);
            k_sbp_r1c_reach64<<<e.grid, kThreads, 0, e.s>>>(e.q[src], jobs64, &e.dc->n_f32_jobs, job_cap, masks);
            CC_LAUNCHED(e.h);
            e.launches++;
        } else {
            k_sbp_r1c_reach64<<<e.grid, kThreads, 0, e.s>>>(e.q[src], r1c_jobs, &e.dc->n_q[dst], job_cap, masks);
            CC_LAUNCHED(e.h);
        }
        CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_q[dst], 0, sizeof(unsigned long long), e.s));
        k_sbp_split_resolve<K><<<e.grid, kThreads, 0, e.s>>>(e.q[src], &e.dc->n_q[src], masks, e.q[dst],
                                                              &e.dc->n_q[dst], e.slice, e.crit, e.crit_cap, gen, e.dc);
        CC_LAUNCHED(e.h);
        e.launches += 3;
        return launch_passes<K + 1>(e, gen, dst);
    } else if constexpr (K < sb::SB_SEVEN_DISK) {
        const int dst = src ^ 1;
        if constexpr (K == sb::SB_UNEVEN_SPLIT || K == sb::SB_MULTI_DISK_STRIP) {
            if (e.fp32) {
                // the jobs live in the seven-disk job buffer (free until then)
                uint32_t* jobs = reinterpret_cast<uint32_t*>(e.jobs);
                const unsigned long long job_cap = e.slice * (sizeof(SevenJob) / sizeof(uint32_t));
                CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_q[dst], 0, sizeof(unsigned long long), e.s));
                CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_f32_jobs, 0, sizeof(unsigned long long), e.s));
                k_sbp_f32<K><<<e.grid, kThreads, 0, e.s>>>(e.q[src], &e.dc->n_q[src], jobs, &e.dc->n_f32_jobs, job_cap,
                                                            e.q[dst], &e.dc->n_q[dst], e.slice, gen, e.dc);
                CC_LAUNCHED(e.h);
                k_sbp_fp64<K><<<e.grid, kThreads, 0, e.s>>>(e.q[src], jobs, &e.dc->n_f32_jobs, job_cap, e.q[dst],
                                                             &e.dc->n_q[dst], e.slice, e.crit, e.crit_cap, gen, e.dc);
                CC_LAUNCHED(e.h);
                e.launches += 2;
                return launch_passes<K + 1>(e, gen, dst);
            }
        }
        CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_q[dst], 0, sizeof(unsigned long long), e.s));
        k_sbp_pass<K><<<e.grid, kThreads, 0, e.s>>>(e.q[src], &e.dc->n_q[src], e.q[dst], &e.dc->n_q[dst], e.slice,
                                                     e.crit, e.crit_cap, gen, e.dc);
        CC_LAUNCHED(e.h);
        e.launches++;
        return launch_passes<K + 1>(e, gen, dst);
    } else {
        static_assert(K == sb::SB_NUM_CRITERIA - 1, "the seven-disk strategies are the last criterion");
        unsigned long long* n_jobs = &e.dc->n_q[src ^ 1];  // the free queue's counter counts the jobs
        CC_CUDA(e.h, cudaMemsetAsync(n_jobs, 0, sizeof(unsigned long long), e.s));
        k_sbp_seven_prefix<<<e.grid, kThreads, 0, e.s>>>(e.q[src], &e.dc->n_q[src], e.jobs, n_jobs, e.slice, e.crit,
                                                          e.crit_cap, gen, e.dc);
        CC_LAUNCHED(e.h);
        k_sbp_seven_pieces<<<e.grid, kThreads, 0, e.s>>>(e.q[src], e.jobs, n_jobs);
        CC_LAUNCHED(e.h);
        k_sbp_seven_resolve<<<e.grid, kThreads, 0, e.s>>>(e.q[src], e.jobs, n_jobs, e.crit, e.crit_cap, gen, e.dc);
        CC_LAUNCHED(e.h);
        e.launches += 3;
        return CC_OK;
    }
}

int sync_counters(Engine& e) {
    CC_CUDA(e.h, cudaMemcpyAsync(e.hc, e.dc, sizeof(SbCounters), cudaMemcpyDeviceToHost, e.s));
    CC_CUDA(e.h, cudaStreamSynchronize(e.s));
    if (e.hc->overflow) return ccrt::fail(e.h, CC_ERR_QUEUE_OVERFLOW, "cc_sb_prove: queue overflow");
    return CC_OK;
}

int drain_criticals(Engine& e) {
    const unsigned long long n = e.hc->n_crit;
    if (!n) return CC_OK;
    size_t old = e.found.size();
    e.found.resize(old + n);
    CC_CUDA(e.h, cudaMemcpyAsync(e.found.data() + old, e.crit, n * sizeof(SbLeaf), cudaMemcpyDeviceToHost, e.s));
    CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_crit, 0, sizeof(unsigned long long), e.s));
    CC_CUDA(e.h, cudaStreamSynchronize(e.s));
    e.hc->n_crit = 0;
    return CC_OK;
}

// one generation: every task of every parent (find_critical_intervals_in)
// A generation after the first stops at a chunk boundary when cc_interrupt
// was called (the initial pass is not interruptible, as in the reference:
// rectangle_size_bound.cu:325, 341).
int run_generation(Engine& e, const std::vector<Box6>& parents, int gen, int nla, const int* rn,
                   unsigned long long task_lo = 0, unsigned long long task_hi = ~0ULL) {
    int st;
    void* p;
    if ((st = ccrt::ensure(e.h, kSlotBase + S_PARENTS, parents.size() * sizeof(Box6), &p))) return st;
    e.parents = (Box6*)p;
    CC_CUDA(e.h, cudaMemcpyAsync(e.parents, parents.data(), parents.size() * sizeof(Box6), cudaMemcpyHostToDevice, e.s));
    const unsigned long long per_parent = (unsigned long long)nla * rn[0] * rn[1];
    const unsigned long long ntasks = parents.size() * per_parent;
    const unsigned long long n456 = (unsigned long long)rn[3] * rn[4] * rn[5];
    // a chunk's cells must fit the cell queue even if every task survives
    unsigned long long chunk = e.cell_cap / (unsigned long long)rn[2];
    if (chunk > e.task_chunk) chunk = e.task_chunk;
    if (chunk < 1) chunk = 1;
    TaskGrid tg{gen, nla, rn[0], rn[1], rn[3], rn[4], rn[5], per_parent};
    LeafGrid lg{gen, rn[3], rn[4], rn[5], 0u, 0ULL};
    const unsigned long long t_end = task_hi < ntasks ? task_hi : ntasks;
    for (unsigned long long t0 = task_lo; t0 < t_end; t0 += chunk) {
        if (gen > 0 && e.h->interrupt.load()) return CC_ERR_INTERRUPTED;
        const unsigned long long t1 = t0 + chunk < t_end ? t0 + chunk : t_end;
        CC_CUDA(e.h, cudaMemsetAsync(e.dc, 0, 2 * sizeof(unsigned long long), e.s));  // n_task, n_cell
        int tgrid = (int)std::min<unsigned long long>((t1 - t0 + kThreads - 1) / kThreads, (unsigned long long)e.grid);
        k_sbp_tasks<<<tgrid, kThreads, 0, e.s>>>(e.parents, t0, t1, tg, e.tasks, chunk, e.dc);
        CC_LAUNCHED(e.h);
        k_sbp_cells<<<e.grid, kThreads, 0, e.s>>>(e.tasks, gen, rn[2], e.cells, e.cell_cap, e.dc);
        CC_LAUNCHED(e.h);
        e.launches += 2;
        if ((st = sync_counters(e))) return st;
        const unsigned long long n_leaves = e.hc->n_cell * n456;
        unsigned long long l0 = 0;
        bool redo_without_filter = false;
        while (l0 < n_leaves) {
            // room for the criticals of a full pass queue
            if (e.hc->n_crit > e.crit_cap - e.slice && (st = drain_criticals(e))) return st;
            const unsigned long long l1 = n_leaves - l0 > e.range ? l0 + e.range : n_leaves;
            CC_CUDA(e.h, cudaMemcpyAsync(e.backup, e.dc, sizeof(SbCounters), cudaMemcpyDeviceToDevice, e.s));
            CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_q[0], 0, 2 * sizeof(unsigned long long), e.s));
            int lgrid = (int)std::min<unsigned long long>((l1 - l0 + kThreads - 1) / kThreads, (unsigned long long)e.grid);
            lg.cell0 = l0 / n456;
            lg.rem0 = (uint32_t)(l0 % n456);
            if (e.plain) {
                k_sbp_leaves_plain<<<lgrid, kThreads, 0, e.s>>>(e.tasks, e.cells, l0, l1, lg, e.crit, e.crit_cap, e.dc);
            } else if (e.fp32 && !redo_without_filter) {
                // the candidate list lives in the second pass queue's memory
                // (free until pass 1) and is counted by its counter; the
                // anchors of the empty leaves in its upper half
                uint32_t* cand = reinterpret_cast<uint32_t*>(e.q[1]);
                const unsigned long long cand_cap = e.slice * (sizeof(SbLeaf) / sizeof(uint32_t)) / 2;
                uint32_t* anchors = cand + cand_cap;
                CC_CUDA(e.h, cudaMemsetAsync(&e.dc->n_anchor, 0, 3 * sizeof(unsigned long long), e.s));
                k_sbp_leaf_filter<<<lgrid, kThreads, 0, e.s>>>(e.tasks, e.cells, l0, l1, lg, cand, &e.dc->n_q[1],
                                                               cand_cap, anchors, cand_cap, e.dc);
                CC_LAUNCHED(e.h);
                k_sbp_empty_cert<<<e.grid, kThreads, 0, e.s>>>(e.tasks, e.cells, l0, l1, lg, anchors, cand_cap, e.dc);
                CC_LAUNCHED(e.h);
                e.launches += 2;
                k_sbp_leaf_check<<<e.grid, kThreads, 0, e.s>>>(e.tasks, e.cells, l0, l1, lg, cand, &e.dc->n_q[1],
                                                               cand_cap, e.q[0], &e.dc->n_q[0], e.slice, e.crit,
                                                               e.crit_cap, e.dc);
            } else {
                k_sbp_leaves<<<lgrid, kThreads, 0, e.s>>>(e.tasks, e.cells, l0, l1, lg, e.q[0], &e.dc->n_q[0],
                                                          e.slice, e.crit, e.crit_cap, e.dc);
            }
            CC_LAUNCHED(e.h);
            e.launches++;
            CC_CUDA(e.h, cudaMemcpyAsync(e.hc, e.dc, sizeof(SbCounters), cudaMemcpyDeviceToHost, e.s));
            CC_CUDA(e.h, cudaStreamSynchronize(e.s));
            if (e.hc->overflow) {  // undo the slice and retry with half of it
                if (e.range == 1) return ccrt::fail(e.h, CC_ERR_QUEUE_OVERFLOW, "cc_sb_prove: queue overflow");
                CC_CUDA(e.h, cudaMemcpyAsync(e.dc, e.backup, sizeof(SbCounters), cudaMemcpyDeviceToDevice, e.s));
                if ((st = sync_counters(e))) return st;
                e.range /= 2;
                continue;
            }
            if (e.fp32 && !redo_without_filter && e.hc->empty_cert_fail) {
                // an empty leaf of the pre-filter failed its FP64 certificate:
                // undo the slice and redo it with FP64 emptiness tests only
                cc::cert_failures_host += e.hc->empty_cert_fail;
                CC_CUDA(e.h, cudaMemcpyAsync(e.dc, e.backup, sizeof(SbCounters), cudaMemcpyDeviceToDevice, e.s));
                if ((st = sync_counters(e))) return st;
                redo_without_filter = true;
                continue;
            }
            redo_without_filter = false;
            e.empty_anchors += e.hc->empty_cert_ok;
            if (e.plain) {  // every leaf was decided in place; at most `slice` criticals per slice
                e.range = e.slice;
                l0 = l1;
                continue;
            }
            // aim the next slice at half of the pass queue
            const unsigned long long open = e.hc->n_q[0] ? e.hc->n_q[0] : 1;
            unsigned long long next = (unsigned long long)((double)(l1 - l0) * (double)(e.slice / 2) / (double)open);
            e.range = std::max<unsigned long long>(std::min<unsigned long long>(1024, e.slice),
                                                   std::min<unsigned long long>(next, 1ULL << 31));
            if ((st = launch_passes<1>(e, gen, 0))) return st;
            if ((st = sync_counters(e))) return st;
            l0 = l1;
        }
    }
    return drain_criticals(e);
}

// Variables::operator< (rectangle_size_bound/variables.hpp:82-94)
bool iv_less(const Iv& a, const Iv& b) { return a.lo < b.lo || (a.lo == b.lo && a.hi < b.hi); }
bool box_less(const Box6& a, const Box6& b) {
    if (iv_less(a.la, b.la)) return true;
    if (iv_less(b.la, a.la)) return false;
    for (int i = 0; i < 6; ++i) {
        if (iv_less(a.r[i], b.r[i])) return true;
        if (iv_less(b.r[i], a.r[i])) return false;
    }
    return false;
}
bool iv_same(const Iv& a, const Iv& b) { return a.lo == b.lo && a.hi == b.hi; }

struct Crit {
    Box6 box;
    uint32_t trapped;
};

// merge_critical_intervals<N> (rectangle_size_bound.cu:103-130)
std::vector<Crit> merge(std::vector<Crit>& v, int n_merged) {
    std::vector<Crit> out;
    if (v.empty()) return out;
    std::sort(v.begin(), v.end(), [](const Crit& a, const Crit& b) { return box_less(a.box, b.box); });
    out.push_back(v.front());
    for (const Crit& x : v) {
        Crit& p = out.back();
        bool same = iv_same(x.box.la, p.box.la);
        for (int i = 0; same && i < n_merged; ++i) same = iv_same(x.box.r[i], p.box.r[i]);
        if (same) {
            for (int i = n_merged; i < 6; ++i) {  // Interval::do_join
                if (x.box.r[i].lo < p.box.r[i].lo) p.box.r[i].lo = x.box.r[i].lo;
                if (x.box.r[i].hi > p.box.r[i].hi) p.box.r[i].hi = x.box.r[i].hi;
            }
            p.trapped |= x.trapped;
        } else {
            out.push_back(x);
        }
    }
    return out;
}

bool grid_ok(const cc_sb_grid* g) {
    auto ok = [](int x) { return x >= 1 && x <= 2047; };
    if (!ok(g->la_splits_init) || g->num_generations < 0 || g->num_generations > CC_MAX_GENERATIONS) return false;
    if (g->num_generations > 0 && !ok(g->la_splits_gen)) return false;
    for (int i = 0; i < 6; ++i) {
        if (!ok(g->r_splits_init[i])) return false;
        if (g->num_generations > 0 && !ok(g->r_splits_gen[i])) return false;
    }
    return true;
}

}  // namespace

extern "C" int cc_sb_prove(cc_handle* h, const cc_sb_box* root, const cc_sb_grid* grid, cc_sb_box** criticals,
                           size_t* n_crit, uint32_t** flags, cc_sb_prove_stats* stats) {
    return cc_sb_prove_ex(h, root, grid, 0, criticals, n_crit, flags, stats);
}

// FP64 certification failures of the size-bound kernels so far (expected 0)
static unsigned long long sb_cert_failures_so_far() {
    unsigned long long v = 0;
    if (cudaMemcpyFromSymbol(&v, cc::cc_cert_fail_count, sizeof(v)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return v + cc::cert_failures_host.load();
}

// the engine's device buffers and work-unit sizes (shared by the entry points)
static int engine_setup(cc_handle* h, int options, Engine& e) {
    e.h = h;
    e.plain = (options & CC_PROVE_PLAIN) != 0;
    e.fp32 = !e.plain && !(options & CC_SB_NO_FP32_PREFILTER);
    e.s = h->stream;
    e.grid = h->sm_count * 8;
    // sizes of the work units (queue capacities follow from them); the
    // environment can shrink them, which only changes how the same work is
    // cut into launches
    auto log2_env = [](const char* name, int dflt, int lo, int hi) {
        const char* v = std::getenv(name);
        int x = v ? std::atoi(v) : dflt;
        return x < lo ? lo : (x > hi ? hi : x);
    };
    e.task_chunk = 1ULL << log2_env("CC_SB_TASK_CHUNK_LOG2", 18, 0, 18);
    e.cell_cap = 1ULL << 22;
    e.slice = 1ULL << log2_env("CC_SB_SLICE_LOG2", 24, 5, 26);
    e.crit_cap = 2 * e.slice;
    e.range = e.slice;
    int st;
    void* p;
    if ((st = ccrt::ensure(h, kSlotBase + S_TASKS, e.task_chunk * sizeof(SbTask), &p))) return st;
    e.tasks = (SbTask*)p;
    if ((st = ccrt::ensure(h, kSlotBase + S_CELLS, e.cell_cap * sizeof(SbCell), &p))) return st;
    e.cells = (SbCell*)p;
    if ((st = ccrt::ensure(h, kSlotBase + S_Q0, e.slice * sizeof(SbLeaf), &p))) return st;
    e.q[0] = (SbLeaf*)p;
    if ((st = ccrt::ensure(h, kSlotBase + S_Q1, e.slice * sizeof(SbLeaf), &p))) return st;
    e.q[1] = (SbLeaf*)p;
    if ((st = ccrt::ensure(h, kSlotBase + S_CRIT, e.crit_cap * sizeof(SbLeaf), &p))) return st;
    e.crit = (SbLeaf*)p;
    if ((st = ccrt::ensure(h, kSlotBase + S_COUNTERS, 2 * sizeof(SbCounters), &p))) return st;
    e.dc = (SbCounters*)p;
    e.backup = e.dc + 1;
    if ((st = ccrt::ensure(h, kSlotBase + S_JOBS, e.slice * sizeof(SevenJob), &p))) return st;
    e.jobs = (SevenJob*)p;
    if ((st = ccrt::ensure_pinned(h, sizeof(SbCounters)))) return st;
    e.hc = (SbCounters*)h->pinned;
    CC_CUDA(h, cudaMemsetAsync(e.dc, 0, sizeof(SbCounters), e.s));

    return CC_OK;
}

static int fill_stats(Engine& e, cc_sb_prove_stats* stats, uint64_t trapped_leaves, const std::vector<uint64_t>& gen_sizes,
                      int generations_run, std::chrono::steady_clock::time_point t_start, unsigned long long fails0);

// criticals of a generation, merged as the reference merges that generation
// (rectangle_size_bound.cu:351-362), to caller-owned arrays
static int emit_criticals(cc_handle* h, std::vector<Crit>& cur, cc_sb_box** criticals, size_t* n_crit,
                          uint32_t** flags) {
    *n_crit = cur.size();
    *criticals = (cc_sb_box*)std::malloc(sizeof(cc_sb_box) * (cur.size() + 1));
    if (flags) *flags = (uint32_t*)std::malloc(sizeof(uint32_t) * (cur.size() + 1));
    if (!*criticals || (flags && !*flags)) return ccrt::fail(h, CC_ERR_OOM, "cc_sb_prove: host allocation");
    for (size_t i = 0; i < cur.size(); ++i) {
        (*criticals)[i].la = cc_iv{cur[i].box.la.lo, cur[i].box.la.hi};
        for (int k = 0; k < 6; ++k) (*criticals)[i].r[k] = cc_iv{cur[i].box.r[k].lo, cur[i].box.r[k].hi};
        if (flags) (*flags)[i] = cur[i].trapped;
    }
    return CC_OK;
}

static int merge_width(int gen) { return gen == 0 ? 0 : (gen % 3 == 0 ? 3 : (gen % 3 == 1 ? 2 : 1)); }

extern "C" int cc_sb_prove_ex(cc_handle* h, const cc_sb_box* root, const cc_sb_grid* grid, int options,
                              cc_sb_box** criticals, size_t* n_crit, uint32_t** flags, cc_sb_prove_stats* stats) {
    if (!h || !root || !grid || !criticals || !n_crit) return CC_ERR_PARAM;
    if (!grid_ok(grid)) return ccrt::fail(h, CC_ERR_PARAM, "cc_sb_prove: split counts must be in [1, 2047]");
    const auto t_start = std::chrono::steady_clock::now();
    const unsigned long long fails0 = sb_cert_failures_so_far();
    h->launches = 0;
    h->interrupt.store(0);
    CC_CUDA(h, cudaSetDevice(h->device));
    *criticals = nullptr;
    *n_crit = 0;
    if (flags) *flags = nullptr;

    Engine e;
    int st = engine_setup(h, options, e);
    if (st) return st;

    std::vector<uint64_t> gen_sizes;
    int generations_run = 0;
    uint64_t trapped_leaves = 0;
    std::vector<Box6> parents(1);
    parents[0].la = Iv{root->la.lb, root->la.ub};
    for (int i = 0; i < 6; ++i) parents[0].r[i] = Iv{root->r[i].lb, root->r[i].ub};
    std::vector<Crit> cur;
    int status = CC_OK;
    for (int gen = 0; gen <= grid->num_generations; ++gen) {
        if (gen > 0) {
            if (cur.empty()) break;
            parents.clear();
            for (const Crit& c : cur) parents.push_back(c.box);
        }
        e.found.clear();
        st = gen == 0 ? run_generation(e, parents, 0, grid->la_splits_init, grid->r_splits_init)
                      : run_generation(e, parents, gen, grid->la_splits_gen, grid->r_splits_gen);
        if (st == CC_ERR_INTERRUPTED) {  // keep the last complete generation's result
            status = st;
            break;
        }
        if (st) return st;
        std::vector<Crit> found(e.found.size());
        for (size_t i = 0; i < e.found.size(); ++i) {
            found[i].box = e.found[i].box;
            found[i].trapped = (uint32_t)(e.found[i].idx >> 63);
            trapped_leaves += found[i].trapped;
        }
        cur = merge(found, merge_width(gen));
        gen_sizes.push_back(cur.size());
        if (gen > 0) generations_run = gen;
    }

    if ((st = emit_criticals(h, cur, criticals, n_crit, flags))) return st;
    if (stats && (st = fill_stats(e, stats, trapped_leaves, gen_sizes, generations_run, t_start, fails0))) return st;
    return status;
}

static int fill_stats(Engine& e, cc_sb_prove_stats* stats, uint64_t trapped_leaves, const std::vector<uint64_t>& gen_sizes,
                      int generations_run, std::chrono::steady_clock::time_point t_start, unsigned long long fails0) {
    cc_handle* h = e.h;
    int st;
    {
        std::memset(stats, 0, sizeof(*stats));
        if ((st = sync_counters(e))) return st;
        std::memcpy(stats->task_counts, e.hc->task_counts, sizeof(stats->task_counts));
        std::memcpy(stats->cell_counts, e.hc->cell_counts, sizeof(stats->cell_counts));
        std::memcpy(stats->leaf_counts, e.hc->leaf_counts, sizeof(stats->leaf_counts));
        stats->digest = e.hc->digest;
        stats->leaf_evals = e.hc->leaf_evals;
        stats->trapped_leaves = trapped_leaves;
        stats->trapped_shortcuts = e.hc->trapped_shortcuts;
        for (size_t g = 0; g < gen_sizes.size() && g <= CC_MAX_GENERATIONS; ++g) stats->gen_sizes[g] = gen_sizes[g];
        stats->generations_run = generations_run;
        stats->fp32_decided = e.hc->fp32_empty;
        stats->widening_samples = e.hc->widen_count;
        stats->widening_mean = e.hc->widen_count ? e.hc->widen_sum / (double)e.hc->widen_count : 0.0;
        double wmax;
        std::memcpy(&wmax, &e.hc->widen_max_bits, sizeof(double));
        stats->widening_max = wmax;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        stats->kernel_launches = h->launches;
        stats->fp32_certified = e.hc->cert_ok;
        stats->empty_anchors = e.empty_anchors;
        stats->cert_failures = sb_cert_failures_so_far() - fails0;
    }
    return CC_OK;
}

// One generation of the size-bound proof over the tasks [task_lo, task_hi)
// (task = parent * (la x r1 x r2 splits) + lambda piece * (r1 x r2) + r1
// piece * r2 splits + r2 piece; rectangle_size_bound.cu:276-310), criticals
// merged as the reference merges generation `gen`.
extern "C" int cc_sb_generation(cc_handle* h, const cc_sb_box* parents, size_t n_parents, int gen, int la_splits,
                                const int r_splits[6], uint64_t task_lo, uint64_t task_hi, int options,
                                cc_sb_box** criticals, size_t* n_crit, uint32_t** flags, cc_sb_prove_stats* stats) {
    if (!h || (n_parents && !parents) || !r_splits || !criticals || !n_crit || task_lo > task_hi || gen < 0 ||
        gen > CC_MAX_GENERATIONS)
        return CC_ERR_PARAM;
    cc_sb_grid g{};
    g.la_splits_init = la_splits;
    g.la_splits_gen = la_splits;
    for (int k = 0; k < 6; ++k) g.r_splits_init[k] = g.r_splits_gen[k] = r_splits[k];
    if (!grid_ok(&g)) return ccrt::fail(h, CC_ERR_PARAM, "cc_sb_generation: split counts must be in [1, 2047]");
    const auto t_start = std::chrono::steady_clock::now();
    const unsigned long long fails0 = sb_cert_failures_so_far();
    h->launches = 0;
    h->interrupt.store(0);
    CC_CUDA(h, cudaSetDevice(h->device));
    *criticals = nullptr;
    *n_crit = 0;
    if (flags) *flags = nullptr;
    Engine e;
    int st = engine_setup(h, options, e);
    if (st) return st;
    std::vector<Box6> ps(n_parents);
    for (size_t i = 0; i < n_parents; ++i) {
        ps[i].la = Iv{parents[i].la.lb, parents[i].la.ub};
        for (int k = 0; k < 6; ++k) ps[i].r[k] = Iv{parents[i].r[k].lb, parents[i].r[k].ub};
    }
    e.found.clear();
    if (n_parents && (st = run_generation(e, ps, gen, la_splits, r_splits, task_lo, task_hi))) return st;
    std::vector<Crit> found(e.found.size());
    uint64_t trapped_leaves = 0;
    for (size_t i = 0; i < e.found.size(); ++i) {
        found[i].box = e.found[i].box;
        found[i].trapped = (uint32_t)(e.found[i].idx >> 63);
        trapped_leaves += found[i].trapped;
    }
    std::vector<Crit> cur = merge(found, merge_width(gen));
    if ((st = emit_criticals(h, cur, criticals, n_crit, flags))) return st;
    if (stats) {
        const std::vector<uint64_t> sizes{cur.size()};
        if ((st = fill_stats(e, stats, trapped_leaves, sizes, 0, t_start, fails0))) return st;
    }
    return CC_OK;
}

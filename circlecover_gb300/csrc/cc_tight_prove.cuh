// Device engine of the tight-rectangle proof (reference:
// tight_rectangle/tight_rectangle.cu:161-320 and 458-498).
//
// The reference launches one kernel per lambda box, each a fixed
// (r1,r2)-blocks x (r3,r4)-threads grid in which every thread re-evaluates
// the outer checks, with a host synchronisation after every launch.  Here all
// lambda boxes ("tasks") of a generation go through the same stages, one
// persistent-grid kernel each, in stream order without host synchronisation:
//
//   stage 1  (task, i1)        r1 cells:  r2 range, r1_strategies
//   stage 2  (r1 cell, i2)     r2 cells:  r1_strategies, r3 range, r1_r2_strategies
//   stage 3  (r2 cell, i3)     r3 cells:  r1_r2_strategies, r4 range, r1_r2_r3_strategies, R4
//   stage 4a (r3 cell, i4)     leaves:    r1_r2_r3_strategies, R, two_by_two
//                                         (prepared form: two_by_two in stage
//                                         4a2 on the compacted leaves that need it)
//
// In the prepared form the per-leaf criteria (two_by_two, the leaf form of
// r1_r2_r3_strategies) are evaluated on FP32 enclosures first and in FP64
// only where those cannot decide (cc_f32.cuh, tight::first_f32): same
// outcomes and trap status, so the same trace.
//   stage 4b (leaf queue)      leaves:    r1_r2_r3_strategies(box, R4), gaps precondition
//   stage 4c (gaps queue)      leaves:    gaps bisection
//
// Each stage reads its item count from device memory and appends survivors
// to the next stage's queue with one atomic per warp (warp-aggregated
// atomics), so every stage runs on full warps of items that need it.
// Critical leaves carry their task index; the host merges them per task by
// r1 (merge_adjacent_r1, tight_rectangle.cu:121-159), which restores the
// reference's order exactly.
//
// Two forms (template parameter Hoist):
//   plain  -- every cell calls the criteria as the reference does;
//   hoist  -- a parent cell prepares the criteria its children evaluate with
//             only their own upper bound changing (cc_tight.cuh, "prepared
//             forms"), e.g. the cover-strip bisection runs once per r3 cell
//             instead of once per leaf.  Identical verdicts.
//
// Every grid cell visited contributes one (level, outcome) count and
// mix64(key) to a digest; the oracle computes the same trace.
#pragma once

#include "cc_tight.cuh"

namespace cc {
namespace prove {

using tight::Box;

struct Task {
    Iv la, weight, r1r;
    int parent;
    int live;  // r1r not empty
};

struct Cell2 {  // a surviving r1 cell
    Iv r1, r2r;
    int task, i1;
    tight::R1Prep p1;
};

struct Cell3 {  // a surviving r2 cell
    Iv r1, r2, r3r;
    int task;
    int16_t i1, i2;
    tight::R12Prep p2;
};

struct Cell4 {  // a surviving r3 cell
    Iv r1, r2, r3, r4r, R4;
    int task;
    int16_t i1, i2, i3;
    int16_t order;  // learned order: 1 = try the r1_r2_r3 leaf criterion before 2x2
    tight::R123Prep p3;
    tight::LeafPrep lp;  // the leaf form of r1_r2_r3 for the leaves whose r4 does not tighten r3
};

struct Leaf {  // a leaf that survived stage 4a
    uint32_t cell4;
    uint16_t i4;
    uint16_t trapped;  // bit 0: a trap site was reached; bit 1: the leaf criterion already failed
};

struct GapsLeaf {  // a leaf that needs the gaps bisection
    tight::GapsJob job;
    uint32_t cell4;
    uint16_t i4;
    uint16_t trapped;
};

struct Critical {
    Box box;
    int task;
    uint32_t flags;
};

// A leaf verdict that the FP32 enclosures decided "true", queued for its
// FP64 certification (k_stage_cert): the leaf, its criterion (0: two_by_two,
// 1: the leaf form of r1_r2_r3_strategies) and the number of the call that
// settled the FP32 run (0: none).
struct CertLeaf {
    uint32_t cell4;
    uint16_t i4;
    uint8_t crit;
    uint8_t call;
};

struct Counters {
    unsigned long long n_cell2, n_cell3, n_cell4, n_leaf, n_gaps, n_crit;
    unsigned long long overflow;
    unsigned long long leaf_evals;
    unsigned long long digest;
    unsigned long long counts[4][8];
    unsigned long long n_leaf2;  // leaves waiting for the 2x2 criterion (split stage 4a)
    // leaf criteria evaluated FP32-first (tight::first_f32_deferred), by
    // outcome: FP64 evaluation, FP32 "false", FP32 "true" certified in FP64
    // (k_stage_cert), certification failed
    unsigned long long fp32[4];
    unsigned long long n_cert;  // FP32 "true" leaf verdicts queued for certification
};

struct Leaf2 {  // a leaf that needs the 2x2 criterion
    Iv r4;
    uint32_t cell4;
    uint16_t i4;
    uint16_t pad;  // bits as Leaf::trapped
};

struct Caps {
    unsigned long long cell2, cell3, cell4, leaf, gaps, crit;
    unsigned long long leaf2;  // leaves waiting for the 2x2 criterion (about half of all leaves)
};

CC_FN uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

// same packing as the oracle's trace_key
CC_FN uint64_t trace_key(uint64_t task, int level, int i1, int i2, int i3, int i4, int outcome) {
    uint64_t packed = ((uint64_t)outcome) | ((uint64_t)i4 << 4) | ((uint64_t)i3 << 15) | ((uint64_t)i2 << 26) |
                      ((uint64_t)i1 << 37) | ((uint64_t)level << 48);
    return mix64(packed ^ mix64(task + 0x9e3779b97f4a7c15ULL));
}

#if CC_DEVICE_BUILD

// per-block trace accumulation in shared memory, flushed once per block
struct BlockTrace {
    unsigned long long counts[8];
    unsigned long long digest;
};

__device__ __forceinline__ void trace_init(BlockTrace& bt) {
    if (threadIdx.x < 8) bt.counts[threadIdx.x] = 0;
    if (threadIdx.x == 0) bt.digest = 0;
    __syncthreads();
}

__device__ __forceinline__ void trace_note(BlockTrace& bt, bool valid, uint64_t key, int outcome) {
    // warp-reduce the digest; one shared atomic per distinct outcome in the
    // warp for the counts (lanes with equal outcomes would serialise)
    uint64_t d = valid ? key : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&bt.digest, (unsigned long long)d);
    const unsigned same = __match_any_sync(0xffffffffu, valid ? outcome : -1);
    if (valid && (threadIdx.x & 31) == (unsigned)(__ffs(same) - 1))
        atomicAdd(&bt.counts[outcome], (unsigned long long)__popc(same));
}

__device__ __forceinline__ void trace_flush(BlockTrace& bt, Counters* c, int level) {
    __syncthreads();
    if (threadIdx.x < 8 && bt.counts[threadIdx.x]) atomicAdd(&c->counts[level][threadIdx.x], bt.counts[threadIdx.x]);
    if (threadIdx.x == 0 && bt.digest) atomicAdd(&c->digest, bt.digest);
}

// Warp-aggregated append: every lane of the warp calls this (full mask);
// lanes with `want` get consecutive slots.  Returns the slot or ~0 if the
// queue is full (then the overflow flag is raised and nothing is written).
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

// per-thread tally of first_f32 outcomes, summed over the warp and added to
// the counters once per warp at the end of a stage kernel (every lane of the
// block reaches it)
struct F32Tally {
    unsigned n[4] = {0, 0, 0, 0};
    __device__ __forceinline__ void note(int how) {
        if (how >= 0) n[how] += 1;
    }
    // a stage's outcomes: the FP32 "true" ones are counted by k_stage_cert
    __device__ __forceinline__ void note_stage(int how) {
        if (how == 0 || how == 1) n[how] += 1;
    }
    __device__ __forceinline__ void flush(Counters* c) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            unsigned v = n[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0 && v) atomicAdd(&c->fp32[k], (unsigned long long)v);
        }
    }
};

// warp-uniform grid-stride loop over [0, total): all 32 lanes enter every
// iteration (lanes past the end with valid = false), so warp collectives are safe
#define CC_WARP_LOOP(total)                                                                              \
    for (unsigned long long base_ = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); \
         base_ < (total); base_ += (unsigned long long)gridDim.x * blockDim.x)

// stage 0: one thread per task
// tasks whose generation-wide index (task_base + t) lies outside [lo, hi)
// belong to another shard: they are marked dead and contribute nothing
__global__ void k_tasks(const Box* __restrict__ parents, int n_parents, int la_splits, Task* __restrict__ tasks,
                        unsigned long long task_base, unsigned long long lo, unsigned long long hi) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_parents * la_splits) return;
    trap_clear();
    int p = t / la_splits;
    int k = t % la_splits;
    Task tk;
    tk.la = subinterval(parents[p].la, k, la_splits);
    tk.weight = tight::required_weight_for(tk.la);
    tk.r1r = intersect(tight::r1_range(tk.la), parents[p].r[0]);
    tk.parent = p;
    const unsigned long long g = task_base + (unsigned long long)t;
    tk.live = !empty(tk.r1r) && g >= lo && g < hi;
    tasks[t] = tk;
}

// stage 1: r1 cells (tight_rectangle.cu:182-191)
template <bool Hoist>
__global__ void __launch_bounds__(128) k_stage1(const Box* __restrict__ parents, const Task* __restrict__ tasks, int n_tasks,
                                                int s1, Cell2* __restrict__ out, Caps caps, Counters* c,
                                                unsigned long long task_base) {
    __shared__ BlockTrace bt;
    trace_init(bt);
    trap_clear();
    const unsigned long long total = (unsigned long long)n_tasks * s1;
    CC_WARP_LOOP(total) {
        unsigned long long idx = base_ + (threadIdx.x & 31);
        bool valid = idx < total;
        int task = valid ? (int)(idx / s1) : 0;
        int i1 = valid ? (int)(idx % s1) : 0;
        int outcome = -1;
        Cell2 cell;
        if (valid) {
            const Task tk = tasks[task];
            if (!tk.live) {
                valid = false;  // the reference returns before its r1 loop
            } else {
                cell.r1 = subinterval(tk.r1r, i1, s1);
                cell.r2r = intersect(tight::r2_range(tk.weight, cell.r1), parents[tk.parent].r[1]);
                cell.task = task;
                cell.i1 = i1;
                if (empty(cell.r2r)) {
                    outcome = CC_T_L1_EMPTY;
                } else {
                    bool ok;
                    if (Hoist) {
                        cell.p1 = tight::r1_prepare(tk.la, tk.weight, cell.r1);
                        ok = tight::r1_check(cell.p1, cell.r2r.hi);
                    } else {
                        ok = tight::r1_strategies(tk.la, tk.weight, cell.r1, cell.r2r.hi);
                    }
                    outcome = ok ? CC_T_L1_R1 : CC_T_L1_SPLIT;
                }
            }
        }
        __syncwarp();
        trace_note(bt, valid, valid ? trace_key(task_base + task, 0, i1, 0, 0, 0, outcome) : 0, outcome);
        unsigned long long slot = warp_append(&c->n_cell2, valid && outcome == CC_T_L1_SPLIT, caps.cell2, &c->overflow);
        if (slot != ~0ULL) out[slot] = cell;
    }
    trace_flush(bt, c, 0);
}

// stage 2: r2 cells (tight_rectangle.cu:193-206)
template <bool Hoist>
__global__ void __launch_bounds__(128) k_stage2(const Box* __restrict__ parents, const Task* __restrict__ tasks,
                                                const Cell2* __restrict__ in, int s2, Cell3* __restrict__ out, Caps caps,
                                                Counters* c, unsigned long long task_base) {
    __shared__ BlockTrace bt;
    trace_init(bt);
    trap_clear();
    const unsigned long long n_in = *(volatile unsigned long long*)&c->n_cell2;
    const unsigned long long total = (n_in < caps.cell2 ? n_in : caps.cell2) * s2;
    CC_WARP_LOOP(total) {
        unsigned long long idx = base_ + (threadIdx.x & 31);
        bool valid = idx < total;
        int outcome = -1;
        Cell3 cell;
        int i2 = 0, task = 0, i1 = 0;
        if (valid) {
            const Cell2& p = in[idx / s2];
            i2 = (int)(idx % s2);
            task = p.task;
            i1 = p.i1;
            const Task tk = tasks[task];
            cell.r1 = p.r1;
            cell.r2 = subinterval(p.r2r, i2, s2);
            cell.task = task;
            cell.i1 = (int16_t)i1;
            cell.i2 = (int16_t)i2;
            bool r1_ok = Hoist ? tight::r1_check(p.p1, cell.r2.hi) : tight::r1_strategies(tk.la, tk.weight, p.r1, cell.r2.hi);
            if (r1_ok) {
                outcome = CC_T_L2_R1;
            } else {
                cell.r3r = intersect(tight::r3_range(tk.weight, cell.r1, cell.r2), parents[tk.parent].r[2]);
                if (empty(cell.r3r)) {
                    outcome = CC_T_L2_EMPTY;
                } else {
                    bool ok;
                    if (Hoist) {
                        cell.p2 = tight::r12_prepare(tk.la, tk.weight, cell.r1, cell.r2);
                        ok = tight::r12_check(cell.p2, cell.r3r.hi);
                    } else {
                        ok = tight::r1_r2_strategies(tk.la, tk.weight, cell.r1, cell.r2, cell.r3r.hi);
                    }
                    outcome = ok ? CC_T_L2_R12 : CC_T_L2_SPLIT;
                }
            }
        }
        __syncwarp();
        trace_note(bt, valid, valid ? trace_key(task_base + task, 1, i1, i2, 0, 0, outcome) : 0, outcome);
        unsigned long long slot = warp_append(&c->n_cell3, valid && outcome == CC_T_L2_SPLIT, caps.cell3, &c->overflow);
        if (slot != ~0ULL) out[slot] = cell;
    }
    trace_flush(bt, c, 1);
}

// stage 3: r3 cells (tight_rectangle.cu:208-227)
template <bool Hoist>
__global__ void __launch_bounds__(128) k_stage3(const Box* __restrict__ parents, const Task* __restrict__ tasks,
                                                const Cell3* __restrict__ in, int s3, Cell4* __restrict__ out, Caps caps,
                                                Counters* c, unsigned long long task_base) {
    __shared__ BlockTrace bt;
    trace_init(bt);
    trap_clear();
    const unsigned long long n_in = *(volatile unsigned long long*)&c->n_cell3;
    const unsigned long long total = (n_in < caps.cell3 ? n_in : caps.cell3) * s3;
    CC_WARP_LOOP(total) {
        unsigned long long idx = base_ + (threadIdx.x & 31);
        bool valid = idx < total;
        int outcome = -1;
        Cell4 cell;
        int i3 = 0, task = 0, i1 = 0, i2 = 0;
        if (valid) {
            const Cell3& p = in[idx / s3];
            i3 = (int)(idx % s3);
            task = p.task;
            i1 = p.i1;
            i2 = p.i2;
            const Task tk = tasks[task];
            cell.r1 = p.r1;
            cell.r2 = p.r2;
            cell.r3 = subinterval(p.r3r, i3, s3);
            cell.task = task;
            cell.i1 = p.i1;
            cell.i2 = p.i2;
            cell.i3 = (int16_t)i3;
            cell.order = 0;
            bool r12_ok = Hoist ? tight::r12_check(p.p2, cell.r3.hi)
                                : tight::r1_r2_strategies(tk.la, tk.weight, p.r1, p.r2, cell.r3.hi);
            if (r12_ok) {
                outcome = CC_T_L3_R12;
            } else {
                cell.r4r = intersect(tight::r4_range(tk.weight, p.r1, p.r2, cell.r3), parents[tk.parent].r[3]);
                if (empty(cell.r4r)) {
                    outcome = CC_T_L3_EMPTY;
                } else {
                    bool ok;
                    if (Hoist) {
                        cell.p3 = tight::r123_prepare(tk.la, tk.weight, cell.r1, cell.r2, cell.r3);
                        ok = tight::r123_check(cell.p3, cell.r4r.hi);
                    } else {
                        ok = tight::r1_r2_r3_strategies(tk.la, tk.weight, cell.r1, cell.r2, cell.r3, cell.r4r.hi);
                    }
                    if (ok) {
                        outcome = CC_T_L3_R123;
                    } else {
                        cell.R4 = tk.weight - cell.r1 - cell.r2 - cell.r3;
                        tighten_lb(cell.R4, 0.0);
                        outcome = empty(cell.R4) ? CC_T_L3_R4EMPTY : CC_T_L3_SPLIT;
                        if (Hoist && outcome == CC_T_L3_SPLIT) {
                            // the leaf box of a leaf whose r4 lower bound is at most r3's
                            Box vb{tk.la, {cell.r1, cell.r2, cell.r3, cell.r3}};
                            tighten_lb(vb.r[1], vb.r[2].lo);
                            tighten_lb(vb.r[0], vb.r[1].lo);
                            cell.lp = tight::leaf123_prepare(vb, cell.R4);
                        }
                    }
                }
            }
        }
        __syncwarp();
        trace_note(bt, valid, valid ? trace_key(task_base + task, 2, i1, i2, i3, 0, outcome) : 0, outcome);
        unsigned long long slot = warp_append(&c->n_cell4, valid && outcome == CC_T_L3_SPLIT, caps.cell4, &c->overflow);
        if (slot != ~0ULL) out[slot] = cell;
    }
    trace_flush(bt, c, 2);
}

__device__ __forceinline__ Box leaf_box(const Cell4& p, Iv la, Iv r4) {
    Box v{la, {p.r1, p.r2, p.r3, r4}};
    tighten_lb(v.r[2], v.r[3].lo);
    tighten_lb(v.r[1], v.r[2].lo);
    tighten_lb(v.r[0], v.r[1].lo);
    return v;
}

// stage 4a: leaves, the cheap checks (tight_rectangle.cu:229-246).  Split
// form: the leaves that reach the 2x2 criterion (about half of them; its six
// bisections are the stage's main cost) are compacted into a queue for
// stage 4a2 instead of being checked here next to lanes that have finished.
// stage 4a over the r3 cells [cell_lo, cell_hi) (the host runs the leaf
// stages in slices of cells that the leaf queues can hold)
template <bool Hoist, bool Split>
__global__ void __launch_bounds__(128) k_stage4a(const Task* __restrict__ tasks, const Cell4* __restrict__ in, int s4,
                                                 unsigned long long cell_lo, unsigned long long cell_hi,
                                                 Leaf* __restrict__ out, Leaf2* __restrict__ out2, Caps caps, Counters* c,
                                                 unsigned long long task_base, CertLeaf* __restrict__ cq) {
    __shared__ BlockTrace bt;
    trace_init(bt);
    const unsigned long long total = (cell_hi - cell_lo) * s4;
    unsigned long long evals = 0;
    F32Tally tally;
    CC_WARP_LOOP(total) {
        unsigned long long idx = base_ + (threadIdx.x & 31);
        bool valid = idx < total;
        int outcome = -1;
        uint32_t pidx = 0;
        int i4 = 0, task = 0, i1 = 0, i2 = 0, i3 = 0;
        bool trapped = false, leaf_tried = false, queue_cert = false;
        int calls = 0;
        Iv r4{0.0, 0.0};
        if (valid) {
            evals += 1;
            pidx = (uint32_t)(cell_lo + idx / s4);
            i4 = (int)(idx % s4);
            const Cell4& p = in[pidx];
            task = p.task;
            i1 = p.i1;
            i2 = p.i2;
            i3 = p.i3;
            const Task tk = tasks[task];
            trap_clear();
            r4 = subinterval(p.r4r, i4, s4);
            bool r123_ok = Hoist ? tight::r123_check(p.p3, r4.hi)
                                 : tight::r1_r2_r3_strategies(tk.la, tk.weight, p.r1, p.r2, p.r3, r4.hi);
            if (r123_ok) {
                outcome = CC_T_L4_R123;
            } else {
                Box v = leaf_box(p, tk.la, r4);
                Iv R = tk.weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
                tighten_lb(R, 0.0);
                if (empty(R)) {
                    outcome = CC_T_L4_REMPTY;
                } else if (Split) {
                    outcome = -3;  // on to stage 4a2
                    if (p.order) {  // learned order: the cheap leaf criterion first
                        int how = -1;
                        // prepared per cell in FP64 where r4 leaves r1..r3 as the cell's, else FP32 first
                        const bool ok4 = r4.lo <= p.r3.lo
                                             ? tight::leaf123_check(p.lp, r4.hi)
                                             : tight::first_f32_deferred(tight::LeafR123{}, v, p.R4, &how, &calls);
                        tally.note_stage(how);
                        if (ok4 && trap_status() == TRAP_NONE) {
                            outcome = CC_T_L4_R123LEAF;
                            queue_cert = how == 2;
                        } else if (!ok4) {
                            leaf_tried = true;  // (a trap leaves it to the plain order)
                        }
                    }
                } else {
                    bool ok = tight::two_by_two_strategies(v, R);
                    trapped = trap_status() != TRAP_NONE;
                    outcome = (ok && !trapped) ? CC_T_L4_2X2 : -2;  // -2: on to stage 4b
                }
            }
            if (Split) trapped = trap_status() != TRAP_NONE;
        }
        __syncwarp();
        bool decided = valid && outcome >= 0;
        trace_note(bt, decided, decided ? trace_key(task_base + task, 3, i1, i2, i3, i4, outcome) : 0, decided ? outcome : 0);
        if (Split) {
            unsigned long long slot = warp_append(&c->n_leaf2, valid && outcome == -3, caps.leaf2, &c->overflow);
            if (slot != ~0ULL)
                out2[slot] = Leaf2{r4, pidx, (uint16_t)i4, (uint16_t)((trapped ? 1 : 0) | (leaf_tried ? 2 : 0))};
            slot = warp_append(&c->n_cert, valid && queue_cert, caps.leaf, &c->overflow);
            if (slot != ~0ULL) cq[slot] = CertLeaf{pidx, (uint16_t)i4, 1, (uint8_t)calls};
        } else {
            unsigned long long slot = warp_append(&c->n_leaf, valid && outcome == -2, caps.leaf, &c->overflow);
            if (slot != ~0ULL) out[slot] = Leaf{pidx, (uint16_t)i4, (uint16_t)(trapped ? 1 : 0)};
        }
    }
    for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
    if ((threadIdx.x & 31) == 0 && evals) atomicAdd(&c->leaf_evals, evals);
    if (Split) tally.flush(c);
    trace_flush(bt, c, 3);
}

// stage 4a2 (split form): the 2x2 criterion on the compacted leaves
// (tight_rectangle.cu:246); failures go on to stage 4b
__global__ void __launch_bounds__(128) k_stage4a2(const Task* __restrict__ tasks, const Cell4* __restrict__ cells,
                                                  const Leaf2* __restrict__ in, Leaf* __restrict__ out, Caps caps,
                                                  Counters* c, unsigned long long task_base, CertLeaf* __restrict__ cq) {
    __shared__ BlockTrace bt;
    trace_init(bt);
    const unsigned long long n_in = *(volatile unsigned long long*)&c->n_leaf2;
    const unsigned long long total = n_in < caps.leaf2 ? n_in : caps.leaf2;
    F32Tally tally;
    CC_WARP_LOOP(total) {
        unsigned long long idx = base_ + (threadIdx.x & 31);
        bool valid = idx < total;
        int outcome = -1;
        Leaf2 lf{Iv{0.0, 0.0}, 0, 0, 0};
        int task = 0, i1 = 0, i2 = 0, i3 = 0;
        bool trapped = false, queue_cert = false;
        int calls = 0;
        if (valid) {
            lf = in[idx];
            const Cell4& p = cells[lf.cell4];
            task = p.task;
            i1 = p.i1;
            i2 = p.i2;
            i3 = p.i3;
            const Task tk = tasks[task];
            trap_clear();
            Box v = leaf_box(p, tk.la, lf.r4);
            Iv R = tk.weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
            tighten_lb(R, 0.0);
            int how = -1;
            bool ok = tight::first_f32_deferred(tight::TwoByTwo{}, v, R, &how, &calls);
            tally.note_stage(how);
            trapped = (lf.pad & 1) != 0 || trap_status() != TRAP_NONE;
            outcome = (ok && !trapped) ? CC_T_L4_2X2 : -2;
            queue_cert = outcome == CC_T_L4_2X2 && how == 2;
        }
        __syncwarp();
        bool decided = valid && outcome >= 0;
        trace_note(bt, decided, decided ? trace_key(task_base + task, 3, i1, i2, i3, lf.i4, outcome) : 0,
                   decided ? outcome : 0);
        unsigned long long slot = warp_append(&c->n_leaf, valid && outcome == -2, caps.leaf, &c->overflow);
        if (slot != ~0ULL) out[slot] = Leaf{lf.cell4, lf.i4, (uint16_t)((trapped ? 1 : 0) | (lf.pad & 2))};
        slot = warp_append(&c->n_cert, valid && queue_cert, caps.leaf, &c->overflow);
        if (slot != ~0ULL) cq[slot] = CertLeaf{lf.cell4, lf.i4, 0, (uint8_t)calls};
    }
    tally.flush(c);
    trace_flush(bt, c, 3);
}

__device__ __forceinline__ void push_critical(Critical* crit, unsigned long long slot, const Box& v, int task, bool trapped) {
    if (slot != ~0ULL) crit[slot] = Critical{v, task, trapped ? 1u : 0u};
}

// stage 4b: r1_r2_r3_strategies(box, R4); leaves that reach the gaps strategy
// go on to its bisection in stage 4c (tight_rectangle.cu:246-255)
// F32: the leaf criterion on FP32 enclosures first (prepared form); the
// plain form evaluates it in FP64 only, as the reference does
template <bool F32>
__global__ void __launch_bounds__(128) k_stage4b(const Task* __restrict__ tasks, const Cell4* __restrict__ cells,
                                                 const Leaf* __restrict__ in, int s4, GapsLeaf* __restrict__ gq,
                                                 Critical* __restrict__ crit, Caps caps, Counters* c,
                                                 unsigned long long task_base, CertLeaf* __restrict__ cq) {
    __shared__ BlockTrace bt;
    trace_init(bt);
    const unsigned long long n_in = *(volatile unsigned long long*)&c->n_leaf;
    const unsigned long long total = n_in < caps.leaf ? n_in : caps.leaf;
    F32Tally tally;
    CC_WARP_LOOP(total) {
        unsigned long long idx = base_ + (threadIdx.x & 31);
        bool valid = idx < total;
        int outcome = -1;
        Leaf lf{0, 0, 0};
        Box v;
        int task = 0, i1 = 0, i2 = 0, i3 = 0;
        bool trapped = false, need_gaps = false, queue_cert = false;
        int calls = 0;
        GapsLeaf gl;
        if (valid) {
            lf = in[idx];
            const Cell4& p = cells[lf.cell4];
            task = p.task;
            i1 = p.i1;
            i2 = p.i2;
            i3 = p.i3;
            const Task tk = tasks[task];
            trap_clear();
            if (lf.trapped & 1) trap(TRAP_BISECTION_CAP);
            Iv r4 = subinterval(p.r4r, lf.i4, s4);
            v = leaf_box(p, tk.la, r4);
            Iv R = tk.weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
            tighten_lb(R, 0.0);
            tight::GapsStart g;
            int how = -1;
            // batched form: the leaf criterion prepared per cell in FP64 where r4
            // leaves r1..r3 as the cell's, else FP32 first
            if (!(lf.trapped & 2) &&
                (F32 ? (r4.lo <= p.r3.lo ? tight::leaf123_check(p.lp, r4.hi)
                                         : tight::first_f32_deferred(tight::LeafR123{}, v, p.R4, &how, &calls))
                     : tight::r1_r2_r3_strategies(v, p.R4))) {
                outcome = CC_T_L4_R123LEAF;
            } else if (tight::gaps_enters(v.r[0].lo, v.r[1].lo, g)) {
                need_gaps = true;
                gl.job = tight::GapsJob{tk.la.hi, v.r[0].lo, v.r[1].lo, v.r[3].lo, v.r[3].hi, g.w1, g.w2, R.lo, R.hi};
                gl.cell4 = lf.cell4;
                gl.i4 = lf.i4;
            } else {
                outcome = CC_T_L4_CRITICAL;
            }
            tally.note_stage(how);
            trapped = trap_status() != TRAP_NONE;
            gl.trapped = trapped ? 1 : 0;
            if (trapped && !need_gaps) outcome = CC_T_L4_TRAPPED;
            queue_cert = F32 && outcome == CC_T_L4_R123LEAF && how == 2;
        }
        __syncwarp();
        bool decided = valid && !need_gaps;
        trace_note(bt, decided, decided ? trace_key(task_base + task, 3, i1, i2, i3, lf.i4, outcome) : 0,
                   decided ? outcome : 0);
        unsigned long long slot = warp_append(&c->n_gaps, valid && need_gaps, caps.gaps, &c->overflow);
        if (slot != ~0ULL) gq[slot] = gl;
        bool keep = decided && (outcome == CC_T_L4_CRITICAL || outcome == CC_T_L4_TRAPPED);
        push_critical(crit, warp_append(&c->n_crit, keep, caps.crit, &c->overflow), v, task, trapped);
        if (F32) {
            const unsigned long long cs = warp_append(&c->n_cert, valid && queue_cert, caps.leaf, &c->overflow);
            if (cs != ~0ULL) cq[cs] = CertLeaf{lf.cell4, lf.i4, 1, (uint8_t)calls};
        }
    }
    if (F32) tally.flush(c);
    trace_flush(bt, c, 3);
}

// FP64 certification of the leaf verdicts the FP32 enclosures decided "true"
// in stages 4a, 4a2 and 4b of the current slice.  Each block takes windows
// of 1024 jobs and sorts them in shared memory by a path key -- criterion,
// the call that settled the FP32 run, and the box features that select the
// criterion's placements on the way (2x2: r1 at least 1/2 takes the
// one-strip form; leaf r1_r2_r3: r2 and r3 above 1/4, where their strips
// exist) -- so that a warp's lanes mostly run the same path, then runs the
// FP64 criterion in record form up to that call (tight::certify_leaf), and
// finally evaluates the recorded calls of the window, sorted again by the
// branches can_recurse_t takes on them.  A failure is counted in fp32[3];
// the host then redoes the chunk in the plain FP64 form.
constexpr int kLeafCertWindow = 1024;
constexpr int kLeafCertKeys = 128;
// A recorded call written earlier in this kernel (by any thread of the
// block, before a barrier): loaded from L2 (ld.global.cg), never through the
// non-coherent read-only path.
__device__ __forceinline__ cc::CertCall load_call(const cc::CertCall* p) {
    const double* d = reinterpret_cast<const double*>(p);
    return cc::CertCall{__ldcg(d), __ldcg(d + 1), __ldcg(d + 2), __ldcg(d + 3)};
}

__global__ void __launch_bounds__(128) k_stage_cert(const Task* __restrict__ tasks, const Cell4* __restrict__ cells,
                                                    const CertLeaf* __restrict__ cq, cc::CertCall* calls, int s4,
                                                    Caps caps, Counters* c) {
    __shared__ CertLeaf s_job[kLeafCertWindow];
    __shared__ int s_cnt[kLeafCertKeys + 1];
    __shared__ uint8_t s_pend[kLeafCertWindow];
    __shared__ uint16_t s_order[kLeafCertWindow];
    constexpr int kPer = kLeafCertWindow / 128;
    constexpr int kNone = tight::kCallPathKeys;  // no recorded call to evaluate
    static_assert(kNone + 1 <= kLeafCertKeys + 1, "s_cnt holds the call keys");
    const unsigned long long n_in = *(volatile unsigned long long*)&c->n_cert;
    const unsigned long long total = n_in < caps.leaf ? n_in : caps.leaf;
    unsigned ok_n = 0, fail_n = 0;
    for (unsigned long long base = (unsigned long long)blockIdx.x * kLeafCertWindow; base < total;
         base += (unsigned long long)gridDim.x * kLeafCertWindow) {
        for (int k = threadIdx.x; k <= kLeafCertKeys; k += 128) s_cnt[k] = 0;
        __syncthreads();
        CertLeaf job[kPer];
        int key[kPer], rank[kPer];
#pragma unroll
        for (int t = 0; t < kPer; ++t) {
            const unsigned long long j = base + (unsigned long long)t * 128 + threadIdx.x;
            job[t] = CertLeaf{0, 0, 0, 0};
            key[t] = kLeafCertKeys;  // past the end: sorted last
            if (j < total) {
                job[t] = cq[j];
                const Cell4& p = cells[job[t].cell4];
                int f;
                if (job[t].crit == 0) f = p.r1.lo >= 0.5 ? 1 : 0;
                else f = (p.r2.lo > 0.25 ? 2 : 0) | (p.r3.lo > 0.25 ? 1 : 0);
                key[t] = (job[t].crit << 6) | ((job[t].call < 15 ? job[t].call : 15) << 2) | f;
            }
            rank[t] = atomicAdd(&s_cnt[key[t]], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // exclusive prefix over the keys
            int acc = 0;
            for (int k = 0; k <= kLeafCertKeys; ++k) {
                const int v = s_cnt[k];
                s_cnt[k] = acc;
                acc += v;
            }
        }
        __syncthreads();
#pragma unroll
        for (int t = 0; t < kPer; ++t) s_job[s_cnt[key[t]] + rank[t]] = job[t];
        __syncthreads();
        const unsigned long long left = total - base;
        const int valid_n = left < (unsigned long long)kLeafCertWindow ? (int)left : kLeafCertWindow;
        // the criteria in record form: a run stops at its chosen call, whose
        // arguments go to calls[base + slot] (cc_cert_out points at the
        // block's 128 entries of this round) ...
#pragma unroll 1
        for (int t = 0; t < kPer; ++t) {
            const int slot = t * 128 + threadIdx.x;
            if (threadIdx.x == 0) cc::cc_cert_out = calls + base + (unsigned long long)t * 128;
            __syncthreads();
            uint8_t pend = 0;
            if (slot < valid_n) {
                const CertLeaf m = s_job[slot];
                const Cell4& p = cells[m.cell4];
                const Task tk = tasks[p.task];
                trap_clear();
                const Box v = leaf_box(p, tk.la, subinterval(p.r4r, m.i4, s4));
                bool ok, reached = false;
                if (m.crit == 0) {
                    Iv R = tk.weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
                    tighten_lb(R, 0.0);
                    ok = tight::certify_leaf(tight::TwoByTwo{}, v, R, m.call, true, &reached);
                } else {
                    ok = tight::certify_leaf(tight::LeafR123{}, v, p.R4, m.call, true, &reached);
                }
                if (ok && reached) pend = 1;
                else if (ok) ++ok_n;
                else ++fail_n;
            }
            s_pend[slot] = pend;
            __syncthreads();  // cc_cert_out is moved next round
        }
        // ... and the chosen calls of the window run afterwards, sorted by the
        // branches can_recurse_t takes on them (tight::call_path_key), so the
        // lanes of a warp follow one path (the block's global writes above are
        // visible to all its threads after the barrier, read with load_call)
        for (int k = threadIdx.x; k <= kNone; k += 128) s_cnt[k] = 0;
        __syncthreads();
        int ckey[kPer], crank[kPer];
#pragma unroll
        for (int t = 0; t < kPer; ++t) {
            const int slot = t * 128 + threadIdx.x;
            ckey[t] = (slot < valid_n && s_pend[slot]) ? tight::call_path_key(load_call(calls + base + slot)) : kNone;
            crank[t] = atomicAdd(&s_cnt[ckey[t]], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int k = 0; k <= kNone; ++k) {
                const int v = s_cnt[k];
                s_cnt[k] = acc;
                acc += v;
            }
        }
        __syncthreads();
#pragma unroll
        for (int t = 0; t < kPer; ++t) {
            const int off = s_cnt[ckey[t]] + crank[t];
            s_order[off] = (uint16_t)(t * 128 + threadIdx.x);
            s_pend[off] = (uint8_t)ckey[t];  // the key, now in sorted order
        }
        __syncthreads();
#pragma unroll 1
        for (int t = 0; t < kPer; ++t) {
            const int pos = t * 128 + threadIdx.x;
            if (s_pend[pos] != kNone) {
                const cc::CertCall a = load_call(calls + base + s_order[pos]);
                trap_clear();
                const bool ok = tight::can_recurse_t<double>(a.w, a.h, a.largest, a.lb) && trap_status() == TRAP_NONE;
                trap_clear();
                if (ok) ++ok_n;
                else ++fail_n;
            }
        }
        __syncthreads();  // s_cnt, s_job, s_pend and s_order are rewritten next iteration
    }
    unsigned v0 = ok_n, v1 = fail_n;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_xor_sync(0xffffffffu, v0, o);
        v1 += __shfl_xor_sync(0xffffffffu, v1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (v0) atomicAdd(&c->fp32[2], (unsigned long long)v0);
        if (v1) atomicAdd(&c->fp32[3], (unsigned long long)v1);
    }
}

// stage 4c: the gaps bisection on full warps of leaves that need it
// (r1_r2_large_r3_r4_gaps_strategy.cu:61-98)
__global__ void __launch_bounds__(128) k_stage4c(const Task* __restrict__ tasks, const Cell4* __restrict__ cells,
                                                 const GapsLeaf* __restrict__ gq, int s4, Critical* __restrict__ crit,
                                                 Caps caps, Counters* c, unsigned long long task_base) {
    __shared__ BlockTrace bt;
    trace_init(bt);
    const unsigned long long n_in = *(volatile unsigned long long*)&c->n_gaps;
    const unsigned long long total = n_in < caps.gaps ? n_in : caps.gaps;
    CC_WARP_LOOP(total) {
        unsigned long long idx = base_ + (threadIdx.x & 31);
        bool valid = idx < total;
        int outcome = -1;
        Box v;
        int task = 0, i1 = 0, i2 = 0, i3 = 0, i4 = 0;
        bool trapped = false;
        if (valid) {
            const GapsLeaf& gl = gq[idx];
            const Cell4& p = cells[gl.cell4];
            task = p.task;
            i1 = p.i1;
            i2 = p.i2;
            i3 = p.i3;
            i4 = gl.i4;
            uint32_t m = tight::gaps_pass(gl.job);
            trapped = gl.trapped || (m >> 31);
            outcome = trapped ? CC_T_L4_TRAPPED : ((m & (1u << 5)) ? CC_T_L4_GAPS : CC_T_L4_CRITICAL);
            if (outcome != CC_T_L4_GAPS) {
                const Task tk = tasks[task];
                v = leaf_box(p, tk.la, subinterval(p.r4r, i4, s4));
            }
        }
        __syncwarp();
        trace_note(bt, valid, valid ? trace_key(task_base + task, 3, i1, i2, i3, i4, outcome) : 0, valid ? outcome : 0);
        bool keep = valid && (outcome == CC_T_L4_CRITICAL || outcome == CC_T_L4_TRAPPED);
        push_critical(crit, warp_append(&c->n_crit, keep, caps.crit, &c->overflow), v, task, trapped);
    }
    trace_flush(bt, c, 3);
}

#endif  // CC_DEVICE_BUILD

}  // namespace prove
}  // namespace cc

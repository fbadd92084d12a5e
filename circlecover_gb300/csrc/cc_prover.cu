// The prover's single CUDA translation unit for sm_103a: kernels and the
// extern "C" entry points of include/circlecover_gb300.h.
//
// One translation unit (no -rdc) so that every criterion inlines into the
// kernels; the reference compiles with separable compilation
// (algcuda/UseCUDA.cmake:30-31, 42), which keeps each criterion an opaque call.
// Built with -fmad=false: the only contraction the reference relies on,
// get_subinterval's FMA, is written out explicitly (cc_iv.cuh).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cc_mlp.cuh"
#include "cc_runtime.cuh"
#include "cc_tight.cuh"
#include "cc_tight_prove.cuh"
#include "cc_tight_summary.cuh"

#include <algorithm>
#include <mutex>

using cc::Iv;
namespace ct = cc::tight;

// ===================================================================== eval
// Layout of a box batch in device memory.
enum class Layout { AoS, SoA };

template <Layout L>
__device__ __forceinline__ ct::Box load_box(const double* __restrict__ in, size_t n, size_t i) {
    ct::Box b;
    double v[10];
    if (L == Layout::SoA) {
#pragma unroll
        for (int k = 0; k < 10; ++k) v[k] = __ldg(in + (size_t)k * n + i);
    } else {
        const double2* p = reinterpret_cast<const double2*>(in + i * 10);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            double2 t = __ldg(p + k);
            v[2 * k] = t.x;
            v[2 * k + 1] = t.y;
        }
    }
    b.la = Iv{v[0], v[1]};
#pragma unroll
    for (int k = 0; k < 4; ++k) b.r[k] = Iv{v[2 + 2 * k], v[3 + 2 * k]};
    return b;
}

// ---- six-pass evaluation --------------------------------------------------
// GB300 issues FP32 instructions at many times the FP64 rate, and a warp pays
// for every path any of its lanes takes.  So:
//   pass 0  every box: the criteria on FP32 enclosures of the FP64 values
//           (ct::eval_group_f32), one kernel per criterion group (the whole
//           FP32 evaluation does not fit the instruction cache), each ORing
//           its bits into the box's mask -- the heavy groups record their
//           can_recurse calls and evaluate them in rounds over compacted
//           queues; then k_eval_collect appends the boxes some group could
//           not decide to the `full` queue, the boxes that need a bisection
//           and every "true" bit to certify to their queues (one atomic per
//           queue and block);
//   pass 1  k_eval_main on the `full` queue: the FP64 criteria (ct::eval_main);
//   pass 2  k_eval_cover: boxes that need the strip-width bisection (~14% of
//           the microbench), with the FP64 steps resumed in a second kernel
//           on full warps;
//   pass 3  k_eval_gaps: boxes that need the gap-width bisection (~31%);
//   pass 4  k_eval_cert: FP64 certification of every verdict bit pass 0
//           decided "true", one kernel per criterion group on its queue, and
//           k_eval_cert_calls for the recorded calls (passes 2 and 3 certify
//           their own true results);
//   pass 5  k_eval_repair: the boxes whose certification failed, evaluated
//           again in FP64 alone.
// The queues hold box indices; each pass reads the box itself.
struct EvalQueues {
    uint32_t* full;
    uint32_t* cover_box;
    uint32_t* gaps_box;
    unsigned long long* counts;  // kCnt* below
    unsigned long long cap;
    // recorded calls of the heavy FP32 groups (null: every group in one kernel)
    ct::CrArgs* args;        // n x kCrRecordSlots
    uint8_t* states;         // kRecGroups x n
    uint32_t* q[2];          // pending boxes of a call round
    unsigned long long* rc;  // the two rounds' queue counters
    ct::EncBox* enc;         // enclosed boxes and weights (n)
    // FP64 certification (cert[0] null: off)
    uint32_t* cert[5];  // FP32 "true" verdicts to certify: record groups r1, r1_r2, 2x2, leaf; three-strip group
    uint8_t* cflags;    // per box: the three-strip group's bits to certify (1: bit 2, 2: bit 6)
    uint32_t* repair;   // boxes whose certification failed
};
enum : int {
    kCntCover = 0, kCntGaps = 1, kCntOverflow = 2, kCntFull = 3,
    kCntCert = 4,          // 4..8: the certification queues
    kCntRepair = 9,        // boxes to evaluate again in FP64 alone
    kCntCoverCert = 10,    // true strip-width results certified
    kCntGapsCert = 11,     // true gap-width results certified
    kCntCoverLoop = 12,    // strip-width jobs whose bisection resumes with FP64 steps (pass 2, second kernel)
};
static constexpr int kEvalCounters = 13;
static constexpr int kCertQueues = 5;
// the groups whose can_recurse calls are recorded, and their verdict bits
static constexpr int kRecGroups = 4;
__host__ __device__ constexpr int rec_group(int k) { return k < 2 ? k : k + 1; }  // 0, 1, 3, 4

// MinB: the register budget (__launch_bounds__ minimum resident blocks per
// SM: 1 = up to 255 registers per thread, 4 = 128, 8 = 64), chosen per
// pass by the autotuner (cc_autotune_eval) together with the grid size.
template <Layout L, int G, int MinB = 1>
__global__ void __launch_bounds__(128, MinB) k_eval_f32(const double* __restrict__ in, size_t n,
                                                        uint32_t* __restrict__ masks, int first,
                                                        ct::EncBox* __restrict__ enc) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (first) {
            masks[i] = ct::eval_group_f32<G>(load_box<L>(in, n, i), enc ? enc + i : nullptr);
        } else {
            const uint32_t prev = masks[i];
            if (prev & ct::kF32Undecided) continue;  // left to the FP64 pass anyway
            masks[i] = prev | ct::eval_group_f32<G>(load_box<L>(in, n, i));
        }
    }
}

// A group with recorded calls: the record pass runs the criterion with
// can_recurse recording instead of evaluating; boxes with calls to make go
// to the first round's queue.
template <int G, int MinB = 1>
__global__ void __launch_bounds__(128, MinB) k_eval_record(const ct::EncBox* __restrict__ enc, size_t n,
                                                           const uint32_t* __restrict__ masks,
                                                           ct::CrArgs* __restrict__ args, uint8_t* __restrict__ state,
                                                           uint32_t* __restrict__ q, unsigned long long* nq,
                                                           unsigned long long* overflow) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n;
         base += stride) {
        unsigned long long i = base + (threadIdx.x & 31);
        bool pending = false;
        if (i < n) {
            uint8_t st = ct::kRecUndecided;  // a box the first kernel left undecided goes to the FP64 pass anyway
            if (!(masks[i] & ct::kF32Undecided)) st = ct::record_group_f32<G>(enc[i], args + i * ct::kCrRecordSlots);
            state[i] = st;
            pending = (st & 3) == ct::kRecPending;
        }
        __syncwarp();
        unsigned long long s = cc::prove::warp_append(nq, pending, n, overflow);
        if (s != ~0ULL) q[s] = (uint32_t)i;
    }
}

// Round `round` of the recorded calls: call `round` of every box still
// pending, on full warps.  A true or undecided answer settles the box (the
// FP64 criterion returns at its first true call); a false one sends it to the
// next round, or, after its last call, to the status its criterion ends with.
__global__ void __launch_bounds__(128) k_eval_calls(const ct::CrArgs* __restrict__ args, uint8_t* __restrict__ state,
                                                    int round, const uint32_t* __restrict__ q_in,
                                                    const unsigned long long* n_in, uint32_t* __restrict__ q_out,
                                                    unsigned long long* n_out, unsigned long long cap,
                                                    unsigned long long* overflow) {
    const unsigned long long total = *n_in < cap ? *n_in : cap;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total;
         base += stride) {
        unsigned long long j = base + (threadIdx.x & 31);
        bool more = false;
        uint32_t i = 0;
        if (j < total) {
            i = q_in[j];
            const uint8_t st = state[i];
            const ct::CrArgs a = args[(size_t)i * ct::kCrRecordSlots + round];
            cc::trap_clear();
            const bool ok = ct::can_recurse(a.w, a.h, a.largest, a.lb);
            const bool undecided = cc::trap_status() != cc::TRAP_NONE;
            cc::trap_clear();
            uint8_t next;
            if (undecided) next = ct::kRecUndecided;
            else if (ok) next = (uint8_t)(ct::kRecTrue | ((round + 1) << 2));  // the call that settled it
            else if (round + 1 < ((st >> 2) & 7)) more = true, next = st;
            else next = (uint8_t)((st >> 5) & 3);
            state[i] = next;
        }
        __syncwarp();
        unsigned long long s = cc::prove::warp_append(n_out, more, cap, overflow);
        if (s != ~0ULL) q_out[s] = i;
    }
}

// The appends of a tile of 128 boxes are aggregated per block: one atomic per
// queue and tile, issued by different threads at once (appended warp by warp,
// a warp waited for eight atomics in a row per 32 boxes).
constexpr int kCollectQueues = 3 + kCertQueues;  // full, cover, gaps, the certification queues
__global__ void __launch_bounds__(128) k_eval_collect(size_t n, uint32_t* __restrict__ masks, EvalQueues q) {
    __shared__ unsigned s_warp[kCollectQueues][4];
    __shared__ unsigned long long s_base[kCollectQueues];
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n_queues = q.cert[0] ? kCollectQueues : 3;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    // block-uniform loop: every thread of the block runs every iteration
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const unsigned long long i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t m = valid ? masks[i] : 0u;
        if (valid && q.states) {
            for (int k = 0; k < kRecGroups; ++k) {
                const uint8_t st = q.states[(size_t)k * n + i] & 3;
                if (st == ct::kRecTrue) m |= 1u << rec_group(k);
                else if (st != ct::kRecFalse) m |= ct::kF32Undecided;
            }
        }
        const bool undecided = (m & ct::kF32Undecided) != 0;
        const bool need_cover = !undecided && (m & ct::kF32Cover);
        const bool need_gaps = !undecided && (m & ct::kF32Gaps);
        if (valid && (q.states || (m & (ct::kF32Undecided | ct::kF32Cover | ct::kF32Gaps))))
            masks[i] = m & ~(ct::kF32Undecided | ct::kF32Cover | ct::kF32Gaps);
        // the FP32 pass's "true" bits, to certify in FP64
        const bool fp32 = valid && !undecided && q.cert[0] != nullptr;
        const uint8_t cf = (uint8_t)(((m >> 2) & 1u) | (((m >> 6) & 1u) << 1));
        bool want[kCollectQueues];
        want[0] = valid && undecided;
        want[1] = valid && need_cover;
        want[2] = valid && need_gaps;
        for (int k = 0; k < kRecGroups; ++k) want[3 + k] = fp32 && ((m >> rec_group(k)) & 1u);
        want[3 + kRecGroups] = fp32 && cf;
        unsigned ballot[kCollectQueues];
#pragma unroll
        for (int k = 0; k < kCollectQueues; ++k) {
            ballot[k] = __ballot_sync(0xffffffffu, want[k]);
            if (lane == 0) s_warp[k][w] = __popc(ballot[k]);
        }
        __syncthreads();
        if ((int)threadIdx.x < n_queues) {
            const int k = threadIdx.x;
            const unsigned tot = s_warp[k][0] + s_warp[k][1] + s_warp[k][2] + s_warp[k][3];
            unsigned long long* ctr = k == 0 ? &q.counts[kCntFull]
                                    : k == 1 ? &q.counts[kCntCover]
                                    : k == 2 ? &q.counts[kCntGaps]
                                             : &q.counts[kCntCert + (k - 3)];
            s_base[k] = tot ? atomicAdd(ctr, (unsigned long long)tot) : 0ULL;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kCollectQueues; ++k) {
            if (!want[k]) continue;
            unsigned before = __popc(ballot[k] & ((1u << lane) - 1u));
            for (unsigned v = 0; v < w; ++v) before += s_warp[k][v];
            const unsigned long long slot = s_base[k] + before;
            if (slot >= q.cap) {
                atomicExch(&q.counts[kCntOverflow], 1ULL);
                continue;
            }
            uint32_t* dst = k == 0 ? q.full : k == 1 ? q.cover_box : k == 2 ? q.gaps_box : q.cert[k - 3];
            dst[slot] = (uint32_t)i;
            if (k == 3 + kRecGroups) q.cflags[i] = cf;
        }
        __syncthreads();  // s_warp and s_base are rewritten next iteration
    }
}

// pass 4: FP64 certification of the FP32 pass's "true" verdicts of group K
// (0..3: the record groups r1, r1_r2, 2x2, leaf; 4: the three-strip group).
// A record group's state byte names the call that settled the criterion
// (bits 2-4, 1-based; 0: none); without record buffers every call is
// evaluated.  Failures go to the repair queue.
// Each block takes a window of 1024 consecutive jobs at a time and sorts it
// in shared memory by a path key: the call that settled the FP32 run (the
// three-strip group: its bits) and the box features that select the
// criterion's blocks on the way to that call (the r1 placements exist for r1
// above 1/4 -- the strip -- and below 1/2 -- the corner; r1_r2's side by side
// needs r2 above 1/4, its stacked placement r1 up to 1/2; the leaf criterion's
// strips need r3 above 1/4), so that the lanes of a warp mostly run the same
// path through the FP64 criterion.
constexpr int kCertWindow = 1024;
constexpr int kCertKeys = 64;

template <Layout L, int K>
__device__ __forceinline__ int cert_path_key(const double* __restrict__ in, size_t n, uint32_t i, int call) {
    auto lo = [&](int k) -> double {  // lower bound of interval k (0 la, 1..4 r1..r4)
        return L == Layout::SoA ? __ldg(in + (size_t)(2 * k) * n + i) : __ldg(in + (size_t)i * 10 + 2 * k);
    };
    int f = 0;
    if (K == 0) {
        const double r1 = lo(1);
        f = (r1 > 0.25 ? 2 : 0) | (r1 < 0.5 ? 1 : 0);
    } else if (K == 1) {
        f = (lo(2) > 0.25 ? 2 : 0) | (lo(1) <= 0.5 ? 1 : 0);
    } else if (K == 3) {
        f = lo(3) > 0.25 ? 1 : 0;
    }
    return ((call & 7) << 3) | f;
}

// With record buffers, a record group's run stops at its chosen call (the
// record form of certify_group): the call's FP64 arguments go to the box's
// record slot K, the state byte is marked pending (kCertPending), and
// k_eval_cert_calls evaluates all those calls afterwards on full warps --
// can_recurse is most of a run's work, and the lanes of a warp reach it at
// different call sites.
constexpr uint8_t kCertPending = 0x80;  // state byte: the chosen call awaits k_eval_cert_calls
static_assert(sizeof(cc::CertCall) == sizeof(ct::CrArgs), "a record slot holds one chosen call");

template <Layout L, int K>
__global__ void __launch_bounds__(128) k_eval_cert(const double* __restrict__ in, size_t n, EvalQueues q) {
    __shared__ uint32_t s_box[kCertWindow];
    __shared__ uint8_t s_key[kCertWindow];
    __shared__ int s_cnt[kCertKeys + 1];
    __shared__ cc::CertCall s_call[128];
    constexpr int kPer = kCertWindow / 128;
    if (K < kRecGroups && threadIdx.x == 0) cc::cc_cert_out = s_call;
    const unsigned long long c = q.counts[kCntCert + K];
    const unsigned long long nq = c < q.cap ? c : q.cap;
    const unsigned long long stride = (unsigned long long)gridDim.x * kCertWindow;
    // block-uniform loop: every thread of the block runs every iteration
    for (unsigned long long base = (unsigned long long)blockIdx.x * kCertWindow; base < nq; base += stride) {
        for (int k = threadIdx.x; k <= kCertKeys; k += 128) s_cnt[k] = 0;
        __syncthreads();
        uint32_t box[kPer];
        int key[kPer], rank[kPer];
#pragma unroll
        for (int t = 0; t < kPer; ++t) {
            const unsigned long long j = base + (unsigned long long)t * 128 + threadIdx.x;
            box[t] = 0;
            key[t] = kCertKeys;  // past the end: sorted last
            if (j < nq) {
                box[t] = q.cert[K][j];
                if (K < kRecGroups) {
                    const int call = q.states ? (int)((q.states[(size_t)K * n + box[t]] >> 2) & 7) : 6;
                    key[t] = cert_path_key<L, K>(in, n, box[t], call);
                } else {
                    key[t] = q.cflags[box[t]] & 3;
                }
            }
            rank[t] = atomicAdd(&s_cnt[key[t]], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // exclusive prefix over the keys
            int acc = 0;
            for (int k = 0; k <= kCertKeys; ++k) {
                const int v = s_cnt[k];
                s_cnt[k] = acc;
                acc += v;
            }
        }
        __syncthreads();
#pragma unroll
        for (int t = 0; t < kPer; ++t) {
            const int off = s_cnt[key[t]] + rank[t];
            s_box[off] = box[t];
            s_key[off] = (uint8_t)(key[t] >> 3);  // the call (record groups)
        }
        __syncthreads();
        const unsigned long long left = nq - base;
        const int valid_n = left < (unsigned long long)kCertWindow ? (int)left : kCertWindow;
#pragma unroll 1
        for (int t = 0; t < kPer; ++t) {
            const int slot = t * 128 + threadIdx.x;
            const bool valid = slot < valid_n;
            bool fail = false;
            uint32_t b_i = 0;
            if (valid) {
                b_i = s_box[slot];
                const ct::Box b = load_box<L>(in, n, b_i);
                if (K < kRecGroups) {
                    bool reached = false;
                    fail = !ct::certify_group<rec_group(K)>(b, q.states ? (int)s_key[slot] : -1, q.args != nullptr,
                                                            &reached);
                    if (q.states) {
                        uint8_t& st = q.states[(size_t)K * n + b_i];
                        const bool pending = !fail && reached;
                        if (pending)
                            reinterpret_cast<cc::CertCall*>(q.args)[(size_t)b_i * ct::kCrRecordSlots + K] =
                                s_call[threadIdx.x];
                        st = (uint8_t)((st & (uint8_t)~kCertPending) | (pending ? kCertPending : 0));
                    }
                } else {
                    const uint8_t f = q.cflags[b_i];
                    fail = !ct::certify_r123(b, ((f & 1) ? (1u << 2) : 0u) | ((f & 2) ? (1u << 6) : 0u));
                }
            }
            __syncwarp();
            const unsigned long long s = cc::prove::warp_append(&q.counts[kCntRepair], valid && fail, q.cap,
                                                                &q.counts[kCntOverflow]);
            if (s != ~0ULL) q.repair[s] = b_i;
        }
        __syncthreads();  // s_cnt and the sorted arrays are rewritten next iteration
    }
}

// pass 4, last kernel: the chosen can_recurse call of every record-form
// certification run that reached it, on the FP64 arguments k_eval_cert
// stored; a false result or a trap fails the certification (the box goes to
// the repair queue).  The calls take different branches of can_recurse_t
// (size-bound ratio or not, orientation, the critical ratio's formula), so
// each block sorts a window of 1,024 jobs by that path (ct::call_path_key)
// before it evaluates them.
__global__ void __launch_bounds__(128) k_eval_cert_calls(size_t n, EvalQueues q) {
    __shared__ uint32_t s_slot[kCertWindow];
    __shared__ uint8_t s_key[kCertWindow];
    __shared__ int s_cnt[ct::kCallPathKeys + 2];
    constexpr int kPer = kCertWindow / 128;
    constexpr int kNone = ct::kCallPathKeys;  // nothing to evaluate (not pending, or past the end)
    if (!q.states || !q.args) return;
    unsigned long long cnt[kRecGroups], total = 0;
#pragma unroll
    for (int k = 0; k < kRecGroups; ++k) {
        const unsigned long long c = q.counts[kCntCert + k];
        cnt[k] = c < q.cap ? c : q.cap;
        total += cnt[k];
    }
    const cc::CertCall* calls = reinterpret_cast<const cc::CertCall*>(q.args);
    const unsigned long long stride = (unsigned long long)gridDim.x * kCertWindow;
    // block-uniform loop: every thread of the block runs every iteration
    for (unsigned long long base = (unsigned long long)blockIdx.x * kCertWindow; base < total; base += stride) {
        for (int k = threadIdx.x; k < ct::kCallPathKeys + 2; k += 128) s_cnt[k] = 0;
        __syncthreads();
        uint32_t slot[kPer];
        int key[kPer], rank[kPer];
#pragma unroll
        for (int t = 0; t < kPer; ++t) {
            const unsigned long long j = base + (unsigned long long)t * 128 + threadIdx.x;
            slot[t] = 0;
            key[t] = kNone;
            if (j < total) {
                unsigned long long jj = j;
                int k = 0;
                while (k < kRecGroups - 1 && jj >= cnt[k]) jj -= cnt[k++];
                const uint32_t b_i = q.cert[k][jj];
                if (q.states[(size_t)k * n + b_i] & kCertPending) {
                    slot[t] = b_i * (uint32_t)ct::kCrRecordSlots + (uint32_t)k;
                    key[t] = ct::call_path_key(calls[slot[t]]);
                }
            }
            rank[t] = atomicAdd(&s_cnt[key[t]], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // exclusive prefix over the keys
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
            const int off = s_cnt[key[t]] + rank[t];
            s_slot[off] = slot[t];
            s_key[off] = (uint8_t)key[t];
        }
        __syncthreads();
#pragma unroll 1
        for (int t = 0; t < kPer; ++t) {
            const int pos = t * 128 + threadIdx.x;
            bool fail = false;
            const uint32_t sl = s_slot[pos];
            if (s_key[pos] != kNone) {
                const cc::CertCall a = calls[sl];
                cc::trap_clear();
                const bool ok = ct::can_recurse_t<double>(a.w, a.h, a.largest, a.lb);
                fail = !ok || cc::trap_status() != cc::TRAP_NONE;
                cc::trap_clear();
            }
            __syncwarp();
            const unsigned long long s = cc::prove::warp_append(&q.counts[kCntRepair], fail, q.cap,
                                                                &q.counts[kCntOverflow]);
            if (s != ~0ULL) q.repair[s] = sl / (uint32_t)ct::kCrRecordSlots;
        }
        __syncthreads();  // s_cnt and the sorted arrays are rewritten next iteration
    }
}

// pass 5: boxes whose certification failed, evaluated again in FP64 alone
// (every criterion and both bisections as the reference computes them)
template <Layout L>
__global__ void __launch_bounds__(128) k_eval_repair(const double* __restrict__ in, size_t n, EvalQueues q,
                                                     uint32_t* __restrict__ masks) {
    const unsigned long long c = q.counts[kCntRepair];
    const unsigned long long nq = c < q.cap ? c : q.cap;
    for (unsigned long long j = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; j < nq;
         j += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t i = q.repair[j];
        masks[i] = ct::eval_all_fp64(load_box<L>(in, n, i));
    }
}

// a failed certificate of a bisection pass: the box to the repair queue
__device__ __forceinline__ void eval_repair_push(const EvalQueues& q, uint32_t i) {
    const unsigned long long s = atomicAdd(&q.counts[kCntRepair], 1ULL);
    if (s < q.cap) q.repair[s] = i;
    else atomicExch(&q.counts[kCntOverflow], 1ULL);
}
// per-thread tally summed over the warp, one atomic per warp (every lane
// of the block reaches the end of the kernel's loop)
__device__ __forceinline__ void warp_tally(unsigned long long* counter, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(counter, v);
}

template <Layout L, int MinB = 1>
__global__ void __launch_bounds__(128, MinB) k_eval_main(const double* __restrict__ in, size_t n,
                                                         uint32_t* __restrict__ masks, EvalQueues q) {
    const unsigned long long nq = q.counts[3] < q.cap ? q.counts[3] : q.cap;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < nq;
         base += stride) {
        unsigned long long j = base + (threadIdx.x & 31);
        bool valid = j < nq;
        bool need_cover = false, need_gaps = false;
        uint32_t i = 0;
        if (valid) {
            i = q.full[j];
            ct::Box b = load_box<L>(in, n, i);
            ct::CoverJob cj;
            ct::GapsJob gj;
            masks[i] = ct::eval_main(b, need_cover, cj, need_gaps, gj);
        }
        __syncwarp();
        unsigned long long s = cc::prove::warp_append(&q.counts[0], valid && need_cover, q.cap, &q.counts[2]);
        if (s != ~0ULL) q.cover_box[s] = i;
        s = cc::prove::warp_append(&q.counts[1], valid && need_gaps, q.cap, &q.counts[2]);
        if (s != ~0ULL) q.gaps_box[s] = i;
    }
}

// pass 2 in two kernels.  The strip-width bisections decide their leading
// steps in FP32 (while the whole warp agrees) and most jobs are settled
// there; the rest need FP64 steps to the fixpoint, which a warp would run
// for its few remaining lanes.  So the first kernel stops a job at its first
// FP64 step and queues its bracket (in the record buffer, unused between the
// call rounds and the certification pass), and the second runs those FP64
// steps on full warps.  Without record buffers (the allocation-free entry)
// the first kernel finishes every job itself.
static_assert(sizeof(ct::CoverResume) <= ct::kCrRecordSlots * sizeof(ct::CrArgs), "a resume state per box slot");
template <Layout L, int MinB = 1, bool Resume = false>
__global__ void __launch_bounds__(128, MinB) k_eval_cover(const double* __restrict__ in, size_t n, EvalQueues q,
                                                          uint32_t* __restrict__ masks) {
    const unsigned long long c = Resume ? q.counts[kCntCoverLoop] : q.counts[0];
    const unsigned long long nq = c < q.cap ? c : q.cap;
    ct::CoverResume* states = reinterpret_cast<ct::CoverResume*>(q.args);
    if (Resume && !states) return;
    const bool certify = q.cert[0] != nullptr;
    unsigned long long certified = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < nq;
         base += stride) {
        const unsigned long long j = base + (threadIdx.x & 31);
        ct::CoverResume st;
        st.it = -1;
        if (j < nq) {
            uint32_t i;
            bool repair = false;
            uint32_t m;
            if (Resume) {
                st = states[j];
                i = st.box;
                m = ct::cover_pass_resume(load_box<L>(in, n, i), q.enc ? q.enc + i : nullptr, certify, &repair, st);
                st.it = -1;
            } else {
                i = q.cover_box[j];
                m = ct::cover_pass_box(load_box<L>(in, n, i), q.enc ? q.enc + i : nullptr, certify, &repair,
                                       states ? &st : nullptr);
                st.box = i;
            }
            if (m) masks[i] |= m;
            if (repair) eval_repair_push(q, i);
            else if (certify && (m & (1u << 2)) && !(m >> 31)) ++certified;
        }
        if (!Resume) {
            __syncwarp();
            const unsigned long long s = cc::prove::warp_append(&q.counts[kCntCoverLoop], st.it >= 0, q.cap,
                                                                &q.counts[kCntOverflow]);
            if (s != ~0ULL) states[s] = st;
        }
    }
    if (certify) warp_tally(&q.counts[kCntCoverCert], certified);
}

template <Layout L, int MinB = 1>
__global__ void __launch_bounds__(128, MinB) k_eval_gaps(const double* __restrict__ in, size_t n, EvalQueues q,
                                                         uint32_t* __restrict__ masks) {
    const unsigned long long nq = q.counts[1] < q.cap ? q.counts[1] : q.cap;
    const bool certify = q.cert[0] != nullptr;
    unsigned long long certified = 0;
    for (unsigned long long j = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; j < nq;
         j += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t i = q.gaps_box[j];
        bool repair = false;
        uint32_t m = ct::gaps_pass_box(load_box<L>(in, n, i), q.enc ? q.enc + i : nullptr, certify, &repair);
        if (m) masks[i] |= m;
        if (repair) eval_repair_push(q, i);
        else if (certify && (m & (1u << 5)) && !(m >> 31)) ++certified;
    }
    if (certify) warp_tally(&q.counts[kCntGapsCert], certified);
}

// queue and record buffers for up to `cap` boxes in handle slots 16..20 and
// 35..39 (about 250 bytes per box)
static int eval_queues(cc_handle* h, size_t cap, EvalQueues* q) {
    void *a, *b, *c, *e, *args, *states, *q0, *q1, *rc;
    int st;
    if ((st = ccrt::ensure(h, 16, cap * sizeof(uint32_t), &a))) return st;
    if ((st = ccrt::ensure(h, 17, cap * sizeof(uint32_t), &b))) return st;
    if ((st = ccrt::ensure(h, 18, cap * sizeof(uint32_t), &c))) return st;
    if ((st = ccrt::ensure(h, 19, kEvalCounters * sizeof(unsigned long long), &e))) return st;
    if ((st = ccrt::ensure(h, 20, cap * ct::kCrRecordSlots * sizeof(ct::CrArgs), &args))) return st;
    if ((st = ccrt::ensure(h, 35, cap * kRecGroups, &states))) return st;
    if ((st = ccrt::ensure(h, 36, cap * sizeof(uint32_t), &q0))) return st;
    if ((st = ccrt::ensure(h, 37, cap * sizeof(uint32_t), &q1))) return st;
    if ((st = ccrt::ensure(h, 38, 2 * sizeof(unsigned long long), &rc))) return st;
    void* enc;
    if ((st = ccrt::ensure(h, 39, cap * sizeof(ct::EncBox), &enc))) return st;
    *q = EvalQueues{(uint32_t*)a, (uint32_t*)b, (uint32_t*)c, (unsigned long long*)e, cap,
                    (ct::CrArgs*)args, (uint8_t*)states, {(uint32_t*)q0, (uint32_t*)q1}, (unsigned long long*)rc,
                    (ct::EncBox*)enc, {}, nullptr, nullptr};
    if (h->eval_certify) {  // certification queues in slots 24..26 (25 bytes per box)
        void *cq, *cf, *rq;
        if ((st = ccrt::ensure(h, 24, cap * kCertQueues * sizeof(uint32_t), &cq))) return st;
        if ((st = ccrt::ensure(h, 25, cap, &cf))) return st;
        if ((st = ccrt::ensure(h, 26, cap * sizeof(uint32_t), &rq))) return st;
        for (int k = 0; k < kCertQueues; ++k) q->cert[k] = (uint32_t*)cq + (size_t)k * cap;
        q->cflags = (uint8_t*)cf;
        q->repair = (uint32_t*)rq;
    }
    return CC_OK;
}

// launch of pass k (0 FP32, 1 FP64 main, 2 cover, 3 gaps) with a register
// budget and grid
// (the register budgets are tuned on device (SoA) batches; the host entry
// point's AoS batches use the default budget)
#define CC_EVAL_LAUNCH(KERNEL, ...)                                                                   \
    template <Layout L>                                                                               \
    static void launch_##KERNEL(int minb, int g, cudaStream_t s, const double* in, size_t n,          \
                                uint32_t* masks, EvalQueues q) {                                      \
        if constexpr (L == Layout::SoA) {                                                             \
            if (minb == 4) KERNEL<L, 4><<<g, 128, 0, s>>>(__VA_ARGS__);                               \
            else if (minb == 8) KERNEL<L, 8><<<g, 128, 0, s>>>(__VA_ARGS__);                          \
            else KERNEL<L, 1><<<g, 128, 0, s>>>(__VA_ARGS__);                                         \
        } else {                                                                                      \
            KERNEL<L, 1><<<g, 128, 0, s>>>(__VA_ARGS__);                                              \
        }                                                                                             \
    }
// pass 0: the FP32 group kernels, then the collection of the queues.  With
// record buffers, the heavy groups (r1, r1_r2, 2x2, leaf) run as a record
// pass plus call rounds; the three-strip group runs in one kernel either way.
template <Layout L>
static cudaError_t launch_k_eval_f32(int minb, int g, cudaStream_t s, const double* in, size_t n, uint32_t* masks,
                                     EvalQueues q) {
    cudaError_t e;
    if (q.args) {
#define CC_F32_RECORD(K)                                                                                      \
    {                                                                                                         \
        constexpr int G = rec_group(K);                                                                       \
        uint8_t* st = q.states + (size_t)(K) * n;                                                             \
        if ((e = cudaMemsetAsync(q.rc, 0, 2 * sizeof(unsigned long long), s)) != cudaSuccess) return e;       \
        if (minb == 4)                                                                                        \
            k_eval_record<G, 4><<<g, 128, 0, s>>>(q.enc, n, masks, q.args, st, q.q[0], &q.rc[0], &q.counts[2]); \
        else if (minb == 8)                                                                                   \
            k_eval_record<G, 8><<<g, 128, 0, s>>>(q.enc, n, masks, q.args, st, q.q[0], &q.rc[0], &q.counts[2]); \
        else                                                                                                  \
            k_eval_record<G, 1><<<g, 128, 0, s>>>(q.enc, n, masks, q.args, st, q.q[0], &q.rc[0], &q.counts[2]); \
        for (int r = 0; r < ct::kCrRecordSlots; ++r) {                                                        \
            e = cudaMemsetAsync(&q.rc[(r + 1) & 1], 0, sizeof(unsigned long long), s);                        \
            if (e != cudaSuccess) return e;                                                                   \
            k_eval_calls<<<g, 128, 0, s>>>(q.args, st, r, q.q[r & 1], &q.rc[r & 1], q.q[(r + 1) & 1],          \
                                          &q.rc[(r + 1) & 1], n, &q.counts[2]);                               \
        }                                                                                                     \
    }
        if (minb == 4 && L == Layout::SoA) k_eval_f32<L, ct::F32_R123, 4><<<g, 128, 0, s>>>(in, n, masks, 1, q.enc);
        else if (minb == 8 && L == Layout::SoA) k_eval_f32<L, ct::F32_R123, 8><<<g, 128, 0, s>>>(in, n, masks, 1, q.enc);
        else k_eval_f32<L, ct::F32_R123, 1><<<g, 128, 0, s>>>(in, n, masks, 1, q.enc);
        CC_F32_RECORD(0)
        CC_F32_RECORD(1)
        CC_F32_RECORD(2)
        CC_F32_RECORD(3)
#undef CC_F32_RECORD
        k_eval_collect<<<g, 128, 0, s>>>(n, masks, q);
        return cudaSuccess;
    }
#define CC_F32_GROUP(G)                                                                         \
    if constexpr (L == Layout::SoA) {                                                           \
        if (minb == 4) k_eval_f32<L, G, 4><<<g, 128, 0, s>>>(in, n, masks, G == 0, nullptr);          \
        else if (minb == 8) k_eval_f32<L, G, 8><<<g, 128, 0, s>>>(in, n, masks, G == 0, nullptr);        \
        else k_eval_f32<L, G, 1><<<g, 128, 0, s>>>(in, n, masks, G == 0, nullptr);                       \
    } else {                                                                                    \
        k_eval_f32<L, G, 1><<<g, 128, 0, s>>>(in, n, masks, G == 0, nullptr);                            \
    }
    CC_F32_GROUP(0)
    CC_F32_GROUP(1)
    CC_F32_GROUP(2)
    CC_F32_GROUP(3)
    CC_F32_GROUP(4)
#undef CC_F32_GROUP
    k_eval_collect<<<g, 128, 0, s>>>(n, masks, q);
    (void)e;
    return cudaSuccess;
}
CC_EVAL_LAUNCH(k_eval_main, in, n, masks, q)
CC_EVAL_LAUNCH(k_eval_gaps, in, n, q, masks)
#undef CC_EVAL_LAUNCH
// pass 2: the counter of the second kernel's queue starts at zero (the
// autotuner reruns the pass on its own); no second kernel without record
// buffers
template <Layout L>
static cudaError_t launch_k_eval_cover(int minb, int g, cudaStream_t s, const double* in, size_t n,
                                       uint32_t* masks, EvalQueues q) {
    const cudaError_t e = cudaMemsetAsync(&q.counts[kCntCoverLoop], 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const bool resume = q.args != nullptr;
    if (L == Layout::SoA && minb == 4) {
        k_eval_cover<L, 4, false><<<g, 128, 0, s>>>(in, n, q, masks);
        if (resume) k_eval_cover<L, 4, true><<<g, 128, 0, s>>>(in, n, q, masks);
    } else if (L == Layout::SoA && minb == 8) {
        k_eval_cover<L, 8, false><<<g, 128, 0, s>>>(in, n, q, masks);
        if (resume) k_eval_cover<L, 8, true><<<g, 128, 0, s>>>(in, n, q, masks);
    } else {
        k_eval_cover<L, 1, false><<<g, 128, 0, s>>>(in, n, q, masks);
        if (resume) k_eval_cover<L, 1, true><<<g, 128, 0, s>>>(in, n, q, masks);
    }
    return cudaSuccess;
}

// kernels launched by pass k beyond one (the FP32 pass's groups, rounds and
// collection; the certification pass's five group kernels) and whether a
// pass launches at all
static int pass_kernels(int pass, const EvalQueues& q) {
    if (pass == 0) return q.args ? 1 + kRecGroups * (1 + ct::kCrRecordSlots) + 1 : ct::F32_GROUPS + 1;
    if (pass == 2) return q.args ? 2 : 1;
    if (pass == 4) return q.cert[0] ? kCertQueues + (q.args ? 1 : 0) : 0;
    if (pass == 5) return q.cert[0] ? 1 : 0;
    return 1;
}

// the launches of one pass; the status of a memory operation among them (a
// launch's own error is left to cudaGetLastError)
template <Layout L>
static cudaError_t launch_pass(int pass, int minb, int g, cudaStream_t s, const double* in, size_t n,
                               uint32_t* masks, EvalQueues q) {
    switch (pass) {
        case 0: return launch_k_eval_f32<L>(minb, g, s, in, n, masks, q);
        case 1: launch_k_eval_main<L>(minb, g, s, in, n, masks, q); break;
        case 2: return launch_k_eval_cover<L>(minb, g, s, in, n, masks, q);
        case 3: launch_k_eval_gaps<L>(minb, g, s, in, n, masks, q); break;
        case 4:
            if (!q.cert[0]) break;
            k_eval_cert<L, 0><<<g, 128, 0, s>>>(in, n, q);
            k_eval_cert<L, 1><<<g, 128, 0, s>>>(in, n, q);
            k_eval_cert<L, 2><<<g, 128, 0, s>>>(in, n, q);
            k_eval_cert<L, 3><<<g, 128, 0, s>>>(in, n, q);
            k_eval_cert<L, 4><<<g, 128, 0, s>>>(in, n, q);
            if (q.args) k_eval_cert_calls<<<g, 128, 0, s>>>(n, q);
            break;
        default:
            if (q.cert[0]) k_eval_repair<L><<<g, 128, 0, s>>>(in, n, q, masks);
            break;
    }
    return cudaSuccess;
}

// the launch sequence of the six passes
template <Layout L>
static int eval_launches(cc_handle* h, const double* in, size_t n, uint32_t* masks, cudaStream_t s,
                         const EvalQueues& q) {
    CC_CUDA(h, cudaMemsetAsync(q.counts, 0, kEvalCounters * sizeof(unsigned long long), s));
    // a small batch takes no more blocks than it has boxes to spread over
    const size_t need = (n + 127) / 128;
    for (int pass = 0; pass < CC_EVAL_STAGES; ++pass) {
        if (h->timing) CC_CUDA(h, cudaEventRecord(h->stage_ev[pass], s));
        int g = h->sm_count * h->tune_grid[pass];
        if ((size_t)g > need) g = (int)need;
        CC_CUDA(h, launch_pass<L>(pass, h->tune_minb[pass], g, s, in, n, masks, q));
        CC_LAUNCHED(h);
        h->launches += pass_kernels(pass, q) - 1;
    }
    if (h->timing) CC_CUDA(h, cudaEventRecord(h->stage_ev[CC_EVAL_STAGES], s));
    return CC_OK;
}

// The six passes on one batch already on the device.  With the handle's
// evaluation graph on (the default) and graph_ok, the launch sequence is captured once
// into a CUDA graph and replayed by one cudaGraphLaunch while the same
// arguments repeat (a batch loop over fixed buffers); a call with other
// arguments re-captures it and updates the executable graph in place.  Not
// while stage timing is on, and not on a stream the caller is capturing
// (the launches then join the caller's graph).
template <Layout L>
static int eval_batch(cc_handle* h, const double* in, size_t n, uint32_t* masks, cudaStream_t s,
                      bool graph_ok = true) {
    EvalQueues q;
    int st = eval_queues(h, n, &q);
    if (st) return st;
    h->stages_recorded = 0;
    h->eval_counts = q.counts;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    bool graph = graph_ok && h->eval_graph && !h->timing && cudaStreamIsCapturing(s, &cap) == cudaSuccess &&
                 cap == cudaStreamCaptureStatusNone;
    if (!graph) cudaGetLastError();
    if (graph) {
        const uintptr_t key_items[] = {(uintptr_t)L, (uintptr_t)in, (uintptr_t)n, (uintptr_t)masks, (uintptr_t)s,
                                       (uintptr_t)q.full, (uintptr_t)q.cover_box, (uintptr_t)q.gaps_box,
                                       (uintptr_t)q.counts, (uintptr_t)q.args, (uintptr_t)q.states,
                                       (uintptr_t)q.q[0], (uintptr_t)q.q[1], (uintptr_t)q.rc, (uintptr_t)q.enc,
                                       (uintptr_t)h->sm_count, (uintptr_t)h->tune_minb[0], (uintptr_t)h->tune_minb[1],
                                       (uintptr_t)h->tune_minb[2], (uintptr_t)h->tune_minb[3],
                                       (uintptr_t)h->tune_grid[0], (uintptr_t)h->tune_grid[1],
                                       (uintptr_t)h->tune_grid[2], (uintptr_t)h->tune_grid[3],
                                       (uintptr_t)q.cert[0], (uintptr_t)q.cflags, (uintptr_t)q.repair};
        std::vector<uintptr_t> key(std::begin(key_items), std::end(key_items));
        if (!h->graph_exec || key != h->graph_key) {
            const uint64_t before = h->launches;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                cudaGetLastError();  // a stream that cannot be captured (the legacy default stream)
                goto direct;
            }
            st = eval_launches<L>(h, in, n, masks, s, q);
            cudaGraph_t g = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (st) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (ce != cudaSuccess) return ccrt::fail(h, CC_ERR_CUDA, "cudaStreamEndCapture", ce);
            bool updated = false;
            if (h->graph_exec) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(h->graph_exec, g, &info) == cudaSuccess;
                if (!updated) {
                    cudaGetLastError();
                    cudaGraphExecDestroy(h->graph_exec);
                    h->graph_exec = nullptr;
                }
            }
            cudaError_t ie = cudaSuccess;
            if (!updated) ie = cudaGraphInstantiate(&h->graph_exec, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) {
                h->graph_exec = nullptr;
                h->graph_key.clear();
                return ccrt::fail(h, CC_ERR_CUDA, "cudaGraphInstantiate", ie);
            }
            h->graph_key = key;
            h->graph_launches = h->launches - before;
            h->graph_captures++;
            h->launches = before;
        }
        CC_CUDA(h, cudaGraphLaunch(h->graph_exec, s));
        h->launches += h->graph_launches;
        h->graph_replays++;
        return CC_OK;
    }
direct:
    st = eval_launches<L>(h, in, n, masks, s, q);
    if (!st && h->timing) h->stages_recorded = CC_EVAL_STAGES;
    return st;
}

static int eval_grid(cc_handle* h, size_t n) {
    size_t blocks = (n + 127) / 128;
    size_t cap = (size_t)h->sm_count * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

// ================================================================ self-test
// Directed-rounding primitives exactly as the criteria call them, for the
// bit-equality test against the host rounding layer.
__global__ void k_selftest_round(int op, int up, const double* a, const double* b, double* out, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = a[i], y = b ? b[i] : 0.0, r = 0.0;
    switch (op) {
        case 0: r = up ? cc::add_up(x, y) : cc::add_dn(x, y); break;
        case 1: r = up ? cc::mul_up(x, y) : cc::mul_dn(x, y); break;
        case 2: r = up ? cc::div_up(x, y) : cc::div_dn(x, y); break;
        case 3: r = up ? cc::sqrt_up(x) : cc::sqrt_dn(x); break;
        case 4: r = up ? cc::rcp_up(x) : cc::rcp_dn(x); break;
    }
    out[i] = r;
}

// FP64 pipe throughput probe: independent chains of directed-rounding adds
// and multiplies (the instructions the criteria issue), or of FMAs.  8
// independent chains per thread hide the pipe latency.
__global__ void __launch_bounds__(256) k_fp64_peak(double* out, int iters, int use_fma) {
    double a[8], b = 1.0000000001, c = 1e-9;
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-7 + k;
    if (use_fma) {
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
        }
    } else {
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int k = 0; k < 8; k += 2) {
                a[k] = __dadd_rd(a[k], c);
                a[k + 1] = __dmul_ru(a[k + 1], b);
            }
        }
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

// FP32 counterpart: chains of directed-rounding adds and multiplies (the
// FP32 enclosures' instructions) or of FMAs.  An FP32 FMA warp instruction
// issues every cycle on each SM sub-partition, so the FMA rate / 32 is also
// the device's warp-instruction issue rate.
__global__ void __launch_bounds__(256) k_fp32_peak(float* out, int iters, int use_fma) {
    float a[8], b = 1.0000001f, c = 1e-7f;
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-4f + k;
    if (use_fma) {
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
        }
    } else {
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int k = 0; k < 8; k += 2) {
                a[k] = __fadd_rd(a[k], c);
                a[k + 1] = __fmul_ru(a[k + 1], b);
            }
        }
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678f) out[0] = s;  // keeps the chains alive
}

extern "C" int cc_selftest_subinterval_contracted(const double* lo, const double* hi, const int* idx, const int* cnt,
                                                  double* out, size_t n, void* stream);

__global__ void k_selftest_subinterval(const double* lo, const double* hi, const int* idx, const int* cnt, double* out,
                                       size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Iv r = cc::subinterval(Iv{lo[i], hi[i]}, idx[i], cnt[i]);
    out[2 * i] = r.lo;
    out[2 * i + 1] = r.hi;
}

// one bisection step decided both ways: the FP32 enclosure's outcome over a
// range of the bisection variable (-1 undecided, 0, 1) and the FP64
// predicate's (0, 1) at the range's lower end
__global__ void k_selftest_bisection_f32(int which, const double* __restrict__ args, size_t n, int8_t* f32_out,
                                         int8_t* f64_out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* a = args + 8 * i;
    const cc::f32::Fv range{__double2float_rd(a[6]), __double2float_ru(a[7])};
    cc::trap_clear();
    if (which == 0) {  // r1, r2, r3; w in [a6, a7]
        f32_out[i] = (int8_t)ct::strip_width_realizable_f32(ct::strip_f32_prepare(a[0], a[1], a[2]), range);
        f64_out[i] = ct::strip_width_realizable(a[0], a[1], a[2], a[6]) ? 1 : 0;
    } else {  // r1, r2, w1, w2, r4; g in [a6, a7]
        f32_out[i] = (int8_t)ct::gap_width_realizable_f32(range, ct::gaps_f32_prepare(a[0], a[1], a[2], a[3], a[4]));
        f64_out[i] = ct::gap_width_realizable(a[6], a[0], a[2], a[1], a[3], a[4]) ? 1 : 0;
    }
    if (cc::trap_status() != cc::TRAP_NONE) f64_out[i] |= 2;
}

// the FP64 certification run of record group K on each box, with the call
// number given per box (1-based; 0 none; -1 every call evaluated): bit 0 the
// direct form, bit 1 the record form (the chosen call evaluated afterwards)
template <int K>
__global__ void __launch_bounds__(128) k_selftest_certify(const double* __restrict__ aos, size_t n,
                                                          const int* __restrict__ call, uint8_t* __restrict__ out) {
    __shared__ cc::CertCall s_call[128];
    if (threadIdx.x == 0) cc::cc_cert_out = s_call;
    __syncthreads();
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ct::Box b = load_box<Layout::AoS>(aos, n, i);
    const bool direct = ct::certify_group<rec_group(K)>(b, call[i]);
    bool reached = false;
    bool record = ct::certify_group<rec_group(K)>(b, call[i], true, &reached);
    if (record && reached) {
        const cc::CertCall a = s_call[threadIdx.x];
        cc::trap_clear();
        record = ct::can_recurse_t<double>(a.w, a.h, a.largest, a.lb) && cc::trap_status() == cc::TRAP_NONE;
        cc::trap_clear();
    }
    out[i] = (uint8_t)((direct ? 1 : 0) | (record ? 2 : 0));
}

// the whole bisection (with the FP32 shortcuts) of each row
__global__ void k_selftest_bisection_width(int which, const double* __restrict__ args, size_t n, double* out,
                                           int8_t* trapped) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* a = args + 8 * i;
    cc::trap_clear();
    if (which == 0) out[i] = ct::cover_strip_width(a[6], a[0], a[1], a[2]);  // la_hi in column 6
    else out[i] = ct::gaps_width(a[0], a[1], a[4], ct::GapsStart{a[2], a[3]});
    trapped[i] = cc::trap_status() != cc::TRAP_NONE ? 1 : 0;
}

// ============================================================== C ABI
extern "C" {

const char* cc_status_str(int s) {
    switch (s) {
        case CC_OK: return "ok";
        case CC_ERR_CUDA: return "CUDA error";
        case CC_ERR_PARAM: return "invalid parameter";
        case CC_ERR_QUEUE_OVERFLOW: return "device queue overflow";
        case CC_ERR_TIMEOUT: return "device wait timed out";
        case CC_ERR_INTERRUPTED: return "interrupted";
        case CC_ERR_NO_DEVICE: return "no usable CUDA device";
        case CC_ERR_OOM: return "out of memory";
        case CC_ERR_TOO_LARGE: return "batch larger than the entry point's fixed capacity";
        default: return "unknown status";
    }
}

int cc_create(cc_handle** out, int device) {
    if (!out) return CC_ERR_PARAM;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return CC_ERR_NO_DEVICE;
    }
    cc_handle* h = new cc_handle();
    h->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        cudaGetLastError();
        return CC_ERR_NO_DEVICE;
    }
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        cudaGetLastError();
        pageable = 0;
    }
    const char* staging = std::getenv("CC_HOST_STAGING");
    h->pageable_access = pageable == 1 && !(staging && staging[0] == '1');
    // the kernels must exist for this device (built for sm_103a only)
    cudaFuncAttributes attr;
    if (cudaFuncGetAttributes(&attr, k_selftest_subinterval) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(h->stream);
        delete h;
        return CC_ERR_NO_DEVICE;
    }
    *out = h;
    return CC_OK;
}

int cc_destroy(cc_handle* h) {
    if (!h) return CC_ERR_PARAM;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto& b : h->bufs)
        if (b.ptr) cudaFree(b.ptr);
    if (h->pinned) cudaFreeHost(h->pinned);
    if (h->mlp_free) h->mlp_free(h);
    for (auto& e : h->stage_ev)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->stream2) {
        cudaStreamSynchronize(h->stream2);
        cudaStreamDestroy(h->stream2);
    }
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    delete h;
    return CC_OK;
}

int cc_set_eval_graph(cc_handle* h, int enable) {
    if (!h) return CC_ERR_PARAM;
    h->eval_graph = enable != 0;
    return CC_OK;
}

int cc_eval_graph_stats(cc_handle* h, unsigned long long* captures, unsigned long long* replays) {
    if (!h || !captures || !replays) return CC_ERR_PARAM;
    *captures = h->graph_captures;
    *replays = h->graph_replays;
    return CC_OK;
}

int cc_set_stage_timing(cc_handle* h, int enable) {
    if (!h) return CC_ERR_PARAM;
    CC_CUDA(h, cudaSetDevice(h->device));
    if (enable && !h->stage_ev[0])
        for (auto& e : h->stage_ev) CC_CUDA(h, cudaEventCreate(&e));
    h->timing = enable != 0;
    h->stages_recorded = 0;
    return CC_OK;
}

int cc_last_eval_counts(cc_handle* h, unsigned long long* counts) {
    if (!h || !counts) return ccrt::fail(h, CC_ERR_PARAM, "cc_last_eval_counts: bad argument");
    if (!h->eval_counts) return ccrt::fail(h, CC_ERR_PARAM, "cc_last_eval_counts: no evaluation recorded");
    CC_CUDA(h, cudaSetDevice(h->device));
    CC_CUDA(h, cudaDeviceSynchronize());
    unsigned long long c[kEvalCounters];
    CC_CUDA(h, cudaMemcpy(c, h->eval_counts, sizeof(c), cudaMemcpyDeviceToHost));
    counts[0] = c[3];
    counts[1] = c[0];
    counts[2] = c[1];
    counts[3] = c[2];
    return CC_OK;
}

int cc_set_eval_certify(cc_handle* h, int enable) {
    if (!h) return CC_ERR_PARAM;
    h->eval_certify = enable != 0;
    return CC_OK;
}

int cc_last_eval_cert(cc_handle* h, unsigned long long* counts) {
    if (!h || !counts) return ccrt::fail(h, CC_ERR_PARAM, "cc_last_eval_cert: bad argument");
    if (!h->eval_counts) return ccrt::fail(h, CC_ERR_PARAM, "cc_last_eval_cert: no evaluation recorded");
    CC_CUDA(h, cudaSetDevice(h->device));
    CC_CUDA(h, cudaDeviceSynchronize());
    unsigned long long c[kEvalCounters];
    CC_CUDA(h, cudaMemcpy(c, h->eval_counts, sizeof(c), cudaMemcpyDeviceToHost));
    for (int k = 0; k < kCertQueues; ++k) counts[k] = c[kCntCert + k];
    counts[5] = c[kCntRepair];
    counts[6] = c[kCntCoverCert];
    counts[7] = c[kCntGapsCert];
    return CC_OK;
}

int cc_last_stage_times(cc_handle* h, float* ms, int max_stages, int* n_stages) {
    if (!h || !ms || !n_stages || max_stages < 0) return ccrt::fail(h, CC_ERR_PARAM, "cc_last_stage_times: bad argument");
    *n_stages = 0;
    if (!h->stages_recorded) return ccrt::fail(h, CC_ERR_PARAM, "cc_last_stage_times: no timed call recorded");
    CC_CUDA(h, cudaSetDevice(h->device));
    CC_CUDA(h, cudaEventSynchronize(h->stage_ev[h->stages_recorded]));
    int k = h->stages_recorded < max_stages ? h->stages_recorded : max_stages;
    for (int i = 0; i < k; ++i) CC_CUDA(h, cudaEventElapsedTime(&ms[i], h->stage_ev[i], h->stage_ev[i + 1]));
    *n_stages = k;
    return CC_OK;
}

const char* cc_last_error(cc_handle* h) { return h ? h->last_error.c_str() : "no handle"; }
uint64_t cc_last_launch_count(cc_handle* h) { return h ? h->launches : 0; }
void cc_interrupt(cc_handle* h) {
    if (h) h->interrupt.store(1);
}
void cc_free(void* p) { std::free(p); }

int cc_tight_eval_device(cc_handle* h, const double* soa, size_t n, uint32_t* masks, void* stream) {
    if (!h || (n && (!soa || !masks))) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    CC_CUDA(h, cudaSetDevice(h->device));
    return eval_batch<Layout::SoA>(h, soa, n, masks, s);
}

// Autotuner (no reference counterpart).  Each pass, with every register
// budget (minimum resident blocks 1, 4, 8) and grid size (2, 4, 8, 16 blocks
// of 128 per SM), is timed with CUDA events on the caller's sample batch, in
// pass order: the FP32 pass from empty queues; the FP64 pass on the queue the
// chosen FP32 run filled, its appends undone before every run (the queue
// counters are restored from a snapshot); the bisection passes on the final
// queues (they only OR bits into the masks, so reruns change nothing).  The
// fastest setting of each pass is kept in the handle for later
// cc_tight_eval_device / cc_tight_eval calls.
extern "C" int cc_autotune_eval(cc_handle* h, const double* soa, size_t n, uint32_t* masks, cc_tune_result* out) {
    if (!h || !soa || !masks || !n) return CC_ERR_PARAM;
    CC_CUDA(h, cudaSetDevice(h->device));
    EvalQueues q;
    int st = eval_queues(h, n, &q);
    if (st) return st;
    cudaStream_t s = h->stream;
    ccrt::EventPair ev;
    CC_CUDA(h, cudaEventCreate(&ev.e0));
    CC_CUDA(h, cudaEventCreate(&ev.e1));
    const cudaEvent_t e0 = ev.e0, e1 = ev.e1;
    const int minbs[3] = {1, 4, 8}, grids[4] = {2, 4, 8, 16};
    unsigned long long snap[kEvalCounters] = {};
    cc_tune_result r{};
    auto time_pass = [&](int pass, int minb, int grid, float* ms) -> int {
        const int g = h->sm_count * grid;
        float best = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            if (pass == 0) CC_CUDA(h, cudaMemsetAsync(q.counts, 0, kEvalCounters * sizeof(unsigned long long), s));
            if (pass == 1) CC_CUDA(h, cudaMemcpyAsync(q.counts, snap, sizeof(snap), cudaMemcpyHostToDevice, s));
            CC_CUDA(h, cudaEventRecord(e0, s));
            CC_CUDA(h, launch_pass<Layout::SoA>(pass, minb, g, s, soa, n, masks, q));
            CC_LAUNCHED(h);
            CC_CUDA(h, cudaEventRecord(e1, s));
            CC_CUDA(h, cudaEventSynchronize(e1));
            float t;
            CC_CUDA(h, cudaEventElapsedTime(&t, e0, e1));
            best = t < best ? t : best;
        }
        *ms = best;
        return CC_OK;
    };
    for (int pass = 0; pass < CC_EVAL_TUNED_STAGES; ++pass) {
        float best = 1e30f;
        int bm = 1, bg = 8;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 4; ++b) {
                float t;
                if ((st = time_pass(pass, minbs[a], grids[b], &t))) return st;
                if (minbs[a] == 1 && grids[b] == 8) r.ms_default[pass] = t;
                if (t < best) best = t, bm = minbs[a], bg = grids[b];
            }
        // leave the queues as the chosen setting of a queue-filling pass leaves them
        if (pass <= 1) {
            float rerun;
            if ((st = time_pass(pass, bm, bg, &rerun))) return st;
            if (pass == 0) {
                CC_CUDA(h, cudaMemcpyAsync(snap, q.counts, sizeof(snap), cudaMemcpyDeviceToHost, s));
                CC_CUDA(h, cudaStreamSynchronize(s));
            }
        }
        h->tune_minb[pass] = bm;
        h->tune_grid[pass] = bg;
        r.min_blocks[pass] = bm;
        r.blocks_per_sm[pass] = bg;
        r.ms[pass] = best;
    }
    if (out) *out = r;
    return CC_OK;
}

// ---- allocation-free evaluation ---------------------------------------------
// For callers that must not allocate device memory once they are running:
// code that executes inside a host framework owning every device allocation
// (an arena or pool it hands out itself), latency-critical loops where a
// cudaMalloc would block on device-wide synchronisation, and processes that
// run close to the memory limit and pre-reserve everything at start-up.
// cc_tight_eval_device_static evaluates a batch already in device memory
// with the same passes as cc_tight_eval_device (FP64 certification
// included), but keeps its queues in the fixed array below instead of
// handle-owned buffers, and needs no handle.  Without room for the record
// buffers its FP32 pass runs every criterion group in one kernel, and the
// certification evaluates every call of a criterion.  The array is part of
// the library image: every GPU that loads the library holds
// CC_STATIC_EVAL_SCRATCH_BYTES for it until the process exits.
static constexpr size_t kStaticMaxBoxes = CC_STATIC_EVAL_MAX_BOXES;
static constexpr size_t kStaticCountersBytes = 256;
// per box: the full, strip-width and gap-width queues, the five
// certification queues and the repair queue (4 bytes each), one flag byte
static constexpr size_t kStaticBytesPerBox = (3 + kCertQueues + 1) * sizeof(uint32_t) + 1;
static constexpr size_t kStaticScratchBytes = kStaticCountersBytes + kStaticMaxBoxes * kStaticBytesPerBox;
static_assert(kEvalCounters * sizeof(unsigned long long) <= kStaticCountersBytes, "counters do not fit");
static_assert(kStaticScratchBytes == CC_STATIC_EVAL_SCRATCH_BYTES, "static scratch size differs from the header");
static __device__ __align__(256) unsigned char cc_static_eval_scratch[CC_STATIC_EVAL_SCRATCH_BYTES];

namespace {
constexpr int kStaticMaxDevices = 64;
std::once_flag g_static_once[kStaticMaxDevices];
void* g_static_scratch[kStaticMaxDevices];  // device address of the array on each device
int g_static_sms[kStaticMaxDevices];
int g_static_setup[kStaticMaxDevices];      // cc_status of the one-time set-up

// once per device, with that device current: the array's device address (its
// name in host code is only a host-side stand-in) and the SM count
void static_setup(int dev) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, cc_static_eval_scratch);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_static_sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        g_static_setup[dev] = CC_ERR_CUDA;
        return;
    }
    g_static_scratch[dev] = p;
    g_static_setup[dev] = CC_OK;
}
}  // namespace

extern "C" int cc_tight_eval_device_static(const double* soa, size_t n, uint32_t* masks, void* stream) {
    if (n && (!soa || !masks)) return CC_ERR_PARAM;
    if (n > kStaticMaxBoxes) return CC_ERR_TOO_LARGE;
    if (n == 0) return CC_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kStaticMaxDevices) {
        cudaGetLastError();
        return CC_ERR_NO_DEVICE;
    }
    std::call_once(g_static_once[dev], static_setup, dev);
    if (g_static_setup[dev] != CC_OK) return g_static_setup[dev];
    unsigned char* base = (unsigned char*)g_static_scratch[dev];
    EvalQueues q;
    q.counts = (unsigned long long*)base;
    unsigned char* p = base + kStaticCountersBytes;
    q.full = (uint32_t*)p;
    p += kStaticMaxBoxes * sizeof(uint32_t);
    q.cover_box = (uint32_t*)p;
    p += kStaticMaxBoxes * sizeof(uint32_t);
    q.gaps_box = (uint32_t*)p;
    q.cap = kStaticMaxBoxes;
    q.args = nullptr;  // no room for the record buffers: every group in one kernel
    q.states = nullptr;
    q.q[0] = q.q[1] = nullptr;
    q.rc = nullptr;
    q.enc = nullptr;
    p += kStaticMaxBoxes * sizeof(uint32_t);
    for (int k = 0; k < kCertQueues; ++k) {
        q.cert[k] = (uint32_t*)p;
        p += kStaticMaxBoxes * sizeof(uint32_t);
    }
    q.repair = (uint32_t*)p;
    p += kStaticMaxBoxes * sizeof(uint32_t);
    q.cflags = p;
    cudaStream_t s = (cudaStream_t)stream;
    // an error the caller left pending is not ours to report or to clear
    if (cudaPeekAtLastError() != cudaSuccess) return CC_ERR_CUDA;
    // the queue counters are the only state that must start at zero
    const cudaError_t me = cudaMemsetAsync(q.counts, 0, kEvalCounters * sizeof(unsigned long long), s);
    if (me != cudaSuccess) {
        cudaGetLastError();  // the memset's own error
        return CC_ERR_CUDA;
    }
    // a small batch takes no more blocks than it has boxes to spread over
    const size_t need = (n + 127) / 128;
    int g = g_static_sms[dev] * 8;
    if ((size_t)g > need) g = (int)need;
    for (int pass = 0; pass < CC_EVAL_STAGES; ++pass) {
        if (launch_pass<Layout::SoA>(pass, 1, g, s, soa, n, masks, q) != cudaSuccess) {
            cudaGetLastError();  // the memory operation's own error
            return CC_ERR_CUDA;
        }
    }
    if (cudaPeekAtLastError() != cudaSuccess) {
        cudaGetLastError();  // a launch of this call failed
        return CC_ERR_CUDA;
    }
    return CC_OK;
}

// AoS boxes (80 bytes each) to the SoA layout of the evaluation passes.
// Consecutive threads load consecutive 16-byte pairs (a warp reads 512
// contiguous bytes per load), which matters when `aos` is host memory read
// over the host link.
__global__ void __launch_bounds__(256) k_aos_to_soa(const double* __restrict__ aos, size_t n, double* __restrict__ soa) {
    const double2* __restrict__ src = reinterpret_cast<const double2*>(aos);
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < 5 * n; j += (size_t)gridDim.x * blockDim.x) {
        const double2 v = src[j];
        const size_t i = j / 5, c = 2 * (j - 5 * i);
        soa[c * n + i] = v.x;
        soa[(c + 1) * n + i] = v.y;
    }
}


// Host-memory entry point.  The boxes move to the device in chunks of 4M by
// the copy engine, on a second stream, so that chunk k+1 travels while chunk
// k is evaluated: straight from the caller's array if it is page-locked, or
// where the device reaches pageable host memory through the host's page
// tables (GB300 with its host over NVLink-C2C: ~190-210 GB/s measured),
// otherwise through two pinned buffers that host threads fill (one thread
// copies at a fraction of the host's memory bandwidth).  The second stream
// also transposes each chunk to SoA (double-buffered), so the transposes
// overlap the evaluation too; above 2^20 boxes the first chunk is a quarter
// of the others, which shortens the time before the first evaluation starts.  Each chunk is
// evaluated by the same passes as cc_tight_eval_device; the masks of all
// chunks return in one copy at the end.
int cc_tight_eval(cc_handle* h, const cc_tight_box* boxes, size_t n, uint32_t* masks) {
    if (!h || (n && (!boxes || !masks))) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    // page-locked input (cudaHostAlloc / cudaHostRegister) is copied as it is
    cudaPointerAttributes pa;
    bool pinned_in = false;
    if (cudaPointerGetAttributes(&pa, boxes) == cudaSuccess) pinned_in = pa.type == cudaMemoryTypeHost;
    else cudaGetLastError();
    const bool direct = h->pageable_access || pinned_in;
    // boxes per chunk (CC_EVAL_CHUNK_LOG2 in the environment, 16..26, changes
    // only how the same work is cut)
    static const int chunk_log2 = [] {
        const char* v = std::getenv("CC_EVAL_CHUNK_LOG2");
        const int x = v ? std::atoi(v) : 22;
        return x < 16 ? 16 : (x > 26 ? 26 : x);
    }();
    const size_t chunk = n < ((size_t)1 << chunk_log2) ? n : ((size_t)1 << chunk_log2);
    const size_t first = n > ((size_t)1 << 20) ? chunk / 4 : chunk;  // small batches: one chunk
    const size_t in_bytes = chunk * sizeof(cc_tight_box);
    void *d_aos[2], *d_soa[2], *d_masks;
    int st = CC_OK;
    for (int b = 0; b < 2 && !st; ++b) st = ccrt::ensure(h, 0 + b, in_bytes, &d_aos[b]);
    for (int b = 0; b < 2 && !st; ++b) st = ccrt::ensure(h, 4 + b, in_bytes, &d_soa[b]);
    if (!st) st = ccrt::ensure(h, 2, n * sizeof(uint32_t), &d_masks);
    if (!st && !direct) st = ccrt::ensure_pinned(h, 2 * in_bytes);
    if (st) return st;
    char* pin[2] = {(char*)h->pinned, (char*)h->pinned + in_bytes};
    if (!h->stream2) CC_CUDA(h, cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking));
    // copied[b]: pin[b] may be refilled; ready[b]: d_soa[b] holds the chunk;
    // used[b]: its evaluation is done, d_soa[b] may be overwritten
    cudaEvent_t copied[2], ready[2], used[2];
    for (int b = 0; b < 2; ++b) {
        CC_CUDA(h, cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming));
        CC_CUDA(h, cudaEventCreateWithFlags(&ready[b], cudaEventDisableTiming));
        CC_CUDA(h, cudaEventCreateWithFlags(&used[b], cudaEventDisableTiming));
    }
    auto fail_cuda = [&](cudaError_t e) { return ccrt::fail(h, CC_ERR_CUDA, "cc_tight_eval", e); };
    cudaError_t e = cudaSuccess;
    int b = 0, k = 0;
    for (size_t off = 0; off < n && e == cudaSuccess && st == CC_OK; ++k, b ^= 1) {
        const size_t want = k == 0 ? first : chunk;
        const size_t cnt = n - off < want ? n - off : want;
        const size_t bytes = cnt * sizeof(cc_tight_box);
        if (k >= 2) {
            // chunk k-2's evaluation has read d_soa[b]; its copy has left pin[b]
            e = cudaStreamWaitEvent(h->stream2, used[b], 0);
            if (e == cudaSuccess && !direct) e = cudaEventSynchronize(copied[b]);
            if (e != cudaSuccess) break;
        }
        if (direct) {
            e = cudaMemcpyAsync(d_aos[b], boxes + off, bytes, cudaMemcpyHostToDevice, h->stream2);
        } else {
            const cc_tight_box* src = boxes + off;
            char* dst = pin[b];
            ccrt::parallel_blocks(cnt, [&](size_t lo, size_t hi) {
                std::memcpy(dst + lo * sizeof(cc_tight_box), src + lo, (hi - lo) * sizeof(cc_tight_box));
            });
            e = cudaMemcpyAsync(d_aos[b], dst, bytes, cudaMemcpyHostToDevice, h->stream2);
        }
        if (e == cudaSuccess) e = cudaEventRecord(copied[b], h->stream2);
        if (e != cudaSuccess) break;
        k_aos_to_soa<<<h->sm_count * 8, 256, 0, h->stream2>>>((const double*)d_aos[b], cnt, (double*)d_soa[b]);
        CC_LAUNCHED(h);
        e = cudaEventRecord(ready[b], h->stream2);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, ready[b], 0);
        if (e != cudaSuccess) break;
        // direct launches: the chunks' arguments differ (a graph would be
        // re-captured for every chunk)
        st = eval_batch<Layout::SoA>(h, (const double*)d_soa[b], cnt, (uint32_t*)d_masks + off, h->stream, false);
        if (st == CC_OK) e = cudaEventRecord(used[b], h->stream);
        off += cnt;
    }
    if (e == cudaSuccess && st == CC_OK)
        e = cudaMemcpyAsync(masks, d_masks, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream);
    cudaError_t e2 = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = e2;
    e2 = cudaStreamSynchronize(h->stream2);
    if (e == cudaSuccess) e = e2;
    for (int j = 0; j < 2; ++j) {
        cudaEventDestroy(copied[j]);
        cudaEventDestroy(ready[j]);
        cudaEventDestroy(used[j]);
    }
    if (st) return st;
    if (e != cudaSuccess) return fail_cuda(e);
    return CC_OK;
}

// Diagnostic: the FP64 certification run of a record group (0 r1, 1 r1_r2,
// 2 2x2, 3 leaf r1_r2_r3) on host boxes, one call number per box.
int cc_selftest_certify(cc_handle* h, int group, const cc_tight_box* boxes, const int* call, size_t n,
                        uint8_t* out) {
    if (!h || !boxes || !call || !out || group < 0 || group >= kRecGroups) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    void *d_b, *d_c, *d_o;
    int st;
    if ((st = ccrt::ensure(h, 0, n * sizeof(cc_tight_box), &d_b))) return st;
    if ((st = ccrt::ensure(h, 1, n * sizeof(int), &d_c))) return st;
    if ((st = ccrt::ensure(h, 2, n, &d_o))) return st;
    CC_CUDA(h, cudaMemcpyAsync(d_b, boxes, n * sizeof(cc_tight_box), cudaMemcpyHostToDevice, h->stream));
    CC_CUDA(h, cudaMemcpyAsync(d_c, call, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    const int g = (int)((n + 127) / 128);
    const double* b = (const double*)d_b;
    switch (group) {
        case 0: k_selftest_certify<0><<<g, 128, 0, h->stream>>>(b, n, (const int*)d_c, (uint8_t*)d_o); break;
        case 1: k_selftest_certify<1><<<g, 128, 0, h->stream>>>(b, n, (const int*)d_c, (uint8_t*)d_o); break;
        case 2: k_selftest_certify<2><<<g, 128, 0, h->stream>>>(b, n, (const int*)d_c, (uint8_t*)d_o); break;
        default: k_selftest_certify<3><<<g, 128, 0, h->stream>>>(b, n, (const int*)d_c, (uint8_t*)d_o); break;
    }
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaMemcpyAsync(out, d_o, n, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

// Diagnostic: measured instruction throughput of this device in operations
// per second (one op = one thread instruction; an FMA counts 1): kind 0 FP64
// directed add/mul, 1 FP64 FMA, 2 FP32 directed add/mul, 3 FP32 FMA.  Best
// of three timed launches (CUDA events) after a warm-up launch.
int cc_selftest_peak(cc_handle* h, int kind, double* ops_per_s) {
    if (!h || !ops_per_s || kind < 0 || kind > 3) return CC_ERR_PARAM;
    CC_CUDA(h, cudaSetDevice(h->device));
    void* d;
    int st = ccrt::ensure(h, 0, 64, &d);
    if (st) return st;
    const int blocks = h->sm_count * 8, threads = 256, iters = kind >= 2 ? 16384 : 4096;
    ccrt::EventPair ev;
    CC_CUDA(h, cudaEventCreate(&ev.e0));
    CC_CUDA(h, cudaEventCreate(&ev.e1));
    auto launch = [&](int it) {
        if (kind < 2) k_fp64_peak<<<blocks, threads, 0, h->stream>>>((double*)d, it, kind & 1);
        else k_fp32_peak<<<blocks, threads, 0, h->stream>>>((float*)d, it, kind & 1);
    };
    launch(64);  // warm-up
    CC_LAUNCHED(h);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        CC_CUDA(h, cudaEventRecord(ev.e0, h->stream));
        launch(iters);
        CC_LAUNCHED(h);
        CC_CUDA(h, cudaEventRecord(ev.e1, h->stream));
        CC_CUDA(h, cudaEventSynchronize(ev.e1));
        float ms = 0;
        CC_CUDA(h, cudaEventElapsedTime(&ms, ev.e0, ev.e1));
        if (ms < best) best = ms;
    }
    *ops_per_s = (double)blocks * threads * iters * 8 / (best * 1e-3);
    return CC_OK;
}

// Diagnostic: FP64 instruction throughput (kind 0 or 1 of cc_selftest_peak).
int cc_selftest_fp64_peak(cc_handle* h, int use_fma, double* ops_per_s) {
    return cc_selftest_peak(h, use_fma ? 1 : 0, ops_per_s);
}

// Diagnostic: the device's directed-rounding primitives on host arrays
// (op: 0 add, 1 mul, 2 div, 3 sqrt, 4 reciprocal; b may be NULL for 3, 4).
int cc_selftest_round(cc_handle* h, int op, int up, const double* a, const double* b, double* out, size_t n) {
    if (!h || !a || !out) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    void *da, *db, *dout;
    int st = ccrt::ensure(h, 0, n * 8, &da);
    if (!st) st = ccrt::ensure(h, 1, n * 8, &db);
    if (!st) st = ccrt::ensure(h, 2, n * 8, &dout);
    if (st) return st;
    CC_CUDA(h, cudaMemcpyAsync(da, a, n * 8, cudaMemcpyHostToDevice, h->stream));
    if (b) CC_CUDA(h, cudaMemcpyAsync(db, b, n * 8, cudaMemcpyHostToDevice, h->stream));
    k_selftest_round<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(op, up, (const double*)da, b ? (const double*)db : nullptr,
                                                                        (double*)dout, n);
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaMemcpyAsync(out, dout, n * 8, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

__global__ void k_selftest_round_to_floats(const double* x, size_t n, float* out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float d, u;
    cc::f32::round_to_floats(x[i], d, u);
    out[4 * i] = d;
    out[4 * i + 1] = u;
    out[4 * i + 2] = __double2float_rd(x[i]);
    out[4 * i + 3] = __double2float_ru(x[i]);
}

// Diagnostic: f32::round_to_floats next to the directed conversions
int cc_selftest_round_to_floats(cc_handle* h, const double* x, size_t n, float* out) {
    if (!h || !x || !out) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    void *dx, *dout;
    int st = ccrt::ensure(h, 0, n * 8, &dx);
    if (!st) st = ccrt::ensure(h, 1, n * 16, &dout);
    if (st) return st;
    CC_CUDA(h, cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, h->stream));
    k_selftest_round_to_floats<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>((const double*)dx, n, (float*)dout);
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaMemcpyAsync(out, dout, n * 16, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

// Diagnostic: subinterval splits computed (a) with the explicit FMA the
// prover uses and (b) by the plain expression `lb + diff*i` compiled with
// nvcc's default contraction (cc_selftest_fmad.cu); out_a/out_b get 2n doubles.
int cc_selftest_subinterval(cc_handle* h, const double* lo, const double* hi, const int* idx, const int* cnt, size_t n,
                            double* out_a, double* out_b) {
    if (!h || !lo || !hi || !idx || !cnt || !out_a || !out_b) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    void *dlo, *dhi, *didx, *dcnt, *da, *db;
    int st = ccrt::ensure(h, 0, n * 8, &dlo);
    if (!st) st = ccrt::ensure(h, 1, n * 8, &dhi);
    if (!st) st = ccrt::ensure(h, 2, n * 4, &didx);
    if (!st) st = ccrt::ensure(h, 3, n * 4, &dcnt);
    if (!st) st = ccrt::ensure(h, 4, n * 16, &da);
    if (!st) st = ccrt::ensure(h, 5, n * 16, &db);
    if (st) return st;
    CC_CUDA(h, cudaMemcpyAsync(dlo, lo, n * 8, cudaMemcpyHostToDevice, h->stream));
    CC_CUDA(h, cudaMemcpyAsync(dhi, hi, n * 8, cudaMemcpyHostToDevice, h->stream));
    CC_CUDA(h, cudaMemcpyAsync(didx, idx, n * 4, cudaMemcpyHostToDevice, h->stream));
    CC_CUDA(h, cudaMemcpyAsync(dcnt, cnt, n * 4, cudaMemcpyHostToDevice, h->stream));
    k_selftest_subinterval<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>((const double*)dlo, (const double*)dhi,
                                                                              (const int*)didx, (const int*)dcnt, (double*)da, n);
    CC_LAUNCHED(h);
    st = cc_selftest_subinterval_contracted((const double*)dlo, (const double*)dhi, (const int*)didx, (const int*)dcnt,
                                            (double*)db, n, h->stream);
    if (st) return ccrt::fail(h, st, "contracted subinterval kernel");
    h->launches += 1;
    CC_CUDA(h, cudaMemcpyAsync(out_a, da, n * 16, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaMemcpyAsync(out_b, db, n * 16, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

int cc_selftest_bisection_f32(cc_handle* h, int which, const double* args, size_t n, int8_t* f32_out,
                              int8_t* f64_out) {
    if (!h || !args || !f32_out || !f64_out || (which != 0 && which != 1)) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    void *da, *d32, *d64;
    int st = ccrt::ensure(h, 0, n * 64, &da);
    if (!st) st = ccrt::ensure(h, 1, n, &d32);
    if (!st) st = ccrt::ensure(h, 2, n, &d64);
    if (st) return st;
    CC_CUDA(h, cudaMemcpyAsync(da, args, n * 64, cudaMemcpyHostToDevice, h->stream));
    k_selftest_bisection_f32<<<(unsigned)((n + 127) / 128), 128, 0, h->stream>>>(which, (const double*)da, n,
                                                                                 (int8_t*)d32, (int8_t*)d64);
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaMemcpyAsync(f32_out, d32, n, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaMemcpyAsync(f64_out, d64, n, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

int cc_selftest_bisection_width(cc_handle* h, int which, const double* args, size_t n, double* out,
                                int8_t* trapped) {
    if (!h || !args || !out || !trapped || (which != 0 && which != 1)) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    void *da, *dout, *dtr;
    int st = ccrt::ensure(h, 0, n * 64, &da);
    if (!st) st = ccrt::ensure(h, 1, n * 8, &dout);
    if (!st) st = ccrt::ensure(h, 2, n, &dtr);
    if (st) return st;
    CC_CUDA(h, cudaMemcpyAsync(da, args, n * 64, cudaMemcpyHostToDevice, h->stream));
    k_selftest_bisection_width<<<(unsigned)((n + 127) / 128), 128, 0, h->stream>>>(which, (const double*)da, n,
                                                                                   (double*)dout, (int8_t*)dtr);
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaMemcpyAsync(out, dout, n * 8, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaMemcpyAsync(trapped, dtr, n, cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

}  // extern "C"

// ========================================================= tight proof host
namespace {

using namespace cc::prove;

// buffer slots in the handle
enum Slot { S_PARENTS = 6, S_TASKS, S_CELL2, S_CELL3, S_CELL4, S_LEAF, S_CRIT, S_COUNTERS, S_GAPS, S_LEAF2 };
static_assert(S_LEAF2 < 16, "proof buffers overlap the evaluation queues");

struct GenTotals {
    unsigned long long counts[4][8] = {};
    unsigned long long digest = 0, leaf_evals = 0, trapped = 0;
    unsigned long long fp32[4] = {};  // first_f32 outcomes (Counters::fp32)
    void add(const GenTotals& g) {
        for (int l = 0; l < 4; ++l)
            for (int o = 0; o < 8; ++o) counts[l][o] += g.counts[l][o];
        digest += g.digest;
        leaf_evals += g.leaf_evals;
        trapped += g.trapped;
        for (int k = 0; k < 4; ++k) fp32[k] += g.fp32[k];
    }
};

// FP64 certification failures of this translation unit's kernels so far
// (cc_cert_fail_count; expected to stay 0)
static unsigned long long cert_failures_so_far() {
    unsigned long long v = 0;
    if (cudaMemcpyFromSymbol(&v, cc::cc_cert_fail_count, sizeof(v)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return v + cc::cert_failures_host.load();
}

int stage_grid(cc_handle* h) { return h->sm_count * 6; }

bool valid_split(int s) { return s >= 1 && s < 2048; }

// merge_adjacent_r1 of one task's critical leaves (tight_rectangle.cu:121-159)
void merge_by_r1(std::vector<cc_tight_box>& v, std::vector<cc_tight_box>& out) {
    if (v.empty()) return;
    std::sort(v.begin(), v.end(), [](const cc_tight_box& a, const cc_tight_box& b) {
        return a.r[0].lb < b.r[0].lb || (a.r[0].lb == b.r[0].lb && a.r[0].ub < b.r[0].ub);
    });
    size_t first = out.size();
    out.push_back(v.front());
    for (const cc_tight_box& b : v) {
        cc_tight_box& p = out.back();
        bool merge = (p.r[0].lb <= b.r[0].lb) ? (p.r[0].ub >= b.r[0].lb) : (b.r[0].ub >= p.r[0].lb);
        if (merge) {
            for (int k = 0; k < 4; ++k) {
                if (b.r[k].lb < p.r[k].lb) p.r[k].lb = b.r[k].lb;
                if (b.r[k].ub > p.r[k].ub) p.r[k].ub = b.r[k].ub;
            }
            continue;
        }
        out.push_back(b);
    }
    (void)first;
}

// ---- learned leaf order ------------------------------------------------------
// Before the leaves of an r3 cell are checked, the network looks at the cell
// (its r4 range in place of a leaf's r4) and predicts whether the leaf
// criterion r1_r2_r3_strategies(box, R4) will certify its leaves.  If so,
// stage 4a tries that criterion (about 31 directed-rounding operations on
// the microbench) before the 2x2 criterion (about 116, six bisections) that
// the reference's order puts first.  The threshold -1.0 on the logit
// (probability 0.27) is about the ratio of the two costs: above it, trying
// the cheap criterion first saves more than it wastes.
constexpr float kLeafFirstLogit = -1.0f;
constexpr unsigned long long kCellLogRate = 64;      // log one cell in 64
constexpr unsigned long long kCellLogCap = 1 << 20;  // cells logged per proof at most

__global__ void k_cell_features(const Task* __restrict__ tasks, const Cell4* __restrict__ cells,
                                const unsigned long long* n_dev, unsigned long long cap, float* __restrict__ feat) {
    const unsigned long long n = *n_dev < cap ? *n_dev : cap;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const Cell4& c = cells[i];
        const Task& t = tasks[c.task];
        const double v[10] = {t.la.lo, t.la.hi, c.r1.lo, c.r1.hi, c.r2.lo, c.r2.hi, c.r3.lo, c.r3.hi, c.r4r.lo, c.r4r.hi};
        cc::mlp::features(v, t.weight, 0.0f, feat + i * cc::mlp::kFeatures);
    }
}

__global__ void k_cell_order(Cell4* __restrict__ cells, const unsigned long long* n_dev, unsigned long long cap,
                             const float* __restrict__ logits) {
    const unsigned long long n = *n_dev < cap ? *n_dev : cap;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        cells[i].order = logits[i * 8 + 4] > kLeafFirstLogit ? 1 : 0;
}

// a sample of the r3 cells (la, r1, r2, r3, r4 range) for training records
__global__ void k_cell_log(const Task* __restrict__ tasks, const Cell4* __restrict__ cells,
                           const unsigned long long* n_dev, unsigned long long cap, unsigned long long salt,
                           cc_tight_box* __restrict__ log, unsigned long long* n_log) {
    const unsigned long long n = *n_dev < cap ? *n_dev : cap;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (mix64(i ^ salt) % kCellLogRate) continue;
        const unsigned long long slot = atomicAdd(n_log, 1ULL);
        if (slot >= kCellLogCap) continue;
        const Cell4& c = cells[i];
        const Task& t = tasks[c.task];
        log[slot] = cc_tight_box{{t.la.lo, t.la.hi}, {{c.r1.lo, c.r1.hi}, {c.r2.lo, c.r2.hi}, {c.r3.lo, c.r3.hi},
                                                      {c.r4r.lo, c.r4r.hi}}};
    }
}

enum { S_CELL_FEAT = 32, S_CELL_LOGITS, S_CELL_LOG };
constexpr int S_CERT = 27;  // FP32 "true" leaf verdicts awaiting their FP64 certification
constexpr int S_CERT_CALLS = 44;  // their chosen can_recurse calls (k_stage_cert)
// run_chunk's answer when an FP64 certification failed: redo the chunk in the
// plain form (FP64 criteria only)
constexpr int kRedoPlain = 1000;

// One chunk of parents [a, b) of a generation; returns CC_QUEUE_OVERFLOW
// (without side effects on `out`/`tot`) when a device queue ran full.
int run_chunk(cc_handle* h, const std::vector<cc_tight_box>& parents, size_t a, size_t b, int k, const int s[4], Caps caps,
              std::vector<cc_tight_box>& out, GenTotals& tot, unsigned long long task_base, bool hoist, int flags,
              unsigned long long task_lo, unsigned long long task_hi, double* demand = nullptr) {
    const bool learned = hoist && (flags & CC_PROVE_LEARNED);
    const bool log_cells = hoist && (flags & CC_PROVE_LOG_CELLS);
    const size_t np = b - a;
    const size_t ntasks = np * (size_t)k;
    void *d_par, *d_tasks, *d_c2, *d_c3, *d_c4, *d_leaf, *d_gaps, *d_crit, *d_cnt, *d_leaf2 = nullptr, *d_cert = nullptr;
    int st;
    if (hoist && (st = ccrt::ensure(h, S_LEAF2, caps.leaf2 * sizeof(Leaf2), &d_leaf2))) return st;
    if (hoist && (st = ccrt::ensure(h, S_CERT, caps.leaf * sizeof(CertLeaf), &d_cert))) return st;
    // the chosen calls of the certification runs, one entry per queued leaf
    // (windows of 1,024 may reach past the count by less than a window)
    void* d_cert_calls = nullptr;
    if (hoist && (st = ccrt::ensure(h, S_CERT_CALLS, (caps.leaf + 1024) * sizeof(cc::CertCall), &d_cert_calls)))
        return st;
    if ((st = ccrt::ensure(h, S_GAPS, caps.gaps * sizeof(GapsLeaf), &d_gaps))) return st;
    if ((st = ccrt::ensure(h, S_PARENTS, np * sizeof(cc_tight_box), &d_par))) return st;
    if ((st = ccrt::ensure(h, S_TASKS, ntasks * sizeof(Task), &d_tasks))) return st;
    if ((st = ccrt::ensure(h, S_CELL2, caps.cell2 * sizeof(Cell2), &d_c2))) return st;
    if ((st = ccrt::ensure(h, S_CELL3, caps.cell3 * sizeof(Cell3), &d_c3))) return st;
    if ((st = ccrt::ensure(h, S_CELL4, caps.cell4 * sizeof(Cell4), &d_c4))) return st;
    if ((st = ccrt::ensure(h, S_LEAF, caps.leaf * sizeof(Leaf), &d_leaf))) return st;
    if ((st = ccrt::ensure(h, S_CRIT, caps.crit * sizeof(Critical), &d_crit))) return st;
    if ((st = ccrt::ensure(h, S_COUNTERS, sizeof(Counters), &d_cnt))) return st;
    Counters* cnt = (Counters*)d_cnt;
    cudaStream_t sm = h->stream;
    CC_CUDA(h, cudaMemcpyAsync(d_par, parents.data() + a, np * sizeof(cc_tight_box), cudaMemcpyHostToDevice, sm));
    CC_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(Counters), sm));
    const int g = stage_grid(h);
    k_tasks<<<(unsigned)((ntasks + 127) / 128), 128, 0, sm>>>((const Box*)d_par, (int)np, k, (Task*)d_tasks, task_base,
                                                              task_lo, task_hi);
    CC_LAUNCHED(h);
    if (hoist) {
        k_stage1<true><<<g, 128, 0, sm>>>((const Box*)d_par, (const Task*)d_tasks, (int)ntasks, s[0], (Cell2*)d_c2, caps, cnt,
                                          task_base);
        CC_LAUNCHED(h);
        k_stage2<true><<<g, 128, 0, sm>>>((const Box*)d_par, (const Task*)d_tasks, (const Cell2*)d_c2, s[1], (Cell3*)d_c3, caps,
                                          cnt, task_base);
        CC_LAUNCHED(h);
        k_stage3<true><<<g, 128, 0, sm>>>((const Box*)d_par, (const Task*)d_tasks, (const Cell3*)d_c3, s[2], (Cell4*)d_c4, caps,
                                          cnt, task_base);
        CC_LAUNCHED(h);
        if (learned) {
            void *d_feat, *d_logits;
            if ((st = ccrt::ensure(h, S_CELL_FEAT, caps.cell4 * cc::mlp::kFeatures * sizeof(float), &d_feat))) return st;
            if ((st = ccrt::ensure(h, S_CELL_LOGITS, caps.cell4 * 8 * sizeof(float), &d_logits))) return st;
            k_cell_features<<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, &cnt->n_cell4, caps.cell4,
                                               (float*)d_feat);
            CC_LAUNCHED(h);
            if ((st = cc_mlp_infer_async(h, (const float*)d_feat, &cnt->n_cell4, caps.cell4, (float*)d_logits, sm)))
                return st;
            k_cell_order<<<g, 128, 0, sm>>>((Cell4*)d_c4, &cnt->n_cell4, caps.cell4, (const float*)d_logits);
            CC_LAUNCHED(h);
        }
        if (log_cells) {
            void* d_log;
            if ((st = ccrt::ensure(h, S_CELL_LOG, kCellLogCap * sizeof(cc_tight_box) + 64, &d_log))) return st;
            unsigned long long* n_log = (unsigned long long*)((char*)d_log + kCellLogCap * sizeof(cc_tight_box));
            CC_CUDA(h, cudaMemsetAsync(n_log, 0, sizeof(unsigned long long), sm));
            k_cell_log<<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, &cnt->n_cell4, caps.cell4,
                                          task_base * 0x9e3779b97f4a7c15ULL, (cc_tight_box*)d_log, n_log);
            CC_LAUNCHED(h);
            unsigned long long nl = 0;
            CC_CUDA(h, cudaMemcpyAsync(&nl, n_log, sizeof(nl), cudaMemcpyDeviceToHost, sm));
            CC_CUDA(h, cudaStreamSynchronize(sm));
            nl = std::min<unsigned long long>(nl, kCellLogCap);
            const size_t room = kCellLogCap - std::min<size_t>(h->cell_log.size(), kCellLogCap);
            const size_t take = std::min<size_t>(nl, room);
            if (take) {
                const size_t old = h->cell_log.size();
                h->cell_log.resize(old + take);
                CC_CUDA(h, cudaMemcpyAsync(h->cell_log.data() + old, d_log, take * sizeof(cc_tight_box),
                                           cudaMemcpyDeviceToHost, sm));
                CC_CUDA(h, cudaStreamSynchronize(sm));
            }
            h->cell_log_splits = s[3];
        }
    } else {
        k_stage1<false><<<g, 128, 0, sm>>>((const Box*)d_par, (const Task*)d_tasks, (int)ntasks, s[0], (Cell2*)d_c2, caps, cnt,
                                           task_base);
        CC_LAUNCHED(h);
        k_stage2<false><<<g, 128, 0, sm>>>((const Box*)d_par, (const Task*)d_tasks, (const Cell2*)d_c2, s[1], (Cell3*)d_c3,
                                           caps, cnt, task_base);
        CC_LAUNCHED(h);
        k_stage3<false><<<g, 128, 0, sm>>>((const Box*)d_par, (const Task*)d_tasks, (const Cell3*)d_c3, s[2], (Cell4*)d_c4,
                                           caps, cnt, task_base);
        CC_LAUNCHED(h);
    }
    // The leaf stages run over slices of the r3 cells small enough that the
    // leaf queues cannot overflow (each cell has s[3] leaves; the queues are
    // emptied between slices), so a chunk never has to be redone for them.
    unsigned long long n_c4 = 0;
    CC_CUDA(h, cudaMemcpyAsync(&n_c4, &cnt->n_cell4, sizeof(n_c4), cudaMemcpyDeviceToHost, sm));
    CC_CUDA(h, cudaStreamSynchronize(sm));
    if (n_c4 > caps.cell4) n_c4 = 0;  // stage 3 overflowed: the chunk is retried smaller
    unsigned long long room = std::min(caps.leaf, caps.gaps);
    if (hoist) room = std::min(room, caps.leaf2);
    const unsigned long long slice = std::max<unsigned long long>(1, room / (unsigned long long)s[3]);
    for (unsigned long long c0 = 0; c0 < n_c4; c0 += slice) {
        const unsigned long long c1 = std::min(n_c4, c0 + slice);
        if (c0) {  // the previous slice's leaf queues are consumed
            CC_CUDA(h, cudaMemsetAsync(&cnt->n_leaf, 0, 2 * sizeof(unsigned long long), sm));  // n_leaf, n_gaps
            CC_CUDA(h, cudaMemsetAsync(&cnt->n_leaf2, 0, sizeof(unsigned long long), sm));
            CC_CUDA(h, cudaMemsetAsync(&cnt->n_cert, 0, sizeof(unsigned long long), sm));
        }
        if (hoist) {
            k_stage4a<true, true><<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, s[3], c0, c1,
                                                     (Leaf*)d_leaf, (Leaf2*)d_leaf2, caps, cnt, task_base,
                                                     (CertLeaf*)d_cert);
            CC_LAUNCHED(h);
            k_stage4a2<<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, (const Leaf2*)d_leaf2, (Leaf*)d_leaf,
                                          caps, cnt, task_base, (CertLeaf*)d_cert);
            CC_LAUNCHED(h);
            k_stage4b<true><<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, (const Leaf*)d_leaf, s[3],
                                               (GapsLeaf*)d_gaps, (Critical*)d_crit, caps, cnt, task_base,
                                               (CertLeaf*)d_cert);
        } else {
            k_stage4a<false, false><<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, s[3], c0, c1,
                                                       (Leaf*)d_leaf, nullptr, caps, cnt, task_base, nullptr);
            CC_LAUNCHED(h);
            k_stage4b<false><<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, (const Leaf*)d_leaf, s[3],
                                                (GapsLeaf*)d_gaps, (Critical*)d_crit, caps, cnt, task_base, nullptr);
        }
        CC_LAUNCHED(h);
        k_stage4c<<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, (const GapsLeaf*)d_gaps, s[3],
                                     (Critical*)d_crit, caps, cnt, task_base);
        CC_LAUNCHED(h);
        if (hoist) {  // FP64 certification of the slice's FP32 "true" leaf verdicts
            k_stage_cert<<<g, 128, 0, sm>>>((const Task*)d_tasks, (const Cell4*)d_c4, (const CertLeaf*)d_cert,
                                            (cc::CertCall*)d_cert_calls, s[3], caps, cnt);
            CC_LAUNCHED(h);
        }
    }
    Counters hc;
    CC_CUDA(h, cudaMemcpyAsync(&hc, cnt, sizeof(Counters), cudaMemcpyDeviceToHost, sm));
    CC_CUDA(h, cudaStreamSynchronize(sm));
    if (hc.overflow) {
        // the queue counters keep counting past their capacity: the first
        // queue that overflowed tells how much too large this chunk was
        auto f = [](unsigned long long n, unsigned long long cap) { return cap ? (double)n / (double)cap : 0.0; };
        double d = std::max({f(hc.n_cell3, caps.cell3), f(hc.n_cell4, caps.cell4), f(hc.n_leaf, caps.leaf),
                             f(hc.n_gaps, caps.gaps), f(hc.n_crit, caps.crit), hoist ? f(hc.n_leaf2, caps.leaf2) : 0.0});
        if (demand) *demand = d;
        return CC_ERR_QUEUE_OVERFLOW;
    }
    if (hc.fp32[3]) {  // an FP32 "true" leaf verdict failed its FP64 certification
        cc::cert_failures_host += hc.fp32[3];
        return kRedoPlain;
    }
    std::vector<Critical> crit(hc.n_crit);
    if (hc.n_crit) {
        CC_CUDA(h, cudaMemcpyAsync(crit.data(), d_crit, hc.n_crit * sizeof(Critical), cudaMemcpyDeviceToHost, sm));
        CC_CUDA(h, cudaStreamSynchronize(sm));
    }
    // group by task (counting sort keeps the per-task lists contiguous)
    std::vector<size_t> start(ntasks + 1, 0);
    for (const Critical& c : crit) start[(size_t)c.task + 1] += 1;
    for (size_t t = 0; t < ntasks; ++t) start[t + 1] += start[t];
    std::vector<cc_tight_box> sorted(crit.size());
    std::vector<size_t> fill(start.begin(), start.end() - 1);
    unsigned long long trapped = 0;
    for (const Critical& c : crit) {
        cc_tight_box bx;
        static_assert(sizeof(bx) == sizeof(c.box), "box layout");
        std::memcpy(&bx, &c.box, sizeof(bx));
        sorted[fill[c.task]++] = bx;
        trapped += c.flags ? 1 : 0;
    }
    std::vector<cc_tight_box> one;
    for (size_t t = 0; t < ntasks; ++t) {
        if (start[t] == start[t + 1]) continue;
        one.assign(sorted.begin() + start[t], sorted.begin() + start[t + 1]);
        merge_by_r1(one, out);
    }
    for (int l = 0; l < 4; ++l)
        for (int o = 0; o < 8; ++o) tot.counts[l][o] += hc.counts[l][o];
    tot.digest += hc.digest;
    tot.leaf_evals += hc.leaf_evals;
    tot.trapped += trapped;
    for (int k = 0; k < 4; ++k) tot.fp32[k] += hc.fp32[k];
    return CC_OK;
}

// All tasks of one generation, in chunks of consecutive tasks that fit the
// device queues.  A chunk may cover part of a parent's lambda pieces (the
// initial pass has one parent with hundreds of pieces); its criticals are
// merged per task, so the chunks' lists concatenate in task order.  After an
// overflow the chunk is retried with the span shrunk by the overflowing
// queue's demand (its counter keeps counting past the capacity); a single
// task that overflows doubles the capacities instead.
int run_generation(cc_handle* h, const std::vector<cc_tight_box>& parents, int k, const int s[4],
                   std::vector<cc_tight_box>& out, GenTotals& tot, Caps& caps, bool hoist, int flags,
                   unsigned long long task_lo = 0, unsigned long long task_hi = ~0ULL) {
    const unsigned long long n_tasks = (unsigned long long)parents.size() * (unsigned long long)k;
    unsigned long long t = std::min(task_lo, n_tasks);
    const unsigned long long t_end = std::min(task_hi, n_tasks);
    unsigned long long span = 1ULL << 16;
    while (t < t_end) {
        const unsigned long long e = std::min(t_end, t + span);
        const size_t a = (size_t)(t / (unsigned long long)k), b = (size_t)((e - 1) / (unsigned long long)k + 1);
        Caps cp = caps;
        cp.cell2 = (e - t) * (unsigned long long)s[0];
        std::vector<cc_tight_box> part;
        GenTotals g;
        double demand = 0.0;
        int st = run_chunk(h, parents, a, b, k, s, cp, part, g, (unsigned long long)a * k, hoist, flags, t, e, &demand);
        if (st == kRedoPlain) {  // the chunk again, FP64 criteria only: the reference's verdicts
            part.clear();
            g = GenTotals();
            st = run_chunk(h, parents, a, b, k, s, cp, part, g, (unsigned long long)a * k, false, flags, t, e, &demand);
        }
        if (st == CC_ERR_QUEUE_OVERFLOW) {
            if (e - t > 1) {
                const double shrink = demand > 1.0 ? 1.25 * demand : 2.0;
                span = std::max<unsigned long long>(1, (unsigned long long)((double)(e - t) / shrink));
                if (span >= e - t) span = (e - t) / 2;
            } else {
                caps.cell3 *= 2;
                caps.cell4 *= 2;
                caps.leaf *= 2;
                caps.leaf2 *= 2;
                caps.gaps *= 2;
                caps.crit *= 2;
                if (caps.cell4 > (1ULL << 31)) return ccrt::fail(h, CC_ERR_QUEUE_OVERFLOW, "tight proof: one box exceeds the queue limit");
            }
            continue;
        }
        if (st) return st;
        out.insert(out.end(), part.begin(), part.end());
        tot.add(g);
        t = e;
    }
    return CC_OK;
}


// ---- checkpoints --------------------------------------------------------------
// State after a completed generation: the grid, the next generation's index,
// the running trace totals and generation sizes, and the parents of the next
// generation (the criticals so far).  Written to `path.tmp` and renamed, so
// a checkpoint file is always complete.
struct CkptHeader {
    char magic[8];
    uint32_t version;
    int32_t next_gen;
    int32_t flags;
    int32_t pad;
    cc_tight_grid grid;
    unsigned long long counts[4][8];
    unsigned long long digest, leaf_evals, trapped;
    uint64_t gen_sizes[CC_MAX_GENERATIONS + 1];
    uint64_t n_parents;
};
static const char kCkptMagic[8] = {'C', 'C', 'T', 'I', 'G', 'H', 'T', '1'};

static int write_checkpoint(cc_handle* h, const cc_tight_grid* grid, int next_gen, int flags, const GenTotals& tot,
                            const uint64_t* gen_sizes, const std::vector<cc_tight_box>& parents) {
    CkptHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, kCkptMagic, 8);
    hd.version = 1;
    hd.next_gen = next_gen;
    hd.flags = flags;
    hd.grid = *grid;
    std::memcpy(hd.counts, tot.counts, sizeof(hd.counts));
    hd.digest = tot.digest;
    hd.leaf_evals = tot.leaf_evals;
    hd.trapped = tot.trapped;
    std::memcpy(hd.gen_sizes, gen_sizes, sizeof(hd.gen_sizes));
    hd.n_parents = parents.size();
    const std::string tmp = h->checkpoint_path + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return ccrt::fail(h, CC_ERR_PARAM, "checkpoint: cannot open the file for writing");
    bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1;
    if (ok && !parents.empty()) ok = std::fwrite(parents.data(), sizeof(cc_tight_box), parents.size(), f) == parents.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), h->checkpoint_path.c_str()) != 0)
        return ccrt::fail(h, CC_ERR_PARAM, "checkpoint: write failed");
    return CC_OK;
}

static int check_grid(cc_handle* h, const cc_tight_grid* grid) {
    if (grid->la_splits_init < 1 || grid->num_generations < 0 || grid->num_generations > CC_MAX_GENERATIONS)
        return ccrt::fail(h, CC_ERR_PARAM, "grid: bad lambda splits or generation count");
    for (int k = 0; k < 4; ++k)
        if (!valid_split(grid->r_splits_init[k]) || (grid->num_generations && !valid_split(grid->r_splits_gen[k])))
            return ccrt::fail(h, CC_ERR_PARAM, "grid: radius splits must be in [1, 2047]");
    for (int g = 0; g < grid->num_generations; ++g)
        if (grid->la_splits_gen[g] < 1) return ccrt::fail(h, CC_ERR_PARAM, "grid: bad lambda splits");
    return CC_OK;
}

// generations start_gen..num_generations from `cur`
static int prove_generations(cc_handle* h, const cc_tight_grid* grid, int flags, int start_gen,
                             std::vector<cc_tight_box>& cur, GenTotals& tot, uint64_t* gen_sizes,
                             cc_tight_box** criticals, size_t* n_crit, cc_prove_stats* stats) {
    const bool hoist = !(flags & CC_PROVE_PLAIN);
    h->launches = 0;
    h->interrupt.store(0);
    CC_CUDA(h, cudaSetDevice(h->device));
    auto t0 = std::chrono::steady_clock::now();
    const unsigned long long fails0 = cert_failures_so_far();
    Caps caps{0, 1ULL << 22, 1ULL << 23, 1ULL << 24, 1ULL << 24, 1ULL << 20, 1ULL << 26};
    std::vector<cc_tight_box> next;
    int gens_run = start_gen > 0 ? start_gen - 1 : 0;
    int status = CC_OK;
    for (int g = start_gen; g <= grid->num_generations; ++g) {
        if (g > 0 && cur.empty()) break;
        const int k = g == 0 ? grid->la_splits_init : grid->la_splits_gen[g - 1];
        const int* s = g == 0 ? grid->r_splits_init : grid->r_splits_gen;
        next.clear();
        int st = run_generation(h, cur, k, s, next, tot, caps, hoist, flags);
        if (st) return st;
        cur.swap(next);
        gen_sizes[g] = cur.size();
        gens_run = g;
        if (!h->checkpoint_path.empty() && (st = write_checkpoint(h, grid, g + 1, flags, tot, gen_sizes, cur)))
            return st;
        if (h->interrupt.load()) {
            status = CC_ERR_INTERRUPTED;
            break;
        }
    }
    *n_crit = cur.size();
    *criticals = (cc_tight_box*)std::malloc(sizeof(cc_tight_box) * (cur.size() + 1));
    if (!*criticals) return ccrt::fail(h, CC_ERR_OOM, "malloc criticals");
    if (!cur.empty()) std::memcpy(*criticals, cur.data(), sizeof(cc_tight_box) * cur.size());
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::memcpy(stats->counts, tot.counts, sizeof(stats->counts));
        stats->digest = tot.digest;
        stats->leaf_evals = tot.leaf_evals;
        stats->trapped_leaves = tot.trapped;
        std::memcpy(stats->gen_sizes, gen_sizes, sizeof(uint64_t) * (CC_MAX_GENERATIONS + 1));
        stats->generations_run = gens_run;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->kernel_launches = h->launches;
        std::memcpy(stats->fp32_first, tot.fp32, sizeof(stats->fp32_first));
        stats->cert_failures = cert_failures_so_far() - fails0;
    }
    return status;
}

}  // namespace

extern "C" int cc_tight_prove_ex(cc_handle* h, const cc_tight_box* root, const cc_tight_grid* grid, int flags,
                                 cc_tight_box** criticals, size_t* n_crit, cc_prove_stats* stats) {
    if (!h || !root || !grid || !criticals || !n_crit) return CC_ERR_PARAM;
    if ((flags & CC_PROVE_LEARNED) && !h->mlp)
        return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_prove_ex: CC_PROVE_LEARNED needs a network (cc_mlp_init)");
    int st = check_grid(h, grid);
    if (st) return st;
    if (flags & CC_PROVE_LOG_CELLS) h->cell_log.clear();
    *criticals = nullptr;
    *n_crit = 0;
    GenTotals tot;
    std::vector<cc_tight_box> cur{*root};
    uint64_t gen_sizes[CC_MAX_GENERATIONS + 1] = {};
    return prove_generations(h, grid, flags, 0, cur, tot, gen_sizes, criticals, n_crit, stats);
}

extern "C" int cc_set_checkpoint(cc_handle* h, const char* path) {
    if (!h) return CC_ERR_PARAM;
    h->checkpoint_path = path ? path : "";
    return CC_OK;
}

extern "C" int cc_tight_resume(cc_handle* h, const char* path, const cc_tight_grid* grid, int flags,
                               cc_tight_box** criticals, size_t* n_crit, cc_prove_stats* stats) {
    if (!h || !path || !criticals || !n_crit) return CC_ERR_PARAM;
    *criticals = nullptr;
    *n_crit = 0;
    FILE* f = std::fopen(path, "rb");
    if (!f) return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_resume: cannot open the checkpoint");
    CkptHeader hd;
    bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, kCkptMagic, 8) == 0 && hd.version == 1 &&
              hd.next_gen >= 1 && hd.next_gen <= CC_MAX_GENERATIONS + 1 && hd.n_parents < (1ULL << 40);
    std::vector<cc_tight_box> cur;
    if (ok) {
        cur.resize(hd.n_parents);
        ok = hd.n_parents == 0 || std::fread(cur.data(), sizeof(cc_tight_box), hd.n_parents, f) == hd.n_parents;
    }
    std::fclose(f);
    if (!ok) return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_resume: not a complete checkpoint");
    cc_tight_grid g = grid ? *grid : hd.grid;
    int st = check_grid(h, &g);
    if (st) return st;
    // the run so far must be the start of the requested schedule
    bool same = g.la_splits_init == hd.grid.la_splits_init && g.num_generations >= hd.next_gen - 1;
    for (int k = 0; k < 4 && same; ++k) same = g.r_splits_init[k] == hd.grid.r_splits_init[k];
    for (int k = 0; k < 4 && same && hd.next_gen > 1; ++k) same = g.r_splits_gen[k] == hd.grid.r_splits_gen[k];
    for (int i = 0; i + 1 < hd.next_gen && same; ++i) same = g.la_splits_gen[i] == hd.grid.la_splits_gen[i];
    if (!same) return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_resume: the checkpoint's schedule is not a prefix of the grid");
    if ((flags & CC_PROVE_LEARNED) && !h->mlp)
        return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_resume: CC_PROVE_LEARNED needs a network (cc_mlp_init)");
    GenTotals tot;
    std::memcpy(tot.counts, hd.counts, sizeof(tot.counts));
    tot.digest = hd.digest;
    tot.leaf_evals = hd.leaf_evals;
    tot.trapped = hd.trapped;
    uint64_t gen_sizes[CC_MAX_GENERATIONS + 1];
    std::memcpy(gen_sizes, hd.gen_sizes, sizeof(gen_sizes));
    return prove_generations(h, &g, flags, hd.next_gen, cur, tot, gen_sizes, criticals, n_crit, stats);
}

extern "C" int cc_tight_prove(cc_handle* h, const cc_tight_box* root, const cc_tight_grid* grid, cc_tight_box** criticals,
                              size_t* n_crit, cc_prove_stats* stats) {
    return cc_tight_prove_ex(h, root, grid, 0, criticals, n_crit, stats);
}

extern "C" int cc_tight_generation(cc_handle* h, const cc_tight_box* parents, size_t n_parents, int la_splits,
                                   const int r_splits[4], uint64_t task_lo, uint64_t task_hi, int flags,
                                   cc_tight_box** criticals, size_t* n_crit, cc_prove_stats* stats) {
    if (!h || (n_parents && !parents) || !r_splits || !criticals || !n_crit || task_lo > task_hi) return CC_ERR_PARAM;
    if (!valid_split(la_splits)) return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_generation: bad lambda splits");
    for (int k = 0; k < 4; ++k)
        if (!valid_split(r_splits[k])) return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_generation: splits in [1, 2047]");
    if ((flags & CC_PROVE_LEARNED) && !h->mlp)
        return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_generation: CC_PROVE_LEARNED needs a network (cc_mlp_init)");
    *criticals = nullptr;
    *n_crit = 0;
    h->launches = 0;
    CC_CUDA(h, cudaSetDevice(h->device));
    auto t0 = std::chrono::steady_clock::now();
    Caps caps{0, 1ULL << 22, 1ULL << 23, 1ULL << 24, 1ULL << 24, 1ULL << 20, 1ULL << 26};
    GenTotals tot;
    const unsigned long long fails0 = cert_failures_so_far();
    std::vector<cc_tight_box> in(parents, parents + n_parents), out;
    int st = run_generation(h, in, la_splits, r_splits, out, tot, caps, !(flags & CC_PROVE_PLAIN), flags, task_lo, task_hi);
    if (st) return st;
    *n_crit = out.size();
    *criticals = (cc_tight_box*)std::malloc(sizeof(cc_tight_box) * (out.size() + 1));
    if (!*criticals) return ccrt::fail(h, CC_ERR_OOM, "malloc criticals");
    if (!out.empty()) std::memcpy(*criticals, out.data(), sizeof(cc_tight_box) * out.size());
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::memcpy(stats->counts, tot.counts, sizeof(stats->counts));
        stats->digest = tot.digest;
        stats->leaf_evals = tot.leaf_evals;
        stats->trapped_leaves = tot.trapped;
        stats->gen_sizes[0] = out.size();
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->kernel_launches = h->launches;
        std::memcpy(stats->fp32_first, tot.fp32, sizeof(stats->fp32_first));
        stats->cert_failures = cert_failures_so_far() - fails0;
    }
    return CC_OK;
}

extern "C" int cc_tight_cell_log(cc_handle* h, cc_tight_box* out, size_t cap, size_t* n, int* r4_splits) {
    if (!h || !n || (cap && !out)) return CC_ERR_PARAM;
    *n = h->cell_log.size();
    if (r4_splits) *r4_splits = h->cell_log_splits;
    const size_t k = std::min(cap, h->cell_log.size());
    if (k) std::memcpy(out, h->cell_log.data(), k * sizeof(cc_tight_box));
    return CC_OK;
}

extern "C" int cc_tight_summary(cc_handle* h, const cc_tight_box* criticals, size_t n, cc_tight_summary_t* out) {
    if (!h || !out || (n && !criticals)) return CC_ERR_PARAM;
    h->launches = 0;
    CC_CUDA(h, cudaSetDevice(h->device));
    void *d_in = nullptr, *d_out = nullptr;
    int st;
    if ((st = ccrt::ensure(h, 0, (n + 1) * sizeof(cc_tight_box), &d_in))) return st;
    if ((st = ccrt::ensure(h, 1, sizeof(cc_tight_summary_t), &d_out))) return st;
    if (n) CC_CUDA(h, cudaMemcpyAsync(d_in, criticals, n * sizeof(cc_tight_box), cudaMemcpyHostToDevice, h->stream));
    void* d_items;
    if ((st = ccrt::ensure(h, 2, (n + 1) * sizeof(cc::summary::Item), &d_items))) return st;
    if (n) {
        const int g = (int)std::min<size_t>((n + 127) / 128, (size_t)h->sm_count * 8);
        cc::summary::k_summary_items<<<g, 128, 0, h->stream>>>((const cc::tight::Box*)d_in, n,
                                                              (cc::summary::Item*)d_items);
        CC_LAUNCHED(h);
    }
    cc::summary::k_summary_fold<<<1, 1, 0, h->stream>>>((const cc::summary::Item*)d_items, (const cc::tight::Box*)d_in,
                                                        n, (cc_tight_summary_t*)d_out);
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaMemcpyAsync(out, d_out, sizeof(cc_tight_summary_t), cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

// ============================================================ refinement
// Adaptive refinement of a set of tight boxes to a depth cap (no reference
// counterpart; the near-critical stress workload).  Every level runs the
// certified evaluation (the six criteria and the emptiness bits, passes 0-5)
// on its boxes -- or the first-success evaluation in the plain or the learned
// order; the split kernels then sort them: certified or empty boxes are
// done, trapped ones are kept as criticals, the others are bisected into the
// next level -- or kept as criticals at the last level.  The boxes of a level
// are independent and of uneven cost (the criteria's branches and
// bisections), so each level is one batch of the evaluation passes over
// compacted queues.
namespace {

enum { S_REF_A = 28, S_REF_B = 29, S_REF_MASKS = 30, S_REF_CRIT = 31, S_REF_SOA = 40, S_REF_FIRST = 41,
       S_REF_MLP = 42, S_REF_BLOCKS = 43 };

struct RefineCounters {
    unsigned long long n_next, n_crit, n_decided, overflow;
    unsigned long long fp64, cover, gaps, cert, steps, warp_max_steps, n_cut;
};

// one evaluation batch's queue sizes added to the level's occupancy
__global__ void k_refine_tally(const unsigned long long* __restrict__ counts, RefineCounters* c) {
    if (threadIdx.x != 0) return;
    c->fp64 += counts[kCntFull];
    c->cover += counts[kCntCover];
    c->gaps += counts[kCntGaps];
    unsigned long long cert = 0;
    for (int k = 0; k < kCertQueues; ++k) cert += counts[kCntCert + k];
    c->cert += cert;
}

// a level's verdicts: the evaluation's masks, or first-success outcomes
struct MaskVerdicts {
    const uint32_t* m;
    __device__ __forceinline__ void get(size_t i, bool& trapped, bool& decided, unsigned& steps) const {
        const uint32_t x = m[i];
        trapped = (x >> 31) != 0;
        decided = !trapped && (x & 0x7Fu) != 0;
        steps = 0;
    }
};
struct FirstVerdicts {
    const uint8_t* o;
    const uint8_t* ev;
    __device__ __forceinline__ void get(size_t i, bool& trapped, bool& decided, unsigned& steps) const {
        const uint8_t x = o[i];
        trapped = (x & 0x80u) != 0;
        decided = !trapped && (x & 0x7Fu) != 7u;
        steps = ev[i];
    }
};

__device__ __forceinline__ void bisect_dim(const cc_tight_box& b, int dim, cc_tight_box& lo_half, cc_tight_box& hi_half) {
    lo_half = b;
    hi_half = b;
    const cc_iv& v = dim == 0 ? b.la : b.r[dim - 1];
    // 0.5 lo + 0.5 hi: no overflow; the halves' union is the interval
    const double mid = 0.5 * v.lb + 0.5 * v.ub;
    cc_iv& l = dim == 0 ? lo_half.la : lo_half.r[dim - 1];
    cc_iv& u = dim == 0 ? hi_half.la : hi_half.r[dim - 1];
    l.ub = mid;
    u.lb = mid;
}

// The split of a level, in three kernels that keep the level's order (so a
// refinement is deterministic and its levels are those of the oracle's
// sequential model): each block owns a contiguous range of the level;
// k_refine_count counts its split candidates (undecided, not trapped, not
// the last level) and its kept boxes (trapped, or undecided at the last
// level); k_refine_scan turns the counts into each block's output offsets,
// carrying at most pair_cap candidates (the first ones in level order) into
// the next level and keeping the others as criticals (flag 3: cut by the
// population cap); k_refine_emit writes the children (lo half, hi half) and
// the criticals at those offsets, in level order within each block.
struct RefineBlocks {
    unsigned long long* cand;  // per block: split candidates, then their offset (exclusive scan)
    unsigned long long* keep;  // per block: kept boxes, then their offset (cut candidates included)
    unsigned long long per_block;
    int n_blocks;
};

template <class V>
__global__ void __launch_bounds__(128) k_refine_count(size_t n, V verdicts, int last, RefineBlocks rb,
                                                      RefineCounters* c) {
    __shared__ unsigned long long s_sum[2][4];
    const unsigned long long lo = (unsigned long long)blockIdx.x * rb.per_block;
    const unsigned long long hi = lo + rb.per_block < n ? lo + rb.per_block : n;
    unsigned long long cand = 0, keep = 0, decided_n = 0, steps_n = 0, warp_max_n = 0;
    for (unsigned long long base = lo + (threadIdx.x & ~31u); base < hi; base += blockDim.x) {
        const unsigned long long i = base + (threadIdx.x & 31);
        unsigned lane_steps = 0;
        if (i < hi) {
            bool trapped, decided;
            verdicts.get(i, trapped, decided, lane_steps);
            steps_n += lane_steps;
            decided_n += decided ? 1 : 0;
            cand += (!trapped && !decided && !last) ? 1 : 0;
            keep += (trapped || (!decided && last)) ? 1 : 0;
        }
        warp_max_n += __reduce_max_sync(0xffffffffu, lane_steps);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_xor_sync(0xffffffffu, cand, o);
        keep += __shfl_xor_sync(0xffffffffu, keep, o);
        decided_n += __shfl_xor_sync(0xffffffffu, decided_n, o);
        steps_n += __shfl_xor_sync(0xffffffffu, steps_n, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_sum[0][w] = cand;
        s_sum[1][w] = keep;
        if (decided_n) atomicAdd(&c->n_decided, decided_n);
        if (steps_n) atomicAdd(&c->steps, steps_n);
        if (warp_max_n) atomicAdd(&c->warp_max_steps, warp_max_n);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        rb.cand[blockIdx.x] = s_sum[0][0] + s_sum[0][1] + s_sum[0][2] + s_sum[0][3];
        rb.keep[blockIdx.x] = s_sum[1][0] + s_sum[1][1] + s_sum[1][2] + s_sum[1][3];
    }
}

__global__ void k_refine_scan(RefineBlocks rb, unsigned long long pair_cap, RefineCounters* c) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long cand_acc = 0, keep_acc = 0, cut_total = 0;
    for (int b = 0; b < rb.n_blocks; ++b) {
        const unsigned long long nc = rb.cand[b], nk = rb.keep[b];
        // candidates of this block past the cap are kept instead
        const unsigned long long room = pair_cap > cand_acc ? pair_cap - cand_acc : 0;
        const unsigned long long cut = nc > room ? nc - room : 0;
        rb.cand[b] = cand_acc;
        rb.keep[b] = keep_acc;
        cand_acc += nc;
        keep_acc += nk + cut;
        cut_total += cut;
    }
    c->n_next = cand_acc < pair_cap ? cand_acc : pair_cap;
    c->n_crit = keep_acc;
    c->n_cut = cut_total;
}

// exclusive rank of `flag` among the block's 128 threads (in thread order),
// and the block's total; every thread calls it
__device__ __forceinline__ unsigned block_rank(bool flag, unsigned* s_warp, unsigned& total) {
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned ballot = __ballot_sync(0xffffffffu, flag);
    if (lane == 0) s_warp[w] = __popc(ballot);
    __syncthreads();
    unsigned before = 0;
    total = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        before += (unsigned)k < w ? s_warp[k] : 0u;
        total += s_warp[k];
    }
    __syncthreads();  // s_warp is rewritten by the next call
    return before + __popc(ballot & ((1u << lane) - 1u));
}

template <class V>
__global__ void __launch_bounds__(128) k_refine_emit(const cc_tight_box* __restrict__ in, size_t n, V verdicts,
                                                     int depth, int last, RefineBlocks rb,
                                                     unsigned long long pair_cap, cc_tight_box* __restrict__ out,
                                                     cc_tight_box* __restrict__ crit,
                                                     uint32_t* __restrict__ crit_flags) {
    __shared__ unsigned s_warp[4];
    const unsigned long long lo = (unsigned long long)blockIdx.x * rb.per_block;
    const unsigned long long hi = lo + rb.per_block < n ? lo + rb.per_block : n;
    unsigned long long cand_at = rb.cand[blockIdx.x], keep_at = rb.keep[blockIdx.x];
    const int dim = depth % 5;
    for (unsigned long long base = lo; base < hi; base += blockDim.x) {  // block-uniform loop
        const unsigned long long i = base + threadIdx.x;
        bool cand = false, keep = false, trapped = false;
        if (i < hi) {
            bool decided;
            unsigned st;
            verdicts.get(i, trapped, decided, st);
            cand = !trapped && !decided && !last;
            keep = trapped || (!decided && last);
        }
        unsigned n_cand;
        const unsigned long long r = cand_at + block_rank(cand, s_warp, n_cand);
        const bool split = cand && r < pair_cap;
        const bool kept = keep || (cand && !split);
        unsigned n_kept;
        const unsigned long long k = keep_at + block_rank(kept, s_warp, n_kept);
        if (split || kept) {
            const cc_tight_box b = in[i];
            if (split) {
                bisect_dim(b, dim, out[2 * r], out[2 * r + 1]);
            } else {
                crit[k] = b;
                crit_flags[k] = trapped ? 1u : (keep ? 2u : 3u);
            }
        }
        cand_at += n_cand;
        keep_at += n_kept;
    }
}

}  // namespace

extern "C" int cc_set_refine_order(cc_handle* h, int order) {
    if (!h || order < CC_REFINE_MASKS || order > CC_REFINE_FIRST_LEARNED) return CC_ERR_PARAM;
    h->refine_order = order;
    return CC_OK;
}

extern "C" int cc_tight_refine(cc_handle* h, const cc_tight_box* boxes, size_t n, int max_depth, size_t max_live,
                               cc_tight_box** criticals, uint32_t** flags, size_t* n_crit, cc_refine_stats* stats) {
    if (!h || (n && !boxes) || !criticals || !n_crit || max_depth < 0 || max_depth > CC_REFINE_MAX_DEPTH)
        return CC_ERR_PARAM;
    *criticals = nullptr;
    if (flags) *flags = nullptr;
    *n_crit = 0;
    CC_CUDA(h, cudaSetDevice(h->device));
    h->launches = 0;
    h->interrupt.store(0);
    const auto t0 = std::chrono::steady_clock::now();
    if (max_live < 2) max_live = (size_t)1 << 26;
    const int order = h->refine_order;
    if (order == CC_REFINE_FIRST_LEARNED && !h->mlp)
        return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_refine: learned order without a trained network (cc_mlp_init)");
    cc_refine_stats st{};
    st.order = order;
    cudaStream_t s = h->stream;
    void *a, *cnt_p;
    int rc;
    if ((rc = ccrt::ensure(h, S_REF_A, std::max<size_t>(n, 1) * sizeof(cc_tight_box), &a))) return rc;
    if (n) CC_CUDA(h, cudaMemcpyAsync(a, boxes, n * sizeof(cc_tight_box), cudaMemcpyHostToDevice, s));
    if ((rc = ccrt::ensure(h, 4, sizeof(RefineCounters), &cnt_p))) return rc;
    RefineCounters* dc = (RefineCounters*)cnt_p;
    ccrt::EventPair ev;
    CC_CUDA(h, cudaEventCreate(&ev.e0));
    CC_CUDA(h, cudaEventCreate(&ev.e1));
    std::vector<cc_tight_box> out;
    std::vector<uint32_t> out_flags;
    int cur_slot = S_REF_A, next_slot = S_REF_B;
    size_t cur_n = n;
    const size_t chunk = (size_t)1 << 24;  // evaluation batches: bounded scratch
    const unsigned long long pair_cap = max_live / 2;  // children pairs a level may carry on
    for (int d = 0; d <= max_depth && cur_n; ++d) {
        const bool last = d == max_depth;
        const size_t next_n = last ? 1 : 2 * std::min<size_t>(cur_n, pair_cap);
        void *cur, *next, *masks, *crit, *blocks;
        if ((rc = ccrt::ensure(h, cur_slot, cur_n * sizeof(cc_tight_box), &cur))) return rc;
        if ((rc = ccrt::ensure(h, next_slot, next_n * sizeof(cc_tight_box), &next))) return rc;
        RefineBlocks rb;
        rb.n_blocks = eval_grid(h, cur_n);
        rb.per_block = (cur_n + rb.n_blocks - 1) / rb.n_blocks;
        if ((rc = ccrt::ensure(h, S_REF_BLOCKS, 2 * (size_t)rb.n_blocks * sizeof(unsigned long long), &blocks)))
            return rc;
        rb.cand = (unsigned long long*)blocks;
        rb.keep = rb.cand + rb.n_blocks;
        if ((rc = ccrt::ensure(h, S_REF_MASKS, cur_n * sizeof(uint32_t), &masks))) return rc;
        if ((rc = ccrt::ensure(h, S_REF_CRIT, cur_n * (sizeof(cc_tight_box) + sizeof(uint32_t)), &crit))) return rc;
        void *soa = nullptr, *first = nullptr, *mlp = nullptr;
        if (order != CC_REFINE_MASKS) {
            const size_t m = std::min(chunk, cur_n);
            if ((rc = ccrt::ensure(h, S_REF_SOA, m * sizeof(cc_tight_box), &soa))) return rc;
            if ((rc = ccrt::ensure(h, S_REF_FIRST, 2 * cur_n, &first))) return rc;
            if (order == CC_REFINE_FIRST_LEARNED &&
                (rc = ccrt::ensure(h, S_REF_MLP, m * kFirstScratchFloats * sizeof(float), &mlp)))
                return rc;
        }
        CC_CUDA(h, cudaMemsetAsync(dc, 0, sizeof(RefineCounters), s));
        CC_CUDA(h, cudaEventRecord(ev.e0, s));
        for (size_t off = 0; off < cur_n; off += chunk) {
            const size_t m = std::min(chunk, cur_n - off);
            const double* part = (const double*)((cc_tight_box*)cur + off);
            if (order == CC_REFINE_MASKS) {
                rc = eval_batch<Layout::AoS>(h, part, m, (uint32_t*)masks + off, s, false);
                if (rc) return rc;
                k_refine_tally<<<1, 32, 0, s>>>(h->eval_counts, dc);
                CC_LAUNCHED(h);
            } else {
                k_aos_to_soa<<<h->sm_count * 8, 256, 0, s>>>(part, m, (double*)soa);
                CC_LAUNCHED(h);
                rc = cc_first_success_async(h, (const double*)soa, m, (float)d, (float*)mlp, (uint8_t*)first + off,
                                            (uint8_t*)first + cur_n + off, s);
                if (rc) return rc;
            }
        }
        cc_tight_box* crit_boxes = (cc_tight_box*)crit;
        uint32_t* crit_fl = (uint32_t*)(crit_boxes + cur_n);
        const int lastf = last ? 1 : 0;
        const MaskVerdicts mv{(const uint32_t*)masks};
        const FirstVerdicts fv{(const uint8_t*)first, (const uint8_t*)first + cur_n};
        if (order == CC_REFINE_MASKS)
            k_refine_count<<<rb.n_blocks, 128, 0, s>>>(cur_n, mv, lastf, rb, dc);
        else
            k_refine_count<<<rb.n_blocks, 128, 0, s>>>(cur_n, fv, lastf, rb, dc);
        CC_LAUNCHED(h);
        k_refine_scan<<<1, 32, 0, s>>>(rb, pair_cap, dc);
        CC_LAUNCHED(h);
        const cc_tight_box* cb = (const cc_tight_box*)cur;
        cc_tight_box* nb = (cc_tight_box*)next;
        if (order == CC_REFINE_MASKS)
            k_refine_emit<<<rb.n_blocks, 128, 0, s>>>(cb, cur_n, mv, d, lastf, rb, pair_cap, nb, crit_boxes, crit_fl);
        else
            k_refine_emit<<<rb.n_blocks, 128, 0, s>>>(cb, cur_n, fv, d, lastf, rb, pair_cap, nb, crit_boxes, crit_fl);
        CC_LAUNCHED(h);
        CC_CUDA(h, cudaEventRecord(ev.e1, s));
        RefineCounters hc;
        CC_CUDA(h, cudaMemcpyAsync(&hc, dc, sizeof(hc), cudaMemcpyDeviceToHost, s));
        CC_CUDA(h, cudaStreamSynchronize(s));
        if (hc.overflow) return ccrt::fail(h, CC_ERR_QUEUE_OVERFLOW, "cc_tight_refine: queue overflow");
        float ms = 0.0f;
        CC_CUDA(h, cudaEventElapsedTime(&ms, ev.e0, ev.e1));
        st.live[d] = cur_n;
        st.decided[d] = hc.n_decided;
        st.ms[d] = ms;
        st.fp64_boxes[d] = hc.fp64;
        st.cover_jobs[d] = hc.cover;
        st.gaps_jobs[d] = hc.gaps;
        st.cert_jobs[d] = hc.cert;
        st.steps[d] = hc.steps;
        st.warp_max_steps[d] = hc.warp_max_steps;
        st.cut[d] = hc.n_cut;
        if (hc.n_cut) st.stopped_at_cap = 1;
        st.depths_run = d + 1;
        if (hc.n_crit) {
            const size_t old = out.size();
            out.resize(old + hc.n_crit);
            out_flags.resize(old + hc.n_crit);
            CC_CUDA(h, cudaMemcpyAsync(out.data() + old, crit, hc.n_crit * sizeof(cc_tight_box), cudaMemcpyDeviceToHost, s));
            CC_CUDA(h, cudaMemcpyAsync(out_flags.data() + old, (cc_tight_box*)crit + cur_n, hc.n_crit * sizeof(uint32_t),
                                       cudaMemcpyDeviceToHost, s));
            CC_CUDA(h, cudaStreamSynchronize(s));
        }
        cur_n = 2 * hc.n_next;
        std::swap(cur_slot, next_slot);
        if (h->interrupt.load()) break;
    }
    *n_crit = out.size();
    *criticals = (cc_tight_box*)std::malloc(sizeof(cc_tight_box) * (out.size() + 1));
    if (!*criticals) return ccrt::fail(h, CC_ERR_OOM, "malloc criticals");
    if (!out.empty()) std::memcpy(*criticals, out.data(), sizeof(cc_tight_box) * out.size());
    if (flags) {
        *flags = (uint32_t*)std::malloc(sizeof(uint32_t) * (out.size() + 1));
        if (!*flags) return ccrt::fail(h, CC_ERR_OOM, "malloc flags");
        if (!out.empty()) std::memcpy(*flags, out_flags.data(), sizeof(uint32_t) * out.size());
    }
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    st.kernel_launches = h->launches;
    if (stats) *stats = st;
    return CC_OK;
}

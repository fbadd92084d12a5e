// Covering-strategy criteria of the tight-rectangle proof: a lambda x 1
// rectangle, lambda in [1, 2.0898841580413818342], is to be covered by disks
// whose total weight (sum of squared radii) is the critical amount
// required_weight_for(lambda).  Every predicate returns true only if its
// covering strategy is certified by outward-rounded FP64 interval arithmetic.
//
// Each function restates the reference function cited next to it with the
// same sequence of directed-rounding operations, so verdicts are
// bit-identical; the structure (names, early exits that cannot change a
// result, hoisted constants) is this project's own.
#pragma once

#include "cc_sb_common.cuh"
#include "cc_f32.cuh"

namespace cc {
#if CC_DEVICE_BUILD
namespace sb {
// one out-of-line copy for the FP32 evaluation (the 2x2 criterion calls it six times)
__device__ __noinline__ inline f32::Fv two_disks_maximize_height(f32::IvF d1, f32::IvF d2, f32::Fv ub_w) {
    return two_disks_maximize_height_t<f32::IvF>(d1, d2, ub_w);
}
}  // namespace sb
#endif
namespace tight {

// A box of the tight proof: aspect ratio and the four largest squared radii
// (reference: tight_rectangle/strategies.cuh:33-50, same 80-byte layout).
template <class I>
struct BoxT {
    I la;
    I r[4];
};
using Box = BoxT<Iv>;

// Break-even aspect ratio lambda_2 = sqrt(sqrt(7)/2 - 1/4) between the
// three-disk and the two-disk worst case, as outward-rounded bounds.  The
// reference recomputes them on every call (critical_ratio.cu:60-61: four
// directed square roots); they are constants, evaluated once with exact
// directed rounding and checked against the formula by the tests.
static constexpr double kBreakEvenLo = 0x1.0929ffddd109ap+0;  // 1.0357971111816711
static constexpr double kBreakEvenHi = 0x1.0929ffddd109bp+0;  // 1.0357971111816713
CC_FN double break_even_lo_formula() { return sqrt_dn(add_dn(mul_dn(0.5, sqrt_dn(7.0)), -0.25)); }
CC_FN double break_even_hi_formula() { return sqrt_up(add_up(mul_up(0.5, sqrt_up(7.0)), -0.25)); }

// Worst-case covering ratio (weight per area) of a lambda x 1 rectangle,
// lambda >= 1 (critical_ratio.cu:58-78):
//   lambda <= lambda_2:  (3/256)/lambda * (16 lambda^2 + 40 + 9/lambda^2)
//   lambda >= lambda_2:  lambda/4 + 1/(2 lambda)
template <class I>
CC_FN I ratio_three_disk(I la) {
    I la2 = square(la);
    return ((3.0 / 256.0) / la) * (16.0 * la2 + 40.0 + 9.0 / la2);
}
template <class I>
CC_FN I ratio_two_disk(I la) { return 0.25 * la + 0.5 * reciprocal(la); }

template <class I>
CC_FN I critical_ratio_t(I la) {
    if (definitely(la <= kBreakEvenLo)) {
        return ratio_three_disk(la);
    }
    if (definitely(la >= kBreakEvenHi)) {
        return ratio_two_disk(la);
    }
    I a = ratio_three_disk(la);
    I b = ratio_two_disk(la);
    return I{lesser(a.lo, b.lo), greater(b.hi, a.hi)};
}

CC_FN Iv critical_ratio(Iv la) { return critical_ratio_t(la); }
#if CC_DEVICE_BUILD
// one out-of-line copy of each FP32 form: the criteria call them from many
// sites, and the evaluation kernels must stay small for the instruction cache
__device__ __noinline__ inline f32::IvF critical_ratio(f32::IvF la) { return critical_ratio_t(la); }
#endif

// ratio for a w x h rectangle in either orientation (critical_ratio.cu:32-52)
template <class I>
CC_FN I critical_ratio_t(I w, I h) {
    if (w.hi <= h.lo) {
        return critical_ratio(h / w);
    }
    if (h.hi <= w.lo) {
        return critical_ratio(w / h);
    }
    I tall = h / w;
    tighten_lb(tall, 1.0);
    I wide = w / h;
    tighten_lb(wide, 1.0);
    I a = critical_ratio(tall);
    I b = critical_ratio(wide);
    return I{lesser(a.lo, b.lo), greater(b.hi, a.hi)};
}
CC_FN Iv critical_ratio(Iv w, Iv h) { return critical_ratio_t(w, h); }
#if CC_DEVICE_BUILD
__device__ __noinline__ inline f32::IvF critical_ratio(f32::IvF w, f32::IvF h) { return critical_ratio_t(w, h); }
#endif

template <class I>
CC_FN I required_weight_for(I w, I h) { return critical_ratio(w, h) * w * h; }  // critical_ratio.cu:80-82
template <class I>
CC_FN I required_weight_for(I la) { return critical_ratio(la) * la; }            // critical_ratio.cu:84-86

// can_apply_size_bounded_covering.cu:49-52
template <class S>
CC_FN S required_weight_for_bounded_size(S ub_w, S ub_h) {
    return mul_up(sb::kCriticalRatio, mul_up(ub_w, ub_h));
}

// Can a rectangle of at most ub_w x ub_h be covered recursively by disks of
// weight <= ub_largest and total weight >= lb_weight?  Best of the worst-case
// ratio, the size-bounded corollary and the 9/64 size-bound ratio
// (can_recurse.cu:32-62).
template <class S>
CC_FN bool can_recurse_t(S ub_w, S ub_h, S ub_largest, S lb_weight) {
    S ub_area = mul_up(ub_w, ub_h);
    S side_min = lesser(ub_w, ub_h);
    S s = rcp_up(side_min);
    S s_sq = mul_up(s, s);
    S largest_norm = mul_up(s_sq, ub_largest);

    S ratio;
    if (largest_norm <= sb::kUbDiskWeight) {
        // the size-bound ratio replaces whatever was computed before
        ratio = sb::kCriticalRatio;
    } else {
        ratio = critical_ratio(ivp(ub_w), ivp(ub_h)).hi;
        S ratio_cor = mul_up(0.5, sqrt_up(add_up(sqrt_up(add_up(mul_up(largest_norm, largest_norm), 1.0)), 1.0)));
        ratio_cor = greater(S(195.0 / 256), ratio_cor);  // at least 195/256
        ratio = lesser(ratio_cor, ratio);                // the better of the two
    }
    S ub_needed = mul_up(ratio, ub_area);
    return lb_weight >= ub_needed;
}
// Certification runs (device only): an FP32 evaluation decided that a
// criterion holds and which of its can_recurse calls settled it; the FP64
// criterion then runs with only that call evaluated and every other call
// answering "false".  Every call site of the criteria is of the form
// "if (... && can_recurse(...)) return true" or "return can_recurse(...)"
// inside placements joined by ||, so a call forced to "false" can only make
// the criterion false: an FP64 run that returns true is an FP64 proof that
// the criterion holds, whatever the FP32 evaluation did.
CC_FN bool can_recurse(double ub_w, double ub_h, double ub_largest, double lb_weight) {
#if CC_DEVICE_BUILD
    const uint8_t mode = cc_trap_words[threadIdx.x];
    if (mode & kCertModeBit) {
        const uint16_t s = cc_cert_state[threadIdx.x];
        cc_cert_state[threadIdx.x] = (uint16_t)(s + 1);
        if ((s & 0xff) + 1 != (s >> 8)) return false;
        if (mode & kCertRecordBit) {  // the chosen call, evaluated later (cert_record_begin)
            cc_cert_out[threadIdx.x] = CertCall{ub_w, ub_h, ub_largest, lb_weight};
            return true;
        }
    }
#endif
    return can_recurse_t<double>(ub_w, ub_h, ub_largest, lb_weight);
}
#if CC_DEVICE_BUILD
// start / end of a certification run that evaluates call number `call`
// (1-based; 0 = no call) of the FP64 criterion; the trap status is cleared
CC_FN void cert_begin(int call) {
    cc_cert_state[threadIdx.x] = (uint16_t)(call << 8);
    cc_trap_words[threadIdx.x] = kCertModeBit;
}
CC_FN void cert_end() { cc_trap_words[threadIdx.x] &= (uint8_t)~(kCertModeBit | kCertRecordBit); }
// The branches can_recurse_t takes on a recorded call, as a sort key for
// running recorded calls on warps that follow one path: 0 the size-bound
// ratio (the largest disk at most 9/64 of the shorter side squared), else 1
// + 3 * (wide rectangle) + the critical ratio's formula (three-disk,
// two-disk, both) for the aspect ratio.  Computed in FP32 near the
// thresholds; it only groups the calls, the evaluation is can_recurse_t's.
static constexpr int kCallPathKeys = 7;
CC_FN int call_path_key(const CertCall& a) {
    const float w = (float)a.w, h = (float)a.h;
    const float side = fminf(w, h);
    const float norm = (float)a.largest / (side * side);
    if (!(norm > 0.140625f)) return 0;
    const bool tall = w <= h;
    const float aspect = tall ? h / w : w / h;
    const int f = aspect <= 1.0357f ? 0 : (aspect >= 1.0359f ? 1 : 2);
    return 1 + (tall ? 0 : 3) + f;
}
// A certification run in record form: the chosen call stores its arguments
// in cc_cert_out[threadIdx.x] and answers "true", so the criterion returns
// true right there (the call sites' form); the call itself is evaluated
// afterwards on the stored arguments, by can_recurse_t.  After the run,
// cert_reached() tells whether the run got to the chosen call.
CC_FN void cert_record_begin(int call) {
    cc_cert_state[threadIdx.x] = (uint16_t)(call << 8);
    cc_trap_words[threadIdx.x] = kCertModeBit | kCertRecordBit;
}
CC_FN bool cert_reached() {
    const uint16_t s = cc_cert_state[threadIdx.x];
    return (s & 0xff) >= (s >> 8);
}
// the FP32 can_recurse counts its calls (low byte of cc_cert_state)
CC_FN void cert_count_reset() { cc_cert_state[threadIdx.x] = 0; }
CC_FN int cert_count() { return cc_cert_state[threadIdx.x] & 0xff; }
// the FP32 run's last can_recurse call answered "true"
CC_FN bool cert_last_true() { return (cc_cert_state[threadIdx.x] & 0x8000) != 0; }

// One out-of-line copy for the FP32 evaluation (it is called from many
// sites), with a shortcut before its costly part.  Where largest_norm is
// certainly above 9/64, can_recurse_t takes ratio = lesser(ratio_cor,
// ratio_wh) with ratio_wh the upper bound of the w x h rectangle's critical
// ratio (critical_ratio(), several interval divisions).  So ratio <=
// ratio_cor, and ratio >= min(ratio_cor, sqrt(2)/2): every critical ratio is
// at least sqrt(2)/2 (the two-disk formula lambda/4 + 1/(2 lambda) has that
// minimum at lambda = sqrt 2; the three-disk one is decreasing on [1,
// lambda_2] down to its value there, 0.74), and the FP64 upper bound of an
// enclosure of it is not below the exact value by more than a few ulps
// (0.7070 leaves a margin of 1e-4); this needs w, h > 0, so that the ratio's
// argument is an aspect ratio >= 1.  As mul_up is monotone, lb_weight above
// the FP32 enclosure of ratio_cor * area (or below that of 0.7070 or
// ratio_cor times area) decides can_recurse_t without ratio_wh; no trap site
// is skipped (the critical ratio has none).  Only certain comparisons are
// used here; anything else falls through to can_recurse_t.
//
// Record mode (mode bit of the trap word, set by record_group_f32): the call
// stores its arguments in the thread's next record slot and answers "false",
// so the criterion goes on exactly as the FP64 one would after a false
// result; the calls are evaluated afterwards, in rounds over compacted
// queues (k_eval_calls), and combined in order (a true call settles the
// criterion, as in the FP64 short circuit).
struct CrArgs {
    f32::Fv w, h, largest, lb;
};
static constexpr int kCrRecordSlots = 4;
static __shared__ CrArgs cc_cr_rec[kCrRecordSlots][128];
// bits 0-2: calls recorded; bit 3 + j: the path to call j was already undecided
static __shared__ uint8_t cc_cr_info[128];

__device__ __noinline__ inline bool can_recurse_record(f32::Fv ub_w, f32::Fv ub_h, f32::Fv ub_largest,
                                                       f32::Fv lb_weight) {
    uint8_t info = cc_cr_info[threadIdx.x];
    const int j = info & 7;
    if (j >= kCrRecordSlots) {  // more calls than slots: the criterion stays undecided
        trap(TRAP_F32_UNDECIDED);
        return false;
    }
    cc_cr_rec[j][threadIdx.x] = CrArgs{ub_w, ub_h, ub_largest, lb_weight};
    if (trap_status() != TRAP_NONE) info |= (uint8_t)(8u << j);
    cc_cr_info[threadIdx.x] = (uint8_t)(info + 1);
    return false;
}

__device__ __forceinline__ bool can_recurse_f32(f32::Fv ub_w, f32::Fv ub_h, f32::Fv ub_largest, f32::Fv lb_weight) {
    using f32::Fv;
    const Fv ub_area = f32::mul(ub_w, ub_h);
    const Fv s = f32::rcp_up(f32::lesser(ub_w, ub_h));
    const Fv largest_norm = f32::mul(f32::mul(s, s), ub_largest);
    // w and h certainly positive and finite: then the critical ratio's
    // argument is an aspect ratio >= 1 and everything stays finite
    const bool sane = ub_w.lo > 0.0f && ub_h.lo > 0.0f && ub_w.hi < 1e30f && ub_h.hi < 1e30f;
    if (sane && largest_norm.lo > 0.140625f && largest_norm.lo <= largest_norm.hi && lb_weight.lo <= lb_weight.hi) {
        const Fv t = f32::add(f32::sqrt_nn(f32::add(f32::mul(largest_norm, largest_norm), Fv{1.0f, 1.0f})),
                              Fv{1.0f, 1.0f});
        const Fv ratio_cor = f32::greater(Fv{0.76171875f, 0.76171875f}, f32::scale(f32::sqrt_nn(t), 0.5f));
        const float need_hi = f32::mul(ratio_cor, ub_area).hi;  // >= the FP64 ub_needed
        if (lb_weight.lo >= need_hi) return true;
        const float r_lo = fminf(ratio_cor.lo, 0.7070f);
        const float need_lo = __fmul_rd(r_lo, ub_area.lo);     // <= the FP64 ub_needed
        if (lb_weight.hi < need_lo) return false;
    }
    return can_recurse_t<f32::Fv>(ub_w, ub_h, ub_largest, lb_weight);
}
// The call count for a later certification run (cert_count) and, in bit 15,
// whether this call answered "true" (cert_last_true).
__device__ __noinline__ inline bool can_recurse(f32::Fv ub_w, f32::Fv ub_h, f32::Fv ub_largest, f32::Fv lb_weight) {
    if (cc_trap_words[threadIdx.x] & kTrapModeBit) return can_recurse_record(ub_w, ub_h, ub_largest, lb_weight);
    const bool r = can_recurse_f32(ub_w, ub_h, ub_largest, lb_weight);
    const uint16_t s = cc_cert_state[threadIdx.x];
    cc_cert_state[threadIdx.x] = (uint16_t)((((s & 0xff) + 1) & 0xff) | (r ? 0x8000 : 0));
    return r;
}
#endif

// ------------------------------------------------------------ one disk
// Place disk 1 as a full-height strip, in a corner, or as an uneven split;
// recurse on the rest (r1_strategies.cu:27-87).  `weight` is
// required_weight_for(la), which the reference recomputes inside every
// criterion; callers compute it once per box (same bits).
template <class I>
CC_FN_INL bool r1_strategies(I la, I weight, I r1, typename I::S ub_r2) {
    using S = typename I::S;
    S square_w = sqrt_dn(mul_dn(2.0, r1.lo));
    S strip_w = add_dn(mul_dn(4.0, r1.lo), -1.0);
    const S lb_rem = (weight - r1).lo;

    if (strip_w > 0.0) {
        strip_w = sqrt_dn(strip_w);
        I w_rest = la - strip_w;
        if (can_recurse(w_rest.hi, 1.0, ub_r2, lb_rem)) {
            return true;
        }
    }

    if (square_w < 1.0) {
        S w_right = add_up(la.hi, -square_w);
        S min_right = lesser(w_right, S(1.0));
        S ub_weight_right;
        if (sb::disk_satisfies_size_bound<S>(ub_r2, min_right)) {
            ub_weight_right = mul_up(w_right, sb::kCriticalRatio);
        } else {
            ub_weight_right = required_weight_for(ivp(w_right), ivp(S(1.0))).hi;
        }
        ub_weight_right = add_up(ub_weight_right, ub_r2);
        S lb_rem_top = add_dn(lb_rem, -ub_weight_right);
        if (lb_rem_top > 0.0) {
            S h_top = add_up(1.0, -square_w);
            if (can_recurse(square_w, h_top, ub_r2, lb_rem_top)) {
                return true;
            }
        }
    }

    S lb_S1 = add_dn(mul_dn(4.0, r1.lo), -1.0);
    if (lb_S1 > 0.0) {
        lb_S1 = sqrt_dn(lb_S1);
        S t = add_up(la.hi, -mul_dn(0.5, lb_S1));
        t = mul_up(t, t);
        S lb_h1 = add_dn(r1.lo, -t);
        if (lb_h1 > 0.0) {
            lb_h1 = mul_dn(2.0, sqrt_dn(lb_h1));
            S ub_pocket_h = mul_up(0.5, add_up(1.0, -lb_h1));
            S ub_pocket_w = add_up(la.hi, -lb_S1);
            S lb_rem_half = mul_dn(0.5, add_dn(lb_rem, -ub_r2));
            if (lb_rem_half > 0.0 && can_recurse(ub_pocket_w, ub_pocket_h, ub_r2, lb_rem_half)) {
                return true;
            }
        }
    }
    return false;
}

// ----------------------------------------------------------- two disks
// Region around the two-disk worst case settled by hand in the paper
// (r1_r2_strategies.cu:29-46).
template <class I>
CC_FN bool two_pocket_by_hand(I la, I r1, I r2) {
    using S = typename I::S;
    if (r2.lo < 0.2400000000000000188 || r1.lo < 0.4900000000000000466) {
        return false;
    }
    I la2 = square(la);
    S r1_need = (0.25 * (la2 + 1.0) - 0.00999999999999999847).hi;
    if (r1.lo < r1_need) {
        return false;
    }
    I S1 = 2.0 * sqrt(r1 - 0.25);
    I pocket = la - S1;
    tighten_lb(pocket, 0.0);
    S r2_need = (0.25 + square(pocket) - 0.00999999999999999847).hi;
    return r2.lo >= r2_need;
}

// disks 1 and 2 side by side as a strip (r1_r2_strategies.cu:48-72)
template <class I>
CC_FN bool r1_r2_side_by_side(I la, I weight, I r1, I r2, typename I::S ub_r3) {
    using S = typename I::S;
    if (two_pocket_by_hand(la, r1, r2)) {
        return true;
    }
    S lb_width = sb::two_disks_maximize_height(r1, r2, 1.0);
    if (lb_width <= 0.0) {
        return false;
    }
    S lb_w2 = add_dn(mul_dn(4.0, r2.lo), -1.0);
    if (lb_w2 > 0.0) {
        lb_w2 = sqrt_dn(lb_w2);
        S lb_w1 = sqrt_dn(add_dn(mul_dn(4.0, r1.lo), -1.0));
        S lb_w = add_dn(lb_w1, lb_w2);
        // the reference: if (lb_w > lb_width) { lb_width = lb_w; if (lb_w > la.hi) return true; }
        if (lb_w > la.hi && lb_w > lb_width) {
            return true;
        }
        lb_width = greater(lb_w, lb_width);
    }
    S w_rem = add_dn(la.hi, lb_width);  // sic: '+' (parity)
    S lb_R3 = (weight - r1 - r2).lo;
    return can_recurse(w_rem, 1.0, ub_r3, lb_R3);
}

// disk 1 in a corner square, disk 2 across the top (r1_r2_strategies.cu:74-129)
template <class I>
CC_FN bool r1_r2_stacked(I la, I weight, I r1, I r2, typename I::S ub_r3) {
    using S = typename I::S;
    S sq_side = sqrt_dn(mul_dn(2.0, r1.lo));
    if (sq_side > 1.0) {
        return false;
    }
    S h_top = add_up(1.0, -sq_side);
    S lb_w2 = add_dn(mul_dn(4.0, r2.lo), -mul_up(h_top, h_top));
    if (lb_w2 < 0.0) {
        return false;
    }
    lb_w2 = sqrt_dn(lb_w2);

    S w_top = add_up(la.hi, -lb_w2);
    S w_bot = add_up(la.hi, -sq_side);
    S top_min = lesser(w_top, h_top);
    S bot_min = lesser(w_bot, sq_side);
    S lb_R3 = (weight - r1 - r2).lo;

    if (sb::disk_satisfies_size_bound<S>(ub_r3, top_min)) {
        S need_top = add_up(required_weight_for_bounded_size<S>(w_top, h_top), ub_r3);
        S left = add_dn(lb_R3, -need_top);
        if (left > 0.0 && can_recurse(w_bot, sq_side, ub_r3, left)) {
            return true;
        }
    } else if (sb::disk_satisfies_size_bound<S>(ub_r3, bot_min)) {
        S need_bot = add_up(required_weight_for_bounded_size<S>(w_bot, sq_side), ub_r3);
        S left = add_dn(lb_R3, -need_bot);
        if (left > 0.0 && can_recurse(w_top, h_top, ub_r3, left)) {
            return true;
        }
    } else {
        S need_top = required_weight_for(ivp(w_top), ivp(h_top)).hi;
        need_top = add_up(need_top, ub_r3);
        S left = add_dn(lb_R3, -need_top);
        if (left > 0.0) {
            return can_recurse(w_bot, sq_side, ub_r3, left);
        }
    }
    return false;
}

// r1_r2_strategies.cu:131-133
template <class I>
CC_FN_INL bool r1_r2_strategies(I la, I weight, I r1, I r2, typename I::S ub_r3) {
    return r1_r2_side_by_side(la, weight, r1, r2, ub_r3) || r1_r2_stacked(la, weight, r1, r2, ub_r3);
}

// --------------------------------------------------------- three disks
// three full-height strips (r1_r2_r3_strategies.cu:28-47)
template <class I>
CC_FN bool r1_r2_r3_three_strips(I la, I weight, I r1, I r2, I r3, typename I::S ub_r4) {
    using S = typename I::S;
    S lb_w3 = add_dn(mul_dn(4.0, r3.lo), -1.0);
    if (lb_w3 <= 0.0) {
        return false;
    }
    lb_w3 = sqrt_dn(lb_w3);
    S lb_w2 = sqrt_dn(add_dn(mul_dn(4.0, r2.lo), -1.0));
    S lb_w1 = sqrt_dn(add_dn(mul_dn(4.0, r1.lo), -1.0));
    S lb_cov = add_dn(lb_w1, add_dn(lb_w2, lb_w3));
    S lb_R4 = (weight - r1 - r2 - r3).lo;
    S ub_rem = add_up(la.hi, -lb_cov);
    if (ub_rem <= 0.0) {
        return true;
    }
    return can_recurse(ub_rem, 1.0, ub_r4, lb_R4);
}

// Disk 1 on top of a strip of width w, disks 2 and 3 below it side by side
// (r1_r2_r3_strategies.cu:49-67).
template <class S>
CC_FN bool strip_width_realizable(S r1, S r2, S r3, S w) {
    S h1 = add_dn(mul_dn(4.0, r1), -mul_up(w, w));
    if (h1 <= 0.0) {
        return false;
    }
    h1 = sqrt_dn(h1);
    S h_rem = add_up(1.0, -h1);
    S h_sq = mul_up(h_rem, h_rem);
    S w2 = add_dn(mul_dn(4.0, r2), -h_sq);
    S w3 = add_dn(mul_dn(4.0, r3), -h_sq);
    if (w3 <= 0.0 || w2 <= 0.0) {
        return false;
    }
    w2 = sqrt_dn(w2);
    w3 = sqrt_dn(w3);
    return add_dn(w2, w3) >= w;
}

#if CC_DEVICE_BUILD
// strip_width_realizable decided with FP32 enclosures of its FP64 values
// (cc_f32.cuh), for every w in the enclosure W at once: YES / NO are the FP64
// predicate's outcome at each such w, UNKNOWN leaves it to the FP64
// predicate.  The operands that do not change during the bisection are
// enclosed once.
struct StripF32 {
    f32::Fv a1, a2, a3;  // 4 r1, 4 r2, 4 r3
};
CC_FN StripF32 strip_f32_prepare(double r1, double r2, double r3) {
    return StripF32{f32::scale(f32::of(r1), 4.0f), f32::scale(f32::of(r2), 4.0f), f32::scale(f32::of(r3), 4.0f)};
}
CC_FN int strip_width_realizable_f32(const StripF32& p, f32::Fv W) {
    using namespace f32;
    const Fv h1 = sub(p.a1, sqr(W));
    if (h1.hi <= 0.0f) return NO;
    if (!(h1.lo > 0.0f)) return UNKNOWN;
    const Fv h_sq = sqr(sub(point(1.0f), sqrt_nn(h1)));
    const Fv w2 = sub(p.a2, h_sq), w3 = sub(p.a3, h_sq);
    if (w3.hi <= 0.0f || w2.hi <= 0.0f) return NO;
    if (!(w3.lo > 0.0f && w2.lo > 0.0f)) return UNKNOWN;
    const Fv sum = add(sqrt_nn(w2), sqrt_nn(w3));
    if (sum.lo >= W.hi) return YES;
    if (sum.hi < W.lo) return NO;
    return UNKNOWN;
}
#endif

// The cover-strip strategy (r1_r2_r3_strategies.cu:69-94) in three pieces,
// so that the bisection can run as its own pass over the boxes that need it:
//   enters: the strip of width 0.3 is realizable (else the strategy fails);
//   width:  the widest realizable strip, by bisection to the FP64 fixpoint;
//   finish: recursion on the rest of the rectangle.
CC_FN bool cover_strip_enters(double r1, double r2, double r3) { return strip_width_realizable(r1, r2, r3, 0.3); }

// The reference's bisections (cover strip, gaps) run to the FP64 fixpoint:
// mid = 0.5 * (lo + hi) until mid is no longer strictly between lo and hi,
// with a trap after CC_BISECTION_CAP steps.  On the device two FP32 shortcuts
// come first, both giving the same lo and the same trap status:
//   * the predicate decided for the whole range [lo, hi] at once (an FP32
//     enclosure of [lo, hi] contains every later mid, and the enclosures are
//     inclusion-isotone).  If it is false everywhere, every step lowers hi and
//     the result is lo; from 0 <= lo < hi <= DBL_MAX that takes fewer than
//     2,100 steps (about 1,075 halvings down to the subnormals, 1,024 more at
//     most for the exponent of hi), so the cap cannot trap.  If it is true
//     everywhere, the steps raise lo and bisect_all_true replays them;
//   * the leading steps decided by the FP32 enclosure of mid, as long as it
//     decides the step for every lane of the warp (a warp vote, so the warp
//     leaves the FP32 steps together); from the first step some lane cannot
//     decide, every step runs the FP64 predicate.  A warp pays for an FP64
//     step if any of its lanes needs one, so per-lane FP32 steps after that
//     would only add work.
CC_FN double bisect_all_true(double lo, double hi) {
    for (int it = 0;; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) {
            break;
        }
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            break;
        }
        lo = mid;
    }
    return lo;
}

#if CC_DEVICE_BUILD
// true while the FP32 decision d may stand for every converged lane
__device__ __forceinline__ bool f32_step_for_all(int d) { return __all_sync(__activemask(), d != f32::UNKNOWN); }
#endif

// A criterion that ends with a bisection needs only its final check of the
// bisection's result, and that result always lies in the current bracket
// [lo, hi].  So the bisections take `early(lo, hi)`: on the device it is
// asked before the first step and where the FP32 steps end for the final
// check's outcome for every result in [lo, hi] (FP32 enclosures: YES, NO or
// UNKNOWN), and a decided answer ends the bisection (*decided; for finite
// brackets only, where the bisection cannot reach its cap, so no trap is
// skipped).  NoEarly never decides.
struct NoEarly {
    CC_METHOD int operator()(double, double) const { return -1; }
};

// A strip-width bisection stopped at its first FP64 step (where the FP32
// steps end and the final check is not decided for the whole bracket), to be
// resumed in a later pass on full warps: its bracket and step count, and the
// box.  *decided is kBisectionDeferred then.
struct CoverResume {
    double lo, hi;
    int32_t it;
    uint32_t box;
};
static constexpr int kBisectionDeferred = 2;

template <class Early>
CC_FN double cover_strip_width_early(double la_hi, double r1, double r2, double r3, Early early, int* decided,
                                     CoverResume* stop = nullptr) {
    double lo = 0.3;
    double hi = la_hi;
    *decided = -1;
#if CC_DEVICE_BUILD
    const bool finite = lo < hi && hi <= CC_DBL_MAX;
    if (finite && (*decided = early(lo, hi)) != f32::UNKNOWN) return lo;
    const StripF32 pf = strip_f32_prepare(r1, r2, r3);
    if (finite) {
        int whole = strip_width_realizable_f32(pf, f32::hull(lo, hi));
        if (whole == f32::NO) return lo;
        if (whole == f32::YES) return bisect_all_true(lo, hi);
    }
    bool f32_steps = true;
#else
    (void)stop;
#endif
    for (int it = 0;; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) {
            break;
        }
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            break;
        }
#if CC_DEVICE_BUILD
        bool ok;
        int d = f32_steps ? strip_width_realizable_f32(pf, f32::of(mid)) : f32::UNKNOWN;
        if (f32_steps && f32_step_for_all(d)) {
            ok = d == f32::YES;
        } else {
            if (f32_steps) {
                f32_steps = false;
                if (finite && (*decided = early(lo, hi)) != f32::UNKNOWN) return lo;
                if (stop) {
                    stop->lo = lo;
                    stop->hi = hi;
                    stop->it = it;
                    *decided = kBisectionDeferred;
                    return lo;
                }
            }
            ok = strip_width_realizable(r1, r2, r3, mid);
        }
#else
        bool ok = strip_width_realizable(r1, r2, r3, mid);
#endif
        if (ok) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    return lo;
}

CC_FN double cover_strip_width_fp64(double la_hi, double r1, double r2, double r3);

// The FP64 steps of a bisection stopped by cover_strip_width_early: the same
// loop from the same bracket and step count.
CC_FN double cover_strip_width_resume(double r1, double r2, double r3, double lo, double hi, int it) {
    for (;; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            break;
        }
        if (strip_width_realizable(r1, r2, r3, mid)) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The widest realizable strip.  On the device the bisection's FP32 steps are
// followed by an FP64 certificate: the width it returns must pass the FP64
// predicate (the reference's bisection keeps lo realizable by construction,
// r1_r2_r3_strategies.cu:90: "a strip width we can definitely achieve").  If
// it does not, the bisection is redone in FP64 alone (cert_failed).
CC_FN double cover_strip_width(double la_hi, double r1, double r2, double r3) {
    int decided;
    const double w = cover_strip_width_early(la_hi, r1, r2, r3, NoEarly{}, &decided);
#if CC_DEVICE_BUILD
    if (!strip_width_realizable(r1, r2, r3, w)) {
        cert_failed();
        return cover_strip_width_fp64(la_hi, r1, r2, r3);
    }
#endif
    return w;
}

// The bisection exactly as the reference runs it (r1_r2_r3_strategies.cu:
// 77-88): FP64 steps only, no FP32 shortcut.  Used to repair a box whose
// FP64 certification failed.
CC_FN double cover_strip_width_fp64(double la_hi, double r1, double r2, double r3) {
    double lo = 0.3, hi = la_hi;
    for (int it = 0;; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            break;
        }
        if (strip_width_realizable(r1, r2, r3, mid)) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <class S>
CC_FN bool cover_strip_finish(S la_hi, S width, S ub_r4, S lb_R4) {
    S ub_rem = add_up(la_hi, -width);
    return can_recurse(ub_rem, 1.0, ub_r4, lb_R4);
}

CC_FN_INL bool r1_r2_r3_cover_strip(Iv la, Iv weight, Iv r1, Iv r2, Iv r3, double ub_r4) {
    if (!cover_strip_enters(r1.lo, r2.lo, r3.lo)) {
        return false;
    }
    double width = cover_strip_width(la.hi, r1.lo, r2.lo, r3.lo);
    return cover_strip_finish(la.hi, width, ub_r4, (weight - r1 - r2 - r3).lo);
}

// r1_r2_r3_strategies.cu:96-99
CC_FN_INL bool r1_r2_r3_strategies(Iv la, Iv weight, Iv r1, Iv r2, Iv r3, double ub_r4) {
    return r1_r2_r3_three_strips(la, weight, r1, r2, r3, ub_r4) || r1_r2_r3_cover_strip(la, weight, r1, r2, r3, ub_r4);
}

// Disks 2 and 3 form a strip, disk 1 covers the rest of a column
// (r1_r2_r3_strategies.cu:101-121).  Each of the three-disk placements below
// is split into the part before its recursion check, returning 0 (fails), 1
// (holds) or 2 (holds iff can_recurse(w, h, ub_r4, lb_R4)), and the check:
// the proof prepares the first part once per r3 cell (leaf123_prepare).
template <class S>
CC_FN int three_disk_big_strip_wh(S ub_la, S r1, S r2, S r3, S& w, S& h) {
    S S_sq = add_dn(add_dn(mul_dn(2.0, r2), add_dn(mul_dn(2.0, r3), -0.25)),
                    add_dn(add_dn(-mul_up(4.0, mul_up(r2, r2)), mul_dn(8.0, mul_dn(r2, r3))),
                           -mul_up(4.0, mul_up(r3, r3))));
    if (S_sq <= 0.0) {
        return 0;
    }
    S side = sqrt_dn(S_sq);
    S la_rem = add_up(ub_la, -side);
    S h1_sq = add_dn(mul_dn(4.0, r1), -mul_up(la_rem, la_rem));
    if (h1_sq <= 0.0) {
        return 0;
    }
    if (h1_sq >= 1.0) {
        return 1;
    }
    w = la_rem;
    h = add_up(1.0, -sqrt_dn(h1_sq));
    return 2;
}
template <class S>
CC_FN bool three_disk_big_strip(S ub_la, S r1, S r2, S r3, S ub_r4, S lb_R4) {
    S w, h;
    const int st = three_disk_big_strip_wh<S>(ub_la, r1, r2, r3, w, h);
    return st == 2 ? can_recurse(w, h, ub_r4, lb_R4) : st == 1;
}

// disk 3 in a corner, disks 1 and 2 along its sides (r1_r2_r3_strategies.cu:123-165)
template <class S>
CC_FN int three_disk_small_corner_wh(S ub_la, S r1, S r2, S r3, S& w, S& h) {
    S c3 = sqrt_dn(mul_dn(2.0, r3));
    if (c3 >= 1.0) {
        return 0;
    }
    S la_left = add_up(ub_la, -c3);
    S la_half = mul_up(la_left, 0.5);
    S one_left = add_up(1.0, -c3);

    if (la_half <= sqrt_dn(r2)) {
        S c1 = sqrt_dn(add_dn(mul_dn(4.0, r1), -mul_up(one_left, one_left)));
        S la_after_1 = add_up(ub_la, -c1);
        S c2 = sqrt_dn(add_dn(mul_dn(4.0, r2), -mul_up(la_left, la_left)));
        S one_after_2 = add_up(1.0, -c2);
        w = la_after_1;
        h = one_after_2;
        return 2;
    }
    if (la_half >= sqrt_dn(r1)) {
        return 0;
    }
    if (one_left >= mul_dn(2.0, sqrt_dn(r2))) {
        return 0;
    }
    S c2 = sqrt_dn(add_dn(mul_dn(4.0, r2), -mul_up(one_left, one_left)));
    S la_after_2 = add_up(ub_la, -c2);
    S c1 = sqrt_dn(add_dn(mul_dn(4.0, r1), -mul_up(la_left, la_left)));
    S one_after_1 = add_up(1.0, -c1);
    w = la_after_2;
    h = one_after_1;
    return 2;
}
template <class S>
CC_FN bool three_disk_small_corner(S ub_la, S r1, S r2, S r3, S ub_r4, S lb_R4) {
    S w, h;
    const int st = three_disk_small_corner_wh<S>(ub_la, r1, r2, r3, w, h);
    return st == 2 ? can_recurse(w, h, ub_r4, lb_R4) : st == 1;
}

// disks 1 and 3 at the sides, 2 in between, a pocket remains
// (r1_r2_r3_strategies.cu:167-204)
template <class I>
CC_FN int three_disk_r1_r3_pocket_wh(I la, I r1, I r2, I r3, typename I::S& w, typename I::S& h) {
    if (r1.lo <= 0.25) {
        return 0;
    }
    I S1 = 2.0 * sqrt(r1 - 0.25);
    I la_m_S1 = la - S1;
    I h2_rest = 0.25 * la_m_S1 * la_m_S1;
    if (r2.lo <= h2_rest.hi) {
        return 0;
    }
    I h2 = 2.0 * sqrt(r2 - h2_rest);
    I one_m_h2 = 1.0 - h2;
    I S3_rest = 0.25 * one_m_h2 * one_m_h2;
    if (r3.lo <= S3_rest.hi) {
        return 0;
    }
    I S3 = 2.0 * sqrt(r3 - S3_rest);
    I X = la - S1 - S3;
    if (X.hi <= 0.0) {
        return 1;
    }
    I t = la - 0.5 * S1 - S3;
    I Y_rest = t * t;
    if (r1.lo <= Y_rest.hi) {
        return 0;
    }
    I Y = 0.5 - sqrt(r1 - Y_rest);
    if (Y.hi <= 0.0) {
        return 1;
    }
    w = X.hi;
    h = Y.hi;
    return 2;
}
template <class I>
CC_FN bool three_disk_r1_r3_pocket(I la, I r1, I r2, I r3, typename I::S ub_r4, typename I::S lb_R4) {
    typename I::S w, h;
    const int st = three_disk_r1_r3_pocket_wh(la, r1, r2, r3, w, h);
    return st == 2 ? can_recurse(w, h, ub_r4, lb_R4) : st == 1;
}

// Region around the three-disk worst case settled by hand in the paper
// (r1_r2_r3_strategies.cu:206-247).
template <class I>
CC_FN bool three_disk_pocket_by_hand(I la, I r1, I r2, I r3) {
    if (la.hi > 1.0499999999999998) {
        return false;
    }
    I la2 = square(la);
    I rstar = 0.0625 * la2 + 0.15625 + 0.03515625 / la2;
    I d1 = rstar - r1;
    if (d1.lo < -0.0009999999999999998 || d1.hi > 0.0009999999999999998) {
        return false;
    }
    I d2 = rstar - r2;
    if (d2.lo < -0.0019999999999999996 || d2.hi > 0.0019999999999999996) {
        return false;
    }
    I d3 = rstar - r3;
    if (d3.lo < -0.0029999999999999996 || d3.hi > 0.0029999999999999996) {
        return false;
    }
    I S1 = 2.0 * sqrt(r1 - 0.25);
    I la_m_S1 = la - S1;
    I h2_rest = 0.25 * la_m_S1 * la_m_S1;
    if (r2.lo <= h2_rest.hi) {
        return false;
    }
    I h2 = 2.0 * sqrt(r2 - h2_rest);
    I one_m_h2 = 1.0 - h2;
    I S3_rest = 0.25 * one_m_h2 * one_m_h2;
    if (r3.lo <= S3_rest.hi) {
        return false;
    }
    I S3 = 2.0 * sqrt(r3 - S3_rest);
    I X = la - S1 - S3;
    return !(X.hi > 0.046999999999999993);
}

// r1_r2_r3_strategies.cu:249-260
template <class I>
CC_FN_INL bool r1_r2_r3_strategies(const BoxT<I>& b, I R4) {
    using S = typename I::S;
    const S ub_la = b.la.hi;
    const S r1 = b.r[0].lo, r2 = b.r[1].lo, r3 = b.r[2].lo;
    const S ub_r4 = b.r[3].hi;
    const S lb_R4 = R4.lo;
    return three_disk_big_strip<S>(ub_la, r1, r2, r3, ub_r4, lb_R4) ||
           three_disk_small_corner<S>(ub_la, r1, r2, r3, ub_r4, lb_R4) ||
           three_disk_r1_r3_pocket(b.la, b.r[0], b.r[1], b.r[2], ub_r4, lb_R4) ||
           three_disk_pocket_by_hand(b.la, b.r[0], b.r[1], b.r[2]);
}

// ------------------------------------------------------------ 2 x 2
// disk 1 as a full-height strip, disks 2..4 stacked beside it
// (two_by_two_strategies.cu:29-53)
template <class I>
CC_FN bool two_by_two_r1_large(const BoxT<I>& b, I R) {
    using S = typename I::S;
    S w1 = sqrt_dn(add_dn(mul_dn(4.0, b.r[0].lo), -1.0));
    S w_rem = add_up(b.la.hi, -w1);
    S w_rem_sq = mul_up(w_rem, w_rem);
    S h4 = add_dn(mul_dn(4.0, b.r[3].lo), -w_rem_sq);
    if (h4 <= 0.0) {
        return false;
    }
    h4 = sqrt_dn(h4);
    S h3 = sqrt_dn(add_dn(mul_dn(4.0, b.r[2].lo), -w_rem_sq));
    S h2 = sqrt_dn(add_dn(mul_dn(4.0, b.r[1].lo), -w_rem_sq));
    S h_tot = add_dn(h2, add_dn(h3, h4));
    if (h_tot >= 1.0) {
        return true;
    }
    S h_rem = add_up(1.0, -h_tot);
    S ub_r5 = lesser(b.r[3].hi, R.hi);
    return can_recurse(w_rem, h_rem, ub_r5, R.lo);
}

// disk 1 in a corner, 2 beside, 4 above, 3 in the opposite corner
// (two_by_two_strategies.cu:55-86)
template <class I>
CC_FN bool two_by_two_lambda_small(const BoxT<I>& b, I R) {
    using S = typename I::S;
    S sq_side = sqrt_dn(mul_dn(2.0, b.r[0].lo));
    if (sq_side >= 1.0) {
        return two_by_two_r1_large(b, R);
    }
    S w_rem = add_up(b.la.hi, -sq_side);
    S h_rem = add_up(1.0, -sq_side);
    S h2 = add_dn(mul_dn(4.0, b.r[1].lo), -mul_up(w_rem, w_rem));
    S w4 = add_dn(mul_dn(4.0, b.r[3].lo), -mul_up(h_rem, h_rem));
    if (h2 <= 0.0 || w4 <= 0.0) {
        return false;
    }
    h2 = sqrt_dn(h2);
    w4 = sqrt_dn(w4);
    w4 = lesser(sq_side, w4);  // the reference: if (w4 > sq_side) w4 = sq_side
    h2 = lesser(sq_side, h2);
    S h = add_up(1.0, -h2);
    S w = add_up(b.la.hi, -w4);
    S diag = add_up(mul_up(h, h), mul_up(w, w));
    return mul_dn(4.0, b.r[2].lo) >= diag;
}

// best pairing of the four disks into two full-height pairs
// (two_by_two_strategies.cu:88-111)
template <class I>
CC_FN bool two_by_two_lambda_big(const BoxT<I>& b, I R) {
    using S = typename I::S;
    S lb_w = add_dn(sb::two_disks_maximize_height(b.r[0], b.r[1], 1.0),
                    sb::two_disks_maximize_height(b.r[2], b.r[3], 1.0));
    S w_1423 = add_dn(sb::two_disks_maximize_height(b.r[0], b.r[3], 1.0),
                      sb::two_disks_maximize_height(b.r[1], b.r[2], 1.0));
    lb_w = greater(w_1423, lb_w);  // the reference: if (w_1423 > lb_w) lb_w = w_1423
    S w_1324 = add_dn(sb::two_disks_maximize_height(b.r[0], b.r[2], 1.0),
                      sb::two_disks_maximize_height(b.r[1], b.r[3], 1.0));
    lb_w = greater(w_1324, lb_w);
    if (lb_w <= 0.0) {
        return false;
    }
    S ub_r5 = lesser(R.hi, b.r[3].hi);
    return can_recurse(add_up(b.la.hi, -lb_w), 1.0, ub_r5, R.lo);
}

// two_by_two_strategies.cu:113-115
template <class I>
CC_FN_INL bool two_by_two_strategies(const BoxT<I>& b, I R) {
    return two_by_two_lambda_small(b, R) || two_by_two_lambda_big(b, R);
}

// ---------------------------------------------- gap closed by disk 4
// Disks 1 and 2 as strips with a gap of width g between them; the gap is
// closed at the bottom by disk 4 (and symmetrically at the top by disk 3)
// (r1_r2_large_r3_r4_gaps_strategy.cu:29-59).
CC_FN bool gap_width_realizable(double g, double r1, double w1, double r2, double w2, double r4) {
    Iv y4 = r4 - 0.25 * ivp(g) * g;
    if (possibly(y4 <= 0.0)) {
        return false;
    }
    Iv x1 = ivp(0.5) * w1;
    Iv x2 = ivp(0.5) * w2 + g + w1;
    Circle c1{Point{x1, ivp(0.5)}, ivp(r1)};
    Circle c2{Point{x2, ivp(0.5)}, ivp(r2)};
    Isect x12 = intersection(c1, c2);
    if (!x12.definitely_intersecting) {
        return false;
    }
    Ub first_lower = x12.p[0].y <= x12.p[1].y;
    if (!is_certain(first_lower)) {
        return false;
    }
    Iv x4 = ivp(0.5) * g + w1;
    y4 = sqrt(y4);
    Point p4{x4, y4};
    const Point& px = x12.p[first_lower.lo ? 0 : 1];
    return definitely(squared_distance(p4, px) <= r4);
}

#if CC_DEVICE_BUILD
// gap_width_realizable decided with FP32 enclosures of its FP64 values
// (cc_f32.cuh), operation for operation, for every g in the enclosure G at
// once: the same quantities, each enclosed by the FP32 interval of the exact
// operation on the enclosures of its operands (`Iv * scalar`, which rounds
// both FP64 bounds down, stays inside that enclosure too).  YES / NO are the
// FP64 predicate's outcome at each such g; UNKNOWN leaves it to the FP64
// predicate.  In the FP64 code the centres' y difference is
// [-0, +0] exactly, so the order of the two intersection points depends on
// dx.lo >= 0 only.
struct GapsF32 {
    f32::Fv w1, x1, hw2, rdiff, rdiff_sq, s2, r4;
};
CC_FN GapsF32 gaps_f32_prepare(double r1, double r2, double w1, double w2, double r4) {
    using namespace f32;
    GapsF32 p;
    const Fv R1 = of(r1), R2 = of(r2);
    p.w1 = of(w1);
    p.x1 = scale(p.w1, 0.5f);
    p.hw2 = scale(of(w2), 0.5f);
    p.rdiff = sub(R1, R2);
    p.rdiff_sq = sqr(p.rdiff);
    p.s2 = scale(add(R1, R2), 2.0f);
    p.r4 = of(r4);
    return p;
}
CC_FN int gap_width_realizable_f32(f32::Fv G, const GapsF32& p) {
    using namespace f32;
    const Fv y4 = sub(p.r4, mul(scale(G, 0.25f), G));
    if (y4.hi <= 0.0f) return NO;
    if (!(y4.lo > 0.0f)) return UNKNOWN;
    const Fv x2 = add(add(p.hw2, G), p.w1);
    // intersection(c1, c2)
    const Fv d2 = sqr(sub(p.x1, x2));
    if (d2.hi == 0.0f) return NO;
    if (!(d2.lo > 0.0f)) return UNKNOWN;
    const Fv d2_sq = sqr(d2);
    if (!(d2_sq.lo > 0.0f)) return UNKNOWN;
    const Fv t = sub(sub(div_pos(p.s2, d2), point(1.0f)), div_pos(p.rdiff_sq, d2_sq));
    if (t.hi < 0.0f) return NO;
    if (!(t.lo >= 0.0f)) return UNKNOWN;
    const Fv half_chord = scale(sqrt_nn(t), 0.5f);
    const Fv shift = div_pos(scale(p.rdiff, 0.5f), d2);
    const Fv dx = sub(x2, p.x1);
    const Fv dy = sub(point(0.5f), point(0.5f));
    const Fv mx = add(scale(add(p.x1, x2), 0.5f), mul(shift, dx));
    const Fv my = add(point(0.5f), mul(shift, dy));
    const Fv ax = add(mx, mul(half_chord, dy)), ay = sub(my, mul(half_chord, dx));
    const Fv bx = sub(mx, mul(half_chord, dy)), by = add(my, mul(half_chord, dx));
    bool a_first;
    if (dx.lo >= 0.0f) a_first = true;
    else if (dx.hi < 0.0f) a_first = false;
    else return UNKNOWN;
    const Fv p0y = a_first ? ay : by, p1y = a_first ? by : ay;
    bool take_a;
    if (p0y.hi <= p1y.lo) take_a = a_first;         // first_lower certainly true: p[0]
    else if (p0y.lo > p1y.hi) take_a = !a_first;    // certainly false: p[1]
    else return UNKNOWN;
    const Fv px = take_a ? ax : bx, py = take_a ? ay : by;
    const Fv x4 = add(scale(G, 0.5f), p.w1);
    const Fv dist = add(sqr(sub(x4, px)), sqr(sub(sqrt_nn(y4), py)));
    if (dist.hi <= p.r4.lo) return YES;
    if (dist.lo > p.r4.hi) return NO;
    return UNKNOWN;
}
#endif

// The gaps strategy (r1_r2_large_r3_r4_gaps_strategy.cu:61-98) in three
// pieces, so that the bisection can run as its own pass over the boxes that
// need it:
//   enters: disks 1 and 2 both cover full-height strips (widths w1, w2);
//   width:  the widest gap disk 4 can close, by bisection to the FP64 fixpoint;
//   finish: recursion on the rest of the rectangle.
struct GapsStart {
    double w1, w2;
};

CC_FN bool gaps_enters(double r1, double r2, GapsStart& g) {
    double w1 = add_dn(mul_dn(4.0, r1), -1.0);
    double w2 = add_dn(mul_dn(4.0, r2), -1.0);
    if (w1 <= 0.0 || w2 <= 0.0) {
        return false;
    }
    g.w1 = sqrt_dn(w1);
    g.w2 = sqrt_dn(w2);
    return true;
}

template <class Early>
CC_FN double gaps_width_early(double r1, double r2, double r4, GapsStart g, Early early, int* decided) {
    const double w1 = g.w1, w2 = g.w2;
    double lo = 0.0, hi = add_dn(sqrt_dn(r1), sqrt_dn(r2));
    *decided = -1;
#if CC_DEVICE_BUILD
    // FP32 shortcuts: see bisect_all_true and cover_strip_width_early
    const bool finite = lo < hi && hi <= CC_DBL_MAX;
    const GapsF32 pf = gaps_f32_prepare(r1, r2, w1, w2, r4);
    if (finite) {
        int whole = gap_width_realizable_f32(f32::Fv{0.0f, f32::round_up(hi)}, pf);
        if (whole == f32::NO) return lo;
        if (whole == f32::YES) return bisect_all_true(lo, hi);
    }
    bool f32_steps = true;
#endif
    for (int it = 0;; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) {
            break;
        }
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            break;
        }
#if CC_DEVICE_BUILD
        bool ok;
        int d = f32_steps ? gap_width_realizable_f32(f32::of(mid), pf) : f32::UNKNOWN;
        if (f32_steps && f32_step_for_all(d)) {
            ok = d == f32::YES;
        } else {
            if (f32_steps) {
                f32_steps = false;
                if (finite && (*decided = early(lo, hi)) != f32::UNKNOWN) return lo;
            }
            ok = gap_width_realizable(mid, r1, w1, r2, w2, r4);
        }
#else
        bool ok = gap_width_realizable(mid, r1, w1, r2, w2, r4);
#endif
        if (ok) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    return lo;
}

CC_FN double gaps_width_fp64(double r1, double r2, double r4, GapsStart g);

// The widest gap disk 4 can close.  On the device the result of the
// bisection with FP32 steps gets an FP64 certificate: 0 (no gap, nothing to
// close) or a width that passes the FP64 predicate, as every lower end of
// the reference's bracket does; otherwise the bisection is redone in FP64.
CC_FN double gaps_width(double r1, double r2, double r4, GapsStart g) {
    int decided;
    const double gap = gaps_width_early(r1, r2, r4, g, NoEarly{}, &decided);
#if CC_DEVICE_BUILD
    if (gap != 0.0 && !gap_width_realizable(gap, r1, g.w1, r2, g.w2, r4)) {
        cert_failed();
        return gaps_width_fp64(r1, r2, r4, g);
    }
#endif
    return gap;
}

// The gap-width bisection exactly as the reference runs it
// (r1_r2_large_r3_r4_gaps_strategy.cu:73-86): FP64 steps only.
CC_FN double gaps_width_fp64(double r1, double r2, double r4, GapsStart g) {
    double lo = 0.0, hi = add_dn(sqrt_dn(r1), sqrt_dn(r2));
    for (int it = 0;; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            break;
        }
        if (gap_width_realizable(mid, r1, g.w1, r2, g.w2, r4)) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <class S>
CC_FN bool gaps_finish_t(S la_hi, S w1, S w2, S gap, S r4_hi, S R_lo, S R_hi) {
    S w_tot = add_dn(w1, add_dn(gap, w2));
    S w_rem = add_up(la_hi, -w_tot);
    if (w_rem <= 0.0) {
        return true;
    }
    S ub_r5 = lesser(r4_hi, R_hi);  // the reference: R.hi, lowered to r4_hi if above it
    return can_recurse(w_rem, 1.0, ub_r5, R_lo);
}
CC_FN bool gaps_finish(double la_hi, GapsStart g, double gap, double r4_hi, Iv R) {
    return gaps_finish_t<double>(la_hi, g.w1, g.w2, gap, r4_hi, R.lo, R.hi);
}

CC_FN_INL bool r1_r2_large_r3_r4_gaps_strategy(const Box& b, Iv R) {
    GapsStart g;
    if (!gaps_enters(b.r[0].lo, b.r[1].lo, g)) {
        return false;
    }
    double gap = gaps_width(b.r[0].lo, b.r[1].lo, b.r[3].lo, g);
    return gaps_finish(b.la.hi, g, gap, b.r[3].hi, R);
}

// --------------------------------------------------- range of each radius
// feasible ranges for r1..r4 given lambda (reference: tight_rectangle.cu:72-102)
CC_FN Iv r1_range(Iv la) {
    double f = div_dn(critical_ratio(la).lo, sb::kCriticalRatio);
    if (f <= 1.0) {
        f = 1.0;
    }
    double lo = mul_dn(sb::kUbDiskWeight, f);
    double hi = mul_up(0.25, add_up(1.0, mul_up(la.hi, la.hi)));
    return Iv{lo, hi};
}
CC_FN Iv r2_range(Iv weight, Iv r1) {
    double u1 = r1.hi;
    double u2 = (weight - r1).hi;
    return Iv{0.0, u1 < u2 ? u1 : u2};
}
CC_FN Iv r3_range(Iv weight, Iv r1, Iv r2) {
    double u1 = r2.hi;
    double u2 = (weight - r1 - r2).hi;
    return Iv{0.0, u1 < u2 ? u1 : u2};
}
CC_FN Iv r4_range(Iv weight, Iv r1, Iv r2, Iv r3) {
    double u1 = r3.hi;
    double u2 = (weight - r1 - r2 - r3).hi;
    return Iv{0.0, u1 < u2 ? u1 : u2};
}

// ------------------------------------------------ per-box verdict mask
// All six exported criteria at the arguments the reference's leaf passes
// them (tight_rectangle.cu:229-248): the first three on the box as given,
// the last three on the box with lower bounds tightened (r3 >= r4 >= ...)
// and with the remaining weights R (all four disks) and R4 (first three).
// Bit layout: CC_TV_* in include/circlecover_gb300.h.
//
// eval_main decides everything except the two bisections and says which of
// them the box still needs; cover_pass / gaps_pass finish them.  eval_all
// chains the three for one box.  The result does not depend on the split:
// every criterion is a pure function of the box, and the trap bit is an OR.

// inputs of the deferred cover-strip bisection (bit 2)
struct CoverJob {
    double la_hi, r1, r2, r3, ub_r4, lb_R4;
};
// inputs of the deferred gaps bisection (bit 5)
struct GapsJob {
    double la_hi, r1, r2, r4, r4_hi, w1, w2, R_lo, R_hi;
};

CC_FN_INL uint32_t eval_main(const Box& in, bool& need_cover, CoverJob& cj, bool& need_gaps, GapsJob& gj) {
    trap_clear();
    const Iv la = in.la, r1 = in.r[0], r2 = in.r[1], r3 = in.r[2], r4 = in.r[3];
    const Iv weight = required_weight_for(la);
    uint32_t m = 0;
    if (r1_strategies(la, weight, r1, r2.hi)) m |= 1u << 0;
    if (r1_r2_strategies(la, weight, r1, r2, r3.hi)) m |= 1u << 1;
    need_cover = false;
    if (r1_r2_r3_three_strips(la, weight, r1, r2, r3, r4.hi)) {
        m |= 1u << 2;
    } else if (cover_strip_enters(r1.lo, r2.lo, r3.lo)) {
        need_cover = true;
        cj = CoverJob{la.hi, r1.lo, r2.lo, r3.lo, r4.hi, (weight - r1 - r2 - r3).lo};
    }
    Iv R4 = weight - r1 - r2 - r3;
    tighten_lb(R4, 0.0);
    Box v{la, {r1, r2, r3, r4}};
    tighten_lb(v.r[2], v.r[3].lo);
    tighten_lb(v.r[1], v.r[2].lo);
    tighten_lb(v.r[0], v.r[1].lo);
    Iv R = weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
    tighten_lb(R, 0.0);
    if (two_by_two_strategies(v, R)) m |= 1u << 3;
    if (r1_r2_r3_strategies(v, R4)) m |= 1u << 4;
    GapsStart g;
    need_gaps = gaps_enters(v.r[0].lo, v.r[1].lo, g);
    if (need_gaps) {
        gj = GapsJob{la.hi, v.r[0].lo, v.r[1].lo, v.r[3].lo, v.r[3].hi, g.w1, g.w2, R.lo, R.hi};
    }
    if (empty(R4) || empty(R)) m |= 1u << 6;
    if (trap_status() != TRAP_NONE) m |= 1u << 31;
    return m;
}

CC_FN_INL uint32_t cover_pass(const CoverJob& j) {
    trap_clear();
    double width = cover_strip_width(j.la_hi, j.r1, j.r2, j.r3);
    uint32_t m = cover_strip_finish(j.la_hi, width, j.ub_r4, j.lb_R4) ? (1u << 2) : 0u;
    if (trap_status() != TRAP_NONE) m |= 1u << 31;
    return m;
}

CC_FN_INL uint32_t gaps_pass(const GapsJob& j) {
    trap_clear();
    GapsStart g{j.w1, j.w2};
    double gap = gaps_width(j.r1, j.r2, j.r4, g);
    uint32_t m = gaps_finish(j.la_hi, g, gap, j.r4_hi, Iv{j.R_lo, j.R_hi}) ? (1u << 5) : 0u;
    if (trap_status() != TRAP_NONE) m |= 1u << 31;
    return m;
}

CC_FN_INL uint32_t eval_all(const Box& in) {
    bool need_cover, need_gaps;
    CoverJob cj;
    GapsJob gj;
    uint32_t m = eval_main(in, need_cover, cj, need_gaps, gj);
    if (need_cover) m |= cover_pass(cj);
    if (need_gaps) m |= gaps_pass(gj);
    return m;
}

// The verdict mask of one box in FP64 alone, both bisections as the
// reference runs them (no FP32 step): the repair of a box one of whose
// FP64 certifications failed.
CC_FN_INL uint32_t eval_all_fp64(const Box& in) {
    bool need_cover, need_gaps;
    CoverJob cj;
    GapsJob gj;
    uint32_t m = eval_main(in, need_cover, cj, need_gaps, gj);
    if (need_cover) {
        trap_clear();
        const double width = cover_strip_width_fp64(cj.la_hi, cj.r1, cj.r2, cj.r3);
        if (cover_strip_finish(cj.la_hi, width, cj.ub_r4, cj.lb_R4)) m |= 1u << 2;
        if (trap_status() != TRAP_NONE) m |= 1u << 31;
    }
    if (need_gaps) {
        trap_clear();
        const GapsStart g{gj.w1, gj.w2};
        const double gap = gaps_width_fp64(gj.r1, gj.r2, gj.r4, g);
        if (gaps_finish(gj.la_hi, g, gap, gj.r4_hi, Iv{gj.R_lo, gj.R_hi})) m |= 1u << 5;
        if (trap_status() != TRAP_NONE) m |= 1u << 31;
    }
    return m;
}

#if CC_DEVICE_BUILD
// ------------------------------------------------ FP32-first evaluation
// eval_main on FP32 enclosures of the box (cc_f32.cuh): the same criteria,
// instantiated with IvF.  A box any of whose comparisons could not be decided
// goes to eval_main; for the others the bits equal eval_main's, and the FP64
// evaluation would not have trapped.
template <class S>
CC_FN bool gaps_enter_test(S r1, S r2) {
    S w1 = add_dn(mul_dn(4.0, r1), -1.0);
    S w2 = add_dn(mul_dn(4.0, r2), -1.0);
    return !(w1 <= 0.0 || w2 <= 0.0);
}

CC_FN_INL BoxT<f32::IvF> enclose(const Box& b) {
    return BoxT<f32::IvF>{f32::of(b.la), {f32::of(b.r[0]), f32::of(b.r[1]), f32::of(b.r[2]), f32::of(b.r[3])}};
}

// The FP32 evaluation is split into criterion groups, one kernel each: the
// whole of it does not fit the instruction cache.  eval_group_f32<G> returns
// the verdict bits of its group, the internal bits kF32Cover / kF32Gaps
// (the box needs the strip-width / gap-width bisection), or kF32Undecided.
enum : uint32_t { kF32Gaps = 1u << 28, kF32Cover = 1u << 29, kF32Undecided = 1u << 30 };
enum F32Group { F32_R1 = 0, F32_R12 = 1, F32_R123 = 2, F32_2X2 = 3, F32_LEAF = 4, F32_GROUPS = 5 };

// criterion G of the group kernels on the enclosed box (G != F32_R123)
template <int G>
CC_FN_INL bool group_criterion_f32(const BoxT<f32::IvF>& in, const f32::IvF& weight) {
    using f32::IvF;
    const IvF la = in.la, r1 = in.r[0], r2 = in.r[1], r3 = in.r[2];
    if (G == F32_R1) return r1_strategies(la, weight, r1, r2.hi);
    if (G == F32_R12) return r1_r2_strategies(la, weight, r1, r2, r3.hi);
    IvF R4 = weight - r1 - r2 - r3;
    tighten_lb(R4, 0.0);
    BoxT<IvF> v = in;
    tighten_lb(v.r[2], v.r[3].lo);
    tighten_lb(v.r[1], v.r[2].lo);
    tighten_lb(v.r[0], v.r[1].lo);
    IvF R = weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
    tighten_lb(R, 0.0);
    if (G == F32_2X2) return two_by_two_strategies(v, R);
    return r1_r2_r3_strategies(v, R4);
}

// State byte of a criterion evaluated with recorded calls: bits 0-1 the
// status; while pending, bits 2-4 the number of calls to evaluate and bits
// 5-6 the status if they all answer false (the criterion's own end).
enum : uint8_t { kRecPending = 0, kRecFalse = 1, kRecTrue = 2, kRecUndecided = 3 };

// The enclosed box and its required weight, computed once by the first FP32
// kernel for the record passes (96 bytes per box).
struct EncBox {
    BoxT<f32::IvF> b;
    f32::IvF weight;
};

// Criterion G in record mode; the calls to evaluate (those before the first
// one reached on an undecided path) go to args[0..).
template <int G>
CC_FN_INL uint8_t record_group_f32(const EncBox& in, CrArgs* __restrict__ args) {
    trap_clear();
    cc_cr_info[threadIdx.x] = 0;
    cc_trap_words[threadIdx.x] |= kTrapModeBit;
    const bool end_value = group_criterion_f32<G>(in.b, in.weight);
    const bool end_undecided = trap_status() != TRAP_NONE;
    trap_clear();
    const uint8_t info = cc_cr_info[threadIdx.x];
    const int m = info & 7;
    int calls = 0;
    while (calls < m && !(info & (8u << calls))) {
        args[calls] = cc_cr_rec[calls][threadIdx.x];
        ++calls;
    }
    const uint8_t end = (calls < m || end_undecided) ? kRecUndecided : (end_value ? kRecTrue : kRecFalse);
    if (calls == 0) return end;
    return (uint8_t)(kRecPending | (calls << 2) | (end << 5));
}

template <int G>
CC_FN_INL uint32_t eval_group_f32(const Box& in64, EncBox* keep = nullptr) {
    using f32::IvF;
    using f32::Fv;
    trap_clear();
    const BoxT<IvF> in = enclose(in64);
    const IvF la = in.la, r1 = in.r[0], r2 = in.r[1], r3 = in.r[2], r4 = in.r[3];
    const IvF weight = required_weight_for(la);
    // a weight whose computation met an undecided comparison need not enclose
    // the FP64 one: kept as NaN, so that every decision on it stays undecided
    if (keep) *keep = EncBox{in, trap_status() == TRAP_NONE ? weight : IvF{f32::nan_fv(), f32::nan_fv()}};
    uint32_t m = 0;
    if (G == F32_R1) {
        if (r1_strategies(la, weight, r1, r2.hi)) m |= 1u << 0;
    } else if (G == F32_R12) {
        if (r1_r2_strategies(la, weight, r1, r2, r3.hi)) m |= 1u << 1;
    } else {
        IvF R4 = weight - r1 - r2 - r3;
        tighten_lb(R4, 0.0);
        BoxT<IvF> v = in;
        tighten_lb(v.r[2], v.r[3].lo);
        tighten_lb(v.r[1], v.r[2].lo);
        tighten_lb(v.r[0], v.r[1].lo);
        IvF R = weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
        tighten_lb(R, 0.0);
        if (G == F32_R123) {
            if (r1_r2_r3_three_strips(la, weight, r1, r2, r3, r4.hi)) {
                m |= 1u << 2;
            } else if (strip_width_realizable<Fv>(r1.lo, r2.lo, r3.lo, 0.3)) {
                m |= kF32Cover;
            }
            if (gaps_enter_test<Fv>(v.r[0].lo, v.r[1].lo)) m |= kF32Gaps;
            if (empty(R4) || empty(R)) m |= 1u << 6;
        } else if (G == F32_2X2) {
            if (two_by_two_strategies(v, R)) m |= 1u << 3;
        } else {
            if (r1_r2_r3_strategies(v, R4)) m |= 1u << 4;
        }
    }
    return trap_status() == TRAP_NONE ? m : kF32Undecided;
}

// FP64 certification of a "true" that the FP32 pass decided for criterion
// group G (F32_R1, F32_R12, F32_2X2, F32_LEAF) at eval_main's arguments: the
// FP64 criterion with only call number `call` evaluated (1-based, the call
// whose FP32 answer settled the criterion; 0: none, the criterion held
// without one), or with all its calls for call < 0.  True if it holds
// without reaching a trap site.
// Record form (record, call > 0): the chosen call only stores its arguments
// (cc_cert_out) and answers "true"; *reached tells whether the run got to it.
// Then true with *reached means "certified if can_recurse_t holds on the
// stored arguments"; true without it, certified outright (the criterion held
// before that call, every earlier call answering "false").
template <int G>
CC_FN_INL bool certify_group(const Box& in, int call, bool record = false, bool* reached = nullptr) {
    const Iv la = in.la, r1 = in.r[0], r2 = in.r[1], r3 = in.r[2];
    const Iv weight = required_weight_for(la);
    record = record && call > 0;
    if (record) cert_record_begin(call);
    else if (call >= 0) cert_begin(call);
    else trap_clear();
    bool ok;
    if (G == F32_R1) {
        ok = r1_strategies(la, weight, r1, r2.hi);
    } else if (G == F32_R12) {
        ok = r1_r2_strategies(la, weight, r1, r2, r3.hi);
    } else {
        Iv R4 = weight - r1 - r2 - r3;
        tighten_lb(R4, 0.0);
        Box v = in;
        tighten_lb(v.r[2], v.r[3].lo);
        tighten_lb(v.r[1], v.r[2].lo);
        tighten_lb(v.r[0], v.r[1].lo);
        Iv R = weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
        tighten_lb(R, 0.0);
        ok = G == F32_2X2 ? two_by_two_strategies(v, R) : r1_r2_r3_strategies(v, R4);
    }
    const bool clean = trap_status() == TRAP_NONE;
    if (reached) *reached = record && cert_reached();
    cert_end();
    trap_clear();
    return ok && clean;
}

// FP64 certification of the bits the FP32 three-strip group decided "true":
// bit 2 by the three-strips placement (one call at most, evaluated in full),
// bit 6 (R or R4 empty).
CC_FN_INL bool certify_r123(const Box& in, uint32_t bits) {
    trap_clear();
    const Iv la = in.la, r1 = in.r[0], r2 = in.r[1], r3 = in.r[2], r4 = in.r[3];
    const Iv weight = required_weight_for(la);
    bool ok = true;
    if (bits & (1u << 2)) ok = r1_r2_r3_three_strips(la, weight, r1, r2, r3, r4.hi);
    if (ok && (bits & (1u << 6))) {
        Iv R4 = weight - r1 - r2 - r3;
        tighten_lb(R4, 0.0);
        Box v = in;
        tighten_lb(v.r[2], v.r[3].lo);
        tighten_lb(v.r[1], v.r[2].lo);
        tighten_lb(v.r[0], v.r[1].lo);
        Iv R = weight - v.r[0] - v.r[1] - v.r[2] - v.r[3];
        tighten_lb(R, 0.0);
        ok = empty(R4) || empty(R);
    }
    ok = ok && trap_status() == TRAP_NONE;
    trap_clear();
    return ok;
}

// A whole criterion on FP32 enclosures first: the same outcome and trap
// status as the FP64 criterion alone (a decided FP32 evaluation stands for an
// FP64 one that did not trap).  A decided "false" stands (the leaf goes on
// to the next criterion, as after an FP64 "false"); a decided "true" is
// certified by the FP64 criterion with only the call that settled the FP32
// run evaluated (cert_begin: the last call it made, or none); an undecided
// run, or a certification that fails (cert_failed), takes the FP64
// criterion's own result.  The caller's pending trap status is kept.
// *how (optional): 0 FP64 evaluation, 1 FP32 "false", 2 FP32 "true" certified
// in FP64, 3 certification failed.
template <class Crit>
CC_FN_INL bool first_f32(Crit crit, const Box& v, Iv rest, int* how = nullptr) {
    const uint32_t saved = trap_status();
    trap_clear();
    cert_count_reset();
    const bool ok32 = crit(enclose(v), f32::of(rest));
    const bool decided = trap_status() == TRAP_NONE;
    const int calls = cert_count();
    trap_clear();
    if (decided && ok32) {
        cert_begin(calls);
        const bool ok64 = crit(v, rest);
        const bool clean = trap_status() == TRAP_NONE;
        cert_end();
        trap_clear();
        if (saved != TRAP_NONE) trap(saved);
        if (ok64 && clean) {
            if (how) *how = 2;
            return true;
        }
        cert_failed();
        if (how) *how = 3;
        return crit(v, rest);
    }
    if (saved != TRAP_NONE) trap(saved);
    if (decided) {
        if (how) *how = 1;
        return false;
    }
    if (how) *how = 0;
    return crit(v, rest);
}
// first_f32 with the certification of a decided "true" left to the caller
// (the proof queues it for a certification pass): *how as first_f32 (2:
// FP32 "true", not yet certified), *calls = the number of the call that
// settled the FP32 run (its last call, if that call answered "true"; 0 if
// none did: the criterion then held with every call "false"), for
// certify_leaf.
template <class Crit>
CC_FN_INL bool first_f32_deferred(Crit crit, const Box& v, Iv rest, int* how, int* calls) {
    const uint32_t saved = trap_status();
    trap_clear();
    cert_count_reset();
    const bool ok32 = crit(enclose(v), f32::of(rest));
    const bool decided = trap_status() == TRAP_NONE;
    *calls = cert_last_true() ? cert_count() : 0;
    trap_clear();
    if (saved != TRAP_NONE) trap(saved);
    if (decided) {
        *how = ok32 ? 2 : 1;
        return ok32;
    }
    *how = 0;
    return crit(v, rest);
}
// The FP64 certification of a deferred "true": the criterion with only call
// number `call` evaluated; true if it holds without reaching a trap site.
// Record form (record, call > 0) as in certify_group: the chosen call only
// stores its arguments (cc_cert_out), *reached tells whether the run got to
// it, and the caller evaluates it afterwards (can_recurse_t).
template <class Crit>
CC_FN_INL bool certify_leaf(Crit crit, const Box& v, Iv rest, int call, bool record = false,
                            bool* reached = nullptr) {
    record = record && call > 0;
    if (record) cert_record_begin(call);
    else cert_begin(call);
    const bool ok = crit(v, rest);
    const bool clean = trap_status() == TRAP_NONE;
    if (reached) *reached = record && cert_reached();
    cert_end();
    trap_clear();
    return ok && clean;
}
struct TwoByTwo {
    template <class I>
    CC_METHOD bool operator()(const BoxT<I>& v, I R) const { return two_by_two_strategies(v, R); }
};
struct LeafR123 {
    template <class I>
    CC_METHOD bool operator()(const BoxT<I>& v, I R4) const { return r1_r2_r3_strategies(v, R4); }
};
// two_by_two_strategies(v, R) and r1_r2_r3_strategies(v, R4), FP32 first
CC_FN_INL bool two_by_two_first_f32(const Box& v, Iv R, int* how = nullptr) {
    return first_f32(TwoByTwo{}, v, R, how);
}
CC_FN_INL bool r1_r2_r3_leaf_first_f32(const Box& v, Iv R4, int* how = nullptr) {
    return first_f32(LeafR123{}, v, R4, how);
}

// The two bisection criteria of one box, from the box itself (the queues
// hold box indices): the bisection in FP64 (with its FP32 shortcuts), then
// the recursion check first on FP32 enclosures and, if that is undecided, in
// FP64.  Same result and trap bit as cover_pass / gaps_pass on eval_main's
// jobs.
// A true result gets an FP64 certificate, the argument the reference's
// criterion makes with the width its bisection reaches: the strip of the
// width used is realizable and the rest of the rectangle can be covered
// recursively (r1_r2_r3_strategies.cu:77-93), resp. the gap of the width used
// is 0 or can be closed by disk 4 and the rest covered
// (r1_r2_large_r3_r4_gaps_strategy.cu:73-97) -- both in FP64.  If it fails
// (*repair), the caller recomputes the box in FP64 alone (eval_all_fp64).
// (enc: the box's enclosure and weight if the FP32 pass kept them)
CC_FN_INL bool cover_certificate(const Box& b, double width) {
    trap_clear();
    const Iv la = b.la, r1 = b.r[0], r2 = b.r[1], r3 = b.r[2];
    bool ok = strip_width_realizable(r1.lo, r2.lo, r3.lo, width) &&
              cover_strip_finish<double>(la.hi, width, b.r[3].hi, (required_weight_for(la) - r1 - r2 - r3).lo);
    ok = ok && trap_status() == TRAP_NONE;
    trap_clear();
    return ok;
}
CC_FN_INL bool gaps_certificate(const Box& b, double gap) {
    trap_clear();
    Box v = b;
    tighten_lb(v.r[2], v.r[3].lo);
    tighten_lb(v.r[1], v.r[2].lo);
    tighten_lb(v.r[0], v.r[1].lo);
    GapsStart g;
    bool ok = gaps_enters(v.r[0].lo, v.r[1].lo, g);
    if (ok && gap != 0.0) ok = gap_width_realizable(gap, v.r[0].lo, g.w1, v.r[1].lo, g.w2, v.r[3].lo);
    if (ok) {
        Iv R = required_weight_for(v.la) - v.r[0] - v.r[1] - v.r[2] - v.r[3];
        tighten_lb(R, 0.0);
        ok = gaps_finish(b.la.hi, g, gap, v.r[3].hi, R);
    }
    ok = ok && trap_status() == TRAP_NONE;
    trap_clear();
    return ok;
}

// FP32 bound of R4 for the strip's final check (from the kept enclosure if
// there is one); *lb_ok: no comparison on the way was undecided
CC_FN_INL f32::Fv cover_lb_R4(const Box& b, const EncBox* enc, bool* lb_ok) {
    trap_clear();
    const f32::Fv lb_R4 = enc ? (enc->weight - enc->b.r[0] - enc->b.r[1] - enc->b.r[2]).lo : [&] {
        const BoxT<f32::IvF> e = enclose(b);
        return (required_weight_for(e.la) - e.r[0] - e.r[1] - e.r[2]).lo;
    }();
    *lb_ok = trap_status() == TRAP_NONE;
    trap_clear();
    return lb_R4;
}
// the strip's final check on the bisection's width, with its certificate
CC_FN_INL uint32_t cover_pass_tail(const Box& b, bool lb_ok, f32::Fv lb_R4, double width, bool certify, bool* repair) {
    uint32_t trapped = trap_status();
    trap_clear();
    bool ok = lb_ok ? cover_strip_finish<f32::Fv>(b.la.hi, width, b.r[3].hi, lb_R4) : false;
    if (!lb_ok || trap_status() != TRAP_NONE) {
        trap_clear();
        ok = cover_strip_finish<double>(b.la.hi, width, b.r[3].hi,
                                        (required_weight_for(b.la) - b.r[0] - b.r[1] - b.r[2]).lo);
        trapped |= trap_status();
    }
    uint32_t m = ok ? (1u << 2) : 0u;
    if (trapped != TRAP_NONE) m |= 1u << 31;
    else if (ok && certify && !cover_certificate(b, width)) *repair = true;
    return m;
}
// resume (optional): a box whose bisection reaches its FP64 steps stops
// there: resume->it >= 0 holds the state (the caller sets resume->box) and
// 0 is returned; cover_pass_resume computes it later (the same result)
CC_FN_INL uint32_t cover_pass_box(const Box& b, const EncBox* enc = nullptr, bool certify = false,
                                  bool* repair = nullptr, CoverResume* resume = nullptr) {
    using f32::Fv;
    const Iv la = b.la, r1 = b.r[0], r2 = b.r[1], r3 = b.r[2];
    bool lb_ok;
    const Fv lb_R4 = cover_lb_R4(b, enc, &lb_ok);
    if (resume) resume->it = -1;
    // cover_strip_finish for every width in [lo, hi]
    auto finish = [&](double lo, double hi) -> int {
        if (!lb_ok) return f32::UNKNOWN;
        bool ok = cover_strip_finish<Fv>(la.hi, f32::hull(lo, hi), b.r[3].hi, lb_R4);
        int d = trap_status() == TRAP_NONE ? (ok ? f32::YES : f32::NO) : f32::UNKNOWN;
        trap_clear();  // no trap can be pending where this is asked
        return d;
    };
    int decided;
    const double width = cover_strip_width_early(la.hi, r1.lo, r2.lo, r3.lo, finish, &decided, resume);
    if (decided == kBisectionDeferred) return 0u;
    if (decided != f32::UNKNOWN) {
        if (decided != f32::YES) return 0u;
        if (certify && !cover_certificate(b, width)) *repair = true;
        return 1u << 2;
    }
    return cover_pass_tail(b, lb_ok, lb_R4, width, certify, repair);
}
CC_FN_INL uint32_t cover_pass_resume(const Box& b, const EncBox* enc, bool certify, bool* repair,
                                     const CoverResume& r) {
    bool lb_ok;
    const f32::Fv lb_R4 = cover_lb_R4(b, enc, &lb_ok);
    const double width = cover_strip_width_resume(b.r[0].lo, b.r[1].lo, b.r[2].lo, r.lo, r.hi, r.it);
    return cover_pass_tail(b, lb_ok, lb_R4, width, certify, repair);
}

CC_FN_INL uint32_t gaps_pass_box(const Box& b, const EncBox* enc = nullptr, bool certify = false,
                                 bool* repair = nullptr) {
    using f32::Fv;
    trap_clear();
    Box v = b;
    tighten_lb(v.r[2], v.r[3].lo);
    tighten_lb(v.r[1], v.r[2].lo);
    tighten_lb(v.r[0], v.r[1].lo);
    GapsStart g;
    if (!gaps_enters(v.r[0].lo, v.r[1].lo, g)) {
        return 0u;
    }
    f32::IvF R;
    if (enc) {  // the same tightening on the kept enclosure encloses v
        BoxT<f32::IvF> e = enc->b;
        tighten_lb(e.r[2], e.r[3].lo);
        tighten_lb(e.r[1], e.r[2].lo);
        tighten_lb(e.r[0], e.r[1].lo);
        R = enc->weight - e.r[0] - e.r[1] - e.r[2] - e.r[3];
    } else {
        BoxT<f32::IvF> e = enclose(v);
        R = required_weight_for(e.la) - e.r[0] - e.r[1] - e.r[2] - e.r[3];
    }
    tighten_lb(R, 0.0);
    const bool R_ok = trap_status() == TRAP_NONE;
    trap_clear();
    // gaps_finish for every gap width in [lo, hi]
    auto finish = [&](double lo, double hi) -> int {
        if (!R_ok) return f32::UNKNOWN;
        bool ok = gaps_finish_t<Fv>(b.la.hi, g.w1, g.w2, f32::hull(lo, hi), v.r[3].hi,
                                    R.lo, R.hi);
        int d = trap_status() == TRAP_NONE ? (ok ? f32::YES : f32::NO) : f32::UNKNOWN;
        trap_clear();  // no trap can be pending where this is asked
        return d;
    };
    int decided;
    const double gap = gaps_width_early(v.r[0].lo, v.r[1].lo, v.r[3].lo, g, finish, &decided);
    if (decided != f32::UNKNOWN) {
        if (decided != f32::YES) return 0u;
        if (certify && !gaps_certificate(b, gap)) *repair = true;
        return 1u << 5;
    }
    uint32_t trapped = trap_status();
    trap_clear();
    bool ok = R_ok ? gaps_finish_t<Fv>(b.la.hi, g.w1, g.w2, gap, v.r[3].hi, R.lo, R.hi) : false;
    if (!R_ok || trap_status() != TRAP_NONE) {
        trap_clear();
        Iv R64 = required_weight_for(v.la) - v.r[0] - v.r[1] - v.r[2] - v.r[3];
        tighten_lb(R64, 0.0);
        ok = gaps_finish(b.la.hi, g, gap, v.r[3].hi, R64);
        trapped |= trap_status();
    }
    uint32_t m = ok ? (1u << 5) : 0u;
    if (trapped != TRAP_NONE) m |= 1u << 31;
    else if (ok && certify && !gaps_certificate(b, gap)) *repair = true;
    return m;
}
#endif

// ------------------------------------------------ prepared (hoisted) forms
// In the proof's nested grid a criterion is evaluated for every cell of the
// next radius with only that radius' upper bound changing: r1_strategies(la,
// r1, r2.hi) for every r2 cell, r1_r2_strategies(la, r1, r2, r3.hi) for every
// r3 cell, r1_r2_r3_strategies(la, r1, r2, r3, r4.hi) for every r4 leaf
// (tight_rectangle.cu:195, 210, 231).  Everything that does not depend on that
// bound -- including the cover-strip bisection -- is computed once per parent
// cell ("prepare"); the per-cell "check" redoes only the operations that
// involve the bound.  check(prepare(x), ub) performs the same directed-rounding
// operations on the same values as the criterion itself, so the verdicts are
// identical for every ub.

// can_recurse(w, h, ub_largest, lb_weight) for fixed w, h (can_recurse.cu:32-62)
struct CrPrep {
    double area, s_sq, ratio_wh;
};
CC_FN CrPrep cr_prepare(double ub_w, double ub_h) {
    CrPrep p;
    p.area = mul_up(ub_w, ub_h);
    double side_min = ub_w < ub_h ? ub_w : ub_h;
    double s = rcp_up(side_min);
    p.s_sq = mul_up(s, s);
    p.ratio_wh = critical_ratio(ivp(ub_w), ivp(ub_h)).hi;
    return p;
}
CC_FN bool cr_check(const CrPrep& p, double ub_largest, double lb_weight) {
    double largest_norm = mul_up(p.s_sq, ub_largest);
    double ratio;
    if (largest_norm <= sb::kUbDiskWeight) {
        ratio = sb::kCriticalRatio;
    } else {
        ratio = p.ratio_wh;
        double ratio_cor = mul_up(0.5, sqrt_up(add_up(sqrt_up(add_up(mul_up(largest_norm, largest_norm), 1.0)), 1.0)));
        if (ratio_cor < 195.0 / 256) {
            ratio_cor = 195.0 / 256;
        }
        if (ratio > ratio_cor) {
            ratio = ratio_cor;
        }
    }
    return lb_weight >= mul_up(ratio, p.area);
}

// r1_strategies(la, r1, ub_r2) for fixed la, r1 (r1_strategies.cu:27-87)
struct R1Prep {
    double lb_rem;
    CrPrep strip;                    // block 1: strip of disk 1
    double min_right, w_sb, w_rec;   // block 2: disk 1 in a corner
    CrPrep corner;
    CrPrep pocket;                   // block 3: uneven split
    uint8_t has_strip, has_corner, has_pocket;
};
CC_FN R1Prep r1_prepare(Iv la, Iv weight, Iv r1) {
    R1Prep p;
    double square_w = sqrt_dn(mul_dn(2.0, r1.lo));
    double strip_w = add_dn(mul_dn(4.0, r1.lo), -1.0);
    p.lb_rem = (weight - r1).lo;
    p.has_strip = strip_w > 0.0;
    if (p.has_strip) {
        strip_w = sqrt_dn(strip_w);
        p.strip = cr_prepare((la - strip_w).hi, 1.0);
    }
    p.has_corner = square_w < 1.0;
    if (p.has_corner) {
        double w_right = add_up(la.hi, -square_w);
        p.min_right = w_right < 1.0 ? w_right : 1.0;
        p.w_sb = mul_up(w_right, sb::kCriticalRatio);
        p.w_rec = required_weight_for(ivp(w_right), ivp(1.0)).hi;
        p.corner = cr_prepare(square_w, add_up(1.0, -square_w));
    }
    p.has_pocket = 0;
    double lb_S1 = add_dn(mul_dn(4.0, r1.lo), -1.0);
    if (lb_S1 > 0.0) {
        lb_S1 = sqrt_dn(lb_S1);
        double t = add_up(la.hi, -mul_dn(0.5, lb_S1));
        t = mul_up(t, t);
        double lb_h1 = add_dn(r1.lo, -t);
        if (lb_h1 > 0.0) {
            lb_h1 = mul_dn(2.0, sqrt_dn(lb_h1));
            p.pocket = cr_prepare(add_up(la.hi, -lb_S1), mul_up(0.5, add_up(1.0, -lb_h1)));
            p.has_pocket = 1;
        }
    }
    return p;
}
CC_FN bool r1_check(const R1Prep& p, double ub_r2) {
    if (p.has_strip && cr_check(p.strip, ub_r2, p.lb_rem)) {
        return true;
    }
    if (p.has_corner) {
        double w = sb::disk_satisfies_size_bound(ub_r2, p.min_right) ? p.w_sb : p.w_rec;
        w = add_up(w, ub_r2);
        double left = add_dn(p.lb_rem, -w);
        if (left > 0 && cr_check(p.corner, ub_r2, left)) {
            return true;
        }
    }
    if (p.has_pocket) {
        double half = mul_dn(0.5, add_dn(p.lb_rem, -ub_r2));
        if (half > 0 && cr_check(p.pocket, ub_r2, half)) {
            return true;
        }
    }
    return false;
}

// r1_r2_strategies(la, r1, r2, ub_r3) for fixed la, r1, r2 (r1_r2_strategies.cu:29-133)
struct R12Prep {
    double lb_R3;
    CrPrep side;                      // side by side: 0 fails, 1 holds, 2 recursion check
    double top_min, bot_min, need_top_sb, need_bot_sb, need_top_rec;
    CrPrep bot, top;                  // stacked: (w_bot x sq_side), (w_top x h_top)
    uint8_t side_state, stacked;
};
CC_FN R12Prep r12_prepare(Iv la, Iv weight, Iv r1, Iv r2) {
    R12Prep p;
    p.lb_R3 = (weight - r1 - r2).lo;
    p.side_state = 2;
    if (two_pocket_by_hand(la, r1, r2)) {
        p.side_state = 1;
    } else {
        double lb_width = sb::two_disks_maximize_height(r1, r2, 1.0);
        if (lb_width <= 0.0) {
            p.side_state = 0;
        } else {
            double lb_w2 = add_dn(mul_dn(4.0, r2.lo), -1.0);
            if (lb_w2 > 0.0) {
                lb_w2 = sqrt_dn(lb_w2);
                double lb_w1 = sqrt_dn(add_dn(mul_dn(4.0, r1.lo), -1.0));
                double lb_w = add_dn(lb_w1, lb_w2);
                if (lb_w > lb_width) {
                    lb_width = lb_w;
                    if (lb_w > la.hi) p.side_state = 1;
                }
            }
            if (p.side_state == 2) p.side = cr_prepare(add_dn(la.hi, lb_width), 1.0);  // sic: '+' (parity)
        }
    }
    if (p.side_state == 1) {
        p.stacked = 0;
        return p;
    }
    p.stacked = 0;
    double sq_side = sqrt_dn(mul_dn(2.0, r1.lo));
    if (sq_side > 1.0) return p;
    double h_top = add_up(1.0, -sq_side);
    double lb_w2 = add_dn(mul_dn(4.0, r2.lo), -mul_up(h_top, h_top));
    if (lb_w2 < 0.0) return p;
    lb_w2 = sqrt_dn(lb_w2);
    double w_top = add_up(la.hi, -lb_w2);
    double w_bot = add_up(la.hi, -sq_side);
    p.top_min = w_top < h_top ? w_top : h_top;
    p.bot_min = w_bot < sq_side ? w_bot : sq_side;
    p.need_top_sb = required_weight_for_bounded_size(w_top, h_top);
    p.need_bot_sb = required_weight_for_bounded_size(w_bot, sq_side);
    p.need_top_rec = required_weight_for(ivp(w_top), ivp(h_top)).hi;
    p.bot = cr_prepare(w_bot, sq_side);
    p.top = cr_prepare(w_top, h_top);
    p.stacked = 1;
    return p;
}
CC_FN bool r12_check(const R12Prep& p, double ub_r3) {
    if (p.side_state == 1) return true;
    if (p.side_state == 2 && cr_check(p.side, ub_r3, p.lb_R3)) return true;
    if (!p.stacked) return false;
    if (sb::disk_satisfies_size_bound(ub_r3, p.top_min)) {
        double left = add_dn(p.lb_R3, -add_up(p.need_top_sb, ub_r3));
        return left > 0.0 && cr_check(p.bot, ub_r3, left);
    }
    if (sb::disk_satisfies_size_bound(ub_r3, p.bot_min)) {
        double left = add_dn(p.lb_R3, -add_up(p.need_bot_sb, ub_r3));
        return left > 0.0 && cr_check(p.top, ub_r3, left);
    }
    double left = add_dn(p.lb_R3, -add_up(p.need_top_rec, ub_r3));
    return left > 0.0 && cr_check(p.bot, ub_r3, left);
}

// r1_r2_r3_strategies(la, r1, r2, r3, ub_r4) for fixed la, r1..r3
// (r1_r2_r3_strategies.cu:28-99); holds the cover-strip bisection result
struct R123Prep {
    double lb_R4;
    CrPrep strips, cover;
    uint8_t strips_state;  // 0 fails, 1 holds, 2 recursion check
    uint8_t has_cover;
    uint8_t trapped;       // the bisection hit its iteration cap
};
CC_FN R123Prep r123_prepare(Iv la, Iv weight, Iv r1, Iv r2, Iv r3) {
    R123Prep p;
    p.lb_R4 = (weight - r1 - r2 - r3).lo;
    p.has_cover = 0;
    p.trapped = 0;
    double lb_w3 = add_dn(mul_dn(4.0, r3.lo), -1.0);
    if (lb_w3 <= 0.0) {
        p.strips_state = 0;
    } else {
        lb_w3 = sqrt_dn(lb_w3);
        double lb_w2 = sqrt_dn(add_dn(mul_dn(4.0, r2.lo), -1.0));
        double lb_w1 = sqrt_dn(add_dn(mul_dn(4.0, r1.lo), -1.0));
        double lb_cov = add_dn(lb_w1, add_dn(lb_w2, lb_w3));
        double ub_rem = add_up(la.hi, -lb_cov);
        if (ub_rem <= 0.0) {
            p.strips_state = 1;
            return p;
        }
        p.strips_state = 2;
        p.strips = cr_prepare(ub_rem, 1.0);
    }
    if (cover_strip_enters(r1.lo, r2.lo, r3.lo)) {
        uint32_t saved = trap_status();
        trap_clear();
        double width = cover_strip_width(la.hi, r1.lo, r2.lo, r3.lo);
        p.trapped = trap_status() != TRAP_NONE;
        if (saved != TRAP_NONE) trap(saved);
        p.cover = cr_prepare(add_up(la.hi, -width), 1.0);
        p.has_cover = 1;
    }
    return p;
}
CC_FN bool r123_check(const R123Prep& p, double ub_r4) {
    if (p.trapped) trap(TRAP_BISECTION_CAP);
    if (p.strips_state == 1) return true;
    if (p.strips_state == 2 && cr_check(p.strips, ub_r4, p.lb_R4)) return true;
    return p.has_cover && cr_check(p.cover, ub_r4, p.lb_R4);
}

// The leaf form r1_r2_r3_strategies(box, R4) for a fixed la, r1..r3 and R4
// as a function of the upper bound of r4 (r1_r2_r3_strategies.cu:101-247):
// the three placements up to their recursion checks, the checks' rectangles
// (cr_prepare) and the pocket settled by hand, computed once.  The trap
// status each placement leaves is replayed when the check gets there, so
// leaf123_check(p, ub_r4) performs the criterion's operations on the same
// values: the same result and trap status as r1_r2_r3_strategies(b, R4)
// with b.r[3].hi = ub_r4.  The proof prepares it per r3 cell, for the
// leaves whose r4 lower bound does not tighten r3 (their tightened r1..r3
// are the cell's own).
struct LeafPrep {
    CrPrep cr[3];
    double lb_R4;
    uint8_t st[3];    // big strip, small corner, r1-r3 pocket: 0 fails, 1 holds, 2 recursion check
    uint8_t trap[4];  // trap status after each placement and after the pocket by hand (0: none)
    uint8_t hand;     // three_disk_pocket_by_hand
};
CC_FN LeafPrep leaf123_prepare(const Box& b, Iv R4) {
    LeafPrep p;
    const uint32_t saved = trap_status();
    trap_clear();
    p.lb_R4 = R4.lo;
    const double ub_la = b.la.hi, r1 = b.r[0].lo, r2 = b.r[1].lo, r3 = b.r[2].lo;
    double w = 0.0, h = 0.0;
    for (int k = 0; k < 3; ++k) {
        const int st = k == 0   ? three_disk_big_strip_wh<double>(ub_la, r1, r2, r3, w, h)
                       : k == 1 ? three_disk_small_corner_wh<double>(ub_la, r1, r2, r3, w, h)
                                : three_disk_r1_r3_pocket_wh(b.la, b.r[0], b.r[1], b.r[2], w, h);
        p.st[k] = (uint8_t)st;
        if (st == 2) p.cr[k] = cr_prepare(w, h);
        p.trap[k] = (uint8_t)trap_status();
        trap_clear();
    }
    p.hand = three_disk_pocket_by_hand(b.la, b.r[0], b.r[1], b.r[2]) ? 1 : 0;
    p.trap[3] = (uint8_t)trap_status();
    trap_clear();
    if (saved != TRAP_NONE) trap(saved);
    return p;
}
CC_FN bool leaf123_check(const LeafPrep& p, double ub_r4) {
    for (int k = 0; k < 3; ++k) {
        if (p.trap[k]) trap(p.trap[k]);
        if (p.st[k] == 1 || (p.st[k] == 2 && cr_check(p.cr[k], ub_r4, p.lb_R4))) return true;
    }
    if (p.trap[3]) trap(p.trap[3]);
    return p.hand != 0;
}

// criteria with the reference's signatures (weight computed inside)
CC_FN_INL bool r1_strategies(Iv la, Iv r1, double ub_r2) { return r1_strategies(la, required_weight_for(la), r1, ub_r2); }
CC_FN_INL bool r1_r2_strategies(Iv la, Iv r1, Iv r2, double ub_r3) {
    return r1_r2_strategies(la, required_weight_for(la), r1, r2, ub_r3);
}
CC_FN_INL bool r1_r2_r3_strategies(Iv la, Iv r1, Iv r2, Iv r3, double ub_r4) {
    return r1_r2_r3_strategies(la, required_weight_for(la), r1, r2, r3, ub_r4);
}

}  // namespace tight
}  // namespace cc

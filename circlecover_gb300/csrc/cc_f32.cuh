// FP32 enclosures of FP64 interval computations (device only).
//
// A bisection criterion evaluates an FP64 predicate dozens of times, and on
// GB300 FP64 instructions cost 64x the FP32 ones.  Far from the bisection's
// fixpoint the predicate's outcome is insensitive to rounding, so it is first
// decided with FP32 intervals that enclose every FP64 value the predicate
// computes; only when that is inconclusive does the FP64 predicate run.
//
// Why a decided FP32 outcome equals the FP64 one.  Every FP64 quantity of the
// predicate is r(f(x, y, ...)), with r rounding down or up (or, for the
// reference's `Iv * scalar`, down where up was meant) and x, y, ... FP64
// quantities computed before.  If x, y, ... lie in the FP32 intervals X, Y,
// ..., then f(x, y, ...) lies in the exact image f(X, Y, ...), and the FP32
// operation below returns [rd32(min f), ru32(max f)] over that image, the
// extremes being taken at the interval corners (f is monotone in each
// argument on the domains used).  A float is also a double, so rd32(v) <=
// rd64(v) <= v <= ru64(v) <= ru32(v): the FP64 value lies in the FP32
// interval again.  By induction every FP64 endpoint lies in the FP32
// interval of the same quantity, and a comparison whose outcome is the same
// for every point of the FP32 intervals has that outcome in FP64 too.
// Inconclusive comparisons, NaNs (every comparison with NaN is false) and
// divisors whose enclosure reaches zero make the FP32 evaluation give up.
//
// The intrinsics are IEEE correctly rounded in the direction named
// (__fadd_rd, __fmul_ru, __fdiv_rd, __fsqrt_ru, __double2float_rd, ...),
// denormals included (the library is built without -ftz); doubles are
// rounded to floats by round_to_floats below.
#pragma once

#include "cc_iv.cuh"

#if CC_DEVICE_BUILD
namespace cc {
namespace f32 {

struct Fv {
    float lo, hi;
    Fv() = default;
    __device__ __forceinline__ Fv(float l, float h) : lo(l), hi(h) {}
    // enclosure of a double (a double that is a float gives {x, x})
    __device__ __forceinline__ Fv(double x);
};

// The double rounded down and up to floats, by integer operations on its
// bits: GB300 runs the conversion instructions on its FP64 unit, at the
// FP64 rate.  For 2^-126 <= |x| < 2^128 (biased exponent 897..1150) the
// float with x's sign, exponent (rebased from 1023 to 127) and leading 23
// mantissa bits is x rounded toward zero, and the next float bit pattern
// away from zero is x rounded away from zero when a discarded mantissa bit
// is set (a mantissa carry moves into the exponent, past the largest float
// to infinity, as rounding does).  Zeros keep their sign.  Other values
// (results below the normal floats, infinities, NaN) take the directed
// conversions.  Plain shifts and bit casts only, so that the compiler folds
// the conversion of a constant.
__device__ __forceinline__ void round_to_floats(double x, float& dn, float& up) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(bits >> 32), lo = (unsigned)bits;
    const unsigned s = hi & 0x80000000u;
    if ((bits << 1) == 0ull) {
        dn = up = __uint_as_float(s);
        return;
    }
    const unsigned e = (hi >> 20) & 0x7ffu;
    if (e - 897u <= 253u) {
        const unsigned mag = (((hi & 0x7fffffffu) - (896u << 20)) << 3) | (lo >> 29);
        const unsigned away = mag + ((lo & 0x1fffffffu) != 0u ? 1u : 0u);
        dn = __uint_as_float(s | (s ? away : mag));
        up = __uint_as_float(s | (s ? mag : away));
        return;
    }
    dn = __double2float_rd(x);
    up = __double2float_ru(x);
}
__device__ __forceinline__ float round_dn(double x) {
    float d, u;
    round_to_floats(x, d, u);
    return d;
}
__device__ __forceinline__ float round_up(double x) {
    float d, u;
    round_to_floats(x, d, u);
    return u;
}

__device__ __forceinline__ Fv::Fv(double x) { round_to_floats(x, lo, hi); }

// enclosure of a double
__device__ __forceinline__ Fv of(double x) { return Fv(x); }
// enclosure of the doubles between lo and hi
__device__ __forceinline__ Fv hull(double lo, double hi) { return Fv{round_dn(lo), round_up(hi)}; }
__device__ __forceinline__ Fv point(float x) { return Fv{x, x}; }
__device__ __forceinline__ float qnan() { return __int_as_float(0x7fffffff); }
__device__ __forceinline__ Fv nan_fv() { return Fv{qnan(), qnan()}; }

// minimum / maximum that return NaN if either operand is NaN (PTX min.NaN)
__device__ __forceinline__ float fmin_nan(float a, float b) {
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float fmax_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ Fv add(Fv a, Fv b) { return Fv{__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)}; }
__device__ __forceinline__ Fv sub(Fv a, Fv b) { return Fv{__fadd_rd(a.lo, -b.hi), __fadd_ru(a.hi, -b.lo)}; }

// Product of two enclosures: the extremes of the four corner products.
// Non-negative operands (the common case) inline; the rest out of line, so
// that the evaluation's code stays small.
__device__ __noinline__ inline Fv mul_mixed(Fv a, Fv b) {
    float p1 = __fmul_rd(a.lo, b.lo), p2 = __fmul_rd(a.lo, b.hi);
    float p3 = __fmul_rd(a.hi, b.lo), p4 = __fmul_rd(a.hi, b.hi);
    float q1 = __fmul_ru(a.lo, b.lo), q2 = __fmul_ru(a.lo, b.hi);
    float q3 = __fmul_ru(a.hi, b.lo), q4 = __fmul_ru(a.hi, b.hi);
    return Fv{fmin_nan(fmin_nan(p1, p2), fmin_nan(p3, p4)), fmax_nan(fmax_nan(q1, q2), fmax_nan(q3, q4))};
}
__device__ __forceinline__ Fv mul(Fv a, Fv b) {
    if (a.lo >= 0.0f && b.lo >= 0.0f) return Fv{__fmul_rd(a.lo, b.lo), __fmul_ru(a.hi, b.hi)};
    return mul_mixed(a, b);
}
// product with a non-negative float constant
__device__ __forceinline__ Fv scale(Fv a, float c) { return Fv{__fmul_rd(a.lo, c), __fmul_ru(a.hi, c)}; }

// square of an enclosure (through |a|); NaN in, NaN out
__device__ __noinline__ inline Fv sqr_mixed(Fv a) {
    if (a.hi <= 0.0f) return Fv{__fmul_rd(a.hi, a.hi), __fmul_ru(a.lo, a.lo)};
    if (a.lo < 0.0f && a.hi > 0.0f) {
        float m = fmax_nan(-a.lo, a.hi);
        return Fv{0.0f, __fmul_ru(m, m)};
    }
    return nan_fv();
}
__device__ __forceinline__ Fv sqr(Fv a) {
    if (a.lo >= 0.0f) return Fv{__fmul_rd(a.lo, a.lo), __fmul_ru(a.hi, a.hi)};
    return sqr_mixed(a);
}

// Reciprocal and square root through the round-to-nearest operations
// (IEEE: within half an ulp, 2^-24 relative, for normal results), widened by
// one ulp in the outward direction: rd(rn(1/x) * (1 - 2^-23)) <= 1/x <=
// ru(rn(1/x) * (1 + 2^-23)).  Arguments outside the range where the results
// are normal take the exactly rounded directed operations, out of line.
static constexpr float kUlpDn = 0x1.fffffcp-1f;  // 1 - 2^-23
static constexpr float kUlpUp = 0x1.000002p+0f;  // 1 + 2^-23

// quotient by a positive enclosure (callers check d.lo > 0 first)
__device__ __noinline__ inline Fv div_pos_exact(Fv a, Fv d) {
    float l = a.lo >= 0.0f ? __fdiv_rd(a.lo, d.hi) : __fdiv_rd(a.lo, d.lo);
    float u = a.hi >= 0.0f ? __fdiv_ru(a.hi, d.lo) : __fdiv_ru(a.hi, d.hi);
    return Fv{l, u};
}
__device__ __forceinline__ Fv div_pos(Fv a, Fv d) {
    if (a.lo >= 0.0f && d.lo >= 0x1p-125f && d.hi <= 0x1p125f) {
        const float r_lo = __fmul_rd(__frcp_rn(d.hi), kUlpDn);  // <= 1/d.hi
        const float r_hi = __fmul_ru(__frcp_rn(d.lo), kUlpUp);  // >= 1/d.lo
        return Fv{__fmul_rd(a.lo, r_lo), __fmul_ru(a.hi, r_hi)};
    }
    return div_pos_exact(a, d);
}

// square root of a non-negative enclosure (callers check a.lo >= 0 first)
__device__ __noinline__ inline Fv sqrt_nn_exact(Fv a) { return Fv{__fsqrt_rd(a.lo), __fsqrt_ru(a.hi)}; }
__device__ __forceinline__ Fv sqrt_nn(Fv a) {
    if (a.lo >= 0x1p-120f) return Fv{__fmul_rd(__fsqrt_rn(a.lo), kUlpDn), __fmul_ru(__fsqrt_rn(a.hi), kUlpUp)};
    return sqrt_nn_exact(a);
}

// three-valued outcome of an FP32 decision
enum : int { UNKNOWN = -1, NO = 0, YES = 1 };

// ------------------------------------------------------------------------
// Enclosure arithmetic for whole criteria.  The criteria are templates over
// their interval type: Iv (FP64, the product's arithmetic) or IvF below
// (FP32 enclosures of the Iv values, with Fv in place of double).  In the
// IvF instantiation every FP64 operation becomes the enclosure of its
// result, and every comparison either has the same outcome for all points of
// its enclosures -- then it is the FP64 comparison's outcome -- or it marks
// the evaluation undecided (the per-thread status word, TRAP_F32_UNDECIDED)
// and answers arbitrarily; the caller discards the result of an undecided
// evaluation.  An FP64 trap site reached by the FP64 evaluation is reached
// by the FP32 one too (its comparisons follow the FP64 branches) and marks it
// undecided, so a decided FP32 evaluation stands for an FP64 evaluation that
// did not trap.  Minima and maxima written as selections in the FP64 code
// (`a < b ? a : b`) are lesser()/greater(), whose enclosures need no decision.

__device__ __forceinline__ void undecided() { trap(TRAP_F32_UNDECIDED); }

// the scalar primitives of cc_base.cuh on enclosures (both roundings of an
// FP64 result lie in the enclosure of the exact result)
__device__ __forceinline__ Fv add_dn(Fv a, Fv b) { return add(a, b); }
__device__ __forceinline__ Fv add_up(Fv a, Fv b) { return add(a, b); }
__device__ __forceinline__ Fv mul_dn(Fv a, Fv b) { return mul(a, b); }
__device__ __forceinline__ Fv mul_up(Fv a, Fv b) { return mul(a, b); }
__device__ __forceinline__ Fv operator-(Fv a) { return Fv{-a.hi, -a.lo}; }

// quotient of enclosures; a divisor enclosure that reaches zero (or a NaN)
// leaves the FP64 quotient unknown
__device__ __forceinline__ Fv quot(Fv a, Fv d) {
    if (d.lo > 0.0f) return div_pos(a, d);
    if (d.hi < 0.0f) return div_pos(-a, -d);
    undecided();
    return nan_fv();
}
__device__ __forceinline__ Fv div_dn(Fv a, Fv b) { return quot(a, b); }
__device__ __forceinline__ Fv div_up(Fv a, Fv b) { return quot(a, b); }
__device__ __forceinline__ Fv rcp_dn(Fv a) { return quot(Fv{1.0f, 1.0f}, a); }
__device__ __forceinline__ Fv rcp_up(Fv a) { return quot(Fv{1.0f, 1.0f}, a); }

// square root: an enclosure reaching below zero leaves the FP64 root (a
// number or NaN) unknown; one entirely below zero gives NaN, as FP64 does
__device__ __forceinline__ Fv root(Fv a) {
    if (a.lo >= 0.0f) return sqrt_nn(a);
    if (!(a.hi < 0.0f)) undecided();
    return nan_fv();
}
__device__ __forceinline__ Fv sqrt_dn(Fv a) { return root(a); }
__device__ __forceinline__ Fv sqrt_up(Fv a) { return root(a); }

// comparisons: the FP64 outcome, or undecided.  An enclosure has lo <= hi
// unless it holds a NaN; any NaN leaves the comparison undecided.
__device__ __forceinline__ bool decide(bool certainly_true, bool certainly_false) {
    if (!certainly_true && !certainly_false) undecided();
    return certainly_true;
}
__device__ __forceinline__ bool operator<(Fv a, Fv b) {
    const bool ok = a.lo <= a.hi && b.lo <= b.hi;
    return decide(ok && a.hi < b.lo, ok && a.lo >= b.hi);
}
__device__ __forceinline__ bool operator<=(Fv a, Fv b) {
    const bool ok = a.lo <= a.hi && b.lo <= b.hi;
    return decide(ok && a.hi <= b.lo, ok && a.lo > b.hi);
}
__device__ __forceinline__ bool operator>(Fv a, Fv b) { return b < a; }
__device__ __forceinline__ bool operator>=(Fv a, Fv b) { return b <= a; }

// lesser(a, b) = a < b ? a : b and greater(a, b) = a > b ? a : b of FP64
// values: the enclosure of the minimum / maximum (NaN in, NaN out)
__device__ __forceinline__ Fv lesser(Fv a, Fv b) { return Fv{fmin_nan(a.lo, b.lo), fmin_nan(a.hi, b.hi)}; }
__device__ __forceinline__ Fv greater(Fv a, Fv b) { return Fv{fmax_nan(a.lo, b.lo), fmax_nan(a.hi, b.hi)}; }

// enclosure of an FP64 interval: lo and hi each enclosed
struct IvF {
    using S = Fv;
    Fv lo, hi;
};

__device__ __forceinline__ IvF ivp(Fv v) { return IvF{v, v}; }
__device__ __forceinline__ IvF of(Iv v) { return IvF{of(v.lo), of(v.hi)}; }

__device__ __forceinline__ IvF operator+(IvF a, IvF b) { return IvF{add(a.lo, b.lo), add(a.hi, b.hi)}; }
__device__ __forceinline__ IvF operator+(IvF a, Fv n) { return IvF{add(a.lo, n), add(a.hi, n)}; }
__device__ __forceinline__ IvF operator+(Fv n, IvF a) { return IvF{add(a.lo, n), add(a.hi, n)}; }
__device__ __forceinline__ IvF operator-(IvF a, IvF b) { return IvF{sub(a.lo, b.hi), sub(a.hi, b.lo)}; }
__device__ __forceinline__ IvF operator-(IvF a, Fv n) { return IvF{sub(a.lo, n), sub(a.hi, n)}; }
__device__ __forceinline__ IvF operator-(Fv n, IvF b) { return IvF{sub(n, b.hi), sub(n, b.lo)}; }
__device__ __forceinline__ IvF operator-(IvF a) { return IvF{-a.hi, -a.lo}; }

// Iv * Iv is the minimum of the four products rounded down and the maximum
// of the four rounded up, empty intervals included (interval.cuh:171-182).
// If all four endpoints are non-negative, the minimum (maximum) product is
// the product of the smaller (larger) endpoints.
__device__ __noinline__ inline IvF mul_iv_mixed(IvF a, IvF b) {
    const Fv p1 = mul(a.lo, b.lo), p2 = mul(a.lo, b.hi), p3 = mul(a.hi, b.lo), p4 = mul(a.hi, b.hi);
    return IvF{lesser(lesser(p1, p2), lesser(p3, p4)), greater(greater(p1, p2), greater(p3, p4))};
}
__device__ __forceinline__ IvF operator*(IvF a, IvF b) {
    if (a.lo.lo >= 0.0f && a.hi.lo >= 0.0f && b.lo.lo >= 0.0f && b.hi.lo >= 0.0f) {
        const Fv amin = lesser(a.lo, a.hi), amax = greater(a.lo, a.hi);
        const Fv bmin = lesser(b.lo, b.hi), bmax = greater(b.lo, b.hi);
        return IvF{Fv{__fmul_rd(amin.lo, bmin.lo), __fmul_ru(amin.hi, bmin.hi)},
                   Fv{__fmul_rd(amax.lo, bmax.lo), __fmul_ru(amax.hi, bmax.hi)}};
    }
    return mul_iv_mixed(a, b);
}
// Iv * scalar (interval.cuh:185-197): the branch on the scalar's sign
__device__ __forceinline__ IvF operator*(IvF a, Fv n) {
    if (n >= Fv{0.0f, 0.0f}) return IvF{mul(a.lo, n), mul(a.hi, n)};
    return IvF{mul(a.hi, n), mul(a.lo, n)};
}
__device__ __forceinline__ IvF operator*(Fv n, IvF a) { return a * n; }

__device__ __forceinline__ IvF operator/(IvF a, Fv n) {
    if (n > Fv{0.0f, 0.0f}) return IvF{quot(a.lo, n), quot(a.hi, n)};
    return IvF{quot(a.hi, n), quot(a.lo, n)};
}
__device__ __forceinline__ IvF operator/(IvF a, IvF o) {
    const Fv z{0.0f, 0.0f};
    if (o.lo > z) {
        if (a.lo >= z) return IvF{quot(a.lo, o.hi), quot(a.hi, o.lo)};
        if (a.hi <= z) return IvF{quot(a.lo, o.lo), quot(a.hi, o.hi)};
        return IvF{quot(a.lo, o.lo), quot(a.hi, o.lo)};
    }
    if (o.hi < z) {
        if (a.lo >= z) return IvF{quot(a.hi, o.hi), quot(a.lo, o.lo)};
        if (a.hi <= z) return IvF{quot(a.hi, o.lo), quot(a.lo, o.hi)};
        return IvF{quot(a.hi, o.hi), quot(a.lo, o.hi)};
    }
    const float inf = __int_as_float(0x7f800000);
    return IvF{Fv{-inf, -inf}, Fv{inf, inf}};
}
__device__ __forceinline__ IvF operator/(Fv n, IvF o) { return ivp(n) / o; }

__device__ __forceinline__ IvF reciprocal(IvF a) {
    const Fv z{0.0f, 0.0f}, one{1.0f, 1.0f};
    if (a.lo > z) return IvF{quot(one, a.hi), quot(one, a.lo)};
    if (a.hi < z) return IvF{quot(one, a.lo), quot(one, a.hi)};
    const float inf = __int_as_float(0x7f800000);
    return IvF{Fv{-inf, -inf}, Fv{inf, inf}};
}

// interval.cuh iv_abs, with its selections as enclosures
__device__ __forceinline__ IvF iv_abs(IvF a) {
    const Fv z{0.0f, 0.0f};
    Fv l = z, u = z;
    if (a.hi > z) {
        u = a.hi;
    } else {
        l = -a.hi;
    }
    if (a.lo < z) {
        u = greater(-a.lo, u);
    } else {
        l = a.lo;
    }
    return IvF{l, u};
}
__device__ __forceinline__ IvF square(IvF a) {
    IvF m = iv_abs(a);
    return IvF{mul(m.lo, m.lo), mul(m.hi, m.hi)};
}
// Interval::sqrt traps for lb < 0: that case is undecided here
__device__ __forceinline__ IvF sqrt(IvF a) {
    if (a.lo < Fv{0.0f, 0.0f}) undecided();
    return IvF{root(a.lo), root(a.hi)};
}

// Uncertain<bool> of an IvF comparison, its two components decided only when
// read: the FP64 code often reads one of them (definitely / possibly), and
// the other may be undecidable without mattering
struct UbF {
    Fv l1, r1, l2, r2;  // component k: lk < rk (strict) or lk <= rk
    bool strict;
};
__device__ __forceinline__ bool ub_part(Fv l, Fv r, bool strict) { return strict ? l < r : l <= r; }
__device__ __forceinline__ bool definitely(UbF b) { return ub_part(b.l1, b.r1, b.strict); }
__device__ __forceinline__ bool possibly(UbF b) { return ub_part(b.l2, b.r2, b.strict); }
__device__ __forceinline__ bool definitely_not(UbF b) { return !possibly(b); }
__device__ __forceinline__ bool possibly_not(UbF b) { return !definitely(b); }
__device__ __forceinline__ bool is_certain(UbF b) { return definitely(b) == possibly(b); }

// the comparisons of cc_iv.cuh, component for component
__device__ __forceinline__ UbF operator<(IvF a, Fv n) { return UbF{a.hi, n, a.lo, n, true}; }
__device__ __forceinline__ UbF operator>(IvF a, Fv n) { return UbF{n, a.lo, n, a.hi, true}; }
__device__ __forceinline__ UbF operator<=(IvF a, Fv n) { return UbF{a.hi, n, a.lo, n, false}; }
__device__ __forceinline__ UbF operator>=(IvF a, Fv n) { return UbF{n, a.lo, n, a.hi, false}; }
__device__ __forceinline__ UbF operator<(IvF a, IvF b) { return UbF{a.hi, b.lo, a.lo, b.hi, true}; }
__device__ __forceinline__ UbF operator<=(IvF a, IvF b) { return UbF{a.hi, b.lo, a.lo, b.hi, false}; }
__device__ __forceinline__ UbF operator>(IvF a, IvF b) { return b < a; }
__device__ __forceinline__ UbF operator>=(IvF a, IvF b) { return b <= a; }

// FP64 `x <= 0 ? 0 : sqrt_dn(x)` for x in the enclosure a: 0, the root, or
// either of them when the sign of x is not certain
__device__ __forceinline__ Fv clipped_root(Fv a) {
    if (a.hi <= 0.0f) return Fv{0.0f, 0.0f};
    if (a.lo > 0.0f) return sqrt_nn(a);
    if (!(a.lo <= a.hi)) return nan_fv();
    return Fv{0.0f, __fsqrt_ru(a.hi)};
}

// The reference's bisection to the FP64 fixpoint from 0 <= lo < hi: mid =
// 0.5 * (lo + hi) while strictly inside the bracket, `pred(mid)` true raises
// lo, a trap after CC_BISECTION_CAP steps; the result is lo.  Run with the
// FP32 shortcuts of the tight bisections (cc_tight.cuh, bisect_all_true):
// `dec(W)` decides the predicate for every point of the enclosure W (YES,
// NO, UNKNOWN) -- first for the whole bracket (false everywhere: the result
// is lo, and a finite bracket reaches its fixpoint in fewer than 2,100
// steps, so the cap cannot trap; true everywhere: the steps are replayed),
// then for the leading steps while every converged lane of the warp has a
// decision; from the first step some lane cannot decide, the FP64 predicate.
// The result gets an FP64 certificate: a lower end that an FP32 decision
// raised must pass the FP64 predicate, as every lower end of the
// reference's bracket does (the initial one, or a midpoint the predicate
// accepted).  If it does not, the bisection is redone on the FP64 predicate
// alone (cert_failed).
template <class Pred>
__device__ __forceinline__ double bisect_fp64(double lo, double hi, const Pred& pred) {
    for (int it = 0;; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) return lo;
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            return lo;
        }
        if (pred(mid)) lo = mid;
        else hi = mid;
    }
}
template <class Dec, class Pred>
__device__ __forceinline__ double bisect_steps(double lo, double hi, const Dec& dec, const Pred& pred,
                                               bool& lo_by_f32) {
    int it = 0;
    lo_by_f32 = false;
    if (lo >= 0.0 && lo < hi && hi <= 1.7976931348623157e308) {
        const int whole = dec(hull(lo, hi));
        if (whole == NO) return lo;
        if (whole == YES) {
            for (;; ++it) {
                const double mid = 0.5 * (lo + hi);
                if (mid <= lo || mid >= hi) return lo;
                if (it >= CC_BISECTION_CAP) {
                    trap(TRAP_BISECTION_CAP);
                    return lo;
                }
                lo = mid;
                lo_by_f32 = true;
            }
        }
    }
    bool f32_steps = true;
    for (;; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) return lo;
        if (it >= CC_BISECTION_CAP) {
            trap(TRAP_BISECTION_CAP);
            return lo;
        }
        bool ok, by_f32;
        const int d = f32_steps ? dec(of(mid)) : UNKNOWN;
        if (f32_steps && __all_sync(__activemask(), d != UNKNOWN)) {
            ok = d == YES;
            by_f32 = true;
        } else {
            f32_steps = false;
            ok = pred(mid);
            by_f32 = false;
        }
        if (ok) {
            lo = mid;
            lo_by_f32 = by_f32;
        } else {
            hi = mid;
        }
    }
}
template <class Dec, class Pred>
__device__ __forceinline__ double bisect(double lo, double hi, const Dec& dec, const Pred& pred) {
    const double lo0 = lo, hi0 = hi;
    bool by_f32;
    const double r = bisect_steps(lo, hi, dec, pred, by_f32);
    if (!by_f32) return r;
    const uint32_t saved = trap_status();
    trap_clear();
    const bool ok = pred(r) && trap_status() == TRAP_NONE;
    trap_clear();
    if (saved != TRAP_NONE) trap(saved);
    if (ok) return r;
    cert_failed();
    return bisect_fp64(lo0, hi0, pred);
}

// The same bisection on FP32 decisions alone, for callers that can go on
// with an enclosure of its result: the steps run while every one is decided
// (they are then the FP64 steps); the exact result if the fixpoint is
// reached that way, else the FP32 enclosure of the bracket at the first
// undecided step, which holds the FP64 result.  For 0 <= lo and a finite hi
// the FP64 bisection ends in fewer than 2,100 steps, so its cap cannot trap;
// other brackets mark the evaluation undecided.
template <class Dec>
__device__ __forceinline__ Fv bisect_enclosure(double lo, double hi, const Dec& dec) {
    if (!(lo >= 0.0 && hi <= 1.7976931348623157e308)) {
        undecided();
        return nan_fv();
    }
    if (!(lo < hi)) return of(lo);  // the first midpoint is not above lo
    const int whole = dec(hull(lo, hi));
    if (whole == NO) return of(lo);
    for (int it = 0; it < CC_BISECTION_CAP; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) return of(lo);
        const int d = whole == YES ? YES : dec(of(mid));
        if (d == UNKNOWN) return hull(lo, hi);
        if (d == YES) lo = mid;
        else hi = mid;
    }
    undecided();
    return nan_fv();
}

// FP64 `a == b`: decided when both are the same point or the enclosures are
// disjoint
__device__ __forceinline__ bool operator==(Fv a, Fv b) {
    const bool ok = a.lo <= a.hi && b.lo <= b.hi;
    return decide(ok && a.lo == a.hi && b.lo == b.hi && a.lo == b.lo, ok && (a.hi < b.lo || b.hi < a.lo));
}

__device__ __forceinline__ void tighten_lb(IvF& a, Fv l) { a.lo = greater(l, a.lo); }
__device__ __forceinline__ void tighten_ub(IvF& a, Fv u) { a.hi = lesser(u, a.hi); }
__device__ __forceinline__ bool empty(IvF a) { return a.lo > a.hi; }

}  // namespace f32
}  // namespace cc
#endif

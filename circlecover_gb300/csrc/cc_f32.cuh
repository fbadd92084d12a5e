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
// denormals included (the library is built without -ftz).
#pragma once

#include "cc_base.cuh"

#if CC_DEVICE_BUILD
namespace cc {
namespace f32 {

struct Fv {
    float lo, hi;
};

// enclosure of a double
__device__ __forceinline__ Fv of(double x) { return Fv{__double2float_rd(x), __double2float_ru(x)}; }
__device__ __forceinline__ Fv point(float x) { return Fv{x, x}; }

__device__ __forceinline__ Fv add(Fv a, Fv b) { return Fv{__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)}; }
__device__ __forceinline__ Fv sub(Fv a, Fv b) { return Fv{__fadd_rd(a.lo, -b.hi), __fadd_ru(a.hi, -b.lo)}; }

// product of two enclosures: the extremes of the four corner products.  A
// NaN corner (infinity times zero) makes the whole product NaN, so that no
// bound is taken from the remaining corners alone.
__device__ __forceinline__ Fv mul(Fv a, Fv b) {
    if (a.lo >= 0.0f && b.lo >= 0.0f) return Fv{__fmul_rd(a.lo, b.lo), __fmul_ru(a.hi, b.hi)};
    float p1 = __fmul_rd(a.lo, b.lo), p2 = __fmul_rd(a.lo, b.hi);
    float p3 = __fmul_rd(a.hi, b.lo), p4 = __fmul_rd(a.hi, b.hi);
    float q1 = __fmul_ru(a.lo, b.lo), q2 = __fmul_ru(a.lo, b.hi);
    float q3 = __fmul_ru(a.hi, b.lo), q4 = __fmul_ru(a.hi, b.hi);
    if (isnan(p1) || isnan(p2) || isnan(p3) || isnan(p4)) return Fv{__int_as_float(0x7fffffff), __int_as_float(0x7fffffff)};
    return Fv{fminf(fminf(p1, p2), fminf(p3, p4)), fmaxf(fmaxf(q1, q2), fmaxf(q3, q4))};
}
// product with a non-negative float constant
__device__ __forceinline__ Fv scale(Fv a, float c) { return Fv{__fmul_rd(a.lo, c), __fmul_ru(a.hi, c)}; }

// square of an enclosure (through |a|); NaN in, NaN out
__device__ __forceinline__ Fv sqr(Fv a) {
    if (a.lo >= 0.0f) return Fv{__fmul_rd(a.lo, a.lo), __fmul_ru(a.hi, a.hi)};
    if (a.hi <= 0.0f) return Fv{__fmul_rd(a.hi, a.hi), __fmul_ru(a.lo, a.lo)};
    if (a.lo < 0.0f && a.hi > 0.0f) {
        float m = fmaxf(-a.lo, a.hi);
        return Fv{0.0f, __fmul_ru(m, m)};
    }
    return Fv{__int_as_float(0x7fffffff), __int_as_float(0x7fffffff)};
}

// quotient by a positive enclosure (callers check d.lo > 0 first)
__device__ __forceinline__ Fv div_pos(Fv a, Fv d) {
    float l = a.lo >= 0.0f ? __fdiv_rd(a.lo, d.hi) : __fdiv_rd(a.lo, d.lo);
    float u = a.hi >= 0.0f ? __fdiv_ru(a.hi, d.lo) : __fdiv_ru(a.hi, d.hi);
    return Fv{l, u};
}

// square root of a non-negative enclosure (callers check a.lo >= 0 first)
__device__ __forceinline__ Fv sqrt_nn(Fv a) { return Fv{__fsqrt_rd(a.lo), __fsqrt_ru(a.hi)}; }

// three-valued outcome of an FP32 decision
enum : int { UNKNOWN = -1, NO = 0, YES = 1 };

}  // namespace f32
}  // namespace cc
#endif

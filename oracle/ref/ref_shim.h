/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Force-included (g++ -include) in front of every reference criteria source
 * when the oracle builds the reference's own code for the host CPU
 * (oracle/ref/Makefile).  It supplies what nvcc would otherwise provide:
 *
 *  - the CUDA FP64 directed-rounding intrinsics the reference calls
 *    (__dadd_rd ... __drcp_ru), implemented exactly on the CPU by
 *    oracle/shim/cc_rounding.h, each one counted (one algorithmic op);
 *  - the FP32 intrinsics referenced by the reference's Interval<float>
 *    specialisations (interval.cuh:30-36 and others; never called by the
 *    criteria), implemented with fesetround;
 *  - algcuda::trap() (reference: algcuda/cuda-utils/cuh/include/algcuda/
 *    exit.cuh:28-31).  On the GPU it kills the context; here it records a
 *    per-box "trapped" status and longjmps back to the box evaluator;
 *  - printf, redirected so that the reference's device printf on an
 *    unresolved seven-disk box (rectangle_size_bound/seven_disk_strategies.cu:
 *    1478-1490) is counted per box rather than written to stdout.
 *
 * macros.hpp (algcuda/cuda-utils/cpp/include/algcuda/macros.hpp:26-40) turns
 * __device__/__host__/__global__ into nothing when __CUDACC__ is undefined,
 * which is what lets the unmodified sources compile as plain C++.
 */
#ifndef CC_ORACLE_REF_SHIM_H
#define CC_ORACLE_REF_SHIM_H

#include <cstdio>
#include <cstdarg>
#include <csetjmp>
#include <cmath>
#include <cfloat>
#include "../shim/cc_rounding.h"

/* skip the reference's exit.cuh; its trap() is replaced below */
#define ALGCUDA_UTILS_EXIT_CUH_INCLUDED_

namespace algcuda {
[[noreturn]] void trap() noexcept;
inline void exit() noexcept {}
}
#define ALGCUDA_ASSERT(expr) ((void)0)

extern "C" int cc_ref_printf(const char* fmt, ...);
#define printf cc_ref_printf

/* CC_REF_FENV selects the fesetround implementation of every operation (the
 * slow exact form; libccref_fe.so, for timing only); the default is the
 * error-free-transform form */
#ifdef CC_REF_FENV
#define CC_REF_ROUND(op) cc_fe_##op
static inline double cc_fe_rcp_rd(double a) { return cc_fe_div_rd(1.0, a); }
static inline double cc_fe_rcp_ru(double a) { return cc_fe_div_ru(1.0, a); }
#else
#define CC_REF_ROUND(op) cc_sw_##op
#endif
static inline double __dadd_rd(double a, double b) { CC_SHIM_TICK(); return CC_REF_ROUND(add_rd)(a, b); }
static inline double __dadd_ru(double a, double b) { CC_SHIM_TICK(); return CC_REF_ROUND(add_ru)(a, b); }
static inline double __dmul_rd(double a, double b) { CC_SHIM_TICK(); return CC_REF_ROUND(mul_rd)(a, b); }
static inline double __dmul_ru(double a, double b) { CC_SHIM_TICK(); return CC_REF_ROUND(mul_ru)(a, b); }
static inline double __ddiv_rd(double a, double b) { CC_SHIM_TICK(); return CC_REF_ROUND(div_rd)(a, b); }
static inline double __ddiv_ru(double a, double b) { CC_SHIM_TICK(); return CC_REF_ROUND(div_ru)(a, b); }
static inline double __dsqrt_rd(double a) { CC_SHIM_TICK(); return CC_REF_ROUND(sqrt_rd)(a); }
static inline double __dsqrt_ru(double a) { CC_SHIM_TICK(); return CC_REF_ROUND(sqrt_ru)(a); }
static inline double __drcp_rd(double a) { CC_SHIM_TICK(); return CC_REF_ROUND(rcp_rd)(a); }
static inline double __drcp_ru(double a) { CC_SHIM_TICK(); return CC_REF_ROUND(rcp_ru)(a); }

#define CC_REF_F32(name, mode, expr)                                          \
    static inline float name(float a, float b) {                             \
        int old = fegetround();                                               \
        fesetround(mode);                                                     \
        volatile float va = a, vb = b;                                        \
        volatile float r = (expr);                                            \
        fesetround(old);                                                      \
        return r;                                                             \
    }
CC_REF_F32(__fadd_rd, FE_DOWNWARD, va + vb)
CC_REF_F32(__fadd_ru, FE_UPWARD, va + vb)
CC_REF_F32(__fmul_rd, FE_DOWNWARD, va * vb)
CC_REF_F32(__fmul_ru, FE_UPWARD, va * vb)
CC_REF_F32(__fdiv_rd, FE_DOWNWARD, va / vb)
CC_REF_F32(__fdiv_ru, FE_UPWARD, va / vb)
#undef CC_REF_F32
static inline float __frcp_rd(float a) { return __fdiv_rd(1.0f, a); }
static inline float __frcp_ru(float a) { return __fdiv_ru(1.0f, a); }
static inline float __fsqrt_rd(float a) {
    int old = fegetround(); fesetround(FE_DOWNWARD);
    volatile float va = a; volatile float r = sqrtf(va);
    fesetround(old); return r;
}
static inline float __fsqrt_ru(float a) {
    int old = fegetround(); fesetround(FE_UPWARD);
    volatile float va = a; volatile float r = sqrtf(va);
    fesetround(old); return r;
}

/*
 * get_subinterval (reference: subintervals.hpp:33-43) computes `lb + diff*i`
 * as a plain expression.  nvcc contracts it into one FMA by default
 * (-fmad=true) in device code, and g++ does the same in the host driver when
 * the target has FMA (the reference builds with -march=native,
 * cmake/util.cmake:111).  The shim pre-empts that header and spells the FMA
 * out, so that the oracle reproduces the contracted form on every host.
 */
#define SUBINTERVALS_HPP_INCLUDED_
#include <algcuda/interval.hpp>
namespace circlecover {
template <typename NumType>
inline algcuda::Interval<NumType> get_subinterval(algcuda::Interval<NumType> interval, int i, int n) {
    double lb = interval.get_lb();
    double ub = interval.get_ub();
    double diff = ub - lb;
    diff /= n;
    double l = std::fma(diff, (double)i, lb);
    double u = std::fma(diff, (double)(i + 1), lb);
    if (i + 1 == n) u = ub;
    return {l, u};
}
}  // namespace circlecover

#endif

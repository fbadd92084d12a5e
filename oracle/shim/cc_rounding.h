/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Host (CPU) implementation of IEEE-754 binary64 arithmetic with directed
 * rounding: add, mul, div, sqrt and reciprocal, each rounded toward -inf
 * ("rd") or +inf ("ru").  These are the exact semantics of the CUDA
 * intrinsics __dadd_rd/__dadd_ru, __dmul_rd/__dmul_ru, __ddiv_rd/__ddiv_ru,
 * __dsqrt_rd/__dsqrt_ru and __drcp_rd/__drcp_ru that the reference's
 * interval type is built on (algcuda/cuda-utils/cuh/include/algcuda/
 * interval.cuh:30-355; every criterion file calls them directly as well).
 *
 * Two implementations:
 *  - cc_fe_*: switch the FPU rounding mode with fesetround() around one
 *    operation.  Exact by definition of IEEE-754, slow (two mode switches).
 *  - cc_sw_*: round-to-nearest result corrected by the sign of its exact
 *    error, obtained with error-free transformations (Knuth TwoSum for add,
 *    FMA residual for mul, exact FMA remainder for div and sqrt; see Boldo &
 *    Muller, "Exact and approximated error of the FMA", IEEE TC 2011).  Where
 *    a residual might itself not be exact (operands or results near the
 *    underflow threshold, infinities, zeros, NaN) it falls back to cc_fe_*.
 *
 * The tests check cc_sw_* against cc_fe_* on random and special operands on
 * the CPU, and against the CUDA intrinsics on the GPU.
 *
 * Compile every user of this file with -frounding-math -ffp-contract=off and
 * without -ffast-math.
 */
#ifndef CC_ORACLE_ROUNDING_H
#define CC_ORACLE_ROUNDING_H

#include <fenv.h>
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <string.h>

#ifdef __cplusplus
#define CC_SHIM_INLINE static inline
#else
#define CC_SHIM_INLINE static inline
#endif

/* ---------------------------------------------------------------- fesetround */

#define CC_FE_BINOP(name, mode, expr)                                         \
    CC_SHIM_INLINE double name(double a, double b) {                          \
        int old = fegetround();                                                \
        fesetround(mode);                                                      \
        volatile double va = a, vb = b;                                        \
        volatile double r = (expr);                                            \
        fesetround(old);                                                       \
        return r;                                                              \
    }

CC_FE_BINOP(cc_fe_add_rd, FE_DOWNWARD, va + vb)
CC_FE_BINOP(cc_fe_add_ru, FE_UPWARD, va + vb)
CC_FE_BINOP(cc_fe_mul_rd, FE_DOWNWARD, va * vb)
CC_FE_BINOP(cc_fe_mul_ru, FE_UPWARD, va * vb)
CC_FE_BINOP(cc_fe_div_rd, FE_DOWNWARD, va / vb)
CC_FE_BINOP(cc_fe_div_ru, FE_UPWARD, va / vb)
#undef CC_FE_BINOP

CC_SHIM_INLINE double cc_fe_sqrt_rd(double a) {
    int old = fegetround();
    fesetround(FE_DOWNWARD);
    volatile double va = a;
    volatile double r = sqrt(va);
    fesetround(old);
    return r;
}
CC_SHIM_INLINE double cc_fe_sqrt_ru(double a) {
    int old = fegetround();
    fesetround(FE_UPWARD);
    volatile double va = a;
    volatile double r = sqrt(va);
    fesetround(old);
    return r;
}

/* ------------------------------------------------------ error-free transforms */

/* next representable double toward -inf / +inf of a finite nonzero x */
CC_SHIM_INLINE double cc_next_down(double x) { return nextafter(x, -INFINITY); }
CC_SHIM_INLINE double cc_next_up(double x) { return nextafter(x, INFINITY); }

/* |x| below this: residuals of products/quotients may underflow -> use fenv */
#define CC_SW_TINY 0x1p-900
/* |x| above this: quotient/product correction may overflow -> use fenv */
#define CC_SW_HUGE 0x1p+1000

CC_SHIM_INLINE double cc_sw_add_rd(double a, double b) {
    double s = a + b;
    if (!isfinite(s) || s == 0.0) return cc_fe_add_rd(a, b);
    double bb = s - a;
    double err = (a - (s - bb)) + (b - bb);
    return err < 0.0 ? cc_next_down(s) : s;
}
CC_SHIM_INLINE double cc_sw_add_ru(double a, double b) {
    double s = a + b;
    if (!isfinite(s) || s == 0.0) return cc_fe_add_ru(a, b);
    double bb = s - a;
    double err = (a - (s - bb)) + (b - bb);
    return err > 0.0 ? cc_next_up(s) : s;
}

CC_SHIM_INLINE int cc_sw_mul_safe(double a, double b, double p) {
    double ap = fabs(p);
    return isfinite(p) && ap > CC_SW_TINY && ap < CC_SW_HUGE && a != 0.0 && b != 0.0;
}
CC_SHIM_INLINE double cc_sw_mul_rd(double a, double b) {
    double p = a * b;
    if (!cc_sw_mul_safe(a, b, p)) return cc_fe_mul_rd(a, b);
    double err = fma(a, b, -p);
    return err < 0.0 ? cc_next_down(p) : p;
}
CC_SHIM_INLINE double cc_sw_mul_ru(double a, double b) {
    double p = a * b;
    if (!cc_sw_mul_safe(a, b, p)) return cc_fe_mul_ru(a, b);
    double err = fma(a, b, -p);
    return err > 0.0 ? cc_next_up(p) : p;
}

CC_SHIM_INLINE int cc_sw_div_safe(double a, double b, double q) {
    double aq = fabs(q), aa = fabs(a), ab = fabs(b);
    return isfinite(q) && aq > CC_SW_TINY && aq < CC_SW_HUGE && aa > CC_SW_TINY &&
           aa < CC_SW_HUGE && ab > CC_SW_TINY && ab < CC_SW_HUGE;
}
/* remainder r = a - q*b is exact; exact quotient - q has the sign of r/b */
CC_SHIM_INLINE double cc_sw_div_rd(double a, double b) {
    double q = a / b;
    if (!cc_sw_div_safe(a, b, q)) return cc_fe_div_rd(a, b);
    double r = fma(-q, b, a);
    if (r == 0.0) return q;
    int below = (r < 0.0) != (b < 0.0); /* exact quotient < q */
    return below ? cc_next_down(q) : q;
}
CC_SHIM_INLINE double cc_sw_div_ru(double a, double b) {
    double q = a / b;
    if (!cc_sw_div_safe(a, b, q)) return cc_fe_div_ru(a, b);
    double r = fma(-q, b, a);
    if (r == 0.0) return q;
    int above = (r < 0.0) == (b < 0.0); /* exact quotient > q */
    return above ? cc_next_up(q) : q;
}

CC_SHIM_INLINE double cc_sw_sqrt_rd(double a) {
    if (!(a > CC_SW_TINY && a < CC_SW_HUGE)) return cc_fe_sqrt_rd(a);
    double s = sqrt(a);
    double r = fma(-s, s, a); /* exact: a - s^2 */
    return r < 0.0 ? cc_next_down(s) : s;
}
CC_SHIM_INLINE double cc_sw_sqrt_ru(double a) {
    if (!(a > CC_SW_TINY && a < CC_SW_HUGE)) return cc_fe_sqrt_ru(a);
    double s = sqrt(a);
    double r = fma(-s, s, a);
    return r > 0.0 ? cc_next_up(s) : s;
}

CC_SHIM_INLINE double cc_sw_rcp_rd(double a) { return cc_sw_div_rd(1.0, a); }
CC_SHIM_INLINE double cc_sw_rcp_ru(double a) { return cc_sw_div_ru(1.0, a); }

/* ------------------------------------------------------------- op counters */
/*
 * Counting mode (CC_SHIM_COUNT defined): every primitive call increments a
 * thread-local counter.  The count per box is the algorithmic work unit of
 * the roofline (one FP64 directed-rounding primitive = 1 op).
 */
#ifdef __cplusplus
/* Thread-local state of the host builds.  Initial-exec TLS makes every access
 * a plain thread-pointer-relative load.  With the default model for
 * shared libraries (TLS descriptors), the port loaded into Python crashed on
 * an aarch64 host (GCC 13, glibc) inside a worker thread's TLS accesses;
 * with initial-exec it runs and agrees bit for bit. */
#ifndef CC_HOST_TLS
#define CC_HOST_TLS thread_local __attribute__((tls_model("initial-exec")))
#endif
#endif

#ifdef CC_SHIM_COUNT
#ifdef __cplusplus
extern CC_HOST_TLS unsigned long long cc_shim_op_count;
#else
extern _Thread_local unsigned long long cc_shim_op_count;
#endif
#define CC_SHIM_TICK() (++cc_shim_op_count)
#else
#define CC_SHIM_TICK() ((void)0)
#endif

#endif /* CC_ORACLE_ROUNDING_H */

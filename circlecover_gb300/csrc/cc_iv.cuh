// Outward-rounded FP64 interval arithmetic and three-valued comparisons.
//
// Semantics follow the reference's algcuda::Interval<double> and
// algcuda::Uncertain<bool> operation for operation, because every verdict and
// every critical box has to come out bit-identical:
//   reference: algcuda/cuda-utils/cpp/include/algcuda/interval.hpp:32-242
//              algcuda/cuda-utils/cuh/include/algcuda/interval.cuh:30-355
// In particular (each one is a parity requirement, not a design choice):
//   * Iv * scalar with scalar >= 0 rounds BOTH bounds down
//     (interval.cuh:185-197);
//   * Iv * Iv takes min/max over the 8 directed products with the `a < b ? a
//     : b` chain of interval.cuh:171-182, which fixes how NaN and signed
//     zeros resolve;
//   * division and reciprocal return (-inf, +inf) when the divisor contains 0
//     (interval.cuh:227-235, 249-292);
//   * sqrt of an interval with lb < 0 traps (interval.cuh:339-346); here it
//     records a trap status for the box instead (cc_base.cuh).
// The struct layout {lo, hi} equals the reference's {lb, ub}.
#pragma once

#include "cc_base.cuh"

namespace cc {

struct Iv {
    using S = double;  // scalar type of the bounds (criteria are templates over Iv and its FP32 enclosure)
    double lo, hi;
};

// Uncertain<bool>: lo = "definitely true", hi = "possibly true"
// (interval.hpp:32-82).
struct Ub {
    bool lo, hi;
};

CC_FN bool definitely(Ub b) { return b.lo; }
CC_FN bool possibly(Ub b) { return b.hi; }
CC_FN bool definitely_not(Ub b) { return !b.hi; }
CC_FN bool possibly_not(Ub b) { return !b.lo; }
CC_FN bool is_certain(Ub b) { return b.lo == b.hi; }
CC_FN Ub operator!(Ub b) { return Ub{!b.hi, !b.lo}; }

CC_FN Iv ivp(double v) { return Iv{v, v}; }
CC_FN Iv ivr(double l, double u) { return Iv{l, u}; }

// ------------------------------------------------------------- + and -
CC_FN Iv operator+(Iv a, Iv b) { return Iv{add_dn(a.lo, b.lo), add_up(a.hi, b.hi)}; }
CC_FN Iv operator+(Iv a, double n) { return Iv{add_dn(a.lo, n), add_up(a.hi, n)}; }
CC_FN Iv operator+(double n, Iv a) { return Iv{add_dn(a.lo, n), add_up(a.hi, n)}; }
CC_FN Iv operator-(Iv a, Iv b) { return Iv{add_dn(a.lo, -b.hi), add_up(a.hi, -b.lo)}; }
CC_FN Iv operator-(Iv a, double n) { return Iv{add_dn(a.lo, -n), add_up(a.hi, -n)}; }
CC_FN Iv operator-(double n, Iv b) { return Iv{add_dn(n, -b.hi), add_up(n, -b.lo)}; }
CC_FN Iv operator-(Iv a) { return Iv{-a.hi, -a.lo}; }

// ------------------------------------------------------------------ *
CC_FN double lesser(double a, double b) { return a < b ? a : b; }
CC_FN double greater(double a, double b) { return a > b ? a : b; }

CC_FN Iv operator*(Iv a, Iv b) {
    // Fast path with identical bits: for non-empty intervals with all four
    // endpoints > 0 the chain below always selects lo*lo rounded down and
    // hi*hi rounded up (directed rounding is monotone, ties are equal bits).
    if (0.0 < a.lo && a.lo <= a.hi && 0.0 < b.lo && b.lo <= b.hi) {
        return Iv{mul_dn(a.lo, b.lo), mul_up(a.hi, b.hi)};
    }
    double l1 = mul_dn(a.lo, b.lo), l2 = mul_dn(a.lo, b.hi);
    double l3 = mul_dn(a.hi, b.lo), l4 = mul_dn(a.hi, b.hi);
    double u1 = mul_up(a.lo, b.lo), u2 = mul_up(a.lo, b.hi);
    double u3 = mul_up(a.hi, b.lo), u4 = mul_up(a.hi, b.hi);
    return Iv{lesser(lesser(l1, l2), lesser(l3, l4)), greater(greater(u1, u2), greater(u3, u4))};
}

CC_FN Iv operator*(Iv a, double n) {
    if (n >= 0) {
        return Iv{mul_dn(a.lo, n), mul_dn(a.hi, n)};  // sic: upper bound rounded down
    }
    return Iv{mul_dn(a.hi, n), mul_up(a.lo, n)};
}
CC_FN Iv operator*(double n, Iv a) { return a * n; }

// ------------------------------------------------------------------ /
CC_FN Iv operator/(Iv a, double n) {
    if (n > 0) {
        return Iv{div_dn(a.lo, n), div_up(a.hi, n)};
    }
    return Iv{div_dn(a.hi, n), div_up(a.lo, n)};
}

CC_FN Iv operator/(Iv a, Iv o) {
    if (o.lo > 0) {
        if (a.lo >= 0) return Iv{div_dn(a.lo, o.hi), div_up(a.hi, o.lo)};
        if (a.hi <= 0) return Iv{div_dn(a.lo, o.lo), div_up(a.hi, o.hi)};
        return Iv{div_dn(a.lo, o.lo), div_up(a.hi, o.lo)};
    }
    if (o.hi < 0) {
        if (a.lo >= 0) return Iv{div_dn(a.hi, o.hi), div_up(a.lo, o.lo)};
        if (a.hi <= 0) return Iv{div_dn(a.hi, o.lo), div_up(a.lo, o.hi)};
        return Iv{div_dn(a.hi, o.hi), div_up(a.lo, o.hi)};
    }
    return Iv{-CC_INF, CC_INF};
}
CC_FN Iv operator/(double n, Iv o) { return ivp(n) / o; }

CC_FN Iv reciprocal(Iv a) {
    if (a.lo > 0) return Iv{rcp_dn(a.hi), rcp_up(a.lo)};
    if (a.hi < 0) return Iv{rcp_dn(a.lo), rcp_up(a.hi)};
    return Iv{-CC_INF, CC_INF};
}

// ------------------------------------------------------ abs, square, sqrt
CC_FN Iv iv_abs(Iv a) {
    double l = 0.0, u = 0.0;
    if (a.hi > 0) {
        u = a.hi;
    } else {
        l = -a.hi;
    }
    if (a.lo < 0) {
        u = u < -a.lo ? -a.lo : u;
    } else {
        l = a.lo;
    }
    return Iv{l, u};
}

CC_FN Iv square(Iv a) {
    Iv m = iv_abs(a);
    return Iv{mul_dn(m.lo, m.lo), mul_up(m.hi, m.hi)};
}

CC_FN Iv sqrt(Iv a) {
    if (a.lo < 0.0) {
        trap(TRAP_SQRT_NEGATIVE);
    }
    return Iv{sqrt_dn(a.lo), sqrt_up(a.hi)};
}

// --------------------------------------------------------- comparisons
CC_FN Ub operator<(Iv a, double n) { return Ub{a.hi < n, a.lo < n}; }
CC_FN Ub operator>(Iv a, double n) { return Ub{a.lo > n, a.hi > n}; }
CC_FN Ub operator<=(Iv a, double n) { return Ub{a.hi <= n, a.lo <= n}; }
CC_FN Ub operator>=(Iv a, double n) { return Ub{a.lo >= n, a.hi >= n}; }
CC_FN Ub operator<(Iv a, Iv b) { return Ub{a.hi < b.lo, a.lo < b.hi}; }
CC_FN Ub operator<=(Iv a, Iv b) { return Ub{a.hi <= b.lo, a.lo <= b.hi}; }
CC_FN Ub operator>(Iv a, Iv b) { return b < a; }
CC_FN Ub operator>=(Iv a, Iv b) { return b <= a; }
CC_FN Ub operator<(double n, Iv a) { return a > n; }
CC_FN Ub operator>(double n, Iv a) { return a < n; }
CC_FN Ub operator<=(double n, Iv a) { return a >= n; }
CC_FN Ub operator>=(double n, Iv a) { return a <= n; }
CC_FN Ub operator==(Iv a, Iv b) {
    return Ub{a.lo == a.hi && b.lo == b.hi && a.lo == b.lo, !(a.lo > b.hi) && !(a.hi < b.lo)};
}
CC_FN Ub operator==(Iv a, double n) { return Ub{a.lo == a.hi && a.lo == n, !(a.lo > n) && !(a.hi < n)}; }

// ------------------------------------------------- set operations
CC_FN Iv intersect(Iv a, Iv o) { return Iv{a.lo < o.lo ? o.lo : a.lo, a.hi > o.hi ? o.hi : a.hi}; }
CC_FN void do_intersect(Iv& a, Iv o) {
    if (o.lo > a.lo) a.lo = o.lo;
    if (o.hi < a.hi) a.hi = o.hi;
}
CC_FN Iv join(Iv a, Iv o) { return Iv{a.lo > o.lo ? o.lo : a.lo, a.hi < o.hi ? o.hi : a.hi}; }
CC_FN void do_join(Iv& a, Iv o) {
    if (o.lo < a.lo) a.lo = o.lo;
    if (o.hi > a.hi) a.hi = o.hi;
}
CC_FN void tighten_ub(Iv& a, double u) {
    if (u < a.hi) a.hi = u;
}
CC_FN void tighten_lb(Iv& a, double l) {
    if (a.lo < l) a.lo = l;
}
CC_FN bool empty(Iv a) { return a.lo > a.hi; }

// The i-th of n equal pieces of an interval, the last one ending exactly at
// the upper bound (reference: subintervals.hpp:33-43).  `lb + diff*i` is
// written there as a plain expression that nvcc contracts into one FMA by
// default; the contraction is spelled out so that host and device agree.
CC_FN Iv subinterval(Iv a, int i, int n) {
    double diff = a.hi - a.lo;
    diff /= n;
    double l = ::fma(diff, (double)i, a.lo);
    double u = ::fma(diff, (double)(i + 1), a.lo);
    if (i + 1 == n) u = a.hi;
    return Iv{l, u};
}

// subinterval() with the step (diff / n) computed once for all pieces of
// the same interval: identical bounds, one division fewer per piece.
CC_FN double subinterval_step(Iv a, int n) {
    double diff = a.hi - a.lo;
    diff /= n;
    return diff;
}
CC_FN Iv subinterval_with_step(Iv a, double step, int i, int n) {
    double l = ::fma(step, (double)i, a.lo);
    double u = ::fma(step, (double)(i + 1), a.lo);
    if (i + 1 == n) u = a.hi;
    return Iv{l, u};
}

}  // namespace cc

// Geometry primitives over interval points: squared distance, circle-circle
// intersection, midpoint.  This is the prover's counterpart of the
// reference's operations.hpp / operations.cuh call surface
// (reference: operations.hpp:32-44, operations.cuh:29-33, operations.cu:25-88);
// the operation order is the reference's, so results are bit-identical.
#pragma once

#include "cc_iv.cuh"

namespace cc {

struct Point {
    Iv x, y;
};

// two intersection points; when definitely_intersecting, p[0] is the one that
// is lexicographically smaller whenever that is certain
struct Isect {
    Point p[2];
    bool definitely_intersecting;
};

struct Circle {
    Point center;
    Iv squared_radius;
};

CC_FN Iv squared_distance(const Point& a, const Point& b) {
    return square(a.x - b.x) + square(a.y - b.y);
}

// reference: operations.cu:30-83
CC_FN Isect intersection(const Circle& c1, const Circle& c2) {
    Isect r;
    r.definitely_intersecting = false;

    Iv d2 = squared_distance(c1.center, c2.center);
    if (d2.lo == 0) {
        return r;
    }

    Iv rdiff = c1.squared_radius - c2.squared_radius;
    Iv rdiff_sq = square(rdiff);

    // squared half-chord relative to the squared centre distance
    Iv t = 2.0 * (c1.squared_radius + c2.squared_radius) / d2 - 1.0 - rdiff_sq / square(d2);
    if (t.lo < 0) {
        return r;
    }
    Iv half_chord = 0.5 * sqrt(t);
    r.definitely_intersecting = true;

    Iv shift = 0.5 * rdiff / d2;
    Iv x1 = c1.center.x, x2 = c2.center.x;
    Iv y1 = c1.center.y, y2 = c2.center.y;

    Iv mx = 0.5 * (x1 + x2);
    Iv my = 0.5 * (y1 + y2);
    Iv dx = x2 - x1;
    Iv dy = y2 - y1;
    mx = mx + shift * dx;
    my = my + shift * dy;

    Point a{mx + half_chord * dy, my - half_chord * dx};
    Point b{mx - half_chord * dy, my + half_chord * dx};

    if (dy.hi < 0 || (dy.hi == 0 && dx.lo >= 0)) {
        r.p[0] = a;
        r.p[1] = b;
    } else {
        r.p[0] = b;
        r.p[1] = a;
    }
    return r;
}

// reference: operations.cu:85-87
CC_FN Point center(const Point& a, const Point& b) {
    return Point{a.x + 0.5 * (b.x - a.x), a.y + 0.5 * (b.y - a.y)};
}

}  // namespace cc

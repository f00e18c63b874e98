// scmath64.h -- double-precision vector and quaternion helpers of the FP64
// host oracle (oracle/scport64.cpp).  TEST INFRASTRUCTURE ONLY.
//
// The same helpers as scmath.h (helper_math's component-wise operators and
// the reference's quaternion functions, spatial_cell_sim/src/math.cuh:15-339)
// with every quantity a double and the elementary functions the C library's
// double ones: the step evaluated as the same algorithm in FP64, the
// reference of the ensemble criterion (MSD and pair-distance histogram after
// many steps) that the single-precision step is compared with.
#pragma once

#include <math.h>

#include "scmath.h"

struct sc_d2 { double x, y; };
struct sc_d3 { double x, y, z; };
struct sc_d4 { double x, y, z, w; };

static inline sc_d3 sc_make_d3(double x, double y, double z) { sc_d3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline sc_d4 sc_make_d4(double x, double y, double z, double w) { sc_d4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }

static inline sc_d3 operator+(sc_d3 a, sc_d3 b) { return sc_make_d3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline sc_d3 operator-(sc_d3 a, sc_d3 b) { return sc_make_d3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline sc_d3 operator-(sc_d3 a) { return sc_make_d3(-a.x, -a.y, -a.z); }
static inline sc_d3 operator*(sc_d3 a, double b) { return sc_make_d3(a.x * b, a.y * b, a.z * b); }
static inline sc_d3 operator*(double b, sc_d3 a) { return sc_make_d3(b * a.x, b * a.y, b * a.z); }
static inline sc_d3 operator*(sc_d3 a, sc_d3 b) { return sc_make_d3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline sc_d3 operator/(sc_d3 a, double b) { return sc_make_d3(a.x / b, a.y / b, a.z / b); }
static inline void operator+=(sc_d3 &a, sc_d3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
static inline void operator-=(sc_d3 &a, sc_d3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
static inline void operator*=(sc_d3 &a, double b) { a.x *= b; a.y *= b; a.z *= b; }
static inline void operator/=(sc_d3 &a, double b) { a.x /= b; a.y /= b; a.z /= b; }
static inline sc_d4 operator+(sc_d4 a, sc_d4 b) { return sc_make_d4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline sc_d4 operator-(sc_d4 a, sc_d4 b) { return sc_make_d4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline sc_d4 operator-(sc_d4 a) { return sc_make_d4(-a.x, -a.y, -a.z, -a.w); }
static inline sc_d4 operator*(sc_d4 a, double b) { return sc_make_d4(a.x * b, a.y * b, a.z * b, a.w * b); }
static inline sc_d4 operator*(double b, sc_d4 a) { return sc_make_d4(b * a.x, b * a.y, b * a.z, b * a.w); }
static inline sc_d4 operator/(sc_d4 a, double b) { return sc_make_d4(a.x / b, a.y / b, a.z / b, a.w / b); }
static inline void operator+=(sc_d4 &a, sc_d4 b) { a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w; }
static inline void operator*=(sc_d4 &a, double b) { a.x *= b; a.y *= b; a.z *= b; a.w *= b; }
static inline void operator/=(sc_d4 &a, double b) { a.x /= b; a.y /= b; a.z /= b; a.w /= b; }

static inline double dot(sc_d3 a, sc_d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double dot(sc_d4 a, sc_d4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline sc_d3 cross(sc_d3 a, sc_d3 b) {
    return sc_make_d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double length(sc_d3 v) { return sqrt(dot(v, v)); }
static inline double length(sc_d4 v) { return sqrt(dot(v, v)); }
static inline sc_d3 normalize(sc_d3 v) { return v * (1.0 / sqrt(dot(v, v))); }
static inline sc_d4 normalize(sc_d4 v) { return v * (1.0 / sqrt(dot(v, v))); }
static inline double sc_d_clamp1(double f, double a, double b) { return fmax(a, fmin(f, b)); }
static inline sc_d3 clamp(sc_d3 v, double a, double b) {
    return sc_make_d3(sc_d_clamp1(v.x, a, b), sc_d_clamp1(v.y, a, b), sc_d_clamp1(v.z, a, b));
}

static inline sc_d3 sc_d_up() { return sc_make_d3(0.0, 1.0, 0.0); }
static inline sc_d3 sc_d_right() { return sc_make_d3(1.0, 0.0, 0.0); }
static inline sc_d3 sc_d_forward() { return sc_make_d3(0.0, 0.0, 1.0); }
static inline sc_d3 sc_d_zero3() { return sc_make_d3(0.0, 0.0, 0.0); }
static inline sc_d4 sc_d_qid() { return sc_make_d4(0.0, 0.0, 0.0, 1.0); }
static inline double sc_d_normsq3(sc_d3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double sc_d_normsq4(sc_d4 a) { return a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w; }
static inline double sc_d_norm3(sc_d3 a) { return sqrt(sc_d_normsq3(a)); }

// math.cuh:90-96
static inline sc_d3 sc_d_safe_cross(sc_d3 a, sc_d3 b) {
    sc_d3 c = cross(a, b);
    if (c.x == 0.0 && c.y == 0.0 && c.z == 0.0) return sc_d_forward();
    return normalize(c);
}
// math.cuh:116-130 (Hamilton product)
static inline sc_d4 sc_d_qmul(sc_d4 a, sc_d4 b) {
    double cx = a.y * b.z - a.z * b.y, cy = a.z * b.x - a.x * b.z, cz = a.x * b.y - a.y * b.x;
    double d = a.x * b.x + a.y * b.y + a.z * b.z;
    return sc_make_d4(a.x * b.w + b.x * a.w + cx, a.y * b.w + b.y * a.w + cy, a.z * b.w + b.z * a.w + cz,
                      a.w * b.w - d);
}
// math.cuh:132-136
static inline double sc_d_angle3(sc_d3 a, sc_d3 b) {
    return acos(sc_d_clamp1(dot(a, b) / (sc_d_norm3(a) * sc_d_norm3(b)), -1.0, 1.0));
}
// math.cuh:143-155
static inline sc_d4 sc_d_quat(sc_d3 axis, double angle) {
    double s = sin(angle * 0.5), c = cos(angle * 0.5);
    return normalize(sc_make_d4(axis.x * s, axis.y * s, axis.z * s, c));
}
// math.cuh:157-160
static inline sc_d4 sc_d_quat_from_to(sc_d3 a, sc_d3 b) { return sc_d_quat(sc_d_safe_cross(a, b), sc_d_angle3(a, b)); }
// math.cuh:171-181
static inline sc_d4 sc_d_qinv(sc_d4 a) {
    double inv = 1.0 / sc_d_normsq4(a);
    return sc_make_d4(-a.x * inv, -a.y * inv, -a.z * inv, a.w * inv);
}
// math.cuh:220-262 (lerp below the reference's 1e-6 threshold)
static inline sc_d4 sc_d_slerp(sc_d4 a, sc_d4 b, double t) {
    const double eps = 1e-6;
    double cosO = a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
    bool flip = false;
    if (cosO < 0.0) { flip = true; cosO = -cosO; }
    double s1, s2;
    if (cosO > 1.0 - eps) {
        s1 = 1.0 - t;
        s2 = flip ? -t : t;
    } else {
        double omega = acos(cosO), invSin = 1.0 / sin(omega);
        s1 = sin((1.0 - t) * omega) * invSin;
        s2 = flip ? -sin(t * omega) * invSin : sin(t * omega) * invSin;
    }
    return sc_make_d4(s1 * a.x + s2 * b.x, s1 * a.y + s2 * b.y, s1 * a.z + s2 * b.z, s1 * a.w + s2 * b.w);
}
// math.cuh:264-277 with the three uniforms already drawn
static inline sc_d4 sc_d_random_rotation(double u, double v, double w) {
    double su = sqrt(u), su1 = sqrt(1.0 - u), tp = 2.0 * 3.14159265358979323846;
    return sc_make_d4(su1 * sin(tp * v), su1 * cos(tp * v), su * sin(tp * w), su * cos(tp * w));
}
// math.cuh:309-338 (rotation-matrix form)
static inline sc_d3 sc_d_rotate(sc_d3 a, sc_d4 q) {
    double x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    double wx2 = q.w * x2, wy2 = q.w * y2, wz2 = q.w * z2;
    double xx2 = q.x * x2, xy2 = q.x * y2, xz2 = q.x * z2;
    double yy2 = q.y * y2, yz2 = q.y * z2, zz2 = q.z * z2;
    return sc_make_d3(a.x * (1.0 - yy2 - zz2) + a.y * (xy2 - wz2) + a.z * (xz2 + wy2),
                      a.x * (xy2 + wz2) + a.y * (1.0 - xx2 - zz2) + a.z * (yz2 - wx2),
                      a.x * (xz2 - wy2) + a.y * (yz2 + wx2) + a.z * (1.0 - xx2 - yy2));
}
// periodic box and reflecting walls (extensions; as scmath.h)
static inline double sc_d_image1(double t, double p, double L) {
    double d = t - p, h = L * 0.5;
    return d > h ? t - L : (d < -h ? t + L : t);
}
static inline sc_d3 sc_d_image3(sc_d3 t, sc_d3 p, double L) {
    return sc_make_d3(sc_d_image1(t.x, p.x, L), sc_d_image1(t.y, p.y, L), sc_d_image1(t.z, p.z, L));
}
static inline double sc_d_wrap1(double x, double L) { return x >= L ? x - L : (x < 0.0 ? x + L : x); }
static inline sc_d3 sc_d_wrap3(sc_d3 v, double L) { return sc_make_d3(sc_d_wrap1(v.x, L), sc_d_wrap1(v.y, L), sc_d_wrap1(v.z, L)); }
static inline double sc_d_reflect1(double x, double L) {
    const double r = x < 0.0 ? -x : (x > L ? L - (x - L) : x);
    return fmin(fmax(r, 0.0), L);
}
static inline sc_d3 sc_d_reflect3(sc_d3 v, double L) {
    return sc_make_d3(sc_d_reflect1(v.x, L), sc_d_reflect1(v.y, L), sc_d_reflect1(v.z, L));
}
// the cell index of a double coordinate (grid.cuh:13-17, saturating)
static inline uint32_t sc_d_grid_idx(double c, double cell, int n) {
    double q = c / cell;
    uint32_t i = !(q > 0.0) ? 0u : (q >= 4294967295.0 ? 0xffffffffu : (uint32_t)q);
    return i < (uint32_t)(n - 1) ? i : (uint32_t)(n - 1);
}

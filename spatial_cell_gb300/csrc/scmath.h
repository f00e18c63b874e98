// scmath.h -- portable (host + sm_103a device) arithmetic that defines the
// floating-point semantics of the spatial-cell step.
//
// Everything here is written with IEEE-754 single/double operations whose
// results are fully specified (+, -, *, /, sqrt, float<->int conversions and
// bit casts) and never with implicit FMA contraction, so the same source gives
// bit-identical results on the CUDA device (built with -fmad=false) and on the
// host (built with -ffp-contract=off).  That is what lets the CUDA step, the
// CPU restatement and the reference's own kernels (compiled for the host with
// this header standing in for CUDA's libraries) agree bit for bit.
//
// Contents
//   * sc_f3 / sc_f4 vector types and the helper_math-style operators the
//     reference uses (spatial_cell_sim/src/math.cuh:8 includes CUDA-samples'
//     helper_math.h; normalize() there is v * rsqrt(dot(v,v)); here the
//     reciprocal square root is the correctly-rounded 1/sqrtf(x), the same
//     definition helper_math.h uses for host code).
//   * Elementary functions sc_sinf/sc_cosf/sc_acosf/sc_logf/sc_expf/sc_powf:
//     Cody-Waite argument reduction (W. J. Cody & W. Waite, "Software Manual
//     for the Elementary Functions", 1980) followed by truncated Taylor
//     series (sin, cos, exp, asin) and the atanh series for log.  Series
//     coefficients are the exact Taylor coefficients rounded to float.
//   * Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
//     "Parallel Random Numbers: As Easy as 1, 2, 3", SC'11) and the uniform /
//     Box-Muller normal maps keyed by (seed, stream, particle id, step, draw).
//   * float -> binary16 round-to-nearest-even conversion for frames.dat.
//   * Restatement of the reference's quaternion helpers
//     (spatial_cell_sim/src/math.cuh:15-339) as sc_* functions.
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define SC_HD __host__ __device__ __forceinline__
// Long functions called from many sites are compiled once per kernel and
// called, which keeps the kernels' instruction footprint small.
#define SC_HD_COLD static __host__ __device__ __noinline__
#define SC_ALIGN16 __align__(16)
#else
#define SC_HD static inline
#define SC_HD_COLD static inline
#define SC_ALIGN16 __attribute__((aligned(16)))
#endif

// ---------------------------------------------------------------------------
// Vector types (layout-compatible with CUDA's float3 / float4)
// ---------------------------------------------------------------------------
struct sc_f2 { float x, y; };
struct sc_f3 { float x, y, z; };
struct SC_ALIGN16 sc_f4 { float x, y, z, w; };

SC_HD sc_f3 sc_make_f3(float x, float y, float z) { sc_f3 r; r.x = x; r.y = y; r.z = z; return r; }
SC_HD sc_f4 sc_make_f4(float x, float y, float z, float w) { sc_f4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }

// helper_math.h semantics: component-wise, left-to-right.
SC_HD sc_f3 operator+(sc_f3 a, sc_f3 b) { return sc_make_f3(a.x + b.x, a.y + b.y, a.z + b.z); }
SC_HD sc_f3 operator-(sc_f3 a, sc_f3 b) { return sc_make_f3(a.x - b.x, a.y - b.y, a.z - b.z); }
SC_HD sc_f3 operator-(sc_f3 a) { return sc_make_f3(-a.x, -a.y, -a.z); }
SC_HD sc_f3 operator*(sc_f3 a, float b) { return sc_make_f3(a.x * b, a.y * b, a.z * b); }
SC_HD sc_f3 operator*(float b, sc_f3 a) { return sc_make_f3(b * a.x, b * a.y, b * a.z); }
SC_HD sc_f3 operator*(sc_f3 a, sc_f3 b) { return sc_make_f3(a.x * b.x, a.y * b.y, a.z * b.z); }
SC_HD sc_f3 operator/(sc_f3 a, float b) { return sc_make_f3(a.x / b, a.y / b, a.z / b); }
SC_HD sc_f3 operator/(sc_f3 a, sc_f3 b) { return sc_make_f3(a.x / b.x, a.y / b.y, a.z / b.z); }
SC_HD void operator+=(sc_f3 &a, sc_f3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
SC_HD void operator-=(sc_f3 &a, sc_f3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
SC_HD void operator*=(sc_f3 &a, float b) { a.x *= b; a.y *= b; a.z *= b; }
SC_HD void operator/=(sc_f3 &a, float b) { a.x /= b; a.y /= b; a.z /= b; }

SC_HD sc_f4 operator+(sc_f4 a, sc_f4 b) { return sc_make_f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
SC_HD sc_f4 operator-(sc_f4 a, sc_f4 b) { return sc_make_f4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
SC_HD sc_f4 operator-(sc_f4 a) { return sc_make_f4(-a.x, -a.y, -a.z, -a.w); }
SC_HD sc_f4 operator*(sc_f4 a, float b) { return sc_make_f4(a.x * b, a.y * b, a.z * b, a.w * b); }
SC_HD sc_f4 operator*(float b, sc_f4 a) { return sc_make_f4(b * a.x, b * a.y, b * a.z, b * a.w); }
SC_HD sc_f4 operator/(sc_f4 a, float b) { return sc_make_f4(a.x / b, a.y / b, a.z / b, a.w / b); }
SC_HD void operator+=(sc_f4 &a, sc_f4 b) { a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w; }
SC_HD void operator*=(sc_f4 &a, float b) { a.x *= b; a.y *= b; a.z *= b; a.w *= b; }
SC_HD void operator/=(sc_f4 &a, float b) { a.x /= b; a.y /= b; a.z /= b; a.w /= b; }

SC_HD float dot(sc_f3 a, sc_f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SC_HD float dot(sc_f4 a, sc_f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
SC_HD sc_f3 cross(sc_f3 a, sc_f3 b) {
    return sc_make_f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
SC_HD float length(sc_f3 v) { return sqrtf(dot(v, v)); }
SC_HD float length(sc_f4 v) { return sqrtf(dot(v, v)); }
SC_HD sc_f3 normalize(sc_f3 v) { float inv = 1.0f / sqrtf(dot(v, v)); return v * inv; }
SC_HD sc_f4 normalize(sc_f4 v) { float inv = 1.0f / sqrtf(dot(v, v)); return v * inv; }
SC_HD float sc_clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
SC_HD sc_f3 clamp(sc_f3 v, float a, float b) {
    return sc_make_f3(sc_clampf(v.x, a, b), sc_clampf(v.y, a, b), sc_clampf(v.z, a, b));
}

// ---------------------------------------------------------------------------
// Bit casts
// ---------------------------------------------------------------------------
SC_HD uint32_t sc_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    union { float f; uint32_t u; } c; c.f = f; return c.u;
#endif
}
SC_HD float sc_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    union { float f; uint32_t u; } c; c.u = u; return c.f;
#endif
}
SC_HD int sc_isfinitef(float x) { return (sc_f2u(x) & 0x7f800000u) != 0x7f800000u; }

// Round-half-away-from-zero to an integer for |x| < 2^23 (exact, portable).
SC_HD int sc_round_int(float x) { return (int)(x >= 0.0f ? x + 0.5f : x - 0.5f); }

// ---------------------------------------------------------------------------
// Elementary functions
// ---------------------------------------------------------------------------
// pi/2 = SC_PIO2_1 + SC_PIO2_2 + SC_PIO2_3 (12 + 12 + 24 significant bits),
// so k * SC_PIO2_1 and k * SC_PIO2_2 are exact for |k| < 2^12.
#define SC_PIO2_1 1.57080078125f
#define SC_PIO2_2 (-4.453584551811218e-06f)
#define SC_PIO2_3 (-8.705515752716053e-10f)
#define SC_2_OVER_PI 0.6366197466850281f
#define SC_PIO2_1D 1.5707963267341256
#define SC_PIO2_2D 6.077100506506192e-11
#define SC_2_OVER_PI_D 0.6366197723675814

// sin / cos of a reduced argument |r| <= ~pi/4 (Taylor through r^13 / r^14).
SC_HD float sc_sin_poly(float r) {
    if (r == 0.0f) return r;  // keeps the sign of zero
    float r2 = r * r;
    float p = 1.6059044372074283e-10f;
    p = p * r2 + (-2.5052107943679403e-08f);
    p = p * r2 + 2.7557318844628753e-06f;
    p = p * r2 + (-0.00019841270113829523f);
    p = p * r2 + 0.008333333767950535f;
    p = p * r2 + (-0.1666666716337204f);
    return r + (r * r2) * p;
}
SC_HD float sc_cos_poly(float r) {
    float r2 = r * r;
    float p = -1.147074536050896e-11f;
    p = p * r2 + 2.0876755879584152e-09f;
    p = p * r2 + (-2.755731998149713e-07f);
    p = p * r2 + 2.4801587642286904e-05f;
    p = p * r2 + (-0.0013888889225199819f);
    p = p * r2 + 0.0416666679084301f;
    return (1.0f - 0.5f * r2) + (r2 * r2) * p;
}

// Reduces x to r in [-pi/4, pi/4] with x = k*pi/2 + r; returns k & 3.
SC_HD int sc_reduce_pio2(float x, float *r) {
    float ax = fabsf(x);
    if (ax <= 1000.0f) {
        int k = sc_round_int(x * SC_2_OVER_PI);
        float fk = (float)k;
        *r = ((x - fk * SC_PIO2_1) - fk * SC_PIO2_2) - fk * SC_PIO2_3;
        return k & 3;
    }
    // Large arguments: the same reduction carried in double precision.
    double xd = (double)x;
    double kd = xd * SC_2_OVER_PI_D;
    kd = (kd >= 0.0) ? (double)(int64_t)(kd + 0.5) : (double)(int64_t)(kd - 0.5);
    *r = (float)((xd - kd * SC_PIO2_1D) - kd * SC_PIO2_2D);
    return (int)(((int64_t)kd) & 3);
}

SC_HD_COLD float sc_sinf(float x) {
    if (!sc_isfinitef(x)) return x - x;  // NaN for +-inf and NaN
    if (x == 0.0f) return x;             // sin(+-0) = +-0
    float r;
    int q = sc_reduce_pio2(x, &r);
    float s = sc_sin_poly(r), c = sc_cos_poly(r);
    return q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
}
SC_HD_COLD float sc_cosf(float x) {
    if (!sc_isfinitef(x)) return x - x;
    float r;
    int q = sc_reduce_pio2(x, &r);
    float s = sc_sin_poly(r), c = sc_cos_poly(r);
    return q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}

// asin on [0, 0.5]: z + z^3 * sum_n c_n z^(2n-2), c_n = (2n)!/(4^n (n!)^2 (2n+1)).
SC_HD float sc_asin_poly(float z) {
    float w = z * z;
    float p = 0.00466014351695776f;
    p = p * w + 0.005153309553861618f;
    p = p * w + 0.005740037653595209f;
    p = p * w + 0.006447210442274809f;
    p = p * w + 0.007312525995075703f;
    p = p * w + 0.008390335366129875f;
    p = p * w + 0.009761609137058258f;
    p = p * w + 0.01155180111527443f;
    p = p * w + 0.013964843936264515f;
    p = p * w + 0.017352763563394547f;
    p = p * w + 0.022372158244252205f;
    p = p * w + 0.0303819440305233f;
    p = p * w + 0.0446428582072258f;
    p = p * w + 0.07500000298023224f;
    p = p * w + 0.1666666716337204f;
    return z + (z * w) * p;
}

#define SC_PI_HI 3.1415927410125732f
#define SC_PI_LO (-8.742277657347586e-08f)
#define SC_PIO2_HI 1.5707963705062866f
#define SC_PIO2_LO (-4.371138828673793e-08f)

SC_HD_COLD float sc_acosf(float x) {
    if (!(x == x)) return x;                       // NaN
    float ax = fabsf(x);
    if (ax > 1.0f) return (x - x) / (x - x);       // NaN outside the domain
    if (ax <= 0.5f) {
        return (SC_PIO2_HI - sc_asin_poly(x > 0.0f ? x : -x) * (x > 0.0f ? 1.0f : -1.0f)) + SC_PIO2_LO;
    }
    float s = sqrtf((1.0f - ax) * 0.5f);
    float a2 = 2.0f * sc_asin_poly(s);
    if (x > 0.0f) return a2;
    return (SC_PI_HI - a2) + SC_PI_LO;
}

#define SC_LN2_HI 0.693145751953125f
#define SC_LN2_LO 1.428606765330187e-06f
#define SC_INV_LN2 1.4426950216293335f

// Natural log for finite x > 0: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
// log(m) = 2*atanh(t), t = (m-1)/(m+1), series through t^13.
SC_HD float sc_logf(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? -INFINITY : (x - x) / (x - x);
    if (!sc_isfinitef(x)) return x;
    uint32_t u = sc_f2u(x);
    int e = 0;
    if ((u & 0x7f800000u) == 0) {           // subnormal: scale into the normal range
        x = x * 16777216.0f;                 // 2^24, exact
        u = sc_f2u(x);
        e = -24;
    }
    e += (int)((u >> 23) & 0xff) - 127;
    float m = sc_u2f((u & 0x007fffffu) | 0x3f800000u);   // [1, 2)
    if (m > 1.4142135381698608f) { m = m * 0.5f; e += 1; }
    float t = (m - 1.0f) / (m + 1.0f);
    float t2 = t * t;
    float p = 0.07692307978868484f;
    p = p * t2 + 0.09090909361839294f;
    p = p * t2 + 0.1111111119389534f;
    p = p * t2 + 0.1428571492433548f;
    p = p * t2 + 0.20000000298023224f;
    p = p * t2 + 0.3333333432674408f;
    float lm = 2.0f * t + (2.0f * t * t2) * p;
    float fe = (float)e;
    return fe * SC_LN2_HI + (lm + fe * SC_LN2_LO);
}

// exp for float z: z = n*ln2 + r, |r| <= ln2/2, exp(r) by Taylor through r^8.
SC_HD float sc_expf(float z) {
    if (!(z == z)) return z;
    if (z > 88.72283935546875f) return INFINITY;
    if (z < -103.0f) return 0.0f;
    int n = sc_round_int(z * SC_INV_LN2);
    float fn = (float)n;
    float r = (z - fn * SC_LN2_HI) - fn * SC_LN2_LO;
    float p = 2.4801587642286904e-05f;
    p = p * r + 0.00019841270113829523f;
    p = p * r + 0.0013888889225199819f;
    p = p * r + 0.008333333767950535f;
    p = p * r + 0.0416666679084301f;
    p = p * r + 0.1666666716337204f;
    p = p * r + 0.5f;
    float er = 1.0f + (r + (r * r) * p);
    // scale by 2^n in two exact steps (keeps n = 128 and subnormal results right)
    int n1 = n / 2, n2 = n - n1;
    float s1 = sc_u2f((uint32_t)(n1 + 127) << 23);
    float s2 = sc_u2f((uint32_t)(n2 + 127) << 23);
    return (er * s1) * s2;
}

// pow for x >= 0 (the step only raises non-negative bases to 0.2):
// exp(y * log(x)) with the IEEE special cases of pow for those inputs.
SC_HD_COLD float sc_powf(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (!(x == x) || !(y == y)) return x + y;
    if (x == 1.0f) return 1.0f;
    if (x < 0.0f) return (x - x) / (x - x);
    if (x == 0.0f) return y > 0.0f ? 0.0f : INFINITY;
    if (!sc_isfinitef(x)) return y > 0.0f ? INFINITY : 0.0f;
    return sc_expf(y * sc_logf(x));
}

// ---------------------------------------------------------------------------
// Philox4x32-10 and the draws of the step (key = seed, counter = (id, step,
// block, stream)).  Streams: 0/1 particle uniform/normal, 2/3 metabolic.
// ---------------------------------------------------------------------------
#define SC_PHILOX_M0 0xD2511F53u
#define SC_PHILOX_M1 0xCD9E8D57u
#define SC_PHILOX_W0 0x9E3779B9u
#define SC_PHILOX_W1 0xBB67AE85u

struct sc_u4 { uint32_t x, y, z, w; };

SC_HD sc_u4 sc_philox4x32_10(sc_u4 c, uint32_t k0, uint32_t k1) {
    for (int i = 0; i < 10; i++) {
        uint64_t p0 = (uint64_t)SC_PHILOX_M0 * (uint64_t)c.x;
        uint64_t p1 = (uint64_t)SC_PHILOX_M1 * (uint64_t)c.z;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        sc_u4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += SC_PHILOX_W0;
        k1 += SC_PHILOX_W1;
    }
    return c;
}

#define SC_STREAM_P_UNIFORM 0u
#define SC_STREAM_P_NORMAL 1u
#define SC_STREAM_M_UNIFORM 2u
#define SC_STREAM_M_NORMAL 3u

// Uniform in the open interval (0, 1): 23 random bits, exact in float.
SC_HD float sc_u01(uint32_t w) { return ((float)(w >> 9) + 0.5f) * 1.1920928955078125e-07f; }

SC_HD sc_u4 sc_draw_block(uint64_t seed, uint32_t stream, uint32_t id, uint32_t step, uint32_t block) {
    sc_u4 c; c.x = id; c.y = step; c.z = block; c.w = stream;
    return sc_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// The d-th uniform of (id, step): word d&3 of block d>>2.
// The binding draw of a rule with a probability (complexify extension): one
// uniform per (rule, step, unordered pair of ids), the same from either side.
// Its stream word carries the top bit and the rule id, so it shares no
// counter with the Brownian draws (streams 0..3).
SC_HD float sc_bind_uniform(uint64_t seed, int rule_id, int id_a, int id_b, int step);

SC_HD float sc_uniform(uint64_t seed, uint32_t stream, uint32_t id, uint32_t step, uint32_t d) {
    sc_u4 b = sc_draw_block(seed, stream, id, step, d >> 2);
    uint32_t w = (d & 3u) == 0 ? b.x : (d & 3u) == 1 ? b.y : (d & 3u) == 2 ? b.z : b.w;
    return sc_u01(w);
}

SC_HD float sc_bind_uniform(uint64_t seed, int rule_id, int id_a, int id_b, int step) {
    const uint32_t lo = (uint32_t)(id_a < id_b ? id_a : id_b), hi = (uint32_t)(id_a < id_b ? id_b : id_a);
    return sc_uniform(seed, 0x80000000u | ((uint32_t)rule_id & 0x7fffffffu), lo, (uint32_t)step, hi);
}

#define SC_2PI_F 6.2831854820251465f

// The d-th standard normal of (id, step): Box-Muller on words 0, 1 of block d.
SC_HD float sc_normal(uint64_t seed, uint32_t stream, uint32_t id, uint32_t step, uint32_t d) {
    sc_u4 b = sc_draw_block(seed, stream, id, step, d);
    float u1 = sc_u01(b.x), u2 = sc_u01(b.y);
    return sqrtf(-2.0f * sc_logf(u1)) * sc_cosf(SC_2PI_F * u2);
}

// ---------------------------------------------------------------------------
// float -> IEEE binary16, round to nearest even (CUDA's __float2half_rn).
// ---------------------------------------------------------------------------
SC_HD uint16_t sc_f2h(float f) {
    uint32_t x = sc_f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(ax > 0x7f800000u ? 0x7fffu : (sign | 0x7c00u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);       // rounds to >= 65520 -> inf
    if (ax < 0x33000001u) return (uint16_t)sign;                     // <= 2^-25 -> +-0
    uint32_t e = ax >> 23;
    uint32_t m = (ax & 0x007fffffu) | 0x00800000u;
    if (e < 113) {                                                   // half subnormal
        uint32_t shift = 126u - e;                                   // 14..24
        uint32_t hm = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1u);
        uint32_t half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (hm & 1u))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t h = ((e - 112u) << 10) | ((m >> 13) & 0x3ffu);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

// ---------------------------------------------------------------------------
// Quaternion / vector helpers of the step (spatial_cell_sim/src/math.cuh)
// ---------------------------------------------------------------------------
#define SC_PI_REF 3.1415926535f   // constants.cuh:4 (PI)

SC_HD sc_f3 sc_up() { return sc_make_f3(0.0f, 1.0f, 0.0f); }
SC_HD sc_f3 sc_right() { return sc_make_f3(1.0f, 0.0f, 0.0f); }
SC_HD sc_f3 sc_forward() { return sc_make_f3(0.0f, 0.0f, 1.0f); }
SC_HD sc_f3 sc_zero3() { return sc_make_f3(0.0f, 0.0f, 0.0f); }
SC_HD sc_f4 sc_qid() { return sc_make_f4(0.0f, 0.0f, 0.0f, 1.0f); }

// math.cuh:15-33
SC_HD float sc_normsq3(sc_f3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
SC_HD float sc_normsq4(sc_f4 a) { return a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w; }
SC_HD float sc_norm3(sc_f3 a) { return sqrtf(sc_normsq3(a)); }

// sqrtf(x) <= d, deciding without the square root wherever the answer is
// certain.  sqrtf rounds to nearest and rounding is monotone, so for a
// normal d > 0: with lo = fl(fl(d*d) * (1 - 2^-20)) <= d^2 (1 - 2^-21),
// x <= lo gives sqrt(x) < d, hence sqrtf(x) <= d; with
// hi = fl(fl(d*d) * (1 + 2^-20)) >= d^2 (1 + 2^-21), x > hi gives
// sqrt(x) > d (1 + 2^-22 - 2^-45), beyond the midpoint d (1 + 2^-24) between
// d and the next float, hence sqrtf(x) > d.  Only x in (lo, hi] (and NaN)
// takes sqrtf; for d outside [1e-10, 1e10] (or NaN) every x does.
typedef struct {
    float d, lo, hi;
} sc_sqrt_le;
SC_HD sc_sqrt_le sc_sqrt_le_make(float d) {
    sc_sqrt_le s;
    s.d = d;
    if (d >= 1e-10f && d <= 1e10f) {
        const float d2 = d * d;
        s.lo = d2 * (1.0f - 0x1p-20f);
        s.hi = d2 * (1.0f + 0x1p-20f);
    } else {
        s.lo = NAN;  // no comparison with NaN holds: every x takes sqrtf
        s.hi = NAN;
    }
    return s;
}
SC_HD bool sc_sqrt_le_test(sc_sqrt_le s, float x) {
    if (x <= s.lo) return true;
    if (x > s.hi) return false;
    return sqrtf(x) <= s.d;
}

// math.cuh:90-96
SC_HD sc_f3 sc_safe_cross(sc_f3 a, sc_f3 b) {
    sc_f3 c = cross(a, b);
    if (c.x == 0.0f && c.y == 0.0f && c.z == 0.0f) return sc_forward();
    return normalize(c);
}

// math.cuh:116-130 (Hamilton product)
SC_HD sc_f4 sc_qmul(sc_f4 a, sc_f4 b) {
    float cx = a.y * b.z - a.z * b.y;
    float cy = a.z * b.x - a.x * b.z;
    float cz = a.x * b.y - a.y * b.x;
    float d = a.x * b.x + a.y * b.y + a.z * b.z;
    return sc_make_f4(a.x * b.w + b.x * a.w + cx,
                      a.y * b.w + b.y * a.w + cy,
                      a.z * b.w + b.z * a.w + cz,
                      a.w * b.w - d);
}

// math.cuh:132-136: acos(clamp(dot(a,b)/(|a||b|), -1, 1))
SC_HD float sc_angle3(sc_f3 a, sc_f3 b) {
    return sc_acosf(sc_clampf(dot(a, b) / (sc_norm3(a) * sc_norm3(b)), -1.0f, 1.0f));
}

// math.cuh:143-155
SC_HD sc_f4 sc_quat(sc_f3 axis, float angle) {
    float s = sc_sinf(angle * 0.5f);
    float c = sc_cosf(angle * 0.5f);
    return normalize(sc_make_f4(axis.x * s, axis.y * s, axis.z * s, c));
}

// math.cuh:157-160
SC_HD sc_f4 sc_quat_from_to(sc_f3 a, sc_f3 b) { return sc_quat(sc_safe_cross(a, b), sc_angle3(a, b)); }

// math.cuh:171-181
SC_HD sc_f4 sc_qinv(sc_f4 a) {
    float inv = 1.0f / sc_normsq4(a);
    return sc_make_f4(-a.x * inv, -a.y * inv, -a.z * inv, a.w * inv);
}

// math.cuh:220-262
// The weights of slerp for an angle whose cosine is cosO (not near 1).
SC_HD_COLD sc_f2 sc_slerp_weights(float cosO, float t, bool flip) {
    float omega = sc_acosf(cosO);
    float invSin = 1.0f / sc_sinf(omega);
    float s1 = sc_sinf((1.0f - t) * omega) * invSin;
    float s2 = flip ? -sc_sinf(t * omega) * invSin : sc_sinf(t * omega) * invSin;
    sc_f2 r;
    r.x = s1;
    r.y = s2;
    return r;
}

SC_HD sc_f4 sc_slerp(sc_f4 a, sc_f4 b, float t) {
    const float eps = 1e-6f;
    float cosO = a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
    bool flip = false;
    if (cosO < 0.0f) { flip = true; cosO = -cosO; }
    float s1, s2;
    if (cosO > (1.0f - eps)) {
        s1 = 1.0f - t;
        s2 = flip ? -t : t;
    } else {
        sc_f2 sw = sc_slerp_weights(cosO, t, flip);
        s1 = sw.x;
        s2 = sw.y;
    }
    return sc_make_f4(s1 * a.x + s2 * b.x, s1 * a.y + s2 * b.y, s1 * a.z + s2 * b.z, s1 * a.w + s2 * b.w);
}

// math.cuh:264-277 with the three uniforms already drawn
SC_HD sc_f4 sc_random_rotation(float u, float v, float w) {
    float su = sqrtf(u), su1 = sqrtf(1.0f - u);
    float tp = 2.0f * SC_PI_REF;
    return sc_make_f4(su1 * sc_sinf(tp * v), su1 * sc_cosf(tp * v), su * sc_sinf(tp * w), su * sc_cosf(tp * w));
}

// math.cuh:309-338 (rotation-matrix form; evaluated literally so signed zeros
// and non-finite inputs behave exactly as in the reference)
SC_HD sc_f3 sc_rotate(sc_f3 a, sc_f4 q) {
    float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    float wx2 = q.w * x2, wy2 = q.w * y2, wz2 = q.w * z2;
    float xx2 = q.x * x2, xy2 = q.x * y2, xz2 = q.x * z2;
    float yy2 = q.y * y2, yz2 = q.y * z2, zz2 = q.z * z2;
    return sc_make_f3(a.x * (1.0f - yy2 - zz2) + a.y * (xy2 - wz2) + a.z * (xz2 + wy2),
                      a.x * (xy2 + wz2) + a.y * (1.0f - xx2 - zz2) + a.z * (yz2 - wx2),
                      a.x * (xz2 - wy2) + a.y * (yz2 + wx2) + a.z * (1.0f - xx2 - yy2));
}

// ---------------------------------------------------------------------------
// Single-precision forms of the reference's double-precision comparisons
// (exactly equivalent; the tests check them against the double forms).
// ---------------------------------------------------------------------------
// (double)|x| > 0.001 for a float x: 0.001 is not a float, so the test is
// |x| >= the smallest float above 0.001 (metabolites.cuh:416).
#define SC_DIFFUSE_THRESHOLD 0.0010000000474974513f
SC_HD bool sc_diffuse_exceeds(float diff) { return fabsf(diff) >= SC_DIFFUSE_THRESHOLD; }

// (double)dist <= (double)s + 0.8 * (double)s * 0.5 (dynamics.cuh:478) for
// float dist, s.  The bound lies within 1e-15 (relative) of 1.4 * s, so
// single precision decides every dist outside [s*1.3999999, s*1.4000001]
// (both products are rounded values of reals strictly below / above the
// bound, and dist < RN(a) implies dist <= a); the rest falls back to double.
SC_HD bool sc_within_lipid_range(float dist, float s) {
    if (dist < s * 1.3999999f) return true;
    if (dist > s * 1.4000001f) return false;
    return (double)dist <= (double)s + 0.8 * (double)s * 0.5;
}

// ---------------------------------------------------------------------------
// Single-precision evaluation of the reference's mixed float/double
// expressions.  GB300 runs double precision at a small fraction of its float
// rate, so these are computed as float-float values and rounded once; where
// the rounding could depend on the last bits, the double expression itself
// is evaluated.  The results are identical to the double expressions for
// every input (the tests compare them on random and adversarial inputs).
// ---------------------------------------------------------------------------
SC_HD float sc_fmaf(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

// Rounds hi + lo (|lo| well below ulp(hi)) to float.  Returns false when a
// value within 2^-40 * |hi + lo| of it could round differently: the float-float
// value carries an error below 2^-46 relative, the double expression below
// 2^-51, so outside that band both round to the same float.
SC_HD bool sc_round_ff(float hi, float lo, float *out) {
    float f = hi + lo;
    float e = (hi - f) + lo;            // hi - f is exact (Sterbenz)
    uint32_t fb = sc_f2u(f) & 0x7fffffffu;
    if (fb < 0x18000000u || fb >= 0x7f000000u) return false;   // tiny, huge, inf, nan
    uint32_t ex = fb & 0x7f800000u;
    float half = sc_u2f(ex - (24u << 23));                     // ulp(f) / 2
    if ((fb & 0x007fffffu) == 0 && e != 0.0f && ((e < 0.0f) == (f > 0.0f)))
        half *= 0.5f;                                           // the gap below a power of two
    float margin = sc_u2f(ex - (40u << 23));
    *out = f;
    return fabsf(e) < half - margin;
}

// (float)((double)(rp + rt) + 0.8 * (double)rp), the metabolic collision
// distance (metabolites.cuh:198,237,324).  0.8 (double) = SC_08_HI + SC_08_LO
// to 2^-50; SC_08_HI * rp is split exactly with an fma.
#define SC_08_HI 0.800000011920929f
#define SC_08_LO (-1.1920929132713809e-08f)
SC_HD float sc_coll_dist(float rp, float rt) {
    float a = rp + rt;
    if (rp > 0.0f && a > 0.0f) {
        float ph = SC_08_HI * rp;
        float pl = sc_fmaf(SC_08_HI, rp, -ph);
        float cl = SC_08_LO * rp;
        float sh = a + ph;
        float bb = sh - a;
        float se = (a - (sh - bb)) + (ph - bb);
        float lo = (se + pl) + cl;
        float f;
        if (sc_round_ff(sh, lo, &f)) return f;
    }
    return (float)((double)(rp + rt) + 0.8 * (double)rp);
}

// (float)((double)x / fmax((double)radius / 2.5, 1.0)), the Brownian step
// length (dynamics.cuh:170): radius <= 2.5 (or NaN) divides by exactly 1.
SC_HD float sc_noise_mag(float x, float radius) {
    if (!(radius > 2.5f)) return x;
    return (float)((double)x / fmax((double)radius / 2.5, 1.0));
}

// (float)((double)rn / ((double)radius / 2.5)), the Brownian rotation weight
// (dynamics.cuh:180): rn * 2.5 / radius as a float-float quotient.
SC_HD float sc_rot_noise(float rn, float radius) {
    uint32_t rb = sc_f2u(radius), nb = sc_f2u(rn) & 0x7fffffffu;
    if (rb >= 0x00800000u && rb < 0x7f000000u && nb >= 0x00800000u && nb < 0x7e000000u) {
        float h = rn * 2.5f;
        float l = sc_fmaf(rn, 2.5f, -h);        // rn * 2.5 = h + l exactly
        float q0 = h / radius;
        float rem = sc_fmaf(-q0, radius, h);    // h - q0 * radius, exact
        float q1 = (rem + l) / radius;
        float f;
        if (sc_round_ff(q0, q1, &f)) return f;
    }
    return (float)((double)rn / ((double)radius / 2.5));
}

// (float)(fmin(fmax((double)L, 1e-6), (double)2.0f) / (double)2.0f), the
// polar attraction factor (dynamics.cuh:496).  SC_ABOVE_1EM6 is the smallest
// float above 1e-6 (double); SC_HALF_1EM6 = (float)5e-7.  NaN gives 5e-7
// (fmax returns the number).
#define SC_ABOVE_1EM6 1.0000001111620804e-06f
#define SC_HALF_1EM6 4.999999987376214e-07f
SC_HD float sc_polar_attr(float L) {
    if (L >= 2.0f) return 1.0f;
    if (L >= SC_ABOVE_1EM6) return L * 0.5f;
    return SC_HALF_1EM6;
}

// ---------------------------------------------------------------------------
// Periodic box (an extension; the reference clamps positions to its walls).
// A neighbour's position is replaced by its nearest periodic image relative
// to the item, so every pair expression keeps its reference form.
// ---------------------------------------------------------------------------
SC_HD float sc_image1(float t, float p, float L) {
    float d = t - p, h = L * 0.5f;
    return d > h ? t - L : (d < -h ? t + L : t);
}
SC_HD sc_f3 sc_image3(sc_f3 t, sc_f3 p, float L) {
    return sc_make_f3(sc_image1(t.x, p.x, L), sc_image1(t.y, p.y, L), sc_image1(t.z, p.z, L));
}
// Brings a coordinate displaced by less than one box length back into [0, L].
SC_HD float sc_wrap1(float x, float L) { return x >= L ? x - L : (x < 0.0f ? x + L : x); }
SC_HD sc_f3 sc_wrap3(sc_f3 v, float L) { return sc_make_f3(sc_wrap1(v.x, L), sc_wrap1(v.y, L), sc_wrap1(v.z, L)); }

// The reference's cell index (grid.cuh:13-17): min((uint)(c / cell), n - 1).
// The float -> unsigned conversion saturates as the GPU's cvt.rzi.u32.f32
// does (negative and NaN -> 0), which keeps the host build defined too.
// A position mirrored back into [0, L] at reflecting walls (an excursion
// longer than the box is clamped after the mirror).
SC_HD float sc_reflect1(float x, float L) {
    const float r = x < 0.0f ? -x : (x > L ? L - (x - L) : x);
    return fminf(fmaxf(r, 0.0f), L);
}
SC_HD sc_f3 sc_reflect3(sc_f3 v, float L) { return sc_make_f3(sc_reflect1(v.x, L), sc_reflect1(v.y, L), sc_reflect1(v.z, L)); }

// Cells per axis of a periodic box and their width: the box split into
// floor(L / cell) equal cells, each at least `cell` wide, so the 27 cells
// around an item hold every item within `cell` of it, across the faces too.
SC_HD int sc_periodic_cells(float L, float cell, float *width) {
    const float q = floorf(L / cell);
    const int n = q >= 1.0f ? (int)q : 1;
    *width = L / (float)n;
    return n;
}

SC_HD uint32_t sc_grid_idx(float c, float cell, int n) {
    float q = c / cell;
    uint32_t g = !(q > 0.0f) ? 0u : (q >= 4294967296.0f ? 0xffffffffu : (uint32_t)q);
    uint32_t m = (uint32_t)(n - 1);
    return g < m ? g : m;
}

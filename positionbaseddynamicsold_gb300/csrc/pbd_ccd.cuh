// pbd_ccd.cuh -- arithmetic shared by the vertex-face and edge-edge
// continuous collision paths: float3 helpers, barycentric coordinates, the
// FP64 cubic root isolation of P/CCD.cpp:48-113, ExtendedVFTest's evaluation
// (P/CCD.cpp:1733-1808), point-triangle distance, the spatial-hash cell and
// bucket functions, warp-aggregated counters and the fixed-point response
// sums.  Include only from translation units compiled with -fmad=false.
#pragma once

#include <cooperative_groups.h>

#include "pbd_common.cuh"

namespace pbd {
namespace {

namespace cg = cooperative_groups;

struct v3 {
    float x, y, z;
};
__device__ __forceinline__ v3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ v3 ld3(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ v3 sub3(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ v3 add3(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ v3 mul3(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ v3 div3(v3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross3(v3 a, v3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// normalize with a correctly rounded reciprocal square root, as the
// reference's host build computes it (1.0f / sqrtf)
__device__ __forceinline__ v3 nrm3(v3 v) {
    float inv = 1.0f / sqrtf(dot3(v, v));
    return mul3(v, inv);
}
__device__ __forceinline__ float dist3(v3 a, v3 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrtf(dx * dx + dy * dy + dz * dz);
}
__device__ __forceinline__ float stp(v3 u, v3 v, v3 w) { return dot3(u, cross3(v, w)); }
// a + t (b - a) with the time rounded to float, as the reference's
// ExtendedVFTest and VFCCDTest interpolate
__device__ __forceinline__ v3 lerp_f(v3 a, v3 b, float tf) {
    v3 d = sub3(b, a);
    return add3(a, mk3(tf * d.x, tf * d.y, tf * d.z));
}
__device__ __forceinline__ v3 lerp_t(v3 a, v3 b, double t) { return lerp_f(a, b, (float)t); }
// BarycentricCoord (P/CCD.cpp:115-130)
__device__ __forceinline__ v3 bary(v3 pos, v3 p0, v3 p1, v3 p2) {
    v3 ab = sub3(p0, p2), ac = sub3(p1, p2), ap = sub3(pos, p2);
    float d00 = dot3(ac, ac), d01 = dot3(ac, ab), d02 = dot3(ac, ap);
    float d11 = dot3(ab, ab), d12 = dot3(ab, ap);
    float inv = 1.0f / (d00 * d11 - d01 * d01);
    float v = (d11 * d02 - d01 * d12) * inv;
    float u = (d00 * d12 - d01 * d02) * inv;
    float w = 1.0f - u - v;
    return mk3(u, v, w);
}

// ---- cubic root isolation (P/CCD.cpp:48-113), double precision ----------
__device__ __forceinline__ double sgnd(double x) { return x < 0 ? -1.0 : 1.0; }

__device__ int solve_quadratic(double a, double b, double c, double x[2]) {
    double d = b * b - 4 * a * c;
    if (d < 0) {
        x[0] = -b / (2 * a);
        return 0;
    }
    double q = -(b + sgnd(b) * sqrt(d)) / 2;
    int i = 0;
    if (fabs(a) > 1e-12 * fabs(q)) x[i++] = q / a;
    if (fabs(q) > 1e-12 * fabs(c)) x[i++] = c / q;
    if (i == 2 && x[0] > x[1]) {
        double s = x[0];
        x[0] = x[1];
        x[1] = s;
    }
    return i;
}

__device__ double newtons_method(double a, double b, double c, double d, double x0, int dir) {
    if (dir != 0) {
        double y0 = d + x0 * (c + x0 * (b + x0 * a));
        double ddy0 = 2 * b + x0 * (6 * a);
        x0 += dir * sqrt(fabs(2 * y0 / ddy0));
    }
    for (int iter = 0; iter < 100; iter++) {
        double y = d + x0 * (c + x0 * (b + x0 * a));
        double dy = c + x0 * (2 * b + x0 * 3 * a);
        if (dy == 0) return x0;
        double x1 = x0 - y / dy;
        if (fabs(x0 - x1) < 1e-6) return x0;
        x0 = x1;
    }
    return x0;
}

// when the derivative has no critical point and none was written, Newton
// starts from 0 (the reference reads an uninitialised value there)
__device__ int solve_cubic(double a, double b, double c, double d, double x[3]) {
    double xc[2] = {0.0, 0.0};
    int ncrit = solve_quadratic(3 * a, 2 * b, c, xc);
    if (ncrit == 0) {
        x[0] = newtons_method(a, b, c, d, xc[0], 0);
        return 1;
    } else if (ncrit == 1) {
        return solve_quadratic(b, c, d, x);
    }
    double yc[2] = {d + xc[0] * (c + xc[0] * (b + xc[0] * a)),
                    d + xc[1] * (c + xc[1] * (b + xc[1] * a))};
    int i = 0;
    if (yc[0] * a >= 0) x[i++] = newtons_method(a, b, c, d, xc[0], -1);
    if (yc[0] * yc[1] <= 0) {
        int closer = fabs(yc[0]) < fabs(yc[1]) ? 0 : 1;
        x[i++] = newtons_method(a, b, c, d, xc[closer], closer == 0 ? 1 : -1);
    }
    if (yc[1] * a <= 0) x[i++] = newtons_method(a, b, c, d, xc[1], 1);
    return i;
}

// A contact's weights are float values (the barycentric coordinates are
// computed in float); the reference stores them as doubles, which the
// contact store does (exactly) when it writes them out.
struct VFResult {
    float t;
    v3 n;
    float w[4];
};

// |d| - 2h < -1e-6 for float d and 2h, the difference taken in double as the
// reference takes it.  The float difference is within 2^-24 of it
// (relative), so it decides whenever it is more than 1e-6 (relative) from
// the bound; otherwise (and for NaN) the double difference decides.
__device__ __forceinline__ bool plane_close(float d, float th2) {
    const float fd = fabsf(d) - th2;
    if (fd < -1.000001e-6f) return true;
    if (fd > -0.999999e-6f) return false;
    return fabs((double)d) - (double)th2 < -1e-6;
}

// one evaluation of ExtendedVFTest's loop body at time tf (the cubic's root
// rounded to float, or 0 or 1)
__device__ __forceinline__ bool vf_eval_at(const v3 *X, const v3 *P, float th, float tf,
                                           VFResult &res) {
    v3 c0 = lerp_f(X[0], P[0], tf), c1 = lerp_f(X[1], P[1], tf);
    v3 c2 = lerp_f(X[2], P[2], tf), c3 = lerp_f(X[3], P[3], tf);
    v3 n = nrm3(cross3(sub3(P[2], P[1]), sub3(P[3], P[1])));
    v3 cn = nrm3(cross3(sub3(c2, c1), sub3(c3, c1)));
    float dist = dot3(sub3(c0, c1), cn);
    v3 w = bary(c0, c1, c2, c3);
    res.t = tf;
    res.n = n;
    res.w[0] = 1.f;
    res.w[1] = w.x;
    res.w[2] = w.y;
    res.w[3] = w.z;
    // the plane test first: the inside test only matters when it passes
    if (!plane_close(dist, 2.0f * th)) return false;
    float e1 = dist3(c1, c2), e2 = dist3(c1, c3), e3 = dist3(c2, c3);
    float es = e1 + e2 + e3;
    // epsilon = thickness / (edge sum / 3.0), a double division rounded to
    // float in the reference.  A float quotient is within a few ulps of it
    // (relative error < 1e-6), so the six inside comparisons come out the
    // same whenever every weight is more than 2^-20 max(1, epsilon) from its
    // bound; otherwise the FP64 division (a long instruction sequence on
    // this GPU) decides.
    float ea = __fdividef(3.0f * th, es);
    const float m = 9.5367431640625e-07f * fmaxf(1.f, ea);  // 2^-20 max(1, eps)
    bool clear = fabsf(w.x - (1 + ea)) > m && fabsf(w.x + ea) > m &&
                 fabsf(w.y - (1 + ea)) > m && fabsf(w.y + ea) > m &&
                 fabsf(w.z - (1 + ea)) > m && fabsf(w.z + ea) > m && isfinite(ea);
    float eps = clear ? ea : (float)((double)th / ((double)es / 3.0));
    return (w.x <= (1 + eps)) && (w.x >= (-eps)) && (w.y <= (1 + eps)) && (w.y >= (-eps)) &&
           (w.z <= (1 + eps)) && (w.z >= (-eps));
}

// true when a3 t^3 + a2 t^2 + a1 t + a0 has no root on [-d, 1+d], d = 1e-3:
// its Bernstein coefficients on that interval share one strict sign
__device__ __forceinline__ bool no_root_near_unit_f64(double a0, double a1, double a2,
                                                      double a3) {
    const double u = -1e-3, L = 1.002;
    double c0 = ((a3 * u + a2) * u + a1) * u + a0;
    double c1 = L * ((3.0 * a3 * u + 2.0 * a2) * u + a1);
    double c2 = L * L * (3.0 * a3 * u + a2);
    double c3 = L * L * L * a3;
    // the Bernstein coefficients only decide a sign with a relative margin
    // of 1e-9, so multiplying by the rounded 1/3 instead of dividing by 3
    // (an FP64 division is a long sequence on this GPU) changes nothing
    const double third = 1.0 / 3.0;
    double b0 = c0, b1 = c0 + c1 * third, b2 = c0 + 2.0 * c1 * third + c2 * third,
           b3 = c0 + c1 + c2 + c3;
    double tol = 1e-9 * (fabs(a0) + fabs(a1) + fabs(a2) + fabs(a3));
    bool pos = b0 > tol && b1 > tol && b2 > tol && b3 > tol;
    bool neg = b0 < -tol && b1 < -tol && b2 < -tol && b3 < -tol;
    return pos || neg;
}

// The same decision, computed in float first.  The coefficients are float
// values (the triple products are float); the float Bernstein coefficients
// are within ~10 ulps of sum |a| of the double ones, so when all four
// clear 1e-5 sum |a| with one sign, the double ones clear the 1e-9 sum |a|
// tolerance with that sign too, and when one clears it above and another
// below, the double ones have both signs as well (no decision of one sign:
// false).  All four zero: false, as in double.  Otherwise the double
// evaluation decides.
__device__ __forceinline__ bool no_root_near_unit(float f0, float f1, float f2, float f3) {
    const float u = -1e-3f, L = 1.002f;
    float c0 = ((f3 * u + f2) * u + f1) * u + f0;
    float c1 = L * ((3.0f * f3 * u + 2.0f * f2) * u + f1);
    float c2 = L * L * (3.0f * f3 * u + f2);
    float c3 = L * L * L * f3;
    const float third = 1.0f / 3.0f;
    float b0 = c0, b1 = c0 + c1 * third, b2 = c0 + 2.0f * c1 * third + c2 * third,
          b3 = c0 + c1 + c2 + c3;
    float tol = 1e-5f * (fabsf(f0) + fabsf(f1) + fabsf(f2) + fabsf(f3));
    if (tol > 0.f && isfinite(tol)) {
        if (b0 > tol && b1 > tol && b2 > tol && b3 > tol) return true;
        if (b0 < -tol && b1 < -tol && b2 < -tol && b3 < -tol) return true;
        const bool above = b0 > tol || b1 > tol || b2 > tol || b3 > tol;
        const bool below = b0 < -tol || b1 < -tol || b2 < -tol || b3 < -tol;
        if (above && below) return false;
    }
    if (f0 == 0.f && f1 == 0.f && f2 == 0.f && f3 == 0.f) return false;
    return no_root_near_unit_f64(f0, f1, f2, f3);
}

// distance from the origin to the segment [a, b]
__device__ __forceinline__ float seg_origin_dist(v3 a, v3 b) {
    v3 d = sub3(b, a);
    float dd = dot3(d, d);
    float t = dd > 0.f ? fminf(fmaxf(-dot3(a, d) / dd, 0.f), 1.f) : 0.f;
    v3 q = add3(a, mul3(d, t));
    return sqrtf(dot3(q, q));
}

// Bernstein coefficients on [0, 1] of a x b for linear a (a0 -> a1) and b
__device__ __forceinline__ void bern_cross(v3 a0, v3 a1, v3 b0, v3 b1, v3 c[3]) {
    c[0] = cross3(a0, b0);
    c[1] = mul3(add3(cross3(a0, b1), cross3(a1, b0)), 0.5f);
    c[2] = cross3(a1, b1);
}
// Bernstein coefficients (degree 4) of u . v for quadratics u and v
__device__ __forceinline__ void bern_dot(const v3 u[3], const v3 v[3], float c[5]) {
    c[0] = dot3(u[0], v[0]);
    c[1] = 0.5f * (dot3(u[0], v[1]) + dot3(u[1], v[0]));
    c[2] = (dot3(u[0], v[2]) + 4.f * dot3(u[1], v[1]) + dot3(u[2], v[0])) * (1.f / 6.f);
    c[3] = 0.5f * (dot3(u[1], v[2]) + dot3(u[2], v[1]));
    c[4] = dot3(u[2], v[2]);
}
__device__ __forceinline__ float len3(v3 a) { return sqrtf(dot3(a, a)); }

// True when no time of the step can pass ExtendedVFTest's inside test
// (every weight >= -eps, eps = h / mean edge): across one edge line the
// point stays outside the triangle by more than eps_max + 0.01 in
// barycentric units for every t in [0, 1], eps_max = h / the mean of the
// edges' smallest lengths over the step (edge vectors move linearly).
// With r_v = v - point (linear in t) and n = (v2 - v1) x (v3 - v1), the
// weight of vertex i is w_i = ((r_j x r_k) . n) / (n . n), (i, j, k) cyclic:
// the barycentric coordinate of the point's projection onto the triangle's
// plane.  Numerator and denominator are quartics in t; their Bernstein
// coefficients follow from the linear factors', and a Bernstein polynomial
// lies between its smallest and largest coefficient.  All five coefficients
// of N_i + e D (e = eps_max + 0.01) below -tol, tol = 1e-4 of their
// magnitude bound (well above this test's float rounding), put w_i below
// -e on the whole interval.  The 0.01 covers the rounding of the
// reference's float evaluation (interpolated positions, barycentric
// coordinates), which the guards keep far below it: the triangle is no
// sliver at either end (sin^2 of its angle at v1 >= 1e-4), n . n does not
// dip below a quarter of its smaller end value, and coordinates are within
// 1000 mean edges of the origin.
__device__ bool vf_outside_all_step(const v3 *X, const v3 *P, float th) {
    const v3 a0 = sub3(X[2], X[1]), a1 = sub3(P[2], P[1]);
    const v3 b0 = sub3(X[3], X[1]), b1 = sub3(P[3], P[1]);
    const v3 c0 = sub3(X[3], X[2]), c1 = sub3(P[3], P[2]);
    const float es = seg_origin_dist(a0, a1) + seg_origin_dist(b0, b1) + seg_origin_dist(c0, c1);
    if (!(es > 0.f)) return false;
    float big = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        big = fmaxf(big, fmaxf(fmaxf(fabsf(X[k].x), fabsf(X[k].y)),
                               fmaxf(fmaxf(fabsf(X[k].z), fabsf(P[k].x)),
                                     fmaxf(fabsf(P[k].y), fabsf(P[k].z)))));
    if (!(big <= 1000.f * (es / 3.f))) return false;
    v3 n[3];
    bern_cross(a0, a1, b0, b1, n);
    float D[5];
    bern_dot(n, n, D);
    if (!(D[0] >= 1e-4f * (dot3(a0, a0) * dot3(b0, b0)) &&
          D[4] >= 1e-4f * (dot3(a1, a1) * dot3(b1, b1))))
        return false;
    const float dmin = 0.25f * fminf(D[0], D[4]);
    if (!(D[1] >= dmin && D[2] >= dmin && D[3] >= dmin)) return false;
    const float e = 3.f * th / es * 1.0001f + 0.01f;
    const float nmag = len3(n[0]) + len3(n[1]) + len3(n[2]);
    const v3 r0[3] = {sub3(X[1], X[0]), sub3(X[2], X[0]), sub3(X[3], X[0])};
    const v3 r1[3] = {sub3(P[1], P[0]), sub3(P[2], P[0]), sub3(P[3], P[0])};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        v3 m[3];
        bern_cross(r0[j], r1[j], r0[k], r1[k], m);
        float C[5];
        bern_dot(m, n, C);
        const float tol =
            1e-4f * ((len3(m[0]) + len3(m[1]) + len3(m[2])) * nmag + e * nmag * nmag);
        if (C[0] + e * D[0] < -tol && C[1] + e * D[1] < -tol && C[2] + e * D[2] < -tol &&
            C[3] + e * D[3] < -tol && C[4] + e * D[4] < -tol)
            return true;
    }
    return false;
}

// ExtendedVFTest (P/CCD.cpp:1733-1808); X/P = start/predicted positions of
// point, f0, f1, f2.  The reference evaluates t = 0, the cubic's roots in
// [0, 1] and t = 1 in ascending order and stops at the first hit.  Three
// shortcuts keep that result: t = 0 is always the first time evaluated, so
// a hit there ends the test before any root is needed; when the
// coplanarity cubic provably has no root within 1e-3 of [0, 1], the root
// solver (Newton iterations converging to roots outside that range) adds no
// time to evaluate, leaving t = 1; and when the point provably stays outside
// the grown triangle over the whole step (vf_outside_all_step), no time can
// hit.  Only the remaining pairs run the FP64 root isolation.
//
// Split in two so a kernel can keep the root isolation off its common path:
// extended_vf_first answers for t = 0 and, when the cubic has no root near
// [0, 1], for t = 1 (returns 1 hit, 0 no hit, 2 roots needed);
// extended_vf_roots finishes a pair that needs roots (t = 0 is known not to
// hit).  extended_vf_test is the composition.
__device__ __forceinline__ void vf_coeffs(const v3 *X, const v3 *P, float a[4]) {
    v3 x0 = X[0], v0 = sub3(P[0], x0);
    v3 x1 = sub3(X[1], x0), x2 = sub3(X[2], x0), x3 = sub3(X[3], x0);
    v3 v1 = sub3(sub3(P[1], X[1]), v0), v2 = sub3(sub3(P[2], X[2]), v0),
       v3_ = sub3(sub3(P[3], X[3]), v0);
    a[0] = stp(x1, x2, x3);
    a[1] = stp(v1, x2, x3) + stp(x1, v2, x3) + stp(x1, x2, v3_);
    a[2] = stp(x1, v2, v3_) + stp(v1, x2, v3_) + stp(v1, v2, x3);
    a[3] = stp(v1, v2, v3_);
}

__device__ __forceinline__ int extended_vf_first(const v3 *X, const v3 *P, float th,
                                                 VFResult &res) {
    float a[4];
    vf_coeffs(X, P, a);
    if (vf_eval_at(X, P, th, 0.0f, res)) return 1;
    if (no_root_near_unit(a[0], a[1], a[2], a[3])) return vf_eval_at(X, P, th, 1.0f, res) ? 1 : 0;
    return 2;
}

__device__ bool extended_vf_roots(const v3 *X, const v3 *P, float th, VFResult &res) {
    float a[4];
    vf_coeffs(X, P, a);
    const double a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
    double t[5];
    int nsol = solve_cubic(a3, a2, a1, a0, t);
    t[nsol] = 1;
    t[nsol + 1] = 0;
    int m = nsol + 2;
    for (int i = 1; i < m; ++i) {
        double v = t[i];
        int j = i - 1;
        while (j >= 0 && t[j] > v) {
            t[j + 1] = t[j];
            --j;
        }
        t[j + 1] = v;
    }
    for (int i = 0; i < m; ++i) {
        if (t[i] < 0 || t[i] > 1) continue;
        if (vf_eval_at(X, P, th, (float)t[i], res)) return true;
    }
    return false;
}

// a pair extended_vf_first left open: no hit when the point stays outside
// over the whole step, else the roots
__device__ bool extended_vf_rest(const v3 *X, const v3 *P, float th, VFResult &res) {
    if (vf_outside_all_step(X, P, th)) return false;
    return extended_vf_roots(X, P, th, res);
}

__device__ bool extended_vf_test(const v3 *X, const v3 *P, float th, VFResult &res) {
    int r = extended_vf_first(X, P, th, res);
    if (r != 2) return r == 1;
    return extended_vf_rest(X, P, th, res);
}

// ---- the reference's other vertex-face tests ------------------------------
// min(a, b, c) of the reference (P/CCD_Basic.h:184): std::min(a, std::min(b, c)),
// whose comparisons decide NaN cases
__device__ __forceinline__ double ref_min3(double a, double b, double c) {
    double m = (c < b) ? c : b;
    return (m < a) ? m : a;
}

// NarrowVFCCDTest (P/CCD.cpp:1810-1872) and VFCCDTest with type VF
// (P/CCD.cpp:2308-2421): the coplanarity cubic's roots in [0, 1], in the
// order solve_cubic returns them (t = 1 is stored but never visited, t = 0
// not at all); a hit where the point lies in the plane (|d| < 1e-6) and
// inside the triangle: within epsilon = thickness / mean predicted edge
// (narrow) or with every weight >= 1e-6 (vfccd).  A miss leaves the last
// evaluated root's t, w and n in res, as the reference leaves its Contact.
__device__ bool vf_roots_test(const v3 *X, const v3 *P, float th, bool narrow, VFResult &res) {
    float a[4];
    vf_coeffs(X, P, a);
    double t[4];
    int nsol = solve_cubic(a[3], a[2], a[1], a[0], t);
    for (int i = 0; i < nsol; ++i) {
        if (t[i] < 0 || t[i] > 1) continue;
        v3 c0 = lerp_t(X[0], P[0], t[i]), c1 = lerp_t(X[1], P[1], t[i]);
        v3 c2 = lerp_t(X[2], P[2], t[i]), c3 = lerp_t(X[3], P[3], t[i]);
        v3 n = nrm3(cross3(sub3(P[2], P[1]), sub3(P[3], P[1])));
        v3 cn = nrm3(cross3(sub3(c2, c1), sub3(c3, c1)));
        double d = dot3(sub3(c0, c1), cn);
        v3 w = bary(c0, c1, c2, c3);
        res.t = (float)t[i];
        res.n = n;
        res.w[0] = 1.f;
        res.w[1] = w.x;
        res.w[2] = w.y;
        res.w[3] = w.z;
        bool in;
        if (narrow) {
            float es = dist3(P[1], P[2]) + dist3(P[1], P[3]) + dist3(P[2], P[3]);
            float eps = (float)((double)th / ((double)es / 3.0));
            in = (w.x <= (1 + eps)) && (w.x >= (-eps)) && (w.y <= (1 + eps)) &&
                 (w.y >= (-eps)) && (w.z <= (1 + eps)) && (w.z >= (-eps));
        } else {
            in = ref_min3(w.x, w.y, w.z) >= 1e-6;
        }
        if (fabs(d) < 1e-6 && in) return true;
    }
    return false;
}

// Point2Plane (P/CCD.cpp:27-44): |N . v + D| / |N|, N the face's
// unnormalised normal, in float
__device__ __forceinline__ float point_to_plane(v3 v, v3 p1, v3 p2, v3 p3) {
    v3 N = cross3(sub3(p2, p1), sub3(p3, p1));
    float D = -(N.x * p1.x + N.y * p1.y + N.z * p1.z);
    float mod = N.x * v.x + N.y * v.y + N.z * v.z + D;
    float area = sqrtf(N.x * N.x + N.y * N.y + N.z * N.z);
    return fabsf(mod) / area;
}

// VFDCDTest (P/CCD.cpp:2265-2306): the predicted point within 2 thickness of
// the predicted face's plane and inside it (every weight >= 1e-6); t = 0,
// the normal of the normalised edges
__device__ bool vf_dcd_test(const v3 *P, float th, VFResult &res) {
    float d = point_to_plane(P[0], P[1], P[2], P[3]);
    if ((double)(d - 2 * th) >= -1e-6) return false;
    v3 w = bary(P[0], P[1], P[2], P[3]);
    res.w[0] = 1.f;
    res.w[1] = w.x;
    res.w[2] = w.y;
    res.w[3] = w.z;
    res.n = nrm3(cross3(nrm3(sub3(P[2], P[1])), nrm3(sub3(P[3], P[1]))));
    res.t = 0.0f;
    return ref_min3(w.x, w.y, w.z) >= 1e-6;
}

// the narrowphase tests by PBD_VFTEST_* value: 0 ExtendedVFTest, 1
// NarrowVFCCDTest, 2 VFCCDTest, 3 VFDCDTest, 4 VFTest = VFCCDTest ||
// VFDCDTest (P/CCD.cpp:2229-2263)
__device__ bool vf_test_mode(const v3 *X, const v3 *P, float th, int mode, VFResult &res) {
    switch (mode) {
        case 1: return vf_roots_test(X, P, th, true, res);
        case 2: return vf_roots_test(X, P, th, false, res);
        case 3: return vf_dcd_test(P, th, res);
        case 4: return vf_roots_test(X, P, th, false, res) || vf_dcd_test(P, th, res);
        default: return extended_vf_test(X, P, th, res);
    }
}

// closest distance from point p to triangle abc (Ericson, Real-Time
// Collision Detection, 5.1.5), float
__device__ float point_tri_dist(v3 p, v3 a, v3 b, v3 c) {
    v3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
    float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) return sqrtf(dot3(ap, ap));
    v3 bp = sub3(p, b);
    float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.f && d4 <= d3) return sqrtf(dot3(bp, bp));
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
        float v = d1 / (d1 - d3);
        v3 q = sub3(p, add3(a, mul3(ab, v)));
        return sqrtf(dot3(q, q));
    }
    v3 cp = sub3(p, c);
    float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.f && d5 <= d6) return sqrtf(dot3(cp, cp));
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
        float w = d2 / (d2 - d6);
        v3 q = sub3(p, add3(a, mul3(ac, w)));
        return sqrtf(dot3(q, q));
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        v3 q = sub3(p, add3(b, mul3(sub3(c, b), w)));
        return sqrtf(dot3(q, q));
    }
    float den = 1.f / (va + vb + vc);
    float v = vb * den, w = vc * den;
    v3 q = sub3(p, add3(a, add3(mul3(ab, v), mul3(ac, w))));
    return sqrtf(dot3(q, q));
}

__device__ __forceinline__ bool sliver(v3 a, v3 b, v3 c) {
    v3 e1 = sub3(b, a), e2 = sub3(c, a);
    v3 n = cross3(e1, e2);
    return !(dot3(n, n) > 1e-10f * (dot3(e1, e1) * dot3(e2, e2)));
}

__device__ __forceinline__ uint32_t teschner(int x, int y, int z) {
    return ((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349663u) ^ ((uint32_t)z * 83492791u);
}

struct GridParams {
    float3 start, cell;
    int3 size;
    int hashed;
    uint32_t nb;  // buckets (bounded: cells; sentinel key = nb)
};

__device__ __forceinline__ bool outside(const GridParams &g, int x, int y, int z) {
    return x < 0 || y < 0 || z < 0 || x >= g.size.x || y >= g.size.y || z >= g.size.z;
}
// bucket of a cell; in hashed mode the instance is mixed in, so instances
// that overlap in space (batched cloths) do not share buckets
__device__ __forceinline__ uint32_t bucket_of(const GridParams &g, int x, int y, int z,
                                              int inst) {
    if (g.hashed) return (teschner(x, y, z) ^ ((uint32_t)inst * 0x9E3779B1u)) & (g.nb - 1u);
    return ((uint32_t)z * (uint32_t)g.size.y) * (uint32_t)g.size.x +
           (uint32_t)y * (uint32_t)g.size.x + (uint32_t)x;
}

// the cell size of an instance (the spatial hash's per-instance cells, or
// its one cell)
__device__ __forceinline__ float3 inst_cell_of(const GridParams &g, const float4 *ic, int n_ic,
                                               int inst) {
    if (inst >= 0 && inst < n_ic) {
        float4 c = ic[inst];
        return make_float3(c.x, c.y, c.z);
    }
    return g.cell;
}

// Append a warp's staged pairs (stage[0, cnt), filled by the whole warp) to
// out with one atomic on *counter; slots at or past cap are dropped and set
// flag_bit in *flags.  Called by all 32 lanes.
__device__ __forceinline__ void warp_flush_pairs(const int2 *stage, int cnt, int lane, int2 *out,
                                                 long long cap, int *counter, int *flags,
                                                 int flag_bit) {
    int base = 0;
    if (lane == 0) base = atomicAdd(counter, cnt);
    base = __shfl_sync(0xffffffffu, base, 0);
    bool over = false;
    for (int l = lane; l < cnt; l += 32) {
        const long long slot = (long long)base + l;
        if (slot < cap)
            out[slot] = stage[l];
        else
            over = true;
    }
    if (__any_sync(0xffffffffu, over) && lane == 0) atomicOr(flags, flag_bit);
    __syncwarp();
}

// Stage this lane's pair (when hit) in the warp's buffer of `size` pairs,
// flushing it first when the 32 new ones might not fit.  Called by all 32
// lanes with the warp's running count cnt.
__device__ __forceinline__ void warp_stage_pair(bool hit, int2 pr, int2 *stage, int size,
                                                int &cnt, int lane, int2 *out, long long cap,
                                                int *counter, int *flags, int flag_bit) {
    const unsigned hm = __ballot_sync(0xffffffffu, hit);
    if (!hm) return;
    if (cnt + 32 > size) {
        warp_flush_pairs(stage, cnt, lane, out, cap, counter, flags, flag_bit);
        cnt = 0;
    }
    if (hit) stage[cnt + __popc(hm & ((1u << lane) - 1u))] = pr;
    cnt += __popc(hm);
    __syncwarp();
}

// one atomic per group of lanes that reach this call together
__device__ __forceinline__ int agg_inc(int *counter) {
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counter, (int)g.size());
    return g.shfl(base, 0) + (int)g.thread_rank();
}

__device__ __forceinline__ void add_fixed(long long *acc, int pt, float dx, float dy, float dz) {
    atomicAdd((unsigned long long *)(acc + 3 * (long long)pt), (unsigned long long)__float2ll_rn(dx * 4294967296.0f));
    atomicAdd((unsigned long long *)(acc + 3 * (long long)pt + 1), (unsigned long long)__float2ll_rn(dy * 4294967296.0f));
    atomicAdd((unsigned long long *)(acc + 3 * (long long)pt + 2), (unsigned long long)__float2ll_rn(dz * 4294967296.0f));
}


GridParams params_of(const pbd_shs *h) {
    GridParams g;
    g.start = make_float3(h->start[0], h->start[1], h->start[2]);
    g.cell = make_float3(h->cell[0], h->cell[1], h->cell[2]);
    g.size = make_int3(h->size[0], h->size[1], h->size[2]);
    g.hashed = h->hashed;
    g.nb = (uint32_t)h->n_buckets;
    return g;
}

}  // namespace
}  // namespace pbd

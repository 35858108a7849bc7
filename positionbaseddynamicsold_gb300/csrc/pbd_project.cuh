// pbd_project.cuh -- the per-constraint projections of the colored
// Gauss-Seidel sweep (distance, dihedral bending, anchor), shared by every
// launch form.  Include only from translation units compiled with
// -fmad=false: the arithmetic mirrors the reference's operation by
// operation, every product rounded before the following add.
//
// Each projection is split into its arithmetic (new positions from old ones
// and the stiffness factor k = 1 - (1 - s)^(1/(iter+1))) and the load /
// store around it, so a launch form may load the points of several records
// before writing any (no two records of a color share a point) or take k
// from a table; the arithmetic, and so the result, is the same either way.
#pragma once

#include <cuda_runtime.h>

namespace pbd {
namespace {

// Position accessor of the per-color kernel: the global array.
struct GlobalPos {
    float4 *p;
    __device__ __forceinline__ float4 ld(int i) const { return p[i]; }
    __device__ __forceinline__ void st(int i, float4 v) const { p[i] = v; }
};

// Stiffness factor k of a constraint with stiffness s in the sweep whose
// exponent is expk = 1/(iter+1), by schedule (PBD_SCHEDULE_*):
//   0  1 - (1 - s)^expk   ProjectContraintsGPUKernel (P/PBD_cuda.cu:1282)
//   1  1                  projectConstraintCPU (P/PBD_cuda.cu:1119, k = 1)
//   2  s                  the stiffness itself, every sweep
__device__ __forceinline__ float stiffness_factor(float s, float expk, int sched) {
    if (sched == 1) return 1.f;
    if (sched == 2) return s;
    return 1.f - powf(1.f - s, expk);
}

// distance constraint of ProjectContraintsGPUKernel (P/PBD_cuda.cu:1264-1294):
// false when the constraint leaves both points where they are
__device__ __forceinline__ bool distance_update(float4 P0, float4 P1, float rest, float k,
                                                float4 &N0, float4 &N1) {
    float m0 = P0.w, m1 = P1.w;
    float msum = m0 + m1;
    float dx = P0.x - P1.x, dy = P0.y - P1.y, dz = P0.z - P1.z;
    float d = sqrtf(dx * dx + dy * dy + dz * dz);
    if (msum == 0.f || d == 0.f) return false;
    float s0 = -m0 / msum * (d - rest);
    float s1 = m1 / msum * (d - rest);
    N0 = make_float4(P0.x + ((dx * s0) / d) * k, P0.y + ((dy * s0) / d) * k,
                     P0.z + ((dz * s0) / d) * k, m0);
    N1 = make_float4(P1.x + ((dx * s1) / d) * k, P1.y + ((dy * s1) / d) * k,
                     P1.z + ((dz * s1) / d) * k, m1);
    return true;
}

template <class Pos>
__device__ __forceinline__ void project_distance(int4 r, const Pos &p, float expk, int sched) {
    float4 P0 = p.ld(r.x), P1 = p.ld(r.y), N0, N1;
    float k = stiffness_factor(__int_as_float(r.w), expk, sched);
    if (!distance_update(P0, P1, __int_as_float(r.z), k, N0, N1)) return;
    p.st(r.x, N0);
    p.st(r.y, N1);
}

struct v3 {
    float x, y, z;
};
__device__ __forceinline__ v3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ v3 sub3(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ v3 add3(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ v3 mul3(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ v3 div3(v3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross3(v3 a, v3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// dihedral bending: signed angle theta = atan2((nA x nB).E/|E|, nA.nB),
// C = theta - theta0, dp_i = w_i * k*C/sum_j w_j|u_j|^2 * u_i with the
// Bridson-Marino-Fedkiw (2003) gradients grad_i theta = -u_i, inside the
// PBD projection of Mueller et al. (2007).  Same operation order as the
// oracle's orc_bending_project_f32.  Q = e0, e1, wA, wB; false when the
// constraint leaves its points where they are.
__device__ __forceinline__ bool bending_update(const float4 Q[4], float theta0, float k,
                                               float4 N[4]) {
    v3 e0 = mk3(Q[0].x, Q[0].y, Q[0].z), e1 = mk3(Q[1].x, Q[1].y, Q[1].z);
    v3 wa = mk3(Q[2].x, Q[2].y, Q[2].z), wb = mk3(Q[3].x, Q[3].y, Q[3].z);
    v3 E = sub3(e1, e0);
    v3 na = cross3(sub3(wa, e0), sub3(wa, e1));
    v3 nb = cross3(sub3(wb, e1), sub3(wb, e0));
    float na2 = dot3(na, na), nb2 = dot3(nb, nb), el2 = dot3(E, E);
    if (na2 == 0.f || nb2 == 0.f || el2 == 0.f) return false;
    float el = sqrtf(el2);
    float sn = dot3(cross3(na, nb), E) / el;
    float cs = dot3(na, nb);
    float c = atan2f(sn, cs) - theta0;
    if (c > 3.14159265f) c -= 6.28318531f;
    if (c < -3.14159265f) c += 6.28318531f;
    v3 a = div3(na, na2), b = div3(nb, nb2);
    v3 uwa = mul3(a, el), uwb = mul3(b, el);
    v3 ue0 = add3(mul3(a, dot3(sub3(wa, e1), E) / el), mul3(b, dot3(sub3(wb, e1), E) / el));
    v3 ue1 = sub3(mul3(a, -dot3(sub3(wa, e0), E) / el), mul3(b, dot3(sub3(wb, e0), E) / el));
    float den = Q[0].w * dot3(ue0, ue0) + Q[1].w * dot3(ue1, ue1) + Q[2].w * dot3(uwa, uwa) +
                Q[3].w * dot3(uwb, uwb);
    if (!(den > 0.f)) return false;
    float s = k * c / den;
    v3 n0 = add3(e0, mul3(ue0, Q[0].w * s));
    v3 n1 = add3(e1, mul3(ue1, Q[1].w * s));
    v3 n2 = add3(wa, mul3(uwa, Q[2].w * s));
    v3 n3 = add3(wb, mul3(uwb, Q[3].w * s));
    N[0] = make_float4(n0.x, n0.y, n0.z, Q[0].w);
    N[1] = make_float4(n1.x, n1.y, n1.z, Q[1].w);
    N[2] = make_float4(n2.x, n2.y, n2.z, Q[2].w);
    N[3] = make_float4(n3.x, n3.y, n3.z, Q[3].w);
    return true;
}

template <class Pos>
__device__ __forceinline__ void project_bending(int4 r, float2 par, const Pos &p, float expk,
                                                int sched) {
    float4 Q[4] = {p.ld(r.x), p.ld(r.y), p.ld(r.z), p.ld(r.w)}, N[4];
    if (!bending_update(Q, par.x, stiffness_factor(par.y, expk, sched), N)) return;
    p.st(r.x, N[0]);
    p.st(r.y, N[1]);
    p.st(r.z, N[2]);
    p.st(r.w, N[3]);
}

// ANCHOR (P/PBD_cuda.cu:1298-1305): snap the point to its rest position
template <class Pos>
__device__ __forceinline__ void project_anchor(float4 a, const Pos &p) {
    int i = __float_as_int(a.w);
    p.st(i, make_float4(a.x, a.y, a.z, p.ld(i).w));
}

}  // namespace
}  // namespace pbd

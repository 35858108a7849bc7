/*
 * pbd_oracle.c -- CPU restatement of the reference PBD cloth step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): loaded by
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg.
 *
 * Reference paths are relative to
 * PositionBasedDynamicsCUDA/PositionBasedDynamicsCUDA/ of
 * vivienldy/PositionBasedDynamicsOld ("P/" below).  Each routine states the
 * reference lines it follows; where the reference reads uninitialised memory
 * or divides by zero the restatement says what it does instead.
 *
 * Build: cc -O2 -ffp-contract=off -fPIC -shared (see oracle/build_oracle.py).
 */
#include "pbd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Host threads for the loops whose iterations are independent (CCD
 * detection per triangle or point, projections within one color, the
 * response's per-contact corrections).  Every merge that the reference does
 * in order (contact storage with its duplicate scan, the sequential GS and
 * response) stays sequential, so results do not depend on the count. */
static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n > 0 ? n : 1; }
int orc_get_threads(void)
{
#ifdef _OPENMP
    return g_threads;
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* float3 arithmetic in the operation order of the reference's host code */
/* ------------------------------------------------------------------ */
typedef struct { float x, y, z; } f3;

static inline f3 mk(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 ld3(const float *p) { return mk(p[0], p[1], p[2]); }
static inline void st3(float *p, f3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
static inline f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 mul(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline f3 divs(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross(f3 a, f3 b)
{
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* normalize: v * (1/sqrt(v.v)) -- the host form used by P/CCD.cpp */
static inline f3 nrm(f3 v)
{
    float inv = 1.0f / sqrtf(dot(v, v));
    return mul(v, inv);
}
/* Distance (P/PBD_cuda.cu:3-6, P/PBD_Basic.cuh:321-324): the sum of the
 * three squared differences, then the square root.  The reference spells
 * both as powf (x^2 and s^0.5); with g_pow_distance set the oracle does the
 * same (used when pinning against the reference's compiled code), otherwise
 * it uses the correctly rounded x*x and sqrtf that the CUDA kernels use. */
static int g_pow_distance = 0;
void orc_set_pow_distance(int on) { g_pow_distance = on; }
static inline float dist3(f3 a, f3 b)
{
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    if (g_pow_distance)
        return powf(powf(dx, 2.0f) + powf(dy, 2.0f) + powf(dz, 2.0f), 0.5f);
    return sqrtf(dx * dx + dy * dy + dz * dz);
}
/* stp (P/CCD_Basic.h:181): u . (v x w) in float */
static inline float stp(f3 u, f3 v, f3 w) { return dot(u, cross(v, w)); }
/* pos (P/CCD.cpp:8-11): the double t is narrowed to float for the product */
static inline f3 lerp_t(f3 a, f3 b, double t)
{
    float tf = (float)t;
    f3 d = sub(b, a);
    return add(a, mk(tf * d.x, tf * d.y, tf * d.z));
}
/* BarycentricCoord (P/CCD.cpp:115-130): weights of p0, p1, p2 from the
 * Gram matrix of the two edges out of p2 (Ericson, Real-Time Collision
 * Detection, 3.4). */
static inline f3 bary(f3 pos, f3 p0, f3 p1, f3 p2)
{
    f3 ab = sub(p0, p2), ac = sub(p1, p2), ap = sub(pos, p2);
    float d00 = dot(ac, ac), d01 = dot(ac, ab), d02 = dot(ac, ap);
    float d11 = dot(ab, ab), d12 = dot(ab, ap);
    float inv = 1.0f / (d00 * d11 - d01 * d01);
    float v = (d11 * d02 - d01 * d12) * inv;
    float u = (d00 * d12 - d01 * d02) * inv;
    float w = 1.0f - u - v;
    return mk(u, v, w);
}

/* ------------------------------------------------------------------ */
/* constraint graph and coloring                                        */
/* ------------------------------------------------------------------ */

int64_t orc_prim2prims(int n_prims, const int *prim_list, const int *indices,
                       int n_points, int *adj_start_num, int *adj_idx)
{
    /* point -> prims map in prim id order (GenePoint2PrimsMap,
     * P/PBD_cuda.cu:155-168) as CSR */
    int *cnt = (int *)calloc((size_t)n_points + 1, sizeof(int));
    for (int p = 0; p < n_prims; ++p)
        for (int i = 0; i < prim_list[2 * p + 1]; ++i)
            cnt[indices[prim_list[2 * p] + i] + 1]++;
    for (int i = 0; i < n_points; ++i) cnt[i + 1] += cnt[i];
    int64_t total_inc = cnt[n_points];
    int *inc = (int *)malloc(sizeof(int) * (size_t)(total_inc > 0 ? total_inc : 1));
    int *fill = (int *)malloc(sizeof(int) * ((size_t)n_points + 1));
    memcpy(fill, cnt, sizeof(int) * ((size_t)n_points + 1));
    for (int p = 0; p < n_prims; ++p)
        for (int i = 0; i < prim_list[2 * p + 1]; ++i)
            inc[fill[indices[prim_list[2 * p] + i]]++] = p;
    /* prim -> linked prims (GenePrim2PrimsMap, P/PBD_cuda.cu:170-202) */
    int64_t total = 0;
    for (int p = 0; p < n_prims; ++p) {
        int64_t start = total;
        for (int i = 0; i < prim_list[2 * p + 1]; ++i) {
            int pt = indices[prim_list[2 * p] + i];
            for (int j = cnt[pt]; j < cnt[pt + 1]; ++j) {
                int q = inc[j];
                if (q == p) continue;
                if (adj_idx) adj_idx[total] = q;
                total++;
            }
        }
        if (adj_start_num) {
            adj_start_num[2 * p] = (int)start;
            adj_start_num[2 * p + 1] = (int)(total - start);
        }
    }
    free(cnt);
    free(inc);
    free(fill);
    return total;
}

/* speculative color of one prim: first color not used by a coloured
 * neighbour, searched in windows of 64 (P/PBD_cuda.cu:335-370) */
static int first_free_color(int idx, const int *adj_start_num, const int *adj_idx,
                            const int *color)
{
    int nidx = adj_start_num[2 * idx];
    int nlast = nidx + adj_start_num[2 * idx + 1];
    int offset = 0;
    for (;;) {
        uint64_t forbidden = 0;
        for (int i = nidx; i < nlast; ++i) {
            int nc = color[adj_idx[i]] - offset;
            if (nc >= 0 && nc < 64) forbidden |= (1ull << nc);
        }
        if (forbidden != ~0ull) return offset + __builtin_ctzll(~forbidden);
        offset += 64;
    }
}

void orc_assign_colors(int n_prims, const int *adj_start_num, const int *adj_idx,
                       const int *color, int *prd_color)
{
    for (int idx = 0; idx < n_prims; ++idx) {
        if (color[idx] >= 0) continue;
        prd_color[idx] = first_free_color(idx, adj_start_num, adj_idx, color);
    }
}

/* conflict test (P/PBD_cuda.cu:400-422): a neighbour with the same
 * speculative color wins if it has more points, or as many and a lower id */
static int loses(int idx, const int *prim_list, const int *adj_start_num,
                 const int *adj_idx, const int *prd_color)
{
    int c = prd_color[idx];
    int npt = prim_list[2 * idx + 1];
    int nidx = adj_start_num[2 * idx];
    int nlast = nidx + adj_start_num[2 * idx + 1];
    for (int i = nidx; i < nlast; ++i) {
        int n = adj_idx[i];
        if (prd_color[n] != c) continue;
        int nnpt = prim_list[2 * n + 1];
        if (nnpt > npt || (nnpt == npt && n < idx)) return 1;
    }
    return 0;
}

int orc_resolve_conflicts_gpu(int n_prims, const int *prim_list,
                              const int *adj_start_num, const int *adj_idx,
                              int *color, const int *prd_color)
{
    int flag = 0;
    for (int idx = 0; idx < n_prims; ++idx) {
        if (color[idx] >= 0) continue;
        if (loses(idx, prim_list, adj_start_num, adj_idx, prd_color))
            flag = 1;
        else
            color[idx] = prd_color[idx];
    }
    return flag;
}

int orc_resolve_conflicts_cpu(int n_prims, const int *prim_list,
                              const int *adj_start_num, const int *adj_idx,
                              int *color, const int *prd_color)
{
    for (int idx = 0; idx < n_prims; ++idx) {
        if (color[idx] >= 0) continue;
        if (loses(idx, prim_list, adj_start_num, adj_idx, prd_color)) return 1;
        color[idx] = prd_color[idx];
    }
    return 0;
}

int orc_edge_coloring_gpu(int n_prims, const int *prim_list,
                          const int *adj_start_num, const int *adj_idx,
                          int *color, int *prd_color, int max_iters)
{
    int it = 0;
    while (it < max_iters) {
        orc_assign_colors(n_prims, adj_start_num, adj_idx, color, prd_color);
        int flag = orc_resolve_conflicts_gpu(n_prims, prim_list, adj_start_num,
                                             adj_idx, color, prd_color);
        ++it;
        if (!flag) break;
    }
    return it;
}

int orc_edge_coloring_cpu(int n_prims, const int *prim_list,
                          const int *adj_start_num, const int *adj_idx,
                          int *color, int *prd_color, int max_iters)
{
    int it = 0;
    while (it < max_iters) {
        orc_assign_colors(n_prims, adj_start_num, adj_idx, color, prd_color);
        int flag = orc_resolve_conflicts_cpu(n_prims, prim_list, adj_start_num,
                                             adj_idx, color, prd_color);
        ++it;
        if (!flag) break;
    }
    return it;
}

void orc_sort_edges_colors(int n, int *color, int *sorted_prim_id)
{
    /* stable counting sort on color (colors are >= -1) */
    if (n <= 0) return;
    int cmax = -1;
    for (int i = 0; i < n; ++i) if (color[i] > cmax) cmax = color[i];
    int nb = cmax + 2;
    int *cnt = (int *)calloc((size_t)nb + 1, sizeof(int));
    for (int i = 0; i < n; ++i) cnt[color[i] + 2]++;
    for (int b = 0; b < nb; ++b) cnt[b + 1] += cnt[b];
    int *c2 = (int *)malloc(sizeof(int) * (size_t)n);
    int *s2 = (int *)malloc(sizeof(int) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        int pos = cnt[color[i] + 1]++;
        c2[pos] = color[i];
        s2[pos] = sorted_prim_id[i];
    }
    memcpy(color, c2, sizeof(int) * (size_t)n);
    memcpy(sorted_prim_id, s2, sizeof(int) * (size_t)n);
    free(cnt);
    free(c2);
    free(s2);
}

int orc_eval_worksets(int n, const int *sorted_color, int *worksets)
{
    int nw = 0;
    int start = 0;
    for (int i = 1; i <= n; ++i) {
        if (i == n || sorted_color[i] != sorted_color[i - 1]) {
            if (n > 0) {
                worksets[2 * nw] = start;
                worksets[2 * nw + 1] = i - start;
                nw++;
            }
            start = i;
        }
    }
    return nw;
}

/* ------------------------------------------------------------------ */
/* solver                                                               */
/* ------------------------------------------------------------------ */

void orc_advect_gpu(int n, float dt, float damp_pow, const float *gravity,
                    const float *mass, float *vel, float *prdp, const float *pos)
{
    f3 g = ld3(gravity);
    for (int i = 0; i < n; ++i) {
        f3 v = ld3(vel + 3 * i);
        /* v += gravity*dt*mass; v *= damping^dt; p = x + v*dt
         * (P/PBD_cuda.cu:968-972) */
        f3 gdt = mul(g, dt);
        v = add(v, mul(gdt, mass[i]));
        v = mul(v, damp_pow);
        st3(vel + 3 * i, v);
        st3(prdp + 3 * i, add(ld3(pos + 3 * i), mul(v, dt)));
    }
}

void orc_advect_cpu(int n, float dt, const float *gravity, float *vel,
                    float *prdp, const float *pos)
{
    f3 g = ld3(gravity);
    for (int i = 0; i < n; ++i) {
        f3 v = add(ld3(vel + 3 * i), mul(g, dt)); /* P/PBD_cuda.cu:1005 */
        st3(vel + 3 * i, v);
        st3(prdp + 3 * i, add(ld3(pos + 3 * i), mul(v, dt)));
    }
}

void orc_integrate(int n, float dt, float *vel, const float *prdp, float *pos)
{
    for (int i = 0; i < n; ++i) {
        f3 p = ld3(prdp + 3 * i);
        st3(vel + 3 * i, divs(sub(p, ld3(pos + 3 * i)), dt));
        st3(pos + 3 * i, p);
    }
}

/* Stiffness schedule (orc_set_stiffness_schedule): 0 = k = 1 - (1-s)^(1/(iter+1))
 * (P/PBD_cuda.cu:1282; the exponent is computed in double and narrowed to
 * float by powf's parameter), 1 = k = 1 (projectConstraintCPU,
 * P/PBD_cuda.cu:1119), 2 = k = s. */
static int g_schedule = 0;

void orc_set_stiffness_schedule(int mode)
{
    g_schedule = mode;
}

static inline float stiff_k(float s, int iter)
{
    if (g_schedule == 1) return 1.0f;
    if (g_schedule == 2) return s;
    return 1.0f - powf(1.0f - s, (float)(1.0 / (double)(iter + 1)));
}

static void project_distance(int i0, int i1, float rest, float k,
                             const float *mass, float *prdp)
{
    f3 p0 = ld3(prdp + 3 * i0), p1 = ld3(prdp + 3 * i1);
    float m0 = mass[i0], m1 = mass[i1];
    float msum = m0 + m1;
    float d = dist3(p0, p1);
    if (msum == 0.0f || d == 0.0f) return;
    f3 v = sub(p0, p1);
    /* P/PBD_cuda.cu:1280-1290 */
    float s0 = -m0 / msum * (d - rest);
    float s1 = m1 / msum * (d - rest);
    f3 dp0 = divs(mul(v, s0), d);
    f3 dp1 = divs(mul(v, s1), d);
    dp0 = mul(dp0, k);
    dp1 = mul(dp1, k);
    st3(prdp + 3 * i0, add(p0, dp0));
    st3(prdp + 3 * i1, add(ld3(prdp + 3 * i1), dp1));
}

/* ---- dihedral bending (no reference code: P/PBD_cuda.cu:110-123 is an
 * empty stub).  Constraint C = theta - theta0 on the signed dihedral angle
 * theta = atan2((n1^ x n2^).e^, n1^.n2^), projected with the PBD step of
 * Mueller et al. 2007 (dp_i = -w_i C grad_i / sum_j w_j |grad_j|^2) using the
 * gradients of Bridson, Marino & Fedkiw 2003: grad_i theta = -u_i with
 *   u_wA = |E| nA/|nA|^2, u_wB = |E| nB/|nB|^2,
 *   u_e0 = ((wA-e1).E/|E|) nA/|nA|^2 + ((wB-e1).E/|E|) nB/|nB|^2,
 *   u_e1 = -((wA-e0).E/|E|) nA/|nA|^2 - ((wB-e0).E/|E|) nB/|nB|^2,
 * nA = (wA-e0)x(wA-e1), nB = (wB-e1)x(wB-e0), E = e1-e0.
 * Point order of a bending prim: e0, e1 (hinge), wA, wB (wings). */
int orc_bending_project_f32(float *P0, float *P1, float *P2, float *P3,
                            const float *w, float rest_angle, float k)
{
    f3 e0 = ld3(P0), e1 = ld3(P1), wa = ld3(P2), wb = ld3(P3);
    f3 E = sub(e1, e0);
    f3 na = cross(sub(wa, e0), sub(wa, e1));
    f3 nb = cross(sub(wb, e1), sub(wb, e0));
    float na2 = dot(na, na), nb2 = dot(nb, nb), el2 = dot(E, E);
    if (na2 == 0.0f || nb2 == 0.0f || el2 == 0.0f) return 0;
    float el = sqrtf(el2);
    float sn = dot(cross(na, nb), E) / el;
    float cs = dot(na, nb);
    float c = atan2f(sn, cs) - rest_angle;
    if (c > 3.14159265f) c -= 6.28318531f;
    if (c < -3.14159265f) c += 6.28318531f;
    f3 a = divs(na, na2), b = divs(nb, nb2);
    f3 uwa = mul(a, el), uwb = mul(b, el);
    f3 ue0 = add(mul(a, dot(sub(wa, e1), E) / el), mul(b, dot(sub(wb, e1), E) / el));
    f3 ue1 = sub(mul(a, -dot(sub(wa, e0), E) / el), mul(b, dot(sub(wb, e0), E) / el));
    float den = w[0] * dot(ue0, ue0) + w[1] * dot(ue1, ue1) + w[2] * dot(uwa, uwa) +
                w[3] * dot(uwb, uwb);
    if (!(den > 0.0f)) return 0;
    float s = k * c / den;
    st3(P0, add(e0, mul(ue0, w[0] * s)));
    st3(P1, add(e1, mul(ue1, w[1] * s)));
    st3(P2, add(wa, mul(uwa, w[2] * s)));
    st3(P3, add(wb, mul(uwb, w[3] * s)));
    return 1;
}

typedef struct { double x, y, z; } d3;
static inline d3 dmk(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 dld(const double *p) { return dmk(p[0], p[1], p[2]); }
static inline void dst(double *p, d3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
static inline d3 dadd(d3 a, d3 b) { return dmk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 dsub(d3 a, d3 b) { return dmk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 dmul(d3 a, double s) { return dmk(a.x * s, a.y * s, a.z * s); }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 dcross(d3 a, d3 b)
{
    return dmk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

double orc_dihedral_angle(const double *P0, const double *P1, const double *P2,
                          const double *P3)
{
    d3 e0 = dld(P0), e1 = dld(P1), wa = dld(P2), wb = dld(P3);
    d3 E = dsub(e1, e0);
    d3 na = dcross(dsub(wa, e0), dsub(wa, e1));
    d3 nb = dcross(dsub(wb, e1), dsub(wb, e0));
    double el = sqrt(ddot(E, E));
    if (el == 0.0) return 0.0;
    return atan2(ddot(dcross(na, nb), E) / el, ddot(na, nb));
}

int orc_bending_project_f64(double *P0, double *P1, double *P2, double *P3,
                            const double *w, double rest_angle, double k)
{
    d3 e0 = dld(P0), e1 = dld(P1), wa = dld(P2), wb = dld(P3);
    d3 E = dsub(e1, e0);
    d3 na = dcross(dsub(wa, e0), dsub(wa, e1));
    d3 nb = dcross(dsub(wb, e1), dsub(wb, e0));
    double na2 = ddot(na, na), nb2 = ddot(nb, nb), el2 = ddot(E, E);
    if (na2 == 0.0 || nb2 == 0.0 || el2 == 0.0) return 0;
    double el = sqrt(el2);
    double c = atan2(ddot(dcross(na, nb), E) / el, ddot(na, nb)) - rest_angle;
    if (c > M_PI) c -= 2.0 * M_PI;
    if (c < -M_PI) c += 2.0 * M_PI;
    d3 a = dmul(na, 1.0 / na2), b = dmul(nb, 1.0 / nb2);
    d3 uwa = dmul(a, el), uwb = dmul(b, el);
    d3 ue0 = dadd(dmul(a, ddot(dsub(wa, e1), E) / el), dmul(b, ddot(dsub(wb, e1), E) / el));
    d3 ue1 = dsub(dmul(a, -ddot(dsub(wa, e0), E) / el), dmul(b, ddot(dsub(wb, e0), E) / el));
    double den = w[0] * ddot(ue0, ue0) + w[1] * ddot(ue1, ue1) + w[2] * ddot(uwa, uwa) +
                 w[3] * ddot(uwb, uwb);
    if (!(den > 0.0)) return 0;
    double s = k * c / den;
    dst(P0, dadd(e0, dmul(ue0, w[0] * s)));
    dst(P1, dadd(e1, dmul(ue1, w[1] * s)));
    dst(P2, dadd(wa, dmul(uwa, w[2] * s)));
    dst(P3, dadd(wb, dmul(uwb, w[3] * s)));
    return 1;
}

static void project_bending(const orc_constraints *c, int prim, float k,
                            const float *mass, float *prdp, int fp64)
{
    const int *ix = c->indices + c->prim_list[2 * prim];
    float rest = c->rest_angle ? c->rest_angle[prim] : 0.0f;
    if (!fp64) {
        float w[4] = {mass[ix[0]], mass[ix[1]], mass[ix[2]], mass[ix[3]]};
        orc_bending_project_f32(prdp + 3 * ix[0], prdp + 3 * ix[1], prdp + 3 * ix[2],
                                prdp + 3 * ix[3], w, rest, k);
        return;
    }
    double p[4][3], w[4];
    for (int j = 0; j < 4; ++j) {
        for (int d = 0; d < 3; ++d) p[j][d] = prdp[3 * ix[j] + d];
        w[j] = mass[ix[j]];
    }
    if (orc_bending_project_f64(p[0], p[1], p[2], p[3], w, rest, k))
        for (int j = 0; j < 4; ++j)
            for (int d = 0; d < 3; ++d) prdp[3 * ix[j] + d] = (float)p[j][d];
}

void orc_project_one(const orc_constraints *c, int prim, int iter,
                     const float *mass, float *prdp, int bending_fp64)
{
    int t = c->ctype[prim];
    int s = c->prim_list[2 * prim];
    if (t == ORC_DISTANCE) {
        float k = stiff_k(c->stiffness[prim], iter);
        project_distance(c->indices[s], c->indices[s + 1], c->rest_length[prim], k,
                         mass, prdp);
    } else if (t == ORC_BENDING) {
        float k = stiff_k(c->stiffness[prim], iter);
        project_bending(c, prim, k, mass, prdp, bending_fp64);
    } else if (t == ORC_ANCHOR) {
        /* anchor: snap the point to its rest position (P/PBD_cuda.cu:1298-1305,
         * with the rest position stored per anchor prim) */
        if (c->rest_pos) {
            int i = c->indices[s];
            prdp[3 * i] = c->rest_pos[3 * prim];
            prdp[3 * i + 1] = c->rest_pos[3 * prim + 1];
            prdp[3 * i + 2] = c->rest_pos[3 * prim + 2];
        }
    }
}

void orc_project_colored(const orc_constraints *c, const int *sorted_prim_id,
                         int n_worksets, const int *worksets, int iter_begin,
                         int iter_end, const float *mass, float *prdp,
                         int bending_fp64)
{
    /* constraints of one color share no point: any order gives the same
     * positions */
    for (int it = iter_begin; it < iter_end; ++it)
        for (int w = 0; w < n_worksets; ++w) {
            const int a = worksets[2 * w], b = worksets[2 * w] + worksets[2 * w + 1];
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1 && b - a > 4096)
#endif
            for (int i = a; i < b; ++i)
                orc_project_one(c, sorted_prim_id[i], it, mass, prdp, bending_fp64);
        }
}

void orc_colli_sphere(int n, float *prdp, const float *center, float radius)
{
    f3 o = ld3(center);
    for (int i = 0; i < n; ++i) {
        f3 p = ld3(prdp + 3 * i);
        float d = dist3(p, o);
        if (d - radius > 0.001f) continue; /* ColliderSphere, P/PBD_cuda.cu:1542-1553 */
        /* GenerateMoveVectorSphere (P/PBD_cuda.cu:1567-1573) */
        float move = radius - dist3(o, p);
        f3 dir = divs(sub(p, o), dist3(o, p));
        st3(prdp + 3 * i, add(p, mul(dir, move)));
    }
}

void orc_project_cpu_range(const orc_constraints *c, const float *mass, float *prdp,
                           int p0, int p1)
{
    for (int i = p0; i < p1; ++i) {
        if (c->prim_list[2 * i + 1] != 2) continue;
        int i0 = c->indices[c->prim_list[2 * i]];
        int i1 = c->indices[c->prim_list[2 * i] + 1];
        f3 p0v = ld3(prdp + 3 * i0), p1v = ld3(prdp + 3 * i1);
        float d = dist3(p0v, p1v);
        /* normalize as compiled in the reference's .cu translation unit:
         * the host rsqrtf there evaluates 1/sqrt in double */
        f3 r0 = sub(p0v, p1v);
        f3 r = mul(r0, (float)(1.0 / sqrt((double)dot(r0, r0))));
        float m0 = mass[i0], m1 = mass[i1];
        float rest = c->rest_length[i];
        /* P/PBD_cuda.cu:1113-1123, k = 1 */
        f3 dp1 = mk(-m0 / (m0 + m1) * (d - rest) * r.x, -m0 / (m0 + m1) * (d - rest) * r.y,
                    -m0 / (m0 + m1) * (d - rest) * r.z);
        f3 dp2 = mk(m1 / (m0 + m1) * (d - rest) * r.x, m1 / (m0 + m1) * (d - rest) * r.y,
                    m1 / (m0 + m1) * (d - rest) * r.z);
        dp1 = mul(dp1, 1.0f);
        dp2 = mul(dp2, 1.0f);
        st3(prdp + 3 * i0, add(p0v, dp1));
        st3(prdp + 3 * i1, add(ld3(prdp + 3 * i1), dp2));
    }
}

void orc_project_cpu(const orc_constraints *c, int iterations,
                     const float *mass, float *prdp, int n_points,
                     const float *sphere_center, float sphere_radius)
{
    for (int ii = 0; ii < iterations; ++ii) {
        orc_project_cpu_range(c, mass, prdp, 0, c->n_prims);
        if (sphere_center) orc_colli_sphere(n_points, prdp, sphere_center, sphere_radius);
    }
}

double orc_residual(const orc_constraints *c, const float *prdp,
                    const float *hinge_rest, double *num_out, double *den_out)
{
    double num = 0.0, den = 0.0;
    for (int p = 0; p < c->n_prims; ++p) {
        const int *ix = c->indices + c->prim_list[2 * p];
        if (c->ctype[p] == ORC_DISTANCE) {
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = (double)prdp[3 * ix[0] + k] - prdp[3 * ix[1] + k];
            double l = c->rest_length[p];
            double cc = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - l;
            num += cc * cc;
            den += l * l;
        } else if (c->ctype[p] == ORC_BENDING) {
            double q[4][3];
            for (int j = 0; j < 4; ++j)
                for (int k = 0; k < 3; ++k) q[j][k] = prdp[3 * ix[j] + k];
            double th = orc_dihedral_angle(q[0], q[1], q[2], q[3]);
            double cc = th - (c->rest_angle ? c->rest_angle[p] : 0.0);
            if (cc > M_PI) cc -= 2.0 * M_PI;
            if (cc < -M_PI) cc += 2.0 * M_PI;
            double e[3];
            for (int k = 0; k < 3; ++k) e[k] = q[1][k] - q[0][k];
            double el = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            double lr = hinge_rest ? hinge_rest[p] : el;
            num += (cc * el) * (cc * el);
            den += lr * lr;
        }
    }
    if (num_out) *num_out = num;
    if (den_out) *den_out = den;
    return den > 0.0 ? sqrt(num) / sqrt(den) : 0.0;
}

/* ------------------------------------------------------------------ */
/* broadphase                                                           */
/* ------------------------------------------------------------------ */

void orc_grid_init(orc_grid *g, const float *center, const int *size,
                   const float *cell, int bounded)
{
    for (int k = 0; k < 3; ++k) {
        g->size[k] = size ? size[k] : 0;
        g->cell[k] = cell[k];
        /* shift = (gridSize * cellSize) / 2 (P/SpatialHashSystem.cpp:91-94) */
        float shift = ((float)(unsigned)g->size[k] * cell[k]) / 2.0f;
        g->start[k] = center[k] - shift;
    }
    g->bounded = bounded;
}

static inline void tri_cell(const orc_grid *g, const int *tri, const float *pos,
                            int *out)
{
    f3 a = ld3(pos + 3 * tri[0]), b = ld3(pos + 3 * tri[1]), c = ld3(pos + 3 * tri[2]);
    /* centroid (P/SpatialHashSystem.cpp:291-293) and cell
     * (P/SpatialHashSystem.cpp:394-396) */
    float cx = (a.x + b.x + c.x) / 3.0f;
    float cy = (a.y + b.y + c.y) / 3.0f;
    float cz = (a.z + b.z + c.z) / 3.0f;
    out[0] = (int)floorf((cx - g->start[0]) / g->cell[0]);
    out[1] = (int)floorf((cy - g->start[1]) / g->cell[1]);
    out[2] = (int)floorf((cz - g->start[2]) / g->cell[2]);
}

void orc_tri_cells(const orc_grid *g, int n_tris, const int *tri_idx,
                   const float *pos, int *cell_xyz)
{
    for (int t = 0; t < n_tris; ++t) tri_cell(g, tri_idx + 3 * t, pos, cell_xyz + 3 * t);
}

static inline int outside(const orc_grid *g, const int *c)
{
    return c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= g->size[0] ||
           c[1] >= g->size[1] || c[2] >= g->size[2];
}

int orc_cell_hash(const orc_grid *g, const int *c)
{
    if (outside(g, c)) return -1;
    return (int)(((unsigned)c[2] * (unsigned)g->size[1]) * (unsigned)g->size[0] +
                 (unsigned)c[1] * (unsigned)g->size[0] + (unsigned)c[0]);
}

/* 64-bit key of an unbounded cell: 21 bits per axis, offset 2^20 */
static inline uint64_t cell_key(const int *c)
{
    return ((uint64_t)(uint32_t)(c[2] + (1 << 20)) << 42) |
           ((uint64_t)(uint32_t)(c[1] + (1 << 20)) << 21) |
           (uint64_t)(uint32_t)(c[0] + (1 << 20));
}

typedef struct { uint64_t key; int id; } keyid;
static int cmp_keyid(const void *a, const void *b)
{
    const keyid *x = (const keyid *)a, *y = (const keyid *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->id - y->id; /* stable: ties by id */
}

/* sorted (cell key, triangle id) table with lookup */
typedef struct { keyid *e; int n; } cell_table;

static cell_table build_table(const orc_grid *g, int n_tris, const int *tri_idx,
                              const float *pos, int *cells)
{
    cell_table t;
    t.e = (keyid *)malloc(sizeof(keyid) * (size_t)(n_tris > 0 ? n_tris : 1));
    t.n = 0;
    for (int i = 0; i < n_tris; ++i) {
        tri_cell(g, tri_idx + 3 * i, pos, cells + 3 * i);
        if (g->bounded && outside(g, cells + 3 * i)) continue;
        uint64_t k = g->bounded ? (uint64_t)orc_cell_hash(g, cells + 3 * i)
                                : cell_key(cells + 3 * i);
        t.e[t.n].key = k;
        t.e[t.n].id = i;
        t.n++;
    }
    qsort(t.e, (size_t)t.n, sizeof(keyid), cmp_keyid);
    return t;
}

static int table_lower(const cell_table *t, uint64_t key)
{
    int lo = 0, hi = t->n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (t->e[mid].key < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* FindNeighbors (P/SpatialHashSystem.cpp:134-187) of one triangle into a
 * growable list; returns the count */
static int neighbors_of(const orc_grid *g, const cell_table *t, const int *cells, int tri,
                        int **buf, int *cap)
{
    int n = 0;
    const int *c = cells + 3 * tri;
    if (g->bounded && outside(g, c)) return 0;
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                int nc[3] = {c[0] + x, c[1] + y, c[2] + z};
                if (g->bounded && outside(g, nc)) continue;
                uint64_t key = g->bounded ? (uint64_t)orc_cell_hash(g, nc) : cell_key(nc);
                for (int i = table_lower(t, key); i < t->n && t->e[i].key == key; ++i) {
                    if (t->e[i].id == tri) continue;
                    if (n == *cap) {
                        *cap *= 2;
                        *buf = (int *)realloc(*buf, sizeof(int) * (size_t)*cap);
                    }
                    (*buf)[n++] = t->e[i].id;
                }
            }
    return n;
}

int64_t orc_find_neighbors_all(const orc_grid *g, int n_tris, const int *tri_idx,
                               const float *pos, int *out_start_num, int *out_idx)
{
    int *cells = (int *)malloc(sizeof(int) * 3 * (size_t)(n_tris > 0 ? n_tris : 1));
    cell_table t = build_table(g, n_tris, tri_idx, pos, cells);
    int cap = 1024;
    int *buf = (int *)malloc(sizeof(int) * (size_t)cap);
    int64_t total = 0;
    for (int tri = 0; tri < n_tris; ++tri) {
        int n = neighbors_of(g, &t, cells, tri, &buf, &cap);
        if (out_idx) memcpy(out_idx + total, buf, sizeof(int) * (size_t)n);
        if (out_start_num) {
            out_start_num[2 * tri] = (int)total;
            out_start_num[2 * tri + 1] = n;
        }
        total += n;
    }
    free(buf);
    free(t.e);
    free(cells);
    return total;
}

/* ------------------------------------------------------------------ */
/* narrowphase                                                          */
/* ------------------------------------------------------------------ */

static inline double sgn(double x) { return x < 0 ? -1.0 : 1.0; }

int orc_solve_quadratic(double a, double b, double c, double x[2])
{
    /* P/CCD.cpp:96-113 */
    double d = b * b - 4 * a * c;
    if (d < 0) {
        x[0] = -b / (2 * a);
        return 0;
    }
    double q = -(b + sgn(b) * sqrt(d)) / 2;
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

double orc_newtons_method(double a, double b, double c, double d, double x0,
                          int init_dir)
{
    /* P/CCD.cpp:75-94 */
    if (init_dir != 0) {
        double y0 = d + x0 * (c + x0 * (b + x0 * a));
        double ddy0 = 2 * b + x0 * (6 * a);
        x0 += init_dir * sqrt(fabs(2 * y0 / ddy0));
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

int orc_solve_cubic(double a, double b, double c, double d, double x[3])
{
    /* P/CCD.cpp:48-73.  When the derivative quadratic yields no critical
     * point without writing one (d >= 0 and both guards fail), the reference
     * starts Newton from an uninitialised value; 0.0 is used here. */
    double xc[2] = {0.0, 0.0};
    int ncrit = orc_solve_quadratic(3 * a, 2 * b, c, xc);
    if (ncrit == 0) {
        x[0] = orc_newtons_method(a, b, c, d, xc[0], 0);
        return 1;
    } else if (ncrit == 1) {
        return orc_solve_quadratic(b, c, d, x);
    } else {
        double yc[2] = {d + xc[0] * (c + xc[0] * (b + xc[0] * a)),
                        d + xc[1] * (c + xc[1] * (b + xc[1] * a))};
        int i = 0;
        if (yc[0] * a >= 0) x[i++] = orc_newtons_method(a, b, c, d, xc[0], -1);
        if (yc[0] * yc[1] <= 0) {
            int closer = fabs(yc[0]) < fabs(yc[1]) ? 0 : 1;
            x[i++] = orc_newtons_method(a, b, c, d, xc[closer], closer == 0 ? 1 : -1);
        }
        if (yc[1] * a <= 0) x[i++] = orc_newtons_method(a, b, c, d, xc[1], 1);
        return i;
    }
}

static void sort_small(double *t, int n)
{
    for (int i = 1; i < n; ++i) {
        double v = t[i];
        int j = i - 1;
        while (j >= 0 && t[j] > v) {
            t[j + 1] = t[j];
            --j;
        }
        t[j + 1] = v;
    }
}

/* cubic coefficients of the coplanarity condition (P/CCD.cpp:1740-1743) */
static void vf_cubic(const float *x, const float *p, double *a)
{
    f3 x0 = ld3(x), v0 = sub(ld3(p), x0);
    f3 x1 = sub(ld3(x + 3), x0), x2 = sub(ld3(x + 6), x0), x3 = sub(ld3(x + 9), x0);
    f3 v1 = sub(sub(ld3(p + 3), ld3(x + 3)), v0);
    f3 v2 = sub(sub(ld3(p + 6), ld3(x + 6)), v0);
    f3 v3 = sub(sub(ld3(p + 9), ld3(x + 9)), v0);
    a[0] = stp(x1, x2, x3);
    a[1] = stp(v1, x2, x3) + stp(x1, v2, x3) + stp(x1, x2, v3);
    a[2] = stp(x1, v2, v3) + stp(v1, x2, v3) + stp(v1, v2, x3);
    a[3] = stp(v1, v2, v3);
}

/* inside test with the thickness-relative epsilon (P/CCD.cpp:1768-1781);
 * the division by 3.0 is in double */
static inline int inside_eps(f3 w, float e1, float e2, float e3, float thickness)
{
    float eps = (float)((double)thickness / ((double)(e1 + e2 + e3) / 3.0));
    return (w.x <= (1 + eps)) && (w.x >= (-eps)) && (w.y <= (1 + eps)) &&
           (w.y >= (-eps)) && (w.z <= (1 + eps)) && (w.z >= (-eps));
}

int orc_extended_vf_test(const float *x, const float *p, float thickness,
                         int i0, int i1, int i2, int i3, orc_contact *ct)
{
    if (i0 == i1 || i0 == i2 || i0 == i3) return 0;
    double a[4];
    vf_cubic(x, p, a);
    double t[5];
    int nsol = orc_solve_cubic(a[3], a[2], a[1], a[0], t);
    t[nsol] = 1;
    t[nsol + 1] = 0;
    sort_small(t, nsol + 2);
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    for (int i = 0; i < nsol + 2; ++i) {
        if (t[i] < 0 || t[i] > 1) continue;
        f3 c0 = lerp_t(X0, P0, t[i]), c1 = lerp_t(X1, P1, t[i]);
        f3 c2 = lerp_t(X2, P2, t[i]), c3 = lerp_t(X3, P3, t[i]);
        f3 n = nrm(cross(sub(P2, P1), sub(P3, P1)));
        f3 cn = nrm(cross(sub(c2, c1), sub(c3, c1)));
        double dist = dot(sub(c0, c1), cn);
        f3 w = bary(c0, c1, c2, c3);
        if (ct) {
            ct->t = (float)t[i];
            ct->n[0] = n.x; ct->n[1] = n.y; ct->n[2] = n.z;
            ct->w[0] = 1; ct->w[1] = w.x; ct->w[2] = w.y; ct->w[3] = w.z;
        }
        int in = inside_eps(w, dist3(c1, c2), dist3(c1, c3), dist3(c2, c3), thickness);
        /* P/CCD.cpp:1800 */
        if ((fabs(dist) - (double)(2.0f * thickness) < -1e-6) && in) return 1;
    }
    return 0;
}

int orc_narrow_vf_ccd_test(const float *x, const float *p, float thickness,
                           int i0, int i1, int i2, int i3, orc_contact *ct)
{
    if (i0 == i1 || i0 == i2 || i0 == i3) return 0;
    double a[4];
    vf_cubic(x, p, a);
    double t[4];
    int nsol = orc_solve_cubic(a[3], a[2], a[1], a[0], t);
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    for (int i = 0; i < nsol; ++i) {
        if (t[i] < 0 || t[i] > 1) continue;
        f3 c0 = lerp_t(X0, P0, t[i]), c1 = lerp_t(X1, P1, t[i]);
        f3 c2 = lerp_t(X2, P2, t[i]), c3 = lerp_t(X3, P3, t[i]);
        f3 n = nrm(cross(sub(P2, P1), sub(P3, P1)));
        f3 cn = nrm(cross(sub(c2, c1), sub(c3, c1)));
        double d = dot(sub(c0, c1), cn);
        f3 w = bary(c0, c1, c2, c3);
        if (ct) {
            ct->t = (float)t[i];
            ct->n[0] = n.x; ct->n[1] = n.y; ct->n[2] = n.z;
            ct->w[0] = 1; ct->w[1] = w.x; ct->w[2] = w.y; ct->w[3] = w.z;
        }
        /* P/CCD.cpp:1845-1863: epsilon from the predicted edges */
        int in = inside_eps(w, dist3(P1, P2), dist3(P1, P3), dist3(P2, P3), thickness);
        if (fabs(d) < 1e-6 && in) return 1;
    }
    return 0;
}

/* min(a, b, c) of the reference (P/CCD_Basic.h:184): std::min(a,
 * std::min(b, c)), whose comparisons decide NaN cases */
static double ref_min3(double a, double b, double c)
{
    double m = (c < b) ? c : b;
    return (m < a) ? m : a;
}

/* free VFCCDTest with type VF (P/CCD.cpp:2308-2421): the cubic's roots in
 * the order solve_cubic returns them (t = 1 is stored but never visited);
 * a hit where the point lies in the triangle's plane (|d| < 1e-6) with
 * every barycentric weight >= 1e-6 (no epsilon) */
int orc_vf_ccd_test(const float *x, const float *p, float thickness, int i0, int i1, int i2,
                    int i3, orc_contact *ct)
{
    (void)thickness;
    (void)i0; (void)i1; (void)i2; (void)i3;
    double a[4];
    vf_cubic(x, p, a);
    double t[4];
    int nsol = orc_solve_cubic(a[3], a[2], a[1], a[0], t);
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    for (int i = 0; i < nsol; ++i) {
        if (t[i] < 0 || t[i] > 1) continue;
        f3 c0 = lerp_t(X0, P0, t[i]), c1 = lerp_t(X1, P1, t[i]);
        f3 c2 = lerp_t(X2, P2, t[i]), c3 = lerp_t(X3, P3, t[i]);
        f3 n = nrm(cross(sub(P2, P1), sub(P3, P1)));
        f3 cn = nrm(cross(sub(c2, c1), sub(c3, c1)));
        double d = dot(sub(c0, c1), cn);
        f3 w = bary(c0, c1, c2, c3);
        if (ct) {
            ct->t = (float)t[i];
            ct->n[0] = n.x; ct->n[1] = n.y; ct->n[2] = n.z;
            ct->w[0] = 1; ct->w[1] = w.x; ct->w[2] = w.y; ct->w[3] = w.z;
        }
        if (fabs(d) < 1e-6 && ref_min3(w.x, w.y, w.z) >= 1e-6) return 1;
    }
    return 0;
}

/* Point2Plane (P/CCD.cpp:27-44): |n . v + D| / |n|, n the unnormalised
 * face normal, in float */
static float point_to_plane(f3 v, f3 p1, f3 p2, f3 p3)
{
    f3 N = cross(sub(p2, p1), sub(p3, p1));
    float D = -(N.x * p1.x + N.y * p1.y + N.z * p1.z);
    float mod = N.x * v.x + N.y * v.y + N.z * v.z + D;
    float area = sqrtf(N.x * N.x + N.y * N.y + N.z * N.z);
    return fabsf(mod) / area;
}

/* free VFDCDTest (P/CCD.cpp:2265-2306): the predicted point closer than
 * 2 thickness to the predicted face's plane and inside it (every weight
 * >= 1e-6); t = 0, the normal of the normalised edges */
int orc_vf_dcd_test(const float *x, const float *p, float thickness, int i0, int i1, int i2,
                    int i3, orc_contact *ct)
{
    (void)x;
    (void)i0; (void)i1; (void)i2; (void)i3;
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    float d = point_to_plane(P0, P1, P2, P3);
    if ((double)(d - 2 * thickness) >= -1e-6) return 0;
    f3 w = bary(P0, P1, P2, P3);
    if (ct) {
        ct->w[0] = 1; ct->w[1] = w.x; ct->w[2] = w.y; ct->w[3] = w.z;
        f3 n = nrm(cross(nrm(sub(P2, P1)), nrm(sub(P3, P1))));
        ct->n[0] = n.x; ct->n[1] = n.y; ct->n[2] = n.z;
        ct->t = 0.0f;
    }
    return ref_min3(w.x, w.y, w.z) >= 1e-6;
}

/* free VFTest (P/CCD.cpp:2229-2263): VFCCDTest, else VFDCDTest (the
 * second writes the contact over whatever the first left) */
int orc_vf_test(const float *x, const float *p, float thickness, int i0, int i1, int i2, int i3,
                orc_contact *ct)
{
    if (orc_vf_ccd_test(x, p, thickness, i0, i1, i2, i3, ct)) return 1;
    return orc_vf_dcd_test(x, p, thickness, i0, i1, i2, i3, ct);
}

/* ExtendedVFTest restated entirely in FP64, the accuracy yardstick of the
 * reference-arithmetic test above (which mixes float geometry with double
 * cubic coefficients and stops Newton at |dx| < 1e-6): the same times 0,
 * roots in [0, 1] and 1, but every quantity in double and every root
 * polished by Newton steps to |dx| < 1e-14.  Returns the same hit
 * decision rule with the double quantities. */
static double polish_root(const double *a, double t)
{
    for (int k = 0; k < 50; ++k) {
        double y = a[0] + t * (a[1] + t * (a[2] + t * a[3]));
        double dy = a[1] + t * (2 * a[2] + t * 3 * a[3]);
        if (dy == 0) break;
        double t1 = t - y / dy;
        if (fabs(t1 - t) < 1e-14) return t1;
        t = t1;
    }
    return t;
}

int orc_extended_vf_test_f64(const float *x, const float *p, float thickness, int i0, int i1,
                             int i2, int i3, orc_contact *ct)
{
    if (i0 == i1 || i0 == i2 || i0 == i3) return 0;
    d3 X[4], P[4];
    for (int j = 0; j < 4; ++j) {
        X[j] = dmk(x[3 * j], x[3 * j + 1], x[3 * j + 2]);
        P[j] = dmk(p[3 * j], p[3 * j + 1], p[3 * j + 2]);
    }
    d3 x0 = X[0], v0 = dsub(P[0], x0);
    d3 x1 = dsub(X[1], x0), x2 = dsub(X[2], x0), x3 = dsub(X[3], x0);
    d3 v1 = dsub(dsub(P[1], X[1]), v0), v2 = dsub(dsub(P[2], X[2]), v0),
       v3 = dsub(dsub(P[3], X[3]), v0);
    double a[4];
    a[0] = ddot(x1, dcross(x2, x3));
    a[1] = ddot(v1, dcross(x2, x3)) + ddot(x1, dcross(v2, x3)) + ddot(x1, dcross(x2, v3));
    a[2] = ddot(x1, dcross(v2, v3)) + ddot(v1, dcross(x2, v3)) + ddot(v1, dcross(v2, x3));
    a[3] = ddot(v1, dcross(v2, v3));
    double t[5];
    int nsol = orc_solve_cubic(a[3], a[2], a[1], a[0], t);
    for (int i = 0; i < nsol; ++i) t[i] = polish_root(a, t[i]);
    t[nsol] = 1;
    t[nsol + 1] = 0;
    sort_small(t, nsol + 2);
    double h = (double)thickness;
    for (int i = 0; i < nsol + 2; ++i) {
        if (t[i] < 0 || t[i] > 1) continue;
        d3 c[4];
        for (int j = 0; j < 4; ++j) c[j] = dadd(X[j], dmul(dsub(P[j], X[j]), t[i]));
        d3 cn = dcross(dsub(c[2], c[1]), dsub(c[3], c[1]));
        double ln = sqrt(ddot(cn, cn));
        if (!(ln > 0)) continue;
        cn = dmul(cn, 1.0 / ln);
        double dist = ddot(dsub(c[0], c[1]), cn);
        /* barycentric weights of c0 in (c1, c2, c3) (Ericson 3.4) */
        d3 ab = dsub(c[1], c[3]), ac = dsub(c[2], c[3]), ap = dsub(c[0], c[3]);
        double d00 = ddot(ac, ac), d01 = ddot(ac, ab), d02 = ddot(ac, ap);
        double d11 = ddot(ab, ab), d12 = ddot(ab, ap);
        double inv = 1.0 / (d00 * d11 - d01 * d01);
        double wv = (d11 * d02 - d01 * d12) * inv;
        double wu = (d00 * d12 - d01 * d02) * inv;
        double ww = 1.0 - wu - wv;
        double e1 = sqrt(ddot(dsub(c[1], c[2]), dsub(c[1], c[2])));
        double e2 = sqrt(ddot(dsub(c[1], c[3]), dsub(c[1], c[3])));
        double e3 = sqrt(ddot(dsub(c[2], c[3]), dsub(c[2], c[3])));
        double eps = h / ((e1 + e2 + e3) / 3.0);
        int in = wu <= 1 + eps && wu >= -eps && wv <= 1 + eps && wv >= -eps && ww <= 1 + eps &&
                 ww >= -eps;
        if (ct) {
            ct->t = (float)t[i];
            ct->w[0] = 1;
            ct->w[1] = wu;
            ct->w[2] = wv;
            ct->w[3] = ww;
            ct->n[0] = (float)cn.x;
            ct->n[1] = (float)cn.y;
            ct->n[2] = (float)cn.z;
        }
        if (fabs(dist) - 2.0 * h < -1e-6 && in) {
            if (ct) ct->t = (float)t[i];
            return 1;
        }
    }
    return 0;
}

static void gather4(const int *ids, const float *src, float *dst)
{
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) dst[3 * j + k] = src[3 * ids[j] + k];
}

int64_t orc_ccd_sh_extended_ref(const orc_grid *g, int n_tris, const int *tri_idx,
                                const float *pos, const float *prdp,
                                float thickness, orc_contact *out, int64_t cap)
{
    return orc_ccd_sh_extended_ref_range(g, n_tris, tri_idx, pos, prdp, thickness, 0, n_tris,
                                         out, cap);
}

struct orc_sh_table {
    int *cells;
    cell_table tb;
};

orc_sh_table *orc_sh_build(const orc_grid *g, int n_tris, const int *tri_idx, const float *prdp)
{
    orc_sh_table *t = (orc_sh_table *)malloc(sizeof(orc_sh_table));
    t->cells = (int *)malloc(sizeof(int) * 3 * (size_t)(n_tris > 0 ? n_tris : 1));
    t->tb = build_table(g, n_tris, tri_idx, prdp, t->cells);
    return t;
}

void orc_sh_free(orc_sh_table *t)
{
    if (!t) return;
    free(t->tb.e);
    free(t->cells);
    free(t);
}

int64_t orc_ccd_sh_extended_ref_range_tab(const orc_grid *g, const orc_sh_table *t, int n_tris,
                                          const int *tri_idx, const float *pos,
                                          const float *prdp, float thickness, int tri_begin,
                                          int tri_end, orc_contact *out, int64_t cap)
{
    /* per triangle of the range, FindNeighbors and the point x neighbor
     * loop (P/CCD.cpp:1541-1586) over a table UpdateSH built */
    const int *cells = t->cells;
    const cell_table tb = t->tb;
    int nbcap = 1024;
    int *nb = (int *)malloc(sizeof(int) * (size_t)nbcap);
    int64_t h = 0;
    int64_t hcap = 1024;
    int *keys = (int *)malloc(sizeof(int) * 4 * (size_t)hcap);
    if (tri_begin < 0) tri_begin = 0;
    if (tri_end > n_tris) tri_end = n_tris;
    for (int tri = tri_begin; tri < tri_end; ++tri) {
        int nn = neighbors_of(g, &tb, cells, tri, &nb, &nbcap);
        for (int j = 0; j < 3; ++j) {
            int ids[4];
            ids[0] = tri_idx[3 * tri + j];
            for (int q = 0; q < nn; ++q) {
                int nt = nb[q];
                ids[1] = tri_idx[3 * nt];
                ids[2] = tri_idx[3 * nt + 1];
                ids[3] = tri_idx[3 * nt + 2];
                float xs[12], ps[12];
                gather4(ids, pos, xs);
                gather4(ids, prdp, ps);
                orc_contact ct;
                if (!orc_extended_vf_test(xs, ps, thickness, ids[0], ids[1], ids[2], ids[3], &ct))
                    continue;
                /* IsDuplicated: linear scan of the stored contacts */
                int dup = 0;
                for (int64_t k = 0; k < h; ++k)
                    if (keys[4 * k] == ids[0] && keys[4 * k + 1] == ids[1] &&
                        keys[4 * k + 2] == ids[2] && keys[4 * k + 3] == ids[3]) {
                        dup = 1;
                        break;
                    }
                if (dup) continue;
                if (h == hcap) {
                    hcap *= 2;
                    keys = (int *)realloc(keys, sizeof(int) * 4 * (size_t)hcap);
                }
                memcpy(keys + 4 * h, ids, sizeof(ids));
                ct.v = ids[0]; ct.f0 = ids[1]; ct.f1 = ids[2]; ct.f2 = ids[3];
                ct.face = nt;
                if (out && h < cap) out[h] = ct;
                h++;
            }
        }
    }
    free(keys);
    free(nb);
    return h;
}

/* Hits of one slice of triangles in the loop order of
 * orc_ccd_sh_extended_ref_range_tab, before the duplicate scan. */
typedef struct {
    int64_t n, cap;
    orc_contact *c;
} raw_hits;

static void detect_slice(const orc_grid *g, const orc_sh_table *t, const int *tri_idx,
                         const float *pos, const float *prdp, float thickness, int tri_begin,
                         int tri_end, raw_hits *out)
{
    int nbcap = 1024;
    int *nb = (int *)malloc(sizeof(int) * (size_t)nbcap);
    out->n = 0;
    out->cap = 256;
    out->c = (orc_contact *)malloc(sizeof(orc_contact) * (size_t)out->cap);
    for (int tri = tri_begin; tri < tri_end; ++tri) {
        int nn = neighbors_of(g, &t->tb, t->cells, tri, &nb, &nbcap);
        for (int j = 0; j < 3; ++j) {
            int ids[4];
            ids[0] = tri_idx[3 * tri + j];
            for (int q = 0; q < nn; ++q) {
                int nt = nb[q];
                ids[1] = tri_idx[3 * nt];
                ids[2] = tri_idx[3 * nt + 1];
                ids[3] = tri_idx[3 * nt + 2];
                float xs[12], ps[12];
                gather4(ids, pos, xs);
                gather4(ids, prdp, ps);
                orc_contact ct;
                if (!orc_extended_vf_test(xs, ps, thickness, ids[0], ids[1], ids[2], ids[3], &ct))
                    continue;
                ct.v = ids[0]; ct.f0 = ids[1]; ct.f1 = ids[2]; ct.f2 = ids[3];
                ct.face = nt;
                if (out->n == out->cap) {
                    out->cap *= 2;
                    out->c = (orc_contact *)realloc(out->c, sizeof(orc_contact) * (size_t)out->cap);
                }
                out->c[out->n++] = ct;
            }
        }
    }
    free(nb);
}

int64_t orc_ccd_sh_extended_ref_range_tab_mt(const orc_grid *g, const orc_sh_table *t,
                                             int n_tris, const int *tri_idx, const float *pos,
                                             const float *prdp, float thickness, int tri_begin,
                                             int tri_end, orc_contact *out, int64_t cap)
{
    /* The triangle loop of CCD_SH_Extended (P/CCD.cpp:1541-1586) split into
     * consecutive slices detected on g_threads threads; the slices' hits
     * are then stored in loop order with the reference's IsDuplicated
     * linear scan (P/CCD.cpp:132-147), so the contact list equals the
     * sequential one. */
    if (tri_begin < 0) tri_begin = 0;
    if (tri_end > n_tris) tri_end = n_tris;
    int n = tri_end - tri_begin;
    if (n <= 0) return 0;
    int nsl = orc_get_threads() * 16;
    if (nsl > n) nsl = n;
    raw_hits *rh = (raw_hits *)calloc((size_t)nsl, sizeof(raw_hits));
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 1)
#endif
    for (int k = 0; k < nsl; ++k) {
        int a = tri_begin + (int)((int64_t)n * k / nsl);
        int b = tri_begin + (int)((int64_t)n * (k + 1) / nsl);
        detect_slice(g, t, tri_idx, pos, prdp, thickness, a, b, rh + k);
    }
    int64_t h = 0, hcap = 1024;
    int *keys = (int *)malloc(sizeof(int) * 4 * (size_t)hcap);
    for (int k = 0; k < nsl; ++k) {
        for (int64_t i = 0; i < rh[k].n; ++i) {
            const orc_contact *ct = rh[k].c + i;
            int ids[4] = {ct->v, ct->f0, ct->f1, ct->f2};
            int dup = 0;
            for (int64_t q = 0; q < h; ++q)
                if (keys[4 * q] == ids[0] && keys[4 * q + 1] == ids[1] &&
                    keys[4 * q + 2] == ids[2] && keys[4 * q + 3] == ids[3]) {
                    dup = 1;
                    break;
                }
            if (dup) continue;
            if (h == hcap) {
                hcap *= 2;
                keys = (int *)realloc(keys, sizeof(int) * 4 * (size_t)hcap);
            }
            memcpy(keys + 4 * h, ids, sizeof(ids));
            if (out && h < cap) out[h] = *ct;
            h++;
        }
        free(rh[k].c);
    }
    free(rh);
    free(keys);
    return h;
}

int64_t orc_ccd_sh_extended_ref_range(const orc_grid *g, int n_tris, const int *tri_idx,
                                      const float *pos, const float *prdp, float thickness,
                                      int tri_begin, int tri_end, orc_contact *out, int64_t cap)
{
    /* UpdateSH(prdP) (binning of every triangle, P/CCD.cpp:1530-1540), then
     * the range */
    orc_sh_table *t = orc_sh_build(g, n_tris, tri_idx, prdp);
    int64_t h = orc_get_threads() > 1
                    ? orc_ccd_sh_extended_ref_range_tab_mt(g, t, n_tris, tri_idx, pos, prdp,
                                                           thickness, tri_begin, tri_end, out, cap)
                    : orc_ccd_sh_extended_ref_range_tab(g, t, n_tris, tri_idx, pos, prdp,
                                                        thickness, tri_begin, tri_end, out, cap);
    orc_sh_free(t);
    return h;
}

typedef struct { int face; orc_contact c; } hit_rec;
static int cmp_hit(const void *a, const void *b)
{
    return ((const hit_rec *)a)->face - ((const hit_rec *)b)->face;
}

/* the test orc_ccd_vf_pairs runs (0 ExtendedVFTest, 1 NarrowVFCCDTest, 2
 * VFCCDTest, 3 VFDCDTest, 4 VFTest) */
static int g_vf_test = 0;
void orc_set_vf_test(int mode) { g_vf_test = mode; }
static int vf_test_by_mode(const float *x, const float *p, float th, int i0, int i1, int i2,
                           int i3, orc_contact *ct)
{
    switch (g_vf_test) {
        case 1: return orc_narrow_vf_ccd_test(x, p, th, i0, i1, i2, i3, ct);
        case 2: return orc_vf_ccd_test(x, p, th, i0, i1, i2, i3, ct);
        case 3: return orc_vf_dcd_test(x, p, th, i0, i1, i2, i3, ct);
        case 4: return orc_vf_test(x, p, th, i0, i1, i2, i3, ct);
        default: return orc_extended_vf_test(x, p, th, i0, i1, i2, i3, ct);
    }
}

/* The hits of point v in face order (orc_ccd_vf_pairs' loop body); hits
 * and cc are the caller's scratch. */
static int vf_pairs_point(const orc_grid *g, const cell_table *t, const int *cells,
                          const int *pc, const int *pt, int v, const int *tri_idx,
                          const int *tri_inst, const int *point_inst, const float *pos,
                          const float *prdp, float thickness, hit_rec **hits, int *hcap,
                          int *cc)
{
    /* centroid cells of the incident triangles (those in the grid) */
    int nc = 0;
    for (int q = pc[v]; q < pc[v + 1] && nc < 64; ++q) {
        const int *c = cells + 3 * pt[q];
        if (g->bounded && outside(g, c)) continue;
        cc[3 * nc] = c[0]; cc[3 * nc + 1] = c[1]; cc[3 * nc + 2] = c[2];
        nc++;
    }
    if (nc == 0) return 0;
    int lo[3], hi[3];
    for (int k = 0; k < 3; ++k) { lo[k] = cc[k]; hi[k] = cc[k]; }
    for (int i = 1; i < nc; ++i)
        for (int k = 0; k < 3; ++k) {
            if (cc[3 * i + k] < lo[k]) lo[k] = cc[3 * i + k];
            if (cc[3 * i + k] > hi[k]) hi[k] = cc[3 * i + k];
        }
    int nh = 0;
    for (int z = lo[2] - 1; z <= hi[2] + 1; ++z)
        for (int y = lo[1] - 1; y <= hi[1] + 1; ++y)
            for (int x = lo[0] - 1; x <= hi[0] + 1; ++x) {
                int cell[3] = {x, y, z};
                int near = 0;
                for (int i = 0; i < nc && !near; ++i)
                    near = abs(cc[3 * i] - x) <= 1 && abs(cc[3 * i + 1] - y) <= 1 &&
                           abs(cc[3 * i + 2] - z) <= 1;
                if (!near) continue;
                if (g->bounded && outside(g, cell)) continue;
                uint64_t key = g->bounded ? (uint64_t)orc_cell_hash(g, cell) : cell_key(cell);
                for (int e = table_lower(t, key); e < t->n && t->e[e].key == key; ++e) {
                    int f = t->e[e].id;
                    if (tri_inst && point_inst && tri_inst[f] != point_inst[v]) continue;
                    int ids[4] = {v, tri_idx[3 * f], tri_idx[3 * f + 1], tri_idx[3 * f + 2]};
                    float xs[12], ps[12];
                    gather4(ids, pos, xs);
                    gather4(ids, prdp, ps);
                    orc_contact ct;
                    memset(&ct, 0, sizeof(ct));
                    if (!vf_test_by_mode(xs, ps, thickness, ids[0], ids[1], ids[2], ids[3], &ct))
                        continue;
                    ct.v = ids[0]; ct.f0 = ids[1]; ct.f1 = ids[2]; ct.f2 = ids[3];
                    ct.face = f;
                    if (nh == *hcap) {
                        *hcap *= 2;
                        *hits = (hit_rec *)realloc(*hits, sizeof(hit_rec) * (size_t)*hcap);
                    }
                    (*hits)[nh].face = f;
                    (*hits)[nh].c = ct;
                    nh++;
                }
            }
    qsort(*hits, (size_t)nh, sizeof(hit_rec), cmp_hit);
    return nh;
}

int64_t orc_ccd_vf_pairs(const orc_grid *g, int n_points, int n_tris,
                         const int *tri_idx, const int *tri_inst,
                         const int *point_inst, const float *pos,
                         const float *prdp, float thickness, orc_contact *out,
                         int64_t cap)
{
    int *cells = (int *)malloc(sizeof(int) * 3 * (size_t)(n_tris > 0 ? n_tris : 1));
    cell_table t = build_table(g, n_tris, tri_idx, prdp, cells);
    /* point -> incident triangles */
    int *pc = (int *)calloc((size_t)n_points + 1, sizeof(int));
    for (int i = 0; i < 3 * n_tris; ++i) pc[tri_idx[i] + 1]++;
    for (int i = 0; i < n_points; ++i) pc[i + 1] += pc[i];
    int *pt = (int *)malloc(sizeof(int) * (size_t)(3 * n_tris > 0 ? 3 * n_tris : 1));
    int *fill = (int *)malloc(sizeof(int) * ((size_t)n_points + 1));
    memcpy(fill, pc, sizeof(int) * ((size_t)n_points + 1));
    for (int i = 0; i < 3 * n_tris; ++i) pt[fill[tri_idx[i]]++] = i / 3;
    /* points in blocks, each block's hits kept in point order; blocks are
     * independent and joined in order */
    const int B = 256;
    int nblk = (n_points + B - 1) / B;
    raw_hits *rh = (raw_hits *)calloc((size_t)(nblk > 0 ? nblk : 1), sizeof(raw_hits));
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads) if (g_threads > 1)
#endif
    {
        int hcap = 256;
        hit_rec *hits = (hit_rec *)malloc(sizeof(hit_rec) * (size_t)hcap);
        int *cc = (int *)malloc(sizeof(int) * 3 * 64);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int k = 0; k < nblk; ++k) {
            raw_hits *o = rh + k;
            o->n = 0;
            o->cap = 0;
            o->c = NULL;
            int v1 = (k + 1) * B < n_points ? (k + 1) * B : n_points;
            for (int v = k * B; v < v1; ++v) {
                int nh = vf_pairs_point(g, &t, cells, pc, pt, v, tri_idx, tri_inst, point_inst,
                                        pos, prdp, thickness, &hits, &hcap, cc);
                if (!nh) continue;
                if (o->n + nh > o->cap) {
                    o->cap = 2 * (o->n + nh);
                    o->c = (orc_contact *)realloc(o->c, sizeof(orc_contact) * (size_t)o->cap);
                }
                for (int i = 0; i < nh; ++i) o->c[o->n++] = hits[i].c;
            }
        }
        free(cc);
        free(hits);
    }
    int64_t h = 0;
    for (int k = 0; k < nblk; ++k) {
        for (int64_t i = 0; i < rh[k].n; ++i) {
            if (out && h < cap) out[h] = rh[k].c[i];
            h++;
        }
        free(rh[k].c);
    }
    free(rh);
    free(pc);
    free(pt);
    free(fill);
    free(t.e);
    free(cells);
    return h;
}

/* RelativePos (P/CCD.cpp:13-25): side of the start-of-step plane */
static inline int side_of(f3 v, f3 p, f3 n) { return dot(sub(v, p), n) >= 0; }

int orc_vf_resolve_test(const float *x, const float *p, float thickness)
{
    /* P/CCD.cpp:1996-2032 */
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    f3 fn = nrm(cross(sub(X2, X1), sub(X3, X1)));
    int dir = side_of(X0, X1, fn);
    f3 pn = nrm(cross(sub(P2, P1), sub(P3, P1)));
    f3 pr = cross(sub(P2, P1), sub(P3, P1));
    if ((double)dot(pr, pr) <= 1e-6) return 0;
    float depth = (float)((double)dot(sub(P0, P1), mul(pn, dir ? 1.0f : -1.0f)) -
                          2.0 * (double)thickness);
    return !(depth >= -1e-6);
}

void orc_vf_resolve_new(const float *x, float *p, float thickness)
{
    /* P/CCD.cpp:2034-2077 */
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    f3 fn = nrm(cross(sub(X2, X1), sub(X3, X1)));
    int dir = side_of(X0, X1, fn);
    f3 pn = nrm(cross(sub(P2, P1), sub(P3, P1)));
    float sg = dir ? 1.0f : -1.0f;
    f3 p1proj = add(P1, mul(mul(mul(pn, sg), 2.0f), thickness));
    float depth = (float)((double)dot(sub(p1proj, P0), mul(pn, sg)) * 0.5);
    f3 vfix = mul(mul(pn, sg), depth);
    f3 ffix = mul(mul(pn, -sg), depth);
    f3 w = bary(P0, P1, P2, P3);
    float sw = w.x * w.x + w.y * w.y + w.z * w.z;
    st3(p, add(P0, vfix));
    st3(p + 3, add(P1, divs(mul(ffix, w.x), sw)));
    st3(p + 6, add(P2, divs(mul(ffix, w.y), sw)));
    st3(p + 9, add(P3, divs(mul(ffix, w.z), sw)));
}

void orc_collision_resolve_ref(int n_contacts, const orc_contact *cts,
                               const float *pos, float *prdp, int iterations,
                               float thickness)
{
    for (int it = 0; it < iterations; ++it)
        for (int c = 0; c < n_contacts; ++c) {
            int ids[4] = {cts[c].v, cts[c].f0, cts[c].f1, cts[c].f2};
            float xs[12], ps[12];
            gather4(ids, pos, xs);
            gather4(ids, prdp, ps);
            if (!orc_vf_resolve_test(xs, ps, thickness)) continue;
            orc_vf_resolve_new(xs, ps, thickness);
            for (int j = 0; j < 4; ++j)
                for (int k = 0; k < 3; ++k) prdp[3 * ids[j] + k] = ps[3 * j + k];
        }
}

/* VFResolve (P/CCD.cpp:2595-2650) on one contact, in place on p[12]:
 * dp = (2h - depth)/2 when the point stayed on its side of the face and is
 * closer than 2h to the predicted plane; (depth + 2h)/2 when it changed
 * sides and some of the four points was never resolved, or VFCCDTest still
 * finds the crossing; the point moves dp along the predicted normal
 * towards its starting side, the face points the other way weighted
 * w_i / sum w^2; the four counters count the contacts that moved them */
static void vf_resolve_old(const float *x, float *p, float thickness, int *rt, const int *ids)
{
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    f3 fn = nrm(cross(sub(X2, X1), sub(X3, X1)));
    int pos_rel = side_of(X0, X1, fn);
    f3 n = nrm(cross(sub(P2, P1), sub(P3, P1)));
    float depth = point_to_plane(P0, P1, P2, P3);
    int prd_rel = side_of(P0, P1, n);
    float dp = 0.0f;
    f3 w = bary(P0, P1, P2, P3);
    if (pos_rel == prd_rel && depth < 2 * thickness) {
        dp = (float)((double)(2 * thickness - depth) * 0.5);
    } else if (pos_rel != prd_rel) {
        if (rt[ids[0]] == 0 || rt[ids[1]] == 0 || rt[ids[2]] == 0 || rt[ids[3]] == 0)
            dp = (float)((double)(depth + 2 * thickness) * 0.5);
        else if (orc_vf_ccd_test(x, p, thickness, ids[0], ids[1], ids[2], ids[3], NULL))
            dp = (float)((double)(depth + 2 * thickness) * 0.5);
    }
    if (dp != 0.0f)
        for (int j = 0; j < 4; ++j) rt[ids[j]] += 1;
    float sw = w.x * w.x + w.y * w.y + w.z * w.z;
    f3 mn = mk(-n.x, -n.y, -n.z);
    f3 a = pos_rel ? n : mn, b = pos_rel ? mn : n;
    st3(p, add(P0, mul(a, dp)));
    st3(p + 3, add(P1, divs(mul(mul(b, dp), w.x), sw)));
    st3(p + 6, add(P2, divs(mul(mul(b, dp), w.y), sw)));
    st3(p + 9, add(P3, divs(mul(mul(b, dp), w.z), sw)));
}

void orc_collision_resolve_old(int n_contacts, const orc_contact *cts, const float *pos,
                               float *prdp, int *resolve_times, float thickness)
{
    /* CollisionResolve (P/CCD.cpp:2423-2593): two passes (its iteration
     * argument is not used), contacts in stored order, in place; a contact
     * is skipped when the point is on its starting side of the predicted
     * face and at least 2h from its plane */
    for (int it = 0; it < 2; ++it)
        for (int c = 0; c < n_contacts; ++c) {
            int ids[4] = {cts[c].v, cts[c].f0, cts[c].f1, cts[c].f2};
            float xs[12], ps[12];
            gather4(ids, pos, xs);
            gather4(ids, prdp, ps);
            f3 X0 = ld3(xs), X1 = ld3(xs + 3), X2 = ld3(xs + 6), X3 = ld3(xs + 9);
            f3 P0 = ld3(ps), P1 = ld3(ps + 3), P2 = ld3(ps + 6), P3 = ld3(ps + 9);
            f3 fn = nrm(cross(sub(X2, X1), sub(X3, X1)));
            int f_rel = side_of(X0, X1, fn);
            f3 nn = nrm(cross(sub(P2, P1), sub(P3, P1)));
            int c_rel = side_of(P0, P1, nn);
            float distance = point_to_plane(P0, P1, P2, P3);
            if (c_rel == f_rel && distance >= 2 * thickness) continue;
            vf_resolve_old(xs, ps, thickness, resolve_times, ids);
            for (int j = 0; j < 4; ++j)
                for (int k = 0; k < 3; ++k) prdp[3 * ids[j] + k] = ps[3 * j + k];
        }
}

int orc_vf_resolve_deltas(const float *x, const float *p, const float *wm,
                          float thickness, int mass_weighted, float *delta)
{
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    f3 e1 = sub(P2, P1), e2 = sub(P3, P1);
    f3 pr = cross(e1, e2);
    float pr2 = dot(pr, pr);
    if (!mass_weighted) {
        /* reference degeneracy guard: |n|^2 <= 1e-6 (P/CCD.cpp:2007) */
        if ((double)pr2 <= 1e-6) return 0;
    } else {
        /* scale-free guard: sin^2 of the corner angle <= 1e-12 */
        if (!(pr2 > 1e-12f * (dot(e1, e1) * dot(e2, e2)))) return 0;
    }
    f3 fn = nrm(cross(sub(X2, X1), sub(X3, X1)));
    int dir = side_of(X0, X1, fn);
    f3 pn = nrm(pr);
    float sg = dir ? 1.0f : -1.0f;
    f3 ns = mul(pn, sg);
    float gap = (float)((double)dot(sub(P0, P1), ns) - 2.0 * (double)thickness);
    if (gap >= -1e-6f) return 0;
    f3 p1proj = add(P1, mul(mul(ns, 2.0f), thickness));
    float depth = (float)((double)dot(sub(p1proj, P0), ns) * 0.5);
    f3 w = bary(P0, P1, P2, P3);
    f3 dv, d1, d2, d3;
    if (!mass_weighted) {
        /* VFResolveNew split: point moves depth, face point moves depth */
        f3 vfix = mul(ns, depth);
        f3 ffix = mul(mul(pn, -sg), depth);
        float sw = w.x * w.x + w.y * w.y + w.z * w.z;
        dv = vfix;
        d1 = divs(mul(ffix, w.x), sw);
        d2 = divs(mul(ffix, w.y), sw);
        d3 = divs(mul(ffix, w.z), sw);
    } else {
        /* inverse-mass split of the separation 2*depth: the point takes
         * alpha = m_v/(m_v + m_f), m_f = sum w_i^2 m_i / sum w_i^2; face
         * point i moves -(1-alpha) 2 depth w_i m_i / sum_j w_j^2 m_j.  Equal
         * masses reduce to the reference split. */
        float sw = w.x * w.x + w.y * w.y + w.z * w.z;
        float swm = w.x * w.x * wm[1] + w.y * w.y * wm[2] + w.z * w.z * wm[3];
        float mf = swm / sw;
        float msum = wm[0] + mf;
        if (!(msum > 0.0f) || !(sw > 0.0f)) return 0;
        float alpha = wm[0] / msum;
        float sep = 2.0f * depth;
        dv = mul(ns, sep * alpha);
        float fs = swm > 0.0f ? -sep * (1.0f - alpha) / swm : 0.0f;
        d1 = mul(ns, fs * w.x * wm[1]);
        d2 = mul(ns, fs * w.y * wm[2]);
        d3 = mul(ns, fs * w.z * wm[3]);
    }
    st3(delta, dv);
    st3(delta + 3, d1);
    st3(delta + 6, d2);
    st3(delta + 9, d3);
    return 1;
}

void orc_collision_resolve_seq(int n_contacts, const orc_contact *cts, const float *pos,
                               float *prdp, const float *mass, int iterations,
                               float thickness, int mass_weighted)
{
    /* CollisionResolveNew's sequential pass (P/CCD.cpp:1874-1994): contacts
     * in stored order, each applied in place before the next is tested;
     * the correction of orc_vf_resolve_deltas (mass_weighted 0: the
     * reference's split and guard, as orc_collision_resolve_ref; 1: the
     * inverse-mass split with the scale-free guard) */
    for (int it = 0; it < iterations; ++it)
        for (int c = 0; c < n_contacts; ++c) {
            int ids[4] = {cts[c].v, cts[c].f0, cts[c].f1, cts[c].f2};
            float xs[12], ps[12], wm[4], dl[12];
            gather4(ids, pos, xs);
            gather4(ids, prdp, ps);
            for (int j = 0; j < 4; ++j) wm[j] = mass ? mass[ids[j]] : 1.0f;
            if (!orc_vf_resolve_deltas(xs, ps, wm, thickness, mass_weighted, dl)) continue;
            for (int j = 0; j < 4; ++j)
                for (int k = 0; k < 3; ++k) prdp[3 * ids[j] + k] = ps[3 * j + k] + dl[3 * j + k];
        }
}

void orc_collision_resolve_jacobi(int n_points, int n_contacts,
                                  const orc_contact *cts, const float *pos,
                                  float *prdp, const float *mass, int iterations,
                                  float thickness, int mass_weighted)
{
    /* Corrections are accumulated in 2^-32 m fixed point (each float
     * correction rounded to the nearest integer multiple, ties to even), so
     * the sum does not depend on the order contacts are visited in; each
     * point then moves by sum * 2^-32 / count (double), rounded to float. */
    int64_t *acc = (int64_t *)malloc(sizeof(int64_t) * 3 * (size_t)(n_points > 0 ? n_points : 1));
    int *cnt = (int *)malloc(sizeof(int) * (size_t)(n_points > 0 ? n_points : 1));
    float *dl = (float *)malloc(sizeof(float) * 12 * (size_t)(n_contacts > 0 ? n_contacts : 1));
    int *act = (int *)malloc(sizeof(int) * (size_t)(n_contacts > 0 ? n_contacts : 1));
    for (int it = 0; it < iterations; ++it) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1 && n_contacts > 1024)
#endif
        for (int c = 0; c < n_contacts; ++c) {
            int ids[4] = {cts[c].v, cts[c].f0, cts[c].f1, cts[c].f2};
            float xs[12], ps[12], wm[4];
            gather4(ids, pos, xs);
            gather4(ids, prdp, ps);
            for (int j = 0; j < 4; ++j) wm[j] = mass ? mass[ids[j]] : 1.0f;
            act[c] = orc_vf_resolve_deltas(xs, ps, wm, thickness, mass_weighted, dl + 12 * c);
        }
        memset(acc, 0, sizeof(int64_t) * 3 * (size_t)n_points);
        memset(cnt, 0, sizeof(int) * (size_t)n_points);
        for (int c = 0; c < n_contacts; ++c) {
            if (!act[c]) continue;
            int ids[4] = {cts[c].v, cts[c].f0, cts[c].f1, cts[c].f2};
            for (int j = 0; j < 4; ++j) {
                for (int k = 0; k < 3; ++k)
                    acc[3 * ids[j] + k] += (int64_t)llrintf(dl[12 * c + 3 * j + k] * 4294967296.0f);
                cnt[ids[j]]++;
            }
        }
        for (int i = 0; i < n_points; ++i)
            if (cnt[i] > 0)
                for (int k = 0; k < 3; ++k)
                    prdp[3 * i + k] = prdp[3 * i + k] +
                        (float)((double)acc[3 * i + k] * (1.0 / 4294967296.0) / (double)cnt[i]);
    }
    free(acc);
    free(cnt);
    free(dl);
    free(act);
}

/* ------------------------------------------------------------------ */
/* edge-edge CCD.  The reference declares the contact kind only          */
/* (Contact::EE, P/CCD_Basic.h:14; EEResolve is commented out,           */
/* P/CCD.cpp:925-928), so this follows ExtendedVFTest's structure         */
/* (P/CCD.cpp:1733-1808): the coplanarity cubic of the four points, the   */
/* times 0, its roots in [0, 1] and 1 in ascending order, and a hit at    */
/* the first time the two edges' lines meet inside both edges closer      */
/* than 2 * thickness.                                                    */
/* ------------------------------------------------------------------ */

static inline float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

/* closest points of the lines through a0a1 and b0b1 (Ericson, Real-Time
 * Collision Detection, 5.1.8): 1 when the lines are not near-parallel and
 * both parameters lie strictly inside (0, 1); *d = A(s) - B(u) */
static int ee_interior(f3 a0, f3 a1, f3 b0, f3 b1, float *s, float *u, f3 *d)
{
    f3 d1 = sub(a1, a0), d2 = sub(b1, b0), r = sub(a0, b0);
    float a = dot(d1, d1), e = dot(d2, d2), b = dot(d1, d2);
    float c = dot(d1, r), f = dot(d2, r);
    float den = a * e - b * b;
    if (!(den > 1e-8f * (a * e))) return 0;
    float ss = (b * f - c * e) / den;
    float uu = (a * f - b * c) / den;
    if (!(ss > 0.0f && ss < 1.0f && uu > 0.0f && uu < 1.0f)) return 0;
    *s = ss;
    *u = uu;
    *d = sub(add(a0, mul(d1, ss)), add(b0, mul(d2, uu)));
    return 1;
}

/* closest points of the segments a0a1 and b0b1 (Ericson 5.1.9) */
static void seg_closest(f3 p1, f3 q1, f3 p2, f3 q2, float *s, float *t)
{
    f3 d1 = sub(q1, p1), d2 = sub(q2, p2), r = sub(p1, p2);
    float a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    float ss, tt;
    if (a <= 1e-20f && e <= 1e-20f) {
        ss = 0.0f;
        tt = 0.0f;
    } else if (a <= 1e-20f) {
        ss = 0.0f;
        tt = clamp01(f / e);
    } else {
        float c = dot(d1, r);
        if (e <= 1e-20f) {
            tt = 0.0f;
            ss = clamp01(-c / a);
        } else {
            float b = dot(d1, d2), den = a * e - b * b;
            ss = den != 0.0f ? clamp01((b * f - c * e) / den) : 0.0f;
            tt = (b * ss + f) / e;
            if (tt < 0.0f) {
                tt = 0.0f;
                ss = clamp01(-c / a);
            } else if (tt > 1.0f) {
                tt = 1.0f;
                ss = clamp01((b - c) / a);
            }
        }
    }
    *s = ss;
    *t = tt;
}

int orc_ee_test(const float *x, const float *p, float thickness, orc_ee_hit *hit)
{
    f3 X0 = ld3(x), X1 = ld3(x + 3), X2 = ld3(x + 6), X3 = ld3(x + 9);
    f3 P0 = ld3(p), P1 = ld3(p + 3), P2 = ld3(p + 6), P3 = ld3(p + 9);
    /* the side the edges start on: the common normal at t = 0 */
    f3 da = sub(X1, X0), db = sub(X3, X2);
    f3 m0 = cross(da, db);
    if (!(dot(m0, m0) > 1e-12f * (dot(da, da) * dot(db, db)))) return 0;
    m0 = nrm(m0);
    float sg = dot(sub(X0, X2), m0) >= 0.0f ? 1.0f : -1.0f;
    double a[4];
    vf_cubic(x, p, a);
    double t[5];
    int nsol = orc_solve_cubic(a[3], a[2], a[1], a[0], t);
    t[nsol] = 1;
    t[nsol + 1] = 0;
    sort_small(t, nsol + 2);
    for (int i = 0; i < nsol + 2; ++i) {
        if (t[i] < 0 || t[i] > 1) continue;
        f3 c0 = lerp_t(X0, P0, t[i]), c1 = lerp_t(X1, P1, t[i]);
        f3 c2 = lerp_t(X2, P2, t[i]), c3 = lerp_t(X3, P3, t[i]);
        float s, u;
        f3 d;
        if (!ee_interior(c0, c1, c2, c3, &s, &u, &d)) continue;
        float dist = sqrtf(dot(d, d));
        if ((double)dist - (double)(2.0f * thickness) < -1e-6) {
            if (hit) {
                hit->t = (float)t[i];
                hit->s = s;
                hit->u = u;
                hit->m0[0] = m0.x;
                hit->m0[1] = m0.y;
                hit->m0[2] = m0.z;
                hit->m0[3] = sg;
            }
            return 1;
        }
    }
    return 0;
}

int64_t orc_ccd_ee_brute(int n_edges, const int *edges, const int *point_inst, const float *x,
                         const float *p, float thickness, int *pairs, orc_ee_hit *hits,
                         int64_t cap)
{
    int64_t n = 0;
    for (int i = 0; i < n_edges; ++i)
        for (int j = i + 1; j < n_edges; ++j) {
            int ids[4] = {edges[2 * i], edges[2 * i + 1], edges[2 * j], edges[2 * j + 1]};
            if (ids[0] == ids[2] || ids[0] == ids[3] || ids[1] == ids[2] || ids[1] == ids[3])
                continue;
            if (point_inst && point_inst[ids[0]] != point_inst[ids[2]]) continue;
            float xs[12], ps[12];
            gather4(ids, x, xs);
            gather4(ids, p, ps);
            orc_ee_hit h;
            if (!orc_ee_test(xs, ps, thickness, &h)) continue;
            if (n < cap) {
                if (pairs) {
                    pairs[2 * n] = i;
                    pairs[2 * n + 1] = j;
                }
                if (hits) hits[n] = h;
            }
            ++n;
        }
    return n;
}

int orc_ee_resolve_deltas(const float *p, const float *wm, const float *m0s, float thickness,
                          float *delta)
{
    f3 A0 = ld3(p), A1 = ld3(p + 3), B0 = ld3(p + 6), B1 = ld3(p + 9);
    f3 d1 = sub(A1, A0), d2 = sub(B1, B0);
    f3 mp = cross(d1, d2);
    if (!(dot(mp, mp) > 1e-12f * (dot(d1, d1) * dot(d2, d2)))) return 0;
    mp = nrm(mp);
    if (dot(mp, ld3(m0s)) < 0.0f) mp = mul(mp, -1.0f);
    float sg = m0s[3];
    float s, u;
    seg_closest(A0, A1, B0, B1, &s, &u);
    f3 d = sub(add(A0, mul(d1, s)), add(B0, mul(d2, u)));
    float g = (float)((double)(sg * dot(d, mp)) - 2.0 * (double)thickness);
    if (!(g < -1e-6f)) return 0;
    float depth = -g;
    float c[4] = {1.0f - s, s, 1.0f - u, u};
    float den = wm[0] * c[0] * c[0] + wm[1] * c[1] * c[1] + wm[2] * c[2] * c[2] +
                wm[3] * c[3] * c[3];
    if (!(den > 0.0f)) return 0;
    float imp = depth / den;
    st3(delta, mul(mp, sg * c[0] * wm[0] * imp));
    st3(delta + 3, mul(mp, sg * c[1] * wm[1] * imp));
    st3(delta + 6, mul(mp, -sg * c[2] * wm[2] * imp));
    st3(delta + 9, mul(mp, -sg * c[3] * wm[3] * imp));
    return 1;
}

void orc_collision_resolve_jacobi_ee(int n_points, int n_vf, const orc_contact *vf,
                                     int n_ee, const int *ee_ids, const float *ee_m0,
                                     const float *pos, float *prdp, const float *mass,
                                     int iterations, float thickness, int mass_weighted)
{
    /* one Jacobi pass over both contact kinds: every correction in 2^-32 m
     * fixed point into per-point sums, then sum * 2^-32 / count per point
     * (orc_collision_resolve_jacobi's scheme) */
    int64_t *acc = (int64_t *)malloc(sizeof(int64_t) * 3 * (size_t)(n_points > 0 ? n_points : 1));
    int *cnt = (int *)malloc(sizeof(int) * (size_t)(n_points > 0 ? n_points : 1));
    int nc = n_vf + n_ee;
    float *dl = (float *)malloc(sizeof(float) * 12 * (size_t)(nc > 0 ? nc : 1));
    int *act = (int *)malloc(sizeof(int) * (size_t)(nc > 0 ? nc : 1));
    int *ids = (int *)malloc(sizeof(int) * 4 * (size_t)(nc > 0 ? nc : 1));
    for (int c = 0; c < n_vf; ++c) {
        ids[4 * c] = vf[c].v;
        ids[4 * c + 1] = vf[c].f0;
        ids[4 * c + 2] = vf[c].f1;
        ids[4 * c + 3] = vf[c].f2;
    }
    for (int c = 0; c < n_ee; ++c)
        for (int j = 0; j < 4; ++j) ids[4 * (n_vf + c) + j] = ee_ids[4 * c + j];
    for (int it = 0; it < iterations; ++it) {
        for (int c = 0; c < nc; ++c) {
            float xs[12], ps[12], wm[4];
            gather4(ids + 4 * c, pos, xs);
            gather4(ids + 4 * c, prdp, ps);
            for (int j = 0; j < 4; ++j) wm[j] = mass ? mass[ids[4 * c + j]] : 1.0f;
            act[c] = c < n_vf ? orc_vf_resolve_deltas(xs, ps, wm, thickness, mass_weighted, dl + 12 * c)
                              : orc_ee_resolve_deltas(ps, wm, ee_m0 + 4 * (c - n_vf), thickness,
                                                      dl + 12 * c);
        }
        memset(acc, 0, sizeof(int64_t) * 3 * (size_t)n_points);
        memset(cnt, 0, sizeof(int) * (size_t)n_points);
        for (int c = 0; c < nc; ++c) {
            if (!act[c]) continue;
            for (int j = 0; j < 4; ++j) {
                for (int k = 0; k < 3; ++k)
                    acc[3 * ids[4 * c + j] + k] +=
                        (int64_t)llrintf(dl[12 * c + 3 * j + k] * 4294967296.0f);
                cnt[ids[4 * c + j]]++;
            }
        }
        for (int i = 0; i < n_points; ++i)
            if (cnt[i] > 0)
                for (int k = 0; k < 3; ++k)
                    prdp[3 * i + k] = prdp[3 * i + k] +
                        (float)((double)acc[3 * i + k] * (1.0 / 4294967296.0) / (double)cnt[i]);
    }
    free(acc);
    free(cnt);
    free(dl);
    free(act);
    free(ids);
}

/* ------------------------------------------------------------------ */
/* substeps                                                             */
/* ------------------------------------------------------------------ */

/* The analytic ground of the GPU path: a point closer than 1 mm above the
 * plane y = h (or below it) is put on it. */
void orc_ground(int n, float *prdp, float h)
{
    for (int i = 0; i < n; ++i)
        if (prdp[3 * i + 1] - h < 0.001f) prdp[3 * i + 1] = h;
}

int64_t orc_substep_gpu_obst(int n_points, const orc_constraints *c,
                             const int *sorted_prim_id, int n_worksets,
                             const int *worksets, int iterations, float dt,
                             float damping, const float *gravity, const float *mass,
                             float *pos, float *vel, float *prdp, int bending_fp64,
                             const orc_colli_params *colli, const float *sphere4,
                             int ground_on, float ground_h)
{
    /* the GPU step's order: per iteration [detection when due], one colored
     * sweep, [one response pass], then the analytic obstacles (the sphere
     * push of ColliWithShpGrd, P/PBD_cuda.cu:1519-1573, and the ground) */
    float damp_pow = powf(damping, dt);
    orc_advect_gpu(n_points, dt, damp_pow, gravity, mass, vel, prdp, pos);
    int64_t nct = 0;
    orc_contact *cts = NULL;
    int use = colli && colli->enabled;
    if (use) cts = (orc_contact *)malloc(sizeof(orc_contact) * (size_t)(colli->contact_cap > 0 ? colli->contact_cap : 1));
    for (int ii = 0; ii < iterations; ++ii) {
        if (use && (ii % colli->ccd_every == 0 || ii == iterations - 1)) {
            nct = orc_ccd_vf_pairs(&colli->grid, n_points, colli->n_tris, colli->tri_idx,
                                   colli->tri_inst, colli->point_inst, pos, prdp,
                                   colli->thickness, cts, colli->contact_cap);
            if (nct > colli->contact_cap) nct = colli->contact_cap;
        }
        orc_project_colored(c, sorted_prim_id, n_worksets, worksets, ii, ii + 1, mass,
                            prdp, bending_fp64);
        if (use && nct > 0)
            orc_collision_resolve_jacobi(n_points, (int)nct, cts, pos, prdp, mass,
                                         colli->resolve_passes, colli->thickness,
                                         colli->mass_weighted);
        if (sphere4) orc_colli_sphere(n_points, prdp, sphere4, sphere4[3]);
        if (ground_on) orc_ground(n_points, prdp, ground_h);
    }
    orc_integrate(n_points, dt, vel, prdp, pos);
    free(cts);
    return nct;
}

int64_t orc_substep_gpu(int n_points, const orc_constraints *c,
                        const int *sorted_prim_id, int n_worksets,
                        const int *worksets, int iterations, float dt,
                        float damping, const float *gravity, const float *mass,
                        float *pos, float *vel, float *prdp, int bending_fp64,
                        const orc_colli_params *colli)
{
    return orc_substep_gpu_obst(n_points, c, sorted_prim_id, n_worksets, worksets, iterations,
                                dt, damping, gravity, mass, pos, vel, prdp, bending_fp64, colli,
                                NULL, 0, 0.0f);
}

int64_t orc_substep_cpu_ref(int n_points, const orc_constraints *c, int iterations,
                            float dt, const float *gravity, const float *mass,
                            float *pos, float *vel, float *prdp,
                            const orc_colli_params *colli,
                            const float *sphere_center, float sphere_radius)
{
    orc_advect_cpu(n_points, dt, gravity, vel, prdp, pos);
    int64_t nct = 0;
    if (!(colli && colli->enabled)) {
        orc_project_cpu(c, iterations, mass, prdp, n_points, sphere_center, sphere_radius);
    } else {
        orc_contact *cts = (orc_contact *)malloc(sizeof(orc_contact) * (size_t)(colli->contact_cap > 0 ? colli->contact_cap : 1));
        for (int ii = 0; ii < iterations; ++ii) {
            if (ii % colli->ccd_every == 0 || ii == iterations - 1) {
                nct = orc_ccd_sh_extended_ref(&colli->grid, colli->n_tris, colli->tri_idx, pos,
                                              prdp, colli->thickness, cts, colli->contact_cap);
                if (nct > colli->contact_cap) nct = colli->contact_cap;
            }
            orc_project_cpu(c, 1, mass, prdp, n_points, NULL, 0.0f);
            if (colli->mass_weighted)
                orc_collision_resolve_seq((int)nct, cts, pos, prdp, mass, 1, colli->thickness, 1);
            else
                orc_collision_resolve_ref((int)nct, cts, pos, prdp, 1, colli->thickness);
            if (sphere_center) orc_colli_sphere(n_points, prdp, sphere_center, sphere_radius);
        }
        free(cts);
    }
    orc_integrate(n_points, dt, vel, prdp, pos);
    return nct;
}

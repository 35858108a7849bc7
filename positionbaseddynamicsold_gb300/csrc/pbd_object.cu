// pbd_object.cu -- PBDObject, ConstraintPBD and SolverPBD on the GPU.
//
// Data layout in HBM (per object):
//   x, p, v        float4 per point; x.w = p.w = massBuffer value (inverse
//                  mass / gravity gate, 0 = pinned), so a projection reads its
//                  weights with the positions in one 16-byte load.
//   drec           int4 per distance constraint {i0, i1, rest, stiffness},
//                  grouped by color (color-major), 16 B per record.
//   bidx / bpar    int4 {e0, e1, wA, wB} + float2 {rest angle, stiffness}
//                  per bending constraint, grouped by color.
//   arec           float4 {rest xyz, point id} per anchor, grouped by color.
// One kernel launch per color applies every constraint of that color; no
// two constraints of a color share a point, so the launch has no races and
// its result does not depend on thread order.  The resident form
// (k_gs_resident) runs whole sweeps in one launch with the points in the
// shared memory of a thread-block cluster and a cluster barrier per color.
// Per-point host transfers go through page-locked staging (or directly from
// a page-locked caller array) and float3 <-> float4 pack kernels.
//
// Arithmetic mirrors the reference kernels operation by operation; this
// translation unit is compiled with -fmad=false so no multiply-add is fused
// (the reference's host path rounds every product separately).
#include <algorithm>
#include <cmath>
#include <cstring>

#include <cooperative_groups.h>

#include "pbd_common.cuh"
#include "pbd_project.cuh"

namespace cg = cooperative_groups;

namespace pbd {

static thread_local std::string g_err;
void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
}

static int bits_for(long long maxval) {
    int b = 0;
    while (b < 63 && (1LL << b) <= maxval) ++b;
    return b < 1 ? 1 : b;
}
static int round8(int b) { return (b + 7) / 8 * 8; }

// ---------------------------------------------------------------------------
// construction kernels
// ---------------------------------------------------------------------------
__global__ void k_pack_state(int n, const float *pos, const float *vel, const float *mass,
                             float4 *x, float4 *p, float4 *v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float m = mass[i];
    float4 a = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], m);
    x[i] = a;
    p[i] = a;
    v[i] = vel ? make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.f)
               : make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_pack_tris(int nt, const int *tri, const int *inst, int4 *out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    out[t] = make_int4(tri[3 * t], tri[3 * t + 1], tri[3 * t + 2], inst ? inst[t] : 0);
}

// entries (point, owner) for CSR builds: owner k emits `cnt` entries
__global__ void k_emit_prim_points(int np, const int2 *prim_list, const int *indices,
                                   const int *eoff, uint32_t *key, int *val) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int2 pl = prim_list[p];
    int o = eoff[p];
    for (int i = 0; i < pl.y; ++i) {
        key[o + i] = (uint32_t)indices[pl.x + i];
        val[o + i] = p;
    }
}

__global__ void k_emit_tri_points(int nt, const int4 *tri, uint32_t *key, int *val) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int4 a = tri[t];
    key[3 * t] = (uint32_t)a.x;
    key[3 * t + 1] = (uint32_t)a.y;
    key[3 * t + 2] = (uint32_t)a.z;
    val[3 * t] = t;
    val[3 * t + 1] = t;
    val[3 * t + 2] = t;
}

// run bounds of a sorted key array: first[k] = start, last[k] = end (excl.)
__global__ void k_run_bounds(long long n, const uint32_t *skey, int *first, int *last) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t k = skey[i];
    if (i == 0 || skey[i - 1] != k) first[k] = (int)i;
    if (i == n - 1 || skey[i + 1] != k) last[k] = (int)(i + 1);
}

__global__ void k_prim_counts(int np, const int2 *prim_list, int *cnt) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) cnt[p] = prim_list[p].y;
}

// GenePrim2PrimsMap (P/PBD_cuda.cu:170-202): for each point of the prim (in
// order), every other prim on that point (ascending id)
__global__ void k_adj_count(int np, const int2 *prim_list, const int *indices, const int *pfirst,
                            const int *plast, const int *pprim, int *deg) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int2 pl = prim_list[p];
    int d = 0;
    for (int i = 0; i < pl.y; ++i) {
        int pt = indices[pl.x + i];
        for (int j = pfirst[pt]; j < plast[pt]; ++j) d += pprim[j] != p;
    }
    deg[p] = d;
}

__global__ void k_adj_fill(int np, const int2 *prim_list, const int *indices, const int *pfirst,
                           const int *plast, const int *pprim, const int *off, int2 *sn,
                           int *adj) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int2 pl = prim_list[p];
    int o = off[p], o0 = o;
    for (int i = 0; i < pl.y; ++i) {
        int pt = indices[pl.x + i];
        for (int j = pfirst[pt]; j < plast[pt]; ++j) {
            int q = pprim[j];
            if (q != p) adj[o++] = q;
        }
    }
    sn[p] = make_int2(o0, o - o0);
}

// ---------------------------------------------------------------------------
// coloring (AssignColorsGPU / ResolveConflictsGPU, P/PBD_cuda.cu:313-431)
// ---------------------------------------------------------------------------
__global__ void k_assign_colors(int np, const int2 *__restrict__ sn, const int *__restrict__ adj,
                                const int *__restrict__ color, int *__restrict__ prd) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np) return;
    if (color[idx] >= 0) return;
    int2 r = sn[idx];
    int offset = 0;
    for (;;) {
        unsigned long long forbidden = 0ull;
        for (int i = r.x; i < r.x + r.y; ++i) {
            int nc = color[adj[i]] - offset;
            if (nc >= 0 && nc < 64) forbidden |= (1ull << nc);
        }
        if (forbidden != ~0ull) {
            prd[idx] = offset + __ffsll((long long)~forbidden) - 1;
            return;
        }
        offset += 64;
    }
}

__global__ void k_resolve_conflicts(int np, const int2 *__restrict__ prim_list,
                                    const int2 *__restrict__ sn, const int *__restrict__ adj,
                                    int *__restrict__ color, const int *__restrict__ prd,
                                    int *flag) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np) return;
    if (color[idx] >= 0) return;
    int c = prd[idx];
    int npt = prim_list[idx].y;
    int2 r = sn[idx];
    for (int i = r.x; i < r.x + r.y; ++i) {
        int n = adj[i];
        if (prd[n] != c) continue;
        int nnpt = prim_list[n].y;
        if (nnpt > npt || (nnpt == npt && n < idx)) {
            *flag = 1;
            return;
        }
    }
    color[idx] = c;
}

__global__ void k_max_color(int np, const int *color, int *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np) atomicMax(out, color[i]);
}

__global__ void k_iota_keys(int np, const int *color, uint32_t *key, int *val) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    key[i] = (uint32_t)color[i];
    val[i] = i;
}

__device__ __forceinline__ int cls_of(int t) {
    return t == PBD_DISTANCE ? 0 : t == PBD_BENDING ? 1 : t == PBD_ANCHOR ? 2 : 3;
}

// class-major key: class * n_colors + color
__global__ void k_class_keys(int np, const int *color, const int *ctype, int nc, uint32_t *key,
                             int *val) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    key[i] = (uint32_t)(cls_of(ctype[i]) * nc + color[i]);
    val[i] = i;
}

// records i0 .. n_rec-1 from the per-prim buffers (sprim = the prim of each
// record, in record order)
__global__ void k_build_records(int i0, int n_rec, const int *sprim, const int2 *prim_list,
                                const int *indices, const float *rest_length,
                                const float *stiffness, const float *rest_angle,
                                const float4 *rest_pos, int nd, int nb, int na, int4 *drec,
                                int4 *bidx, float2 *bpar, float4 *arec) {
    int i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rec) return;
    int p = sprim[i];
    int s = prim_list[p].x;
    if (i < nd) {
        drec[i] = make_int4(indices[s], indices[s + 1], __float_as_int(rest_length[p]),
                            __float_as_int(stiffness[p]));
    } else if (i < nd + nb) {
        int j = i - nd;
        bidx[j] = make_int4(indices[s], indices[s + 1], indices[s + 2], indices[s + 3]);
        bpar[j] = make_float2(rest_angle ? rest_angle[p] : 0.f, stiffness[p]);
    } else if (i < nd + nb + na) {
        int j = i - nd - nb;
        float4 r = rest_pos ? rest_pos[p] : make_float4(0.f, 0.f, 0.f, 0.f);
        arec[j] = make_float4(r.x, r.y, r.z, __int_as_float(indices[s]));
    }
}

__global__ void k_set_type_stiffness(int np, const int *__restrict__ ctype, unsigned mask,
                                     float v, float *stiffness) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np && ((unsigned)ctype[p] & mask)) stiffness[p] = v;
}

__global__ void k_set_rest_pos(int n, const int *__restrict__ prims, const float *__restrict__ t3,
                               float4 *rest_pos) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rest_pos[prims[i]] = make_float4(t3[3 * i], t3[3 * i + 1], t3[3 * i + 2], 0.f);
}

// ---------------------------------------------------------------------------
// solver kernels
// ---------------------------------------------------------------------------

// AdvectGPUKernel (P/PBD_cuda.cu:949-979): v += (g*dt)*m; v *= damping^dt;
// p = x + v*dt.  gdt = g*dt and damp_pow = powf(damping, dt) come from the host.
__global__ void __launch_bounds__(256) k_advect(int n, float dt, float damp_pow, float3 gdt,
                                                const float4 *__restrict__ x,
                                                float4 *__restrict__ v, float4 *__restrict__ p,
                                                float4 *__restrict__ p0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 X = x[i], V = v[i];
    float m = X.w;
    V.x = V.x + gdt.x * m;
    V.y = V.y + gdt.y * m;
    V.z = V.z + gdt.z * m;
    V.x = V.x * damp_pow;
    V.y = V.y * damp_pow;
    V.z = V.z * damp_pow;
    v[i] = make_float4(V.x, V.y, V.z, 0.f);
    float4 P = make_float4(X.x + V.x * dt, X.y + V.y * dt, X.z + V.z * dt, m);
    p[i] = P;
    if (p0) p0[i] = P;  // kept for the warm start and the correction record
}

// IntegrationGPUKernel (P/PBD_cuda.cu:1467-1482): v = (p - x)/dt; x = p
__global__ void __launch_bounds__(256) k_integrate(int n, float dt, float4 *__restrict__ x,
                                                   float4 *__restrict__ v,
                                                   const float4 *__restrict__ p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 P = p[i], X = x[i];
    v[i] = make_float4((P.x - X.x) / dt, (P.y - X.y) / dt, (P.z - X.z) / dt, 0.f);
    x[i] = make_float4(P.x, P.y, P.z, X.w);
}

// one color phase: distance, then bending, then anchor records of the color.
// Launched with programmatic stream serialization: the records (which no
// phase writes) are loaded first, the next phase is allowed to launch, and
// positions are touched only after griddepcontrol.wait, i.e. after the
// previous phase has completed and its writes are visible.
__global__ void __launch_bounds__(512) k_project_color(const int4 *__restrict__ drec, int nd,
                                                       const int4 *__restrict__ bidx,
                                                       const float2 *__restrict__ bpar, int nb,
                                                       const float4 *__restrict__ arec, int na,
                                                       float4 *__restrict__ p, float expk,
                                                       const float *__restrict__ expk_dev,
                                                       int sched) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int4 r = make_int4(0, 0, 0, 0);
    float2 bp = make_float2(0.f, 0.f);
    float4 ar = make_float4(0.f, 0.f, 0.f, 0.f);
    int kind = 0;
    if (t < nd) {
        r = drec[t];
        kind = 1;
    } else if (t < nd + nb) {
        r = bidx[t - nd];
        bp = bpar[t - nd];
        kind = 2;
    } else if (t < nd + nb + na) {
        ar = arec[t - nd - nb];
        kind = 3;
    }
    asm volatile("griddepcontrol.launch_dependents;");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // the solve-to-residual loop keeps the sweep's exponent on the device
    if (expk_dev) expk = *expk_dev;
    GlobalPos P{p};
    if (kind == 1)
        project_distance(r, P, expk, sched);
    else if (kind == 2)
        project_bending(r, bp, P, expk, sched);
    else if (kind == 3)
        project_anchor(ar, P);
}

// ColliWithShpGrd (P/PBD_cuda.cu:1519-1573) on one point
__device__ __forceinline__ float4 obstacle_point(float4 P, int sphere_on, float3 c, float r,
                                                 int ground_on, float gh) {
    if (sphere_on) {
        float dx = P.x - c.x, dy = P.y - c.y, dz = P.z - c.z;
        float d = sqrtf(dx * dx + dy * dy + dz * dz);
        if (!(d - r > 0.001f)) {
            float ex = c.x - P.x, ey = c.y - P.y, ez = c.z - P.z;
            float d2 = sqrtf(ex * ex + ey * ey + ez * ez);
            float move = r - d2;
            float mx = (dx / d2) * move, my = (dy / d2) * move, mz = (dz / d2) * move;
            P.x = P.x + mx;
            P.y = P.y + my;
            P.z = P.z + mz;
        }
    }
    if (ground_on && P.y - gh < 0.001f) P.y = gh;
    return P;
}

// Resident form of the colored GS: every point lives in shared memory for a
// whole launch of one or more sweeps.  A thread-block cluster of S blocks
// (S = 1: a single block, no cluster) keeps point i in block i % S at slot
// i / S (distributed shared memory for S > 1), so a color phase costs one
// cluster barrier instead of a kernel launch.  Block r takes the r-th of S
// even shares of every color's flat record list (distance | bending |
// anchor, the per-color kernel's order; no two records of
// a color share a point), one record per thread and round.  The first
// record of each thread in the next phase is fetched before the barrier.  The
// stiffness factors 1 - (1 - s)^(1/(it+1)) of the object's distinct
// stiffness values are computed once per sweep into a table; a record whose
// value is not in the table computes its own.  Same records, same arithmetic
// per record, so the same result as the per-color launches.
constexpr int kResThreads = 1024;
constexpr int kResMaxColors = 256;
constexpr int kResTab = 8;

template <int S>
struct ResPos {
    float4 *local;
    __device__ __forceinline__ float4 *at(int i) const {
        if constexpr (S == 1)
            return local + i;
        else
            return cg::this_cluster().map_shared_rank(local + (unsigned)i / S,
                                                      (unsigned)i % S);
    }
    __device__ __forceinline__ float4 ld(int i) const { return *at(i); }
    __device__ __forceinline__ void st(int i, float4 v) const { *at(i) = v; }
};

template <int S>
__device__ __forceinline__ void res_sync() {
    if constexpr (S == 1)
        __syncthreads();
    else
        cg::this_cluster().sync();
}

struct ResRec {
    int kind;  // 0 none, 1 distance, 2 bending, 3 anchor
    int4 r;    // distance {i0, i1, rest, s}; bending {e0, e1, wA, wB}
    float4 f;  // bending {rest angle, s}; anchor {rest xyz, point id}
};

// the object's factor for stiffness s (table hit) or s's own
__device__ __forceinline__ float res_factor(float s, float expk, int sched, const float *ts,
                                            const float *tk, int ntab) {
    for (int j = 0; j < ntab; ++j)
        if (ts[j] == s) return tk[j];
    return stiffness_factor(s, expk, sched);
}

template <int S>
__device__ __forceinline__ void res_project(const ResRec &A, const ResPos<S> &P, float expk,
                                            int sched, const float *ts, const float *tk,
                                            int ntab) {
    if (A.kind == 1) {
        float4 N0, N1;
        if (distance_update(P.ld(A.r.x), P.ld(A.r.y), __int_as_float(A.r.z),
                            res_factor(__int_as_float(A.r.w), expk, sched, ts, tk, ntab), N0,
                            N1)) {
            P.st(A.r.x, N0);
            P.st(A.r.y, N1);
        }
    } else if (A.kind == 2) {
        float4 Q[4] = {P.ld(A.r.x), P.ld(A.r.y), P.ld(A.r.z), P.ld(A.r.w)}, N[4];
        if (bending_update(Q, A.f.x, res_factor(A.f.y, expk, sched, ts, tk, ntab), N)) {
            P.st(A.r.x, N[0]);
            P.st(A.r.y, N[1]);
            P.st(A.r.z, N[2]);
            P.st(A.r.w, N[3]);
        }
    } else if (A.kind == 3) {
        int i = __float_as_int(A.f.w);
        P.st(i, make_float4(A.f.x, A.f.y, A.f.z, P.ld(i).w));
    }
}

// seg = dseg | bseg | aseg (n_colors + 1 starts each); tab = the distinct
// stiffness values; sweeps it0..it1-1, the analytic obstacles after each
// sweep when sphere_on / ground_on.
template <int S>
__global__ void __launch_bounds__(kResThreads, 1) k_gs_resident(
    const int *__restrict__ seg, const int4 *__restrict__ drec, const int4 *__restrict__ bidx,
    const float2 *__restrict__ bpar, const float4 *__restrict__ arec,
    const float *__restrict__ tab, int ntab, int n_colors, int n, float4 *__restrict__ p,
    int it0, int it1, int sched, int sphere_on, float3 sc, float sr, int ground_on, float gh) {
    extern __shared__ float4 sp[];
    __shared__ int sg[3 * (kResMaxColors + 1)];
    __shared__ float tab_s[kResTab], tab_k[kResTab];
    int r = 0;
    if constexpr (S > 1) r = (int)cg::this_cluster().block_rank();
    const int tid = threadIdx.x;
    const int nc1 = n_colors + 1;
    const int nloc = (n - r + S - 1) / S;  // this block's points: r, r + S, r + 2S, ...
    for (int c = tid; c < 3 * nc1; c += kResThreads) sg[c] = seg[c];
    if (tid < ntab) tab_s[tid] = tab[tid];
    for (int j = tid; j < nloc; j += kResThreads) sp[j] = p[j * S + r];
    __syncthreads();
    const ResPos<S> P{sp};
    // block r's share [lo, hi) of color c's flat record list
    auto share = [&](int c, int &lo, int &hi, int &dn, int &bn) {
        dn = sg[c + 1] - sg[c];
        bn = sg[nc1 + c + 1] - sg[nc1 + c];
        int an = sg[2 * nc1 + c + 1] - sg[2 * nc1 + c];
        long long tot = dn + bn + an;
        lo = (int)(tot * r / S);
        hi = (int)(tot * (r + 1) / S);
    };
    auto fetch = [&](int c, int f, int hi, int dn, int bn) {
        ResRec q;
        q.kind = 0;
        q.r = make_int4(0, 0, 0, 0);
        q.f = make_float4(0.f, 0.f, 0.f, 0.f);
        if (f >= hi) return q;
        if (f < dn) {
            q.kind = 1;
            q.r = drec[sg[c] + f];
        } else if (f < dn + bn) {
            q.kind = 2;
            int k = sg[nc1 + c] + (f - dn);
            q.r = bidx[k];
            float2 bp = bpar[k];
            q.f = make_float4(bp.x, bp.y, 0.f, 0.f);
        } else {
            q.kind = 3;
            q.f = arec[sg[2 * nc1 + c] + (f - dn - bn)];
        }
        return q;
    };
    int lo, hi, dn, bn;
    share(0, lo, hi, dn, bn);
    ResRec A = fetch(0, lo + tid, hi, dn, bn);
    res_sync<S>();  // every block's points are in place before any remote access
    for (int it = it0; it < it1; ++it) {
        const float expk = (float)(1.0 / (double)(it + 1));
        if (tid < ntab) tab_k[tid] = stiffness_factor(tab_s[tid], expk, sched);
        __syncthreads();
        for (int c = 0; c < n_colors; ++c) {
            share(c, lo, hi, dn, bn);
            res_project<S>(A, P, expk, sched, tab_s, tab_k, ntab);
            for (int f = lo + tid + kResThreads; f < hi; f += kResThreads)
                res_project<S>(fetch(c, f, hi, dn, bn), P, expk, sched, tab_s, tab_k, ntab);
            // the next phase's first record, before the barrier
            const int cn = c + 1 < n_colors ? c + 1 : 0;
            int lo2, hi2, dn2, bn2;
            share(cn, lo2, hi2, dn2, bn2);
            A = fetch(cn, lo2 + tid, hi2, dn2, bn2);
            res_sync<S>();
        }
        if (sphere_on || ground_on) {
            for (int j = tid; j < nloc; j += kResThreads)
                sp[j] = obstacle_point(sp[j], sphere_on, sc, sr, ground_on, gh);
            res_sync<S>();
        }
    }
    for (int j = tid; j < nloc; j += kResThreads) p[j * S + r] = sp[j];
}

// ColliWithShpGrd (P/PBD_cuda.cu:1519-1573): sphere push-out and ground plane
__global__ void k_obstacles(int n, float4 *p, int sphere_on, float3 c, float r, int ground_on,
                            float gh) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    p[i] = obstacle_point(p[i], sphere_on, c, r, ground_on, gh);
}

// the sphere of each point's instance (ColliWithShpGrd's sphere push with a
// per-instance centre and radius)
__global__ void k_obstacles_inst(int n, float4 *p, const int *point_inst, const float4 *spheres,
                                 int n_spheres) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = point_inst[i];
    if (k < 0 || k >= n_spheres) return;
    float4 sp = spheres[k];
    p[i] = obstacle_point(p[i], 1, make_float3(sp.x, sp.y, sp.z), sp.w, 0, 0.f);
}

// residual: FP64 per constraint, warp-shuffle + block reduction
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) k_residual(const int4 *__restrict__ drec, int nd,
                                                  const int4 *__restrict__ bidx,
                                                  const float2 *__restrict__ bpar, int nb,
                                                  const float4 *__restrict__ p, double *part) {
    __shared__ double ws[8];
    double acc = 0.0;
    int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nd + nb; t += stride) {
        if (t < nd) {
            int4 r = drec[t];
            float4 a = p[r.x], b = p[r.y];
            double dx = (double)a.x - b.x, dy = (double)a.y - b.y, dz = (double)a.z - b.z;
            double c = sqrt(dx * dx + dy * dy + dz * dz) - (double)__int_as_float(r.z);
            acc += c * c;
        } else {
            int j = t - nd;
            int4 r = bidx[j];
            float4 q0 = p[r.x], q1 = p[r.y], q2 = p[r.z], q3 = p[r.w];
            double E[3] = {(double)q1.x - q0.x, (double)q1.y - q0.y, (double)q1.z - q0.z};
            double A0[3] = {(double)q2.x - q0.x, (double)q2.y - q0.y, (double)q2.z - q0.z};
            double A1[3] = {(double)q2.x - q1.x, (double)q2.y - q1.y, (double)q2.z - q1.z};
            double B1[3] = {(double)q3.x - q1.x, (double)q3.y - q1.y, (double)q3.z - q1.z};
            double B0[3] = {(double)q3.x - q0.x, (double)q3.y - q0.y, (double)q3.z - q0.z};
            double na[3] = {A0[1] * A1[2] - A0[2] * A1[1], A0[2] * A1[0] - A0[0] * A1[2],
                            A0[0] * A1[1] - A0[1] * A1[0]};
            double nb_[3] = {B1[1] * B0[2] - B1[2] * B0[1], B1[2] * B0[0] - B1[0] * B0[2],
                             B1[0] * B0[1] - B1[1] * B0[0]};
            double cx[3] = {na[1] * nb_[2] - na[2] * nb_[1], na[2] * nb_[0] - na[0] * nb_[2],
                            na[0] * nb_[1] - na[1] * nb_[0]};
            double el = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
            double th = el > 0.0 ? atan2((cx[0] * E[0] + cx[1] * E[1] + cx[2] * E[2]) / el,
                                         na[0] * nb_[0] + na[1] * nb_[1] + na[2] * nb_[2])
                                 : 0.0;
            double c = th - (double)bpar[j].x;
            if (c > 3.141592653589793) c -= 6.283185307179586;
            if (c < -3.141592653589793) c += 6.283185307179586;
            acc += (c * el) * (c * el);
        }
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += ws[w];
        part[blockIdx.x] = s;
    }
}

__global__ void k_sum_parts(int n, const double *part, double *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += part[i];
        out[0] = s;
    }
}

constexpr int kResidualBlocks = 4 * kNumSMs;

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
int launch_obstacles(pbd_solver *s);

static int advect(pbd_object *o, float dt, float4 *p0) {
    float dp = powf(o->damping, dt);
    float3 gdt = make_float3(o->gravity[0] * dt, o->gravity[1] * dt, o->gravity[2] * dt);
    k_advect<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, dt, dp, gdt, o->x.p, o->v.p, o->p.p,
                                                         p0);
    PBD_LAUNCH();
    return PBD_OK;
}
int launch_advect(pbd_object *o, float dt) { return advect(o, dt, nullptr); }
// advect and keep the advected positions in o->p0 (allocated by the caller)
int launch_advect_p0(pbd_object *o, float dt) { return advect(o, dt, o->p0.p); }

int launch_residual_parts(pbd_object *o, bool dist, bool bend, const float4 *pos) {
    int nd = o->h_dseg.empty() ? 0 : o->h_dseg.back();
    int nb = o->h_bseg.empty() ? 0 : o->h_bseg.back();
    k_residual<<<kResidualBlocks, 256, 0, o->stream>>>(o->drec.p, dist ? nd : 0, o->bidx.p,
                                                       o->bpar.p, bend ? nb : 0, pos,
                                                       o->res_part.p);
    PBD_LAUNCH();
    return PBD_OK;
}

int launch_integrate(pbd_object *o, float dt) {
    k_integrate<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, dt, o->x.p, o->v.p, o->p.p);
    PBD_LAUNCH();
    return PBD_OK;
}

static inline int __float_as_int_host(float f) {
    int i;
    memcpy(&i, &f, sizeof(i));
    return i;
}

static int launch_sweep_per_color(pbd_object *o, int iter, const float *expk_dev = nullptr) {
    float expk = (float)(1.0 / (double)(iter + 1));
    for (int c = 0; c < o->n_colors; ++c) {
        int d0 = o->h_dseg[c], nd = o->h_dseg[c + 1] - d0;
        int b0 = o->h_bseg[c], nb = o->h_bseg[c + 1] - b0;
        int a0 = o->h_aseg[c], na = o->h_aseg[c + 1] - a0;
        int tot = nd + nb + na;
        if (!tot) continue;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid_for(tot, o->gs_block));
        cfg.blockDim = dim3(o->gs_block);
        cfg.stream = o->stream;
        cudaLaunchAttribute at[2];
        at[0].id = cudaLaunchAttributePriority;
        at[0].val.priority = gs_priority();
        at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = o->pdl ? 2 : 1;
        PBD_CUDA(cudaLaunchKernelEx(&cfg, k_project_color, (const int4 *)(o->drec.p + d0), nd,
                                    (const int4 *)(o->bidx.p + b0), (const float2 *)(o->bpar.p + b0),
                                    nb, (const float4 *)(o->arec.p + a0), na, o->p.p, expk,
                                    expk_dev, o->sched));
    }
    return PBD_OK;
}

int gs_priority() {
    static int prio = 1;
    if (prio == 1) {
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
            cudaGetLastError();
            greatest = 0;
        }
        prio = greatest;
    }
    return prio;
}

int launch_sweep_dev(pbd_solver *s, const float *expk_dev, bool obstacles_inside) {
    PBD_TRY(launch_sweep_per_color(s->obj, 0, expk_dev));
    if (obstacles_inside) PBD_TRY(launch_obstacles(s));
    return PBD_OK;
}

// The kernel attribute is process-wide, so it is set to the device's opt-in
// limit (net of the static shared memory), the same value for every object:
// a small object planned after a large one must not lower the limit that
// the large object's launches need.
template <int S>
static bool resident_fits(int n, int smem_optin) {
    size_t smem = sizeof(float4) * (size_t)((n + S - 1) / S);
    if (smem < 16) smem = 16;
    if ((long long)smem > smem_optin) return false;
    if (cudaFuncSetAttribute(k_gs_resident<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_optin) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (S > 8 && cudaFuncSetAttribute(k_gs_resident<S>,
                                      cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                     cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(S);
    cfg.blockDim = dim3(kResThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = S;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_gs_resident<S>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return nclusters >= 1;
}

// Once per coloring: which cluster sizes hold every point in shared memory,
// the device copy of the per-color record starts and the table of distinct
// stiffness values.  The records themselves are the per-color ones.
static int resident_plan(pbd_object *o) {
    if (o->cl_state != 0) return PBD_OK;
    o->cl_state = -1;
    o->cl_fit = 0;
    const int nc = o->n_colors;
    if (o->np == 0 || nc == 0 || nc > kResMaxColors) return PBD_OK;
    int dev = 0, optin = 0;
    PBD_CUDA(cudaGetDevice(&dev));
    PBD_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    optin -= (int)(sizeof(int) * 3 * (kResMaxColors + 1) + 2 * sizeof(float) * kResTab) + 1024;
    if (resident_fits<1>(o->n, optin)) o->cl_fit |= 1;
    if (resident_fits<2>(o->n, optin)) o->cl_fit |= 2;
    if (resident_fits<4>(o->n, optin)) o->cl_fit |= 4;
    if (resident_fits<8>(o->n, optin)) o->cl_fit |= 8;
    if (resident_fits<16>(o->n, optin)) o->cl_fit |= 16;
    if (!o->cl_fit) return PBD_OK;
    cudaStream_t s = o->stream;
    const int nd = o->h_dseg[nc], nb = o->h_bseg[nc];
    std::vector<int4> d(nd);
    std::vector<float2> bp(nb);
    if (nd) PBD_CUDA(cudaMemcpyAsync(d.data(), o->drec.p, sizeof(int4) * nd, cudaMemcpyDeviceToHost, s));
    if (nb) PBD_CUDA(cudaMemcpyAsync(bp.data(), o->bpar.p, sizeof(float2) * nb, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    // the first kResTab distinct stiffness values, in record order
    std::vector<float> tab;
    auto add = [&](float v) {
        if (v != v || (int)tab.size() >= kResTab) return;
        for (float t : tab)
            if (t == v) return;
        tab.push_back(v);
    };
    for (int k = 0; k < nd; ++k) {
        float v;
        std::memcpy(&v, &d[k].w, sizeof(float));
        add(v);
    }
    for (int k = 0; k < nb; ++k) add(bp[k].y);
    std::vector<int> seg;
    seg.insert(seg.end(), o->h_dseg.begin(), o->h_dseg.end());
    seg.insert(seg.end(), o->h_bseg.begin(), o->h_bseg.end());
    seg.insert(seg.end(), o->h_aseg.begin(), o->h_aseg.end());
    PBD_TRY(o->cl_seg.upload(seg.data(), seg.size(), s));
    // full capacity once: graphs captured earlier keep the table's address
    PBD_TRY(o->cl_tab.alloc(kResTab));
    if (!tab.empty()) PBD_TRY(o->cl_tab.upload(tab.data(), tab.size(), s));
    PBD_CUDA(cudaStreamSynchronize(s));
    o->cl_ntab = (int)tab.size();
    o->cl_state = 1;
    return PBD_OK;
}

// cluster size in use: the one set, else the largest that fits
static int resident_size(const pbd_object *o) {
    if (o->cl_S) return (o->cl_fit & o->cl_S) ? o->cl_S : 0;
    for (int S = 16; S >= 1; S >>= 1)
        if (o->cl_fit & S) return S;
    return 0;
}

template <int S>
static int launch_resident_s(pbd_solver *s, int it0, int it1, bool ob) {
    pbd_object *o = s->obj;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(S);
    cfg.blockDim = dim3(kResThreads);
    cfg.dynamicSmemBytes = std::max<size_t>(16, sizeof(float4) * (size_t)((o->n + S - 1) / S));
    cfg.stream = o->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = S;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = S > 1 ? 1 : 0;
    PBD_CUDA(cudaLaunchKernelEx(
        &cfg, k_gs_resident<S>, (const int *)o->cl_seg.p, (const int4 *)o->drec.p,
        (const int4 *)o->bidx.p, (const float2 *)o->bpar.p, (const float4 *)o->arec.p,
        (const float *)o->cl_tab.p, o->cl_ntab, o->n_colors, o->n, o->p.p, it0, it1, o->sched,
        ob ? s->sphere_on : 0, make_float3(s->sphere_c[0], s->sphere_c[1], s->sphere_c[2]),
        s->sphere_r, ob ? s->ground_on : 0, s->ground_h));
    return PBD_OK;
}

static int launch_resident(pbd_solver *s, int it0, int it1, bool ob) {
    switch (resident_size(s->obj)) {
        case 1: return launch_resident_s<1>(s, it0, it1, ob);
        case 2: return launch_resident_s<2>(s, it0, it1, ob);
        case 4: return launch_resident_s<4>(s, it0, it1, ob);
        case 8: return launch_resident_s<8>(s, it0, it1, ob);
        case 16: return launch_resident_s<16>(s, it0, it1, ob);
    }
    PBD_CHECK(false, PBD_ERR_STATE, "no cluster size holds this object's points");
}

// PBD_GS_AUTO takes the per-color launches, which apply to every object; the
// autotuner picks the block size, or the resident form and its cluster size
// where that is faster, per object.
static int resolved_path(pbd_solver *s) {
    if (s->gs_path != PBD_GS_CLUSTER) return PBD_GS_PER_COLOR;
    if (s->n_inst_spheres > 0) return -2;  // per-instance spheres: per-color form only
    if (resident_plan(s->obj) != PBD_OK) return -1;
    return s->obj->cl_state == 1 && resident_size(s->obj) ? PBD_GS_CLUSTER : -2;
}

// Everything a launch form needs before a stream capture (plans and
// uploads); capture forbids allocation and synchronisation.
int prepare_gs_path(pbd_solver *s) {
    pbd_object *o = s->obj;
    if (s->gs_path == PBD_GS_CLUSTER) PBD_TRY(resident_plan(o));
    return PBD_OK;
}

// GS sweeps it0..it1-1, each followed by the analytic obstacles when
// obstacles_inside (otherwise the caller applies them)
int launch_sweeps(pbd_solver *s, int it0, int it1, bool obstacles_inside) {
    pbd_object *o = s->obj;
    PBD_CHECK(o->sorted, PBD_ERR_STATE,
              "no color-sorted constraints: run edge coloring and SortEdgesColors first");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    PBD_CUDA(cudaStreamIsCapturing(o->stream, &cap));
    if (cap == cudaStreamCaptureStatusNone) PBD_TRY(prepare_gs_path(s));
    int path = resolved_path(s);
    PBD_CHECK(path != -1, PBD_ERR_CUDA, "launch plan failed: %s", pbd_last_error());
    PBD_CHECK(path != -2, PBD_ERR_STATE,
              "the requested Gauss-Seidel form does not apply to this object (%d points)", o->n);
    if (path == PBD_GS_CLUSTER)
        return launch_resident(s, it0, it1, obstacles_inside && (s->sphere_on || s->ground_on));
    for (int it = it0; it < it1; ++it) {
        PBD_TRY(launch_sweep_per_color(o, it));
        if (obstacles_inside) PBD_TRY(launch_obstacles(s));
    }
    return PBD_OK;
}

int launch_obstacles(pbd_solver *s) {
    pbd_object *o = s->obj;
    if (s->sphere_on || s->ground_on) {
        k_obstacles<<<grid_for(o->n, 256), 256, 0, o->stream>>>(
            o->n, o->p.p, s->sphere_on,
            make_float3(s->sphere_c[0], s->sphere_c[1], s->sphere_c[2]), s->sphere_r,
            s->ground_on, s->ground_h);
        PBD_LAUNCH();
    }
    if (s->n_inst_spheres > 0 && o->has_inst) {
        k_obstacles_inst<<<grid_for(o->n, 256), 256, 0, o->stream>>>(
            o->n, o->p.p, o->point_inst.p, s->inst_spheres.p, s->n_inst_spheres);
        PBD_LAUNCH();
    }
    return PBD_OK;
}

static int build_point_csr(pbd_object *o, int n_entries, const int *d_owner_counts, int n_owners,
                           bool tris, DBuf<int> &first, DBuf<int> &last, DBuf<int> &owner) {
    cudaStream_t s = o->stream;
    DBuf<uint32_t> key, key2;
    DBuf<int> val, val2, eoff;
    PBD_TRY(key.alloc(n_entries));
    PBD_TRY(key2.alloc(n_entries));
    PBD_TRY(val.alloc(n_entries));
    PBD_TRY(val2.alloc(n_entries));
    if (tris) {
        k_emit_tri_points<<<grid_for(o->nt, 256), 256, 0, s>>>(o->nt, o->tri.p, key.p, val.p);
    } else {
        PBD_TRY(eoff.alloc(n_owners + 1));
        PBD_TRY(exclusive_scan(d_owner_counts, eoff.p, n_owners, nullptr, s));
        k_emit_prim_points<<<grid_for(n_owners, 256), 256, 0, s>>>(n_owners, o->prim_list.p,
                                                                    o->indices.p, eoff.p, key.p,
                                                                    val.p);
    }
    PBD_LAUNCH();
    uint32_t *sk;
    int *sv;
    PBD_TRY(radix_sort<uint32_t>(key.p, val.p, key2.p, val2.p, n_entries, nullptr,
                                 round8(bits_for(o->n)), o->scr, s, &sk, &sv));
    PBD_TRY(first.alloc(o->n + 1));
    PBD_TRY(last.alloc(o->n + 1));
    PBD_TRY(owner.alloc(n_entries));
    PBD_CUDA(cudaMemsetAsync(first.p, 0, sizeof(int) * (o->n + 1), s));
    PBD_CUDA(cudaMemsetAsync(last.p, 0, sizeof(int) * (o->n + 1), s));
    if (n_entries) {
        k_run_bounds<<<grid_for(n_entries, 256), 256, 0, s>>>(n_entries, sk, first.p, last.p);
        PBD_CUDA(cudaMemcpyAsync(owner.p, sv, sizeof(int) * n_entries, cudaMemcpyDeviceToDevice, s));
    }
    PBD_LAUNCH();
    PBD_CUDA(cudaStreamSynchronize(s));
    return PBD_OK;
}

}  // namespace pbd

using namespace pbd;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *pbd_last_error(void) { return pbd::g_err.c_str(); }
int pbd_version(void) { return 1; }

int pbd_object_create(const pbd_object_desc *d, pbd_object **out) {
    PBD_CHECK(d && out, PBD_ERR_ARG, "null argument");
    *out = nullptr;
    PBD_CHECK(d->n_points > 0 && d->pos && d->mass, PBD_ERR_ARG, "need n_points > 0, pos, mass");
    PBD_CHECK(d->n_tris >= 0 && (d->n_tris == 0 || d->tri_idx), PBD_ERR_ARG, "bad triangles");
    PBD_CHECK(d->n_prims >= 0 && (d->n_prims == 0 || (d->prim_list && d->indices &&
                                                      d->constraint_type && d->stiffness)),
              PBD_ERR_ARG, "bad constraint buffers");
    // host-side validation of the constraint topology
    int n_idx = 0;
    std::vector<int> cnt(d->n_prims), ct(d->n_prims);
    for (int p = 0; p < d->n_prims; ++p) {
        int s = d->prim_list[2 * p], c = d->prim_list[2 * p + 1];
        int t = d->constraint_type[p];
        int need = t == PBD_DISTANCE ? 2 : t == PBD_BENDING ? 4 : t == PBD_ANCHOR ? 1 : -1;
        PBD_CHECK(need > 0, PBD_ERR_ARG, "prim %d: unknown constraint type %d", p, t);
        PBD_CHECK(c == need && s >= 0, PBD_ERR_ARG, "prim %d: type %d needs %d points, has %d", p,
                  t, need, c);
        PBD_CHECK(t != PBD_DISTANCE || d->rest_length, PBD_ERR_ARG, "rest_length missing");
        if (s + c > n_idx) n_idx = s + c;
        cnt[p] = c;
        ct[p] = t;
    }
    for (int i = 0; i < n_idx; ++i)
        PBD_CHECK(d->indices[i] >= 0 && d->indices[i] < d->n_points, PBD_ERR_ARG,
                  "constraint index %d out of range", i);
    for (long long i = 0; i < 3LL * d->n_tris; ++i)
        PBD_CHECK(d->tri_idx[i] >= 0 && d->tri_idx[i] < d->n_points, PBD_ERR_ARG,
                  "triangle index %lld out of range", i);

    pbd_object *o = new pbd_object();
    auto fail = [&](int r) {
        pbd_object_destroy(o);
        return r;
    };
    o->n = d->n_points;
    o->nt = d->n_tris;
    o->np = d->n_prims;
    o->n_idx = n_idx;
    o->damping = d->damping_rate;
    for (int k = 0; k < 3; ++k) o->gravity[k] = d->gravity[k];
    o->h_prim_count = cnt;
    o->h_ctype = ct;
    o->h_mass.assign(d->mass, d->mass + d->n_points);
    int r;
    if (cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed: %s", cudaGetErrorString(cudaGetLastError()));
        delete o;
        return PBD_ERR_CUDA;
    }
    cudaStream_t s = o->stream;
    {
        DBuf<float> hp, hv, hm;
        if ((r = hp.upload(d->pos, 3 * (size_t)o->n, s)) || (r = hm.upload(d->mass, o->n, s)))
            return fail(r);
        if (d->vel && (r = hv.upload(d->vel, 3 * (size_t)o->n, s))) return fail(r);
        if ((r = o->x.alloc(o->n)) || (r = o->p.alloc(o->n)) || (r = o->v.alloc(o->n)) ||
            (r = o->mass.upload(d->mass, o->n, s)))
            return fail(r);
        k_pack_state<<<grid_for(o->n, 256), 256, 0, s>>>(o->n, hp.p, d->vel ? hv.p : nullptr,
                                                         hm.p, o->x.p, o->p.p, o->v.p);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("state upload failed: %s", cudaGetErrorString(cudaGetLastError()));
            return fail(PBD_ERR_CUDA);
        }
    }
    // triangles
    if (o->nt) {
        DBuf<int> ht, hi;
        if ((r = ht.upload(d->tri_idx, 3 * (size_t)o->nt, s))) return fail(r);
        if (d->tri_inst && (r = hi.upload(d->tri_inst, o->nt, s))) return fail(r);
        if ((r = o->tri.alloc(o->nt))) return fail(r);
        k_pack_tris<<<grid_for(o->nt, 256), 256, 0, s>>>(o->nt, ht.p, d->tri_inst ? hi.p : nullptr,
                                                         o->tri.p);
        if ((r = build_point_csr(o, 3 * o->nt, nullptr, 0, true, o->pt_tri_first, o->pt_tri_last,
                                 o->pt_tri)))
            return fail(r);
    }
    o->has_inst = d->point_inst != nullptr;
    if (d->point_inst && (r = o->point_inst.upload(d->point_inst, o->n, s))) return fail(r);
    if (d->point_inst) {
        std::vector<int> ti(o->nt, 0);
        if (d->tri_inst) ti.assign(d->tri_inst, d->tri_inst + o->nt);
        if ((r = o->tri_inst.upload(ti.data(), o->nt, s))) return fail(r);
        if (cudaStreamSynchronize(s) != cudaSuccess) return fail(PBD_ERR_CUDA);
    }
    // constraint buffers
    if (o->np) {
        if ((r = o->prim_list.upload((const int2 *)d->prim_list, o->np, s)) ||
            (r = o->indices.upload(d->indices, n_idx, s)) ||
            (r = o->ctype.upload(d->constraint_type, o->np, s)) ||
            (r = o->stiffness.upload(d->stiffness, o->np, s)))
            return fail(r);
        std::vector<float> zero(o->np, 0.f);
        if ((r = o->rest_length.upload(d->rest_length ? d->rest_length : zero.data(), o->np, s)) ||
            (r = o->rest_angle.upload(d->rest_angle ? d->rest_angle : zero.data(), o->np, s)))
            return fail(r);
        std::vector<float4> rp(o->np, make_float4(0, 0, 0, 0));
        if (d->rest_pos)
            for (int p = 0; p < o->np; ++p)
                rp[p] = make_float4(d->rest_pos[3 * p], d->rest_pos[3 * p + 1],
                                    d->rest_pos[3 * p + 2], 0.f);
        if ((r = o->rest_pos.upload(rp.data(), o->np, s))) return fail(r);
        if (cudaStreamSynchronize(s) != cudaSuccess) return fail(PBD_ERR_CUDA);
        // Point2PrimsMap as CSR, then Prim2PrimsMap
        DBuf<int> pc, pfirst, plast, pprim, deg, off;
        if ((r = pc.alloc(o->np))) return fail(r);
        k_prim_counts<<<grid_for(o->np, 256), 256, 0, s>>>(o->np, o->prim_list.p, pc.p);
        long long n_entries = 0;
        for (int p = 0; p < o->np; ++p) n_entries += cnt[p];
        if ((r = build_point_csr(o, (int)n_entries, pc.p, o->np, false, pfirst, plast, pprim)))
            return fail(r);
        if ((r = deg.alloc(o->np)) || (r = off.alloc(o->np)) || (r = o->flag.alloc(4)))
            return fail(r);
        k_adj_count<<<grid_for(o->np, 256), 256, 0, s>>>(o->np, o->prim_list.p, o->indices.p,
                                                          pfirst.p, plast.p, pprim.p, deg.p);
        if ((r = exclusive_scan(deg.p, off.p, o->np, o->flag.p, s))) return fail(r);
        int total = 0;
        if (cudaMemcpyAsync(&total, o->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s) ||
            cudaStreamSynchronize(s)) {
            set_error("adjacency count failed: %s", cudaGetErrorString(cudaGetLastError()));
            return fail(PBD_ERR_CUDA);
        }
        o->n_adj = total;
        if ((r = o->adj_sn.alloc(o->np)) || (r = o->adj.alloc(total))) return fail(r);
        k_adj_fill<<<grid_for(o->np, 256), 256, 0, s>>>(o->np, o->prim_list.p, o->indices.p,
                                                         pfirst.p, plast.p, pprim.p, off.p,
                                                         o->adj_sn.p, o->adj.p);
        if ((r = o->color.alloc(o->np)) || (r = o->prd_color.alloc(o->np))) return fail(r);
        if (cudaMemsetAsync(o->color.p, 0xff, sizeof(int) * o->np, s) ||
            cudaMemsetAsync(o->prd_color.p, 0xff, sizeof(int) * o->np, s) ||
            cudaStreamSynchronize(s)) {
            set_error("adjacency build failed: %s", cudaGetErrorString(cudaGetLastError()));
            return fail(PBD_ERR_CUDA);
        }
        // residual denominator: rest lengths and hinge lengths of the
        // initial positions
        double den = 0.0, den_d = 0.0;
        for (int p = 0; p < o->np; ++p) {
            const int *ix = d->indices + d->prim_list[2 * p];
            if (ct[p] == PBD_DISTANCE) {
                double l = d->rest_length[p];
                den += l * l;
                den_d += l * l;
            } else if (ct[p] == PBD_BENDING) {
                double e2 = 0.0;
                for (int k = 0; k < 3; ++k) {
                    double dd = (double)d->pos[3 * ix[1] + k] - d->pos[3 * ix[0] + k];
                    e2 += dd * dd;
                }
                den += e2;
            }
        }
        o->res_den = den;
        o->res_den_d = den_d;
        o->h_prim_list.assign(d->prim_list, d->prim_list + 2 * (size_t)o->np);
        o->h_indices.assign(d->indices, d->indices + n_idx);
        o->h_rest_length.assign(o->np, 0.f);
        if (d->rest_length)
            for (int p = 0; p < o->np; ++p) o->h_rest_length[p] = d->rest_length[p];
    }
    if ((r = o->res_part.alloc(kResidualBlocks)) || (r = o->res_out.alloc(1))) return fail(r);
    *out = o;
    return PBD_OK;
}

int pbd_object_create_grid(float damping, const float *gravity, int res_x, int res_y,
                           float size_x, float size_y, unsigned ct_mask, const float *stiffness,
                           pbd_object **out) {
    PBD_CHECK(gravity && stiffness && out && res_x >= 2 && res_y >= 2, PBD_ERR_ARG,
              "bad grid arguments");
    int n = res_x * res_y;
    // initPosition (P/PBD_cuda.cu:831-852)
    std::vector<float> pos(3 * (size_t)n), vel(3 * (size_t)n, 0.f), mass(n, 1.f);
    float lx = size_x / (res_x - 1), lz = size_y / (res_y - 1);
    for (int i = 0; i < res_y; ++i)
        for (int j = 0; j < res_x; ++j) {
            int k = i * res_x + j;
            pos[3 * k] = 0.0f + j * lx;
            pos[3 * k + 1] = 0.0f;
            pos[3 * k + 2] = 0.0f + i * lz;
        }
    // initMeshTopolIndices (P/PBD_cuda.cu:854-869)
    std::vector<int> tri;
    for (int i = 0; i < n - res_x; ++i) {
        if (i % res_x == res_x - 1) continue;
        int t[6] = {i, i + res_x, i + res_x + 1, i, i + res_x + 1, i + 1};
        tri.insert(tri.end(), t, t + 6);
    }
    std::vector<int> pl, idx, ctv;
    std::vector<float> rl, st, ra, rp;
    auto dist = [&](int a, int b) {  // Distance (P/PBD_cuda.cu:3-6)
        float dx = pos[3 * a] - pos[3 * b], dy = pos[3 * a + 1] - pos[3 * b + 1],
              dz = pos[3 * a + 2] - pos[3 * b + 2];
        return powf(powf(dx, 2) + powf(dy, 2) + powf(dz, 2), 0.5f);
    };
    auto add_prim = [&](std::initializer_list<int> pts, int type, float rest, float stf) {
        pl.push_back((int)idx.size());
        pl.push_back((int)pts.size());
        for (int q : pts) idx.push_back(q);
        ctv.push_back(type);
        rl.push_back(rest);
        st.push_back(stf);
        ra.push_back(0.f);
        rp.push_back(0.f);
        rp.push_back(0.f);
        rp.push_back(0.f);
    };
    if (ct_mask & PBD_DISTANCE) {
        // InitDistanceIndices stencil (P/PBD_cuda.cu:19-54)
        std::vector<int> e;
        for (int i = 0; i < n - res_x; ++i) {
            if (i % res_x == 0) {
                int a[4] = {i, i + 1, i, i + res_x};
                e.insert(e.end(), a, a + 4);
            } else if (i % res_x == res_x - 1) {
                int a[4] = {i, i + res_x, i, i + res_x - 1};
                e.insert(e.end(), a, a + 4);
            } else {
                int a[6] = {i, i + 1, i, i + res_x, i, i + res_x - 1};
                e.insert(e.end(), a, a + 6);
            }
        }
        for (int i = n - res_x; i < n - 1; ++i) {
            e.push_back(i);
            e.push_back(i + 1);
        }
        for (size_t k = 0; k < e.size(); k += 2)
            add_prim({e[k], e[k + 1]}, PBD_DISTANCE, dist(e[k], e[k + 1]), stiffness[0]);
    }
    if (ct_mask & PBD_BENDING) {
        // InitBendingConstr is an empty stub in the reference (P/PBD_cuda.cu:
        // 110-123); here BENDING adds a dihedral constraint on every interior
        // mesh edge, rest angle 0 (the grid is flat).
        std::vector<long long> keys;
        std::vector<int> opp;
        int ntri = (int)tri.size() / 3;
        for (int t = 0; t < ntri; ++t)
            for (int k = 0; k < 3; ++k) {
                int a = tri[3 * t + k], b = tri[3 * t + (k + 1) % 3], c = tri[3 * t + (k + 2) % 3];
                keys.push_back(((long long)std::min(a, b) << 32) | (unsigned)std::max(a, b));
                opp.push_back(c);
                (void)c;
            }
        std::vector<int> order(keys.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return keys[a] < keys[b]; });
        for (size_t i = 0; i + 1 < order.size(); ++i) {
            if (keys[order[i]] != keys[order[i + 1]]) continue;
            int ea = order[i], eb = order[i + 1];
            int t = ea / 3, k = ea % 3;
            int e0 = tri[3 * t + k], e1 = tri[3 * t + (k + 1) % 3];
            add_prim({e0, e1, opp[ea], opp[eb]}, PBD_BENDING, 0.f, stiffness[1]);
            ++i;
        }
    }
    if (ct_mask & PBD_ANCHOR) {
        // InitAnchorConstr (P/PBD_cuda.cu:125-153): points 0 and res_y-1, rest
        // positions of points 0 and res_x-1 (initPosition, :850-851)
        int pts[2] = {0, res_y - 1}, restp[2] = {0, res_x - 1};
        for (int a = 0; a < 2; ++a) {
            add_prim({pts[a]}, PBD_ANCHOR, 0.f, stiffness[2]);
            for (int k = 0; k < 3; ++k) rp[rp.size() - 3 + k] = pos[3 * restp[a] + k];
        }
    }
    pbd_object_desc d;
    memset(&d, 0, sizeof(d));
    d.n_points = n;
    d.pos = pos.data();
    d.vel = vel.data();
    d.mass = mass.data();
    d.n_tris = (int)tri.size() / 3;
    d.tri_idx = tri.data();
    d.n_prims = (int)ctv.size();
    d.prim_list = pl.data();
    d.indices = idx.data();
    d.constraint_type = ctv.data();
    d.rest_length = rl.data();
    d.stiffness = st.data();
    d.rest_angle = ra.data();
    d.rest_pos = rp.data();
    d.damping_rate = damping;
    for (int k = 0; k < 3; ++k) d.gravity[k] = gravity[k];
    return pbd_object_create(&d, out);
}

int pbd_object_destroy(pbd_object *o) {
    if (!o) return PBD_OK;
    if (o->stream) cudaStreamSynchronize(o->stream);
    cudaStream_t s = o->stream;
    if (o->in_done) cudaEventDestroy(o->in_done);
    delete o;  // DBuf / HBuf members free their memory
    if (s) cudaStreamDestroy(s);
    return PBD_OK;
}

int pbd_object_sizes(const pbd_object *o, int *n, int *nt, int *np) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    if (n) *n = o->n;
    if (nt) *nt = o->nt;
    if (np) *np = o->np;
    return PBD_OK;
}

// float3 <-> float4 (w = massBuffer value, or 0) on the device, so that host
// transfers move 12 bytes per point through page-locked staging
__global__ void k_pack3(int n, const float *__restrict__ src, const float *__restrict__ mass,
                        float4 *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], mass ? mass[i] : 0.f);
}

__global__ void k_unpack3(int n, const float4 *__restrict__ src, float *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = src[i];
    dst[3 * i] = v.x;
    dst[3 * i + 1] = v.y;
    dst[3 * i + 2] = v.z;
}

static int staging(pbd_object *o) {
    size_t m = 3 * (size_t)o->n;
    PBD_TRY(o->h_in.alloc(2 * m));
    PBD_TRY(o->h_out.alloc(2 * m));
    PBD_TRY(o->d3.alloc(2 * m));
    if (!o->in_done) PBD_CUDA(cudaEventCreateWithFlags(&o->in_done, cudaEventDisableTiming));
    return PBD_OK;
}

// page-locked (cudaHostAlloc / cudaHostRegister) host memory is copied
// directly; anything else goes through the object's staging
static bool page_locked(const void *h) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// Device float4 arrays src[k] -> host float3 arrays dst[k] (k < cnt); blocks
// until every dst holds its values.
static int copy_out3n(pbd_object *o, int cnt, const float4 *const *src, float *const *dst) {
    for (int k = 0; k < cnt; ++k) PBD_CHECK(dst[k], PBD_ERR_ARG, "null argument");
    if (o->n == 0) return PBD_OK;
    PBD_TRY(staging(o));
    const size_t m = 3 * (size_t)o->n, bytes = sizeof(float) * m;
    bool direct[2];
    for (int k = 0; k < cnt; ++k) {
        direct[k] = page_locked(dst[k]);
        float *d3 = o->d3.p + k * m;
        k_unpack3<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, src[k], d3);
        PBD_LAUNCH();
        PBD_CUDA(cudaMemcpyAsync(direct[k] ? dst[k] : o->h_out.p + k * m, d3, bytes,
                                 cudaMemcpyDeviceToHost, o->stream));
    }
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    for (int k = 0; k < cnt; ++k)
        if (!direct[k]) std::memcpy(dst[k], o->h_out.p + k * m, bytes);
    return PBD_OK;
}

// Host float3 arrays src[k] -> device float4 arrays dst[k] (w = massBuffer
// value when keep_w[k], else 0).  Returns once every src has been read; the
// copies are ordered before later work on the object's stream.
static int copy_in3n(pbd_object *o, int cnt, float4 *const *dst, const float *const *src,
                     const bool *keep_w) {
    for (int k = 0; k < cnt; ++k) PBD_CHECK(src[k], PBD_ERR_ARG, "null argument");
    if (o->n == 0) return PBD_OK;
    PBD_TRY(staging(o));
    const size_t m = 3 * (size_t)o->n, bytes = sizeof(float) * m;
    // the previous upload out of the staging (or a caller's page-locked
    // array) has to be done before the staging is overwritten
    PBD_CUDA(cudaEventSynchronize(o->in_done));
    bool any_direct = false;
    for (int k = 0; k < cnt; ++k) {
        const bool direct = page_locked(src[k]);
        any_direct |= direct;
        if (!direct) std::memcpy(o->h_in.p + k * m, src[k], bytes);
        float *d3 = o->d3.p + k * m;
        PBD_CUDA(cudaMemcpyAsync(d3, direct ? src[k] : o->h_in.p + k * m, bytes,
                                 cudaMemcpyHostToDevice, o->stream));
        k_pack3<<<grid_for(o->n, 256), 256, 0, o->stream>>>(
            o->n, d3, keep_w[k] ? o->mass.p : nullptr, dst[k]);
        PBD_LAUNCH();
    }
    PBD_CUDA(cudaEventRecord(o->in_done, o->stream));
    // a caller's page-locked array is read by the copy itself: wait for it
    if (any_direct) PBD_CUDA(cudaEventSynchronize(o->in_done));
    return PBD_OK;
}

static int copy_out3(pbd_object *o, const float4 *src, float *dst) {
    PBD_CHECK(o, PBD_ERR_ARG, "null argument");
    return copy_out3n(o, 1, &src, &dst);
}

static int copy_in3(pbd_object *o, float4 *dst, const float *src, bool keep_w) {
    PBD_CHECK(o, PBD_ERR_ARG, "null argument");
    return copy_in3n(o, 1, &dst, &src, &keep_w);
}

int pbd_object_get_positions(pbd_object *o, float *v) { return copy_out3(o, o ? o->x.p : nullptr, v); }
int pbd_object_get_velocities(pbd_object *o, float *v) { return copy_out3(o, o ? o->v.p : nullptr, v); }
int pbd_object_get_predicted(pbd_object *o, float *v) { return copy_out3(o, o ? o->p.p : nullptr, v); }
int pbd_object_set_positions(pbd_object *o, const float *v) { return copy_in3(o, o ? o->x.p : nullptr, v, true); }
int pbd_object_set_velocities(pbd_object *o, const float *v) { return copy_in3(o, o ? o->v.p : nullptr, v, false); }
int pbd_object_set_predicted(pbd_object *o, const float *v) { return copy_in3(o, o ? o->p.p : nullptr, v, true); }

int pbd_object_get_state(pbd_object *o, float *pos3, float *vel3) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    const float4 *src[2] = {o->x.p, o->v.p};
    float *dst[2] = {pos3, vel3};
    return copy_out3n(o, 2, src, dst);
}

int pbd_object_set_state(pbd_object *o, const float *pos3, const float *vel3) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    float4 *dst[2] = {o->x.p, o->v.p};
    const float *src[2] = {pos3, vel3};
    const bool keep[2] = {true, false};
    return copy_in3n(o, 2, dst, src, keep);
}

// records i0.. from the per-prim buffers, after a per-prim change
static int rebuild_records(pbd_object *o, int i0) {
    const int n_rec = o->n_rec[0] + o->n_rec[1] + o->n_rec[2];
    if (!o->sorted || i0 >= n_rec) return PBD_OK;
    k_build_records<<<grid_for(n_rec - i0, 256), 256, 0, o->stream>>>(
        i0, n_rec, o->rec_prim.p, o->prim_list.p, o->indices.p, o->rest_length.p,
        o->stiffness.p, o->rest_angle.p, o->rest_pos.p, o->n_rec[0], o->n_rec[1], o->n_rec[2],
        o->drec.p, o->bidx.p, o->bpar.p, o->arec.p);
    PBD_LAUNCH();
    return PBD_OK;
}

int pbd_object_set_stiffness_schedule(pbd_object *o, int schedule) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    PBD_CHECK(schedule >= PBD_SCHEDULE_REFERENCE && schedule <= PBD_SCHEDULE_DIRECT, PBD_ERR_ARG,
              "unknown stiffness schedule %d", schedule);
    o->sched = schedule;
    return PBD_OK;
}

int pbd_object_get_stiffness_schedule(pbd_object *o, int *schedule) {
    PBD_CHECK(o && schedule, PBD_ERR_ARG, "null argument");
    *schedule = o->sched;
    return PBD_OK;
}

int pbd_object_set_stiffness(pbd_object *o, unsigned ct_mask, float value) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    PBD_CHECK(value == value, PBD_ERR_ARG, "stiffness is NaN");
    if (!o->np || !ct_mask) return PBD_OK;
    k_set_type_stiffness<<<grid_for(o->np, 256), 256, 0, o->stream>>>(o->np, o->ctype.p, ct_mask,
                                                                       value, o->stiffness.p);
    PBD_LAUNCH();
    PBD_TRY(rebuild_records(o, 0));
    o->cl_state = 0;  // the resident form's table of distinct values
    return PBD_OK;
}

int pbd_object_set_anchor_targets(pbd_object *o, int n, const int *prims, const float *targets) {
    PBD_CHECK(o && n >= 0 && (n == 0 || (prims && targets)), PBD_ERR_ARG, "bad argument");
    for (int i = 0; i < n; ++i) {
        PBD_CHECK(prims[i] >= 0 && prims[i] < o->np, PBD_ERR_ARG, "prim %d out of range", prims[i]);
        PBD_CHECK(o->h_ctype[prims[i]] == PBD_ANCHOR, PBD_ERR_ARG, "prim %d is not an ANCHOR",
                  prims[i]);
        PBD_CHECK(targets[3 * i] == targets[3 * i] && targets[3 * i + 1] == targets[3 * i + 1] &&
                      targets[3 * i + 2] == targets[3 * i + 2],
                  PBD_ERR_ARG, "target %d is NaN", i);
    }
    if (!n) return PBD_OK;
    // both uploads read the caller's arrays before returning
    PBD_TRY(o->anc_prim.upload(prims, n, o->stream));
    PBD_TRY(o->anc_t.upload(targets, 3 * (size_t)n, o->stream));
    k_set_rest_pos<<<grid_for(n, 256), 256, 0, o->stream>>>(n, o->anc_prim.p, o->anc_t.p,
                                                             o->rest_pos.p);
    PBD_LAUNCH();
    return rebuild_records(o, o->n_rec[0] + o->n_rec[1]);
}

int pbd_object_stream(pbd_object *o, void **s) {
    PBD_CHECK(o && s, PBD_ERR_ARG, "null argument");
    *s = (void *)o->stream;
    return PBD_OK;
}

int pbd_object_sync(pbd_object *o) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    return PBD_OK;
}

// ---- ConstraintPBD --------------------------------------------------------
static int finish_coloring(pbd_object *o) {
    cudaStream_t s = o->stream;
    PBD_TRY(o->flag.alloc(4));
    PBD_CUDA(cudaMemsetAsync(o->flag.p, 0xff, sizeof(int), s));
    k_max_color<<<grid_for(o->np, 256), 256, 0, s>>>(o->np, o->color.p, o->flag.p);
    PBD_LAUNCH();
    int mx = -1;
    PBD_CUDA(cudaMemcpyAsync(&mx, o->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    o->n_colors = mx + 1;
    o->colored = true;
    o->sorted = false;
    o->cl_state = 0;
    return PBD_OK;
}

int pbd_constraints_edge_coloring(pbd_object *o, int max_iterations, int *sweeps) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    if (sweeps) *sweeps = 0;
    if (!o->np) {
        o->colored = true;
        o->n_colors = 0;
        return PBD_OK;
    }
    cudaStream_t s = o->stream;
    PBD_CUDA(cudaMemsetAsync(o->color.p, 0xff, sizeof(int) * o->np, s));
    PBD_CUDA(cudaMemsetAsync(o->prd_color.p, 0xff, sizeof(int) * o->np, s));
    const int window = 16;
    int done = 0, it = 0;
    while (it < max_iterations && !done) {
        int w = std::min(window, max_iterations - it);
        for (int k = 0; k < w; ++k) {
            k_assign_colors<<<grid_for(o->np, 256), 256, 0, s>>>(o->np, o->adj_sn.p, o->adj.p,
                                                                 o->color.p, o->prd_color.p);
            if (k == w - 1) PBD_CUDA(cudaMemsetAsync(o->flag.p, 0, sizeof(int), s));
            k_resolve_conflicts<<<grid_for(o->np, 256), 256, 0, s>>>(
                o->np, o->prim_list.p, o->adj_sn.p, o->adj.p, o->color.p, o->prd_color.p,
                o->flag.p);
        }
        PBD_LAUNCH();
        it += w;
        int f = 1;
        PBD_CUDA(cudaMemcpyAsync(&f, o->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaStreamSynchronize(s));
        done = (f == 0);
    }
    if (sweeps) *sweeps = it;
    PBD_CHECK(done, PBD_ERR_TIMEOUT, "edge coloring did not converge in %d sweeps", max_iterations);
    return finish_coloring(o);
}

int pbd_constraints_set_colors(pbd_object *o, const int *color) {
    PBD_CHECK(o && (color || !o->np), PBD_ERR_ARG, "null argument");
    for (int p = 0; p < o->np; ++p) PBD_CHECK(color[p] >= 0, PBD_ERR_ARG, "color %d < 0", p);
    if (o->np) PBD_CUDA(cudaMemcpyAsync(o->color.p, color, sizeof(int) * o->np, cudaMemcpyHostToDevice, o->stream));
    return finish_coloring(o);
}

int pbd_constraints_get_colors(pbd_object *o, int *color) {
    PBD_CHECK(o && color, PBD_ERR_ARG, "null argument");
    if (!o->np) return PBD_OK;
    PBD_CUDA(cudaMemcpyAsync(color, o->color.p, sizeof(int) * o->np, cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    return PBD_OK;
}

int pbd_constraints_sort_edges_colors(pbd_object *o) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    PBD_CHECK(o->colored, PBD_ERR_STATE, "constraints are not colored");
    int np = o->np;
    cudaStream_t s = o->stream;
    o->h_worksets.assign(2 * (size_t)o->n_colors, 0);
    o->cl_state = 0;  // the cluster plan follows the records
    o->h_dseg.assign(o->n_colors + 1, 0);
    o->h_bseg.assign(o->n_colors + 1, 0);
    o->h_aseg.assign(o->n_colors + 1, 0);
    if (!np) {
        o->sorted = true;
        return PBD_OK;
    }
    int nc = o->n_colors;
    DBuf<uint32_t> k1, k2;
    DBuf<int> v1, v2, first, last;
    PBD_TRY(k1.alloc(np));
    PBD_TRY(k2.alloc(np));
    PBD_TRY(v1.alloc(np));
    PBD_TRY(v2.alloc(np));
    PBD_TRY(o->sorted_color.alloc(np));
    PBD_TRY(o->sorted_prim.alloc(np));
    // SortEdgesColors: stable sort of prim ids by color
    k_iota_keys<<<grid_for(np, 256), 256, 0, s>>>(np, o->color.p, k1.p, v1.p);
    PBD_LAUNCH();
    uint32_t *sk;
    int *sv;
    PBD_TRY(radix_sort<uint32_t>(k1.p, v1.p, k2.p, v2.p, np, nullptr, round8(bits_for(nc)), o->scr,
                                 s, &sk, &sv));
    PBD_CUDA(cudaMemcpyAsync(o->sorted_color.p, sk, sizeof(int) * np, cudaMemcpyDeviceToDevice, s));
    PBD_CUDA(cudaMemcpyAsync(o->sorted_prim.p, sv, sizeof(int) * np, cudaMemcpyDeviceToDevice, s));
    // solver records: class-major, then color, then prim id
    k_class_keys<<<grid_for(np, 256), 256, 0, s>>>(np, o->color.p, o->ctype.p, nc, k1.p, v1.p);
    PBD_LAUNCH();
    PBD_TRY(radix_sort<uint32_t>(k1.p, v1.p, k2.p, v2.p, np, nullptr, round8(bits_for(4LL * nc)),
                                 o->scr, s, &sk, &sv));
    PBD_TRY(first.alloc(4 * (size_t)nc + 1));
    PBD_TRY(last.alloc(4 * (size_t)nc + 1));
    PBD_CUDA(cudaMemsetAsync(first.p, 0, sizeof(int) * (4 * nc + 1), s));
    PBD_CUDA(cudaMemsetAsync(last.p, 0, sizeof(int) * (4 * nc + 1), s));
    k_run_bounds<<<grid_for(np, 256), 256, 0, s>>>(np, sk, first.p, last.p);
    PBD_LAUNCH();
    std::vector<int> hf(4 * nc), hl(4 * nc);
    PBD_CUDA(cudaMemcpyAsync(hf.data(), first.p, sizeof(int) * 4 * nc, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaMemcpyAsync(hl.data(), last.p, sizeof(int) * 4 * nc, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    int nrec[4] = {0, 0, 0, 0};
    std::vector<int> *segs[3] = {&o->h_dseg, &o->h_bseg, &o->h_aseg};
    for (int c = 0; c < 4; ++c)
        for (int col = 0; col < nc; ++col) {
            int cntv = hl[c * nc + col] - hf[c * nc + col];
            if (c < 3) (*segs[c])[col + 1] = (*segs[c])[col] + cntv;
            nrec[c] += cntv;
        }
    PBD_TRY(o->drec.alloc(nrec[0]));
    PBD_TRY(o->bidx.alloc(nrec[1]));
    PBD_TRY(o->bpar.alloc(nrec[1]));
    PBD_TRY(o->arec.alloc(nrec[2]));
    PBD_TRY(o->bend_prim.alloc(nrec[1]));
    if (nrec[1])
        PBD_CUDA(cudaMemcpyAsync(o->bend_prim.p, sv + nrec[0], sizeof(int) * nrec[1],
                                 cudaMemcpyDeviceToDevice, s));
    o->feat_built = false;
    // the prim of every record, for rebuilding records after the per-prim
    // stiffness or anchor targets change
    const int n_rec = nrec[0] + nrec[1] + nrec[2];
    PBD_TRY(o->rec_prim.alloc(std::max(n_rec, 1)));
    if (n_rec)
        PBD_CUDA(cudaMemcpyAsync(o->rec_prim.p, sv, sizeof(int) * n_rec, cudaMemcpyDeviceToDevice, s));
    o->n_rec[0] = nrec[0];
    o->n_rec[1] = nrec[1];
    o->n_rec[2] = nrec[2];
    k_build_records<<<grid_for(np, 256), 256, 0, s>>>(
        0, n_rec, sv, o->prim_list.p, o->indices.p, o->rest_length.p, o->stiffness.p,
        o->rest_angle.p, o->rest_pos.p, nrec[0], nrec[1], nrec[2], o->drec.p, o->bidx.p,
        o->bpar.p, o->arec.p);
    PBD_LAUNCH();
    PBD_CUDA(cudaStreamSynchronize(s));
    // worksets over the color-sorted prim list
    int start = 0;
    for (int col = 0; col < nc; ++col) {
        int cntv = 0;
        for (int c = 0; c < 4; ++c) cntv += hl[c * nc + col] - hf[c * nc + col];
        o->h_worksets[2 * col] = start;
        o->h_worksets[2 * col + 1] = cntv;
        start += cntv;
    }
    o->sorted = true;
    return PBD_OK;
}

int pbd_constraints_eval_worksets(pbd_object *o, int *n) {
    PBD_CHECK(o, PBD_ERR_ARG, "null object");
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "SortEdgesColors has not run");
    if (n) *n = o->n_colors;
    return PBD_OK;
}

int pbd_constraints_get_sorted(pbd_object *o, int *sc, int *sp) {
    PBD_CHECK(o && sc && sp, PBD_ERR_ARG, "null argument");
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "SortEdgesColors has not run");
    if (!o->np) return PBD_OK;
    PBD_CUDA(cudaMemcpyAsync(sc, o->sorted_color.p, sizeof(int) * o->np, cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaMemcpyAsync(sp, o->sorted_prim.p, sizeof(int) * o->np, cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    return PBD_OK;
}

int pbd_constraints_get_worksets(pbd_object *o, int *ws, int cap, int *n) {
    PBD_CHECK(o && n, PBD_ERR_ARG, "null argument");
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "SortEdgesColors has not run");
    *n = o->n_colors;
    for (int i = 0; i < o->n_colors && i < cap && ws; ++i) {
        ws[2 * i] = o->h_worksets[2 * i];
        ws[2 * i + 1] = o->h_worksets[2 * i + 1];
    }
    return PBD_OK;
}

int pbd_constraints_get_adjacency(pbd_object *o, int *sn, int *adj, long long cap,
                                  long long *total) {
    PBD_CHECK(o && total, PBD_ERR_ARG, "null argument");
    *total = o->n_adj;
    if (sn && o->np)
        PBD_CUDA(cudaMemcpyAsync(sn, o->adj_sn.p, sizeof(int2) * o->np, cudaMemcpyDeviceToHost, o->stream));
    if (adj && o->n_adj) {
        long long m = std::min(cap, o->n_adj);
        PBD_CUDA(cudaMemcpyAsync(adj, o->adj.p, sizeof(int) * m, cudaMemcpyDeviceToHost, o->stream));
    }
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    return PBD_OK;
}

int pbd_constraints_residual(pbd_object *o, double *res) {
    PBD_CHECK(o && res, PBD_ERR_ARG, "null argument");
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "SortEdgesColors has not run");
    int nd = o->h_dseg.empty() ? 0 : o->h_dseg.back();
    int nb = o->h_bseg.empty() ? 0 : o->h_bseg.back();
    k_residual<<<kResidualBlocks, 256, 0, o->stream>>>(o->drec.p, nd, o->bidx.p, o->bpar.p, nb,
                                                       o->p.p, o->res_part.p);
    k_sum_parts<<<1, 32, 0, o->stream>>>(kResidualBlocks, o->res_part.p, o->res_out.p);
    PBD_LAUNCH();
    double num = 0.0;
    PBD_CUDA(cudaMemcpyAsync(&num, o->res_out.p, sizeof(double), cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    *res = o->res_den > 0.0 ? sqrt(num) / sqrt(o->res_den) : 0.0;
    return PBD_OK;
}

// ---- SolverPBD ------------------------------------------------------------
int pbd_solver_create(pbd_solver **out) {
    PBD_CHECK(out, PBD_ERR_ARG, "null argument");
    *out = new pbd_solver();
    return PBD_OK;
}

int pbd_solver_destroy(pbd_solver *s) {
    if (!s) return PBD_OK;
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    if (s->rexec) cudaGraphExecDestroy(s->rexec);
    delete s;
    return PBD_OK;
}

int pbd_solver_set_target(pbd_solver *s, pbd_object *o) {
    PBD_CHECK(s && o, PBD_ERR_ARG, "null argument");
    s->obj = o;
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
    if (s->rexec) cudaGraphExecDestroy(s->rexec);
    s->rexec = nullptr;
    return PBD_OK;
}

int pbd_solver_advect(pbd_solver *s, float dt) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    return launch_advect(s->obj, dt);
}

int pbd_solver_integration(pbd_solver *s, float dt) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    return launch_integrate(s->obj, dt);
}

int pbd_solver_project_constraint(pbd_solver *s, int st, int iterations) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(st == PBD_GAUSSSEIDEL, PBD_ERR_ARG, "only Gauss-Seidel is implemented");
    if (iterations <= 0) return PBD_OK;
    return launch_sweeps(s, 0, iterations, true);
}

int pbd_solver_set_sphere(pbd_solver *s, int on, const float *c, float r) {
    PBD_CHECK(s && (!on || c), PBD_ERR_ARG, "null argument");
    s->sphere_on = on;
    if (c)
        for (int k = 0; k < 3; ++k) s->sphere_c[k] = c[k];
    s->sphere_r = r;
    return PBD_OK;
}

int pbd_solver_set_ground(pbd_solver *s, int on, float h) {
    PBD_CHECK(s, PBD_ERR_ARG, "null argument");
    s->ground_on = on;
    s->ground_h = h;
    return PBD_OK;
}

int pbd_solver_set_instance_spheres(pbd_solver *s, int n, const float *spheres4) {
    PBD_CHECK(s && s->obj && n >= 0 && (n == 0 || spheres4), PBD_ERR_ARG, "bad argument");
    PBD_CHECK(n == 0 || s->obj->has_inst, PBD_ERR_STATE, "the target object has no instances");
    if (n > 0) PBD_TRY(s->inst_spheres.upload((const float4 *)spheres4, n, s->obj->stream));
    PBD_CUDA(cudaStreamSynchronize(s->obj->stream));
    s->n_inst_spheres = n;
    return PBD_OK;
}

// projectConstraintWithColli's iteration (P/PBD_cuda.cu:1130-1210): CCD when
// due, one sweep, the response, the analytic obstacles.  A due detection
// reads the positions at the iteration's start and its contacts are first
// used by the response after the sweep, so it runs beside the sweep on the
// collision solver's side stream (from a copy of those positions) and the
// response waits for it: the same contacts as a detection before the
// sweep.
static int project_with_colli(pbd_solver *s, int iterations, pbd_colli *c) {
    if (!c) return iterations > 0 ? launch_sweeps(s, 0, iterations, true) : PBD_OK;
    for (int ii = 0; ii < iterations; ++ii) {
        bool forked = false;
        if (ii % 10 == 0 || ii == iterations - 1) PBD_TRY(ccd_detect_fork(c, &forked));
        PBD_TRY(launch_sweeps(s, ii, ii + 1, false));
        if (forked) PBD_TRY(ccd_join(c));
        PBD_TRY(ccd_resolve(c, c->iterations));
        PBD_TRY(launch_obstacles(s));
    }
    return PBD_OK;
}

int pbd_solver_project_constraint_with_colli(pbd_solver *s, int st, int iterations,
                                             pbd_colli *c) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(st == PBD_GAUSSSEIDEL, PBD_ERR_ARG, "only Gauss-Seidel is implemented");
    PBD_CHECK(!c || c->obj == s->obj, PBD_ERR_ARG, "collision solver targets another object");
    return project_with_colli(s, iterations, c);
}

static int record_steps(pbd_solver *s, float dt, int substeps, int iterations, pbd_colli *c) {
    for (int k = 0; k < substeps; ++k) {
        PBD_TRY(launch_advect(s->obj, dt));
        PBD_TRY(project_with_colli(s, iterations, c));
        PBD_TRY(launch_integrate(s->obj, dt));
    }
    return PBD_OK;
}

int pbd_solver_step(pbd_solver *s, float dt, int substeps, int iterations, pbd_colli *c,
                    int use_graph) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(s->obj->sorted, PBD_ERR_STATE, "constraints are not color-sorted");
    PBD_CHECK(!c || c->obj == s->obj, PBD_ERR_ARG, "collision solver targets another object");
    if (!use_graph) return record_steps(s, dt, substeps, iterations, c);
    int sig = s->sphere_on * 3 + s->ground_on * 7 +
              (c ? c->response * 11 + c->iterations * 13 + c->ee_on * 101 : 0) +
              (s->n_inst_spheres > 0) * 17 +
              s->gs_path * 1009 + s->obj->sched * 7919;
    if (s->gexec && (s->g_dt != dt || s->g_sub != substeps || s->g_it != iterations ||
                     s->g_colli != c || s->g_sig != sig)) {
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
    }
    cudaStream_t st = s->obj->stream;
    if (!s->gexec) {
        if (c) PBD_TRY(ccd_detect(c));  // sizes every buffer before capture
        PBD_TRY(prepare_gs_path(s));    // plans and uploads outside the capture
        PBD_CUDA(cudaStreamSynchronize(st));
        cudaGraph_t g;
        PBD_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int r = record_steps(s, dt, substeps, iterations, c);
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (r != PBD_OK) {
            if (e == cudaSuccess) cudaGraphDestroy(g);
            return r;
        }
        PBD_CUDA(e);
        size_t nn = 0;
        cudaGraphGetNodes(g, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(g, nodes.data(), &nn);
        long long nk = 0;
        for (size_t i = 0; i < nn; ++i) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++nk;
        }
        s->g_kernels = nk;
        // node priorities: the color phases before an overlapped detection
        cudaError_t ei = cudaGraphInstantiate(&s->gexec, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        PBD_CUDA(ei);
        s->g_dt = dt;
        s->g_sub = substeps;
        s->g_it = iterations;
        s->g_colli = c;
        s->g_sig = sig;
    }
    PBD_CUDA(cudaGraphLaunch(s->gexec, st));
    return PBD_OK;
}

int pbd_solver_set_gs_path(pbd_solver *s, int path) {
    PBD_CHECK(s && path >= PBD_GS_AUTO && path <= PBD_GS_CLUSTER, PBD_ERR_ARG, "bad path");
    if (s->gs_path != path) {  // cached graphs hold the old form's launches
        if (s->gexec) cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
        if (s->rexec) cudaGraphExecDestroy(s->rexec);
        s->rexec = nullptr;
    }
    s->gs_path = path;
    return PBD_OK;
}

int pbd_solver_get_gs_path(pbd_solver *s, int *path) {
    PBD_CHECK(s && path && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(s->obj->sorted, PBD_ERR_STATE, "constraints are not color-sorted");
    int p = resolved_path(s);
    PBD_CHECK(p != -1, PBD_ERR_CUDA, "launch plan failed");
    *path = p == -2 ? PBD_GS_PER_COLOR : p;
    return PBD_OK;
}

int pbd_solver_graph_kernels(pbd_solver *s, long long *n) {
    PBD_CHECK(s && n, PBD_ERR_ARG, "null argument");
    *n = s->gexec ? s->g_kernels : 0;
    return PBD_OK;
}

// Times `iterations` sweeps, one launch sequence per sweep as a substep with
// collisions issues them, replayed from a CUDA graph, for every launch form
// that applies to the object (per-color launches with 64..512 threads per
// block; the resident form with every cluster size whose shared memory holds
// the object), keeps the fastest and restores the predicted positions.
// Every form gives the same result, so the choice only changes speed.
int pbd_solver_autotune(pbd_solver *s, int iterations, int reps, pbd_autotune_result *res) {
    PBD_CHECK(s && s->obj && res, PBD_ERR_ARG, "null argument");
    PBD_CHECK(iterations >= 1 && reps >= 1, PBD_ERR_ARG, "need iterations, reps >= 1");
    pbd_object *o = s->obj;
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "constraints are not color-sorted");
    memset(res, 0, sizeof(*res));
    cudaStream_t st = o->stream;
    DBuf<float4> save;
    PBD_TRY(save.alloc(o->n));
    PBD_CUDA(cudaMemcpyAsync(save.p, o->p.p, sizeof(float4) * o->n, cudaMemcpyDeviceToDevice, st));
    struct Cand {
        int path, block;
    };
    std::vector<Cand> cands = {{PBD_GS_PER_COLOR, 64}, {PBD_GS_PER_COLOR, 128},
                               {PBD_GS_PER_COLOR, 256}, {PBD_GS_PER_COLOR, 512}};
    if (s->n_inst_spheres == 0) {
        PBD_TRY(resident_plan(o));
        if (o->cl_state == 1)
            for (int S = 1; S <= 16; S <<= 1)
                if (o->cl_fit & S) cands.push_back({PBD_GS_CLUSTER, S});
    }
    const int keep_path = s->gs_path, keep_block = o->gs_block, keep_cl = o->cl_S;
    cudaEvent_t e0, e1;
    PBD_CUDA(cudaEventCreate(&e0));
    PBD_CUDA(cudaEventCreate(&e1));
    int best = -1;
    double best_us = 0.0;
    int rc = PBD_OK;
    for (size_t k = 0; k < cands.size() && k < 12 && rc == PBD_OK; ++k) {
        s->gs_path = cands[k].path;
        if (cands[k].path == PBD_GS_CLUSTER)
            o->cl_S = cands[k].block;
        else
            o->gs_block = cands[k].block;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        rc = prepare_gs_path(s);  // plans outside the capture
        if (rc != PBD_OK) break;
        if (resolved_path(s) != cands[k].path) continue;  // does not apply to this object
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            rc = PBD_ERR_CUDA;
            break;
        }
        int r = PBD_OK;
        for (int it = 0; it < iterations && r == PBD_OK; ++it) r = launch_sweeps(s, it, it + 1, true);
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (r != PBD_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            rc = r != PBD_OK ? r : PBD_ERR_CUDA;
            break;
        }
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            rc = PBD_ERR_CUDA;
            break;
        }
        float ms = 0.f;
        if (cudaGraphLaunch(ge, st) != cudaSuccess || cudaEventRecord(e0, st) != cudaSuccess) rc = PBD_ERR_CUDA;
        for (int i = 0; i < reps && rc == PBD_OK; ++i)
            if (cudaGraphLaunch(ge, st) != cudaSuccess) rc = PBD_ERR_CUDA;
        if (rc == PBD_OK && (cudaEventRecord(e1, st) != cudaSuccess ||
                             cudaEventSynchronize(e1) != cudaSuccess ||
                             cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            rc = PBD_ERR_CUDA;
        cudaGraphExecDestroy(ge);
        cudaMemcpyAsync(o->p.p, save.p, sizeof(float4) * o->n, cudaMemcpyDeviceToDevice, st);
        if (rc != PBD_OK) break;
        double us = 1e3 * ms / ((double)reps * iterations);
        const int m = res->n;
        res->path[m] = cands[k].path;
        res->block[m] = cands[k].block;
        res->us_per_sweep[m] = us;
        res->n = m + 1;
        if (best < 0 || us < best_us) {
            best = m;
            best_us = us;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != PBD_OK || best < 0) {
        s->gs_path = keep_path;
        o->gs_block = keep_block;
        o->cl_S = keep_cl;
        set_error("autotune failed: %s", cudaGetErrorString(cudaGetLastError()));
        return rc != PBD_OK ? rc : PBD_ERR_CUDA;
    }
    s->gs_path = res->path[best];
    if (res->path[best] == PBD_GS_CLUSTER)
        o->cl_S = res->block[best];
    else
        o->gs_block = res->block[best];
    if (res->path[best] != PBD_GS_CLUSTER) o->cl_S = keep_cl;
    res->best = best;
    PBD_TRY(prepare_gs_path(s));
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
    if (s->rexec) cudaGraphExecDestroy(s->rexec);
    s->rexec = nullptr;
    PBD_CUDA(cudaStreamSynchronize(st));
    return PBD_OK;
}

int pbd_solver_set_gs_block(pbd_solver *s, int block) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(block >= 32 && block <= 512 && block % 32 == 0, PBD_ERR_ARG,
              "block must be a multiple of 32 in [32, 512], got %d", block);
    s->obj->gs_block = block;
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
    if (s->rexec) cudaGraphExecDestroy(s->rexec);
    s->rexec = nullptr;
    return PBD_OK;
}

int pbd_solver_get_gs_block(pbd_solver *s, int *block) {
    PBD_CHECK(s && s->obj && block, PBD_ERR_ARG, "null argument");
    *block = s->obj->gs_block;
    return PBD_OK;
}

int pbd_solver_set_gs_cluster(pbd_solver *s, int size) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(size == 0 || size == 1 || size == 2 || size == 4 || size == 8 || size == 16,
              PBD_ERR_ARG, "cluster size must be 0, 1, 2, 4, 8 or 16, got %d", size);
    s->obj->cl_S = size;
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
    if (s->rexec) cudaGraphExecDestroy(s->rexec);
    s->rexec = nullptr;
    return PBD_OK;
}

int pbd_solver_get_gs_cluster(pbd_solver *s, int *size) {
    PBD_CHECK(s && s->obj && size, PBD_ERR_ARG, "null argument");
    PBD_CHECK(s->obj->sorted, PBD_ERR_STATE, "constraints are not color-sorted");
    PBD_TRY(resident_plan(s->obj));
    *size = s->obj->cl_state == 1 ? resident_size(s->obj) : 0;
    return PBD_OK;
}

}  // extern "C"

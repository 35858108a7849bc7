// ref_adapter.cpp -- C entry points over the reference's own compiled code.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
// reference's sources, where they lie, into oracle/_ref/libpbdref.so by
// oracle/build_oracle.py; nothing of the reference is copied here.  It exists
// to pin the oracle restatement (oracle/pbd_oracle.c) and to generate the
// golden fixtures under tests/golden/.  The reference exists only in this
// container, so the library is never built on a GPU host.
//
// Paths below are relative to PositionBasedDynamicsCUDA/PositionBasedDynamicsCUDA/.
#include <cstdio>
#include <cstring>
#include <unistd.h>
#include <fcntl.h>

#include "PBD_Basic.cuh"
#include "CCD_Basic.h"
#include "SpatialHashSystem.h"

namespace {

// The reference prints progress lines from inside the routines called here
// (PBD_DEBUG at PBD_Basic.cuh:25-32, Buffer device messages); silence fd 1
// around each call.
struct Quiet {
    int saved;
    Quiet() {
        fflush(stdout);
        saved = dup(1);
        int nul = open("/dev/null", O_WRONLY);
        dup2(nul, 1);
        close(nul);
    }
    ~Quiet() {
        fflush(stdout);
        std::cout.flush();
        dup2(saved, 1);
        close(saved);
    }
};

void fill_f3(BufferVector3f &b, const float *p, int n) {
    b.m_Data.resize(n);
    for (int i = 0; i < n; ++i) b.m_Data[i] = make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
void read_f3(BufferVector3f &b, float *p) {
    for (size_t i = 0; i < b.m_Data.size(); ++i) {
        p[3 * i] = b.m_Data[i].x;
        p[3 * i + 1] = b.m_Data[i].y;
        p[3 * i + 2] = b.m_Data[i].z;
    }
}
void fill_topol(Topology &t, int n_prims, const int *prim_list, const int *indices) {
    t.primList.m_Data.resize(n_prims);
    int n_idx = 0;
    for (int p = 0; p < n_prims; ++p) {
        t.primList.m_Data[p] = make_int2(prim_list[2 * p], prim_list[2 * p + 1]);
        int e = prim_list[2 * p] + prim_list[2 * p + 1];
        if (e > n_idx) n_idx = e;
    }
    t.indices.m_Data.assign(indices, indices + n_idx);
}
void fill_tris(Topology &t, int n_tris, const int *tri_idx) {
    t.indices.m_Data.assign(tri_idx, tri_idx + 3 * n_tris);
    t.primList.m_Data.resize(n_tris);
    for (int i = 0; i < n_tris; ++i) t.primList.m_Data[i] = make_int2(3 * i, 3);
}

}  // namespace

extern "C" {

// GenePoint2PrimsMap + GenePrim2PrimsMap (PBD_cuda.cu:155-202)
long long ref_prim2prims(int n_prims, const int *prim_list, const int *indices,
                         int *adj_start_num, int *adj_idx) {
    ConstraintPBD c;
    fill_topol(c.topol, n_prims, prim_list, indices);
    c.GenePoint2PrimsMap(c.topol);
    c.GenePrim2PrimsMap(c.topol);
    for (int p = 0; p < n_prims; ++p) {
        adj_start_num[2 * p] = c.Prim2PrimsMap.startNumList.m_Data[p].x;
        adj_start_num[2 * p + 1] = c.Prim2PrimsMap.startNumList.m_Data[p].y;
    }
    if (adj_idx)
        for (size_t i = 0; i < c.Prim2PrimsMap.indices.m_Data.size(); ++i)
            adj_idx[i] = c.Prim2PrimsMap.indices.m_Data[i];
    return (long long)c.Prim2PrimsMap.indices.m_Data.size();
}

// EdgeColoringCPU (PBD_cuda.cu:448-485), `iterations` sweeps
void ref_edge_coloring_cpu(int n_prims, const int *prim_list, const int *indices,
                           int iterations, int *color_out) {
    ConstraintPBD c;
    fill_topol(c.topol, n_prims, prim_list, indices);
    c.color.m_Data.assign(n_prims, -1);
    c.prdColor.m_Data.assign(n_prims, -1);
    c.GenePoint2PrimsMap(c.topol);
    c.GenePrim2PrimsMap(c.topol);
    c.ht = CPU;
    c.EdgeColoring(iterations);
    for (int p = 0; p < n_prims; ++p) color_out[p] = c.color.m_Data[p];
}

// One AssignColorsCPU sweep (PBD_cuda.cu:204-254) from a given state.
void ref_assign_colors_cpu(int n_prims, const int *prim_list, const int *indices,
                           const int *color, int *prd_color) {
    ConstraintPBD c;
    fill_topol(c.topol, n_prims, prim_list, indices);
    c.color.m_Data.assign(color, color + n_prims);
    c.prdColor.m_Data.assign(prd_color, prd_color + n_prims);
    c.GenePoint2PrimsMap(c.topol);
    c.GenePrim2PrimsMap(c.topol);
    c.AssignColorsCPU();
    for (int p = 0; p < n_prims; ++p) prd_color[p] = c.prdColor.m_Data[p];
}

// SortEdgesColors + EvalWorksets (PBD_cuda.cu:546-625); returns #worksets
int ref_sort_worksets(int n, int *color, int *sorted_prim_id, int *worksets) {
    ConstraintPBD c;
    c.color.m_Data.assign(color, color + n);
    c.sortedPrimId.m_Data.assign(sorted_prim_id, sorted_prim_id + n);
    {
        Quiet q;
        c.SortEdgesColors();
    }
    c.EvalWorksets();
    for (int i = 0; i < n; ++i) {
        color[i] = c.color.m_Data[i];
        sorted_prim_id[i] = c.sortedPrimId.m_Data[i];
    }
    for (size_t w = 0; w < c.colorWorksets.m_Data.size(); ++w) {
        worksets[2 * w] = c.colorWorksets.m_Data[w].x;
        worksets[2 * w + 1] = c.colorWorksets.m_Data[w].y;
    }
    return (int)c.colorWorksets.m_Data.size();
}

// SolverPBD CPU substeps: Advect + ProjectConstraint(GAUSSSEIDEL) +
// Integration (PBD_cuda.cu:981-1127, 1437-1465).  The reference's
// ProjectConstraint also applies ColliWithShpGrd (unit sphere at origin).
void ref_substeps_cpu(int n_points, float *pos, float *vel, const float *mass,
                      int n_prims, const int *prim_list, const int *indices,
                      const float *rest_length, const float *stiffness,
                      const int *ctype, float damping, const float *gravity,
                      float dt, int iterations, int substeps) {
    Quiet q;
    PBDObject obj(damping, make_float3(gravity[0], gravity[1], gravity[2]), CPU);
    fill_f3(obj.meshTopol.posBuffer, pos, n_points);
    fill_f3(obj.velBuffer, vel, n_points);
    obj.massBuffer.m_Data.assign(mass, mass + n_points);
    fill_topol(obj.constrPBDBuffer.topol, n_prims, prim_list, indices);
    obj.constrPBDBuffer.prdPBuffer = obj.meshTopol.posBuffer;
    obj.constrPBDBuffer.restLengthBuffer.m_Data.assign(rest_length, rest_length + n_prims);
    obj.constrPBDBuffer.stiffnessBuffer.m_Data.assign(stiffness, stiffness + n_prims);
    obj.constrPBDBuffer.constraintType.m_Data.assign(ctype, ctype + n_prims);
    Timer timer;
    SolverPBD solver;
    solver.SetTarget(&obj);
    solver.SetTimer(&timer);
    for (int s = 0; s < substeps; ++s) {
        solver.Advect(dt);
        solver.ProjectConstraint(GAUSSSEIDEL, iterations);
        solver.Integration(dt);
    }
    read_f3(obj.meshTopol.posBuffer, pos);
    read_f3(obj.velBuffer, vel);
    obj.ht = CPU;  // keep the destructor away from device frees
}

// SpatialHashSystem on a fresh grid + FindNeighbors for every triangle
// (SpatialHashSystem.cpp:45-187).  Returns the total neighbor count.
long long ref_find_neighbors_all(const float *center, const int *size,
                                 const float *cell, int n_tris, const int *tri_idx,
                                 int n_points, const float *pos,
                                 int *out_start_num, int *out_idx) {
    Quiet q;
    BufferVector3f p;
    fill_f3(p, pos, n_points);
    BufferInt ti;
    ti.m_Data.assign(tri_idx, tri_idx + 3 * n_tris);
    SpatialHashSystem shs(p, ti, CPU, make_float3(center[0], center[1], center[2]),
                          make_uint3(size[0], size[1], size[2]),
                          make_float3(cell[0], cell[1], cell[2]));
    shs.InitSH();
    long long total = 0;
    BufferInt nb;
    for (int t = 0; t < n_tris; ++t) {
        shs.FindNeighbors(nb, t);
        out_start_num[2 * t] = (int)total;
        out_start_num[2 * t + 1] = nb.GetSize();
        if (out_idx)
            for (int i = 0; i < nb.GetSize(); ++i) out_idx[total + i] = nb.m_Data[i];
        total += nb.GetSize();
    }
    return total;
}

// solve_cubic (CCD.cpp:48-73)
int ref_solve_cubic(double a, double b, double c, double d, double *x) {
    return solve_cubic(a, b, c, d, x);
}

// The reference's solve_cubic reads xc[0] uninitialised when the derivative
// quadratic has no usable root (a face moving with its point gives a = b =
// 0, P/CCD.cpp:48-54); Newton then starts from whatever an earlier call left
// on the stack and the root's last bits follow it.  Zeroing the stack below
// the caller's frame before each test makes that start 0, the oracle's
// choice, and the fixtures independent of call order.
__attribute__((noinline)) static void scrub_stack() {
    volatile char buf[32768];
    memset((char *)buf, 0, sizeof(buf));
    __asm__ __volatile__("" : : "r"(buf) : "memory");
}

static int vf_call(int which, const float *x, const float *p, float thickness,
                   int i0, int i1, int i2, int i3, float *t, double *w, float *n) {
    float3 X[4], P[4];
    for (int j = 0; j < 4; ++j) {
        X[j] = make_float3(x[3 * j], x[3 * j + 1], x[3 * j + 2]);
        P[j] = make_float3(p[3 * j], p[3 * j + 1], p[3 * j + 2]);
    }
    Contact ct;
    memset(&ct, 0, sizeof(ct));
    bool hit;
    Quiet q;  // VFCCDTest prints for one hard-coded id quadruple
    scrub_stack();
    if (which == 0)
        hit = ExtendedVFTest(X[0], X[1], X[2], X[3], P[0], P[1], P[2], P[3], ct, thickness,
                             i0, i1, i2, i3);
    else if (which == 1)
        hit = NarrowVFCCDTest(X[0], X[1], X[2], X[3], P[0], P[1], P[2], P[3], ct, thickness,
                              i0, i1, i2, i3);
    else if (which == 2)
        hit = VFCCDTest(X[0], X[1], X[2], X[3], P[0], P[1], P[2], P[3], Contact::VF, ct,
                        thickness, i0, i1, i2, i3);
    else if (which == 3)
        hit = VFDCDTest(X[0], X[1], X[2], X[3], P[0], P[1], P[2], P[3], ct, thickness, i0, i1,
                        i2, i3);
    else
        hit = VFTest(X[0], X[1], X[2], X[3], P[0], P[1], P[2], P[3], ct, thickness, i0, i1, i2,
                     i3);
    *t = ct.t;
    for (int k = 0; k < 4; ++k) w[k] = ct.w[k];
    n[0] = ct.n.x; n[1] = ct.n.y; n[2] = ct.n.z;
    return hit ? 1 : 0;
}

// free ExtendedVFTest (CCD.cpp:1733-1808)
int ref_extended_vf_test(const float *x, const float *p, float thickness, int i0, int i1,
                         int i2, int i3, float *t, double *w, float *n) {
    return vf_call(0, x, p, thickness, i0, i1, i2, i3, t, w, n);
}

// free NarrowVFCCDTest (CCD.cpp:1810-1872)
int ref_narrow_vf_ccd_test(const float *x, const float *p, float thickness, int i0, int i1,
                           int i2, int i3, float *t, double *w, float *n) {
    return vf_call(1, x, p, thickness, i0, i1, i2, i3, t, w, n);
}

// free VFCCDTest with type VF (CCD.cpp:2308-2421), VFDCDTest
// (CCD.cpp:2265-2306) and VFTest (CCD.cpp:2229-2263)
int ref_vf_ccd_test(const float *x, const float *p, float thickness, int i0, int i1, int i2,
                    int i3, float *t, double *w, float *n) {
    return vf_call(2, x, p, thickness, i0, i1, i2, i3, t, w, n);
}
int ref_vf_dcd_test(const float *x, const float *p, float thickness, int i0, int i1, int i2,
                    int i3, float *t, double *w, float *n) {
    return vf_call(3, x, p, thickness, i0, i1, i2, i3, t, w, n);
}
int ref_vf_test(const float *x, const float *p, float thickness, int i0, int i1, int i2, int i3,
                float *t, double *w, float *n) {
    return vf_call(4, x, p, thickness, i0, i1, i2, i3, t, w, n);
}

// free CCD_SH_Extended (CCD.cpp:1522-1587).  The grid is built on prdp so
// that InitSH and the UpdateSH inside the call bin identically (the
// reference never clears cell ranges between updates).  out_ids: 4 per
// contact; out_t, out_w (4 doubles), out_n (3 floats).  Returns #contacts.
long long ref_ccd_sh_extended(const float *center, const int *size, const float *cell,
                              int n_tris, const int *tri_idx, int n_points,
                              const float *pos, const float *prdp, float thickness,
                              long long cap, int *out_ids, float *out_t, double *out_w,
                              float *out_n) {
    Quiet q;
    BufferVector3f P, X;
    fill_f3(P, prdp, n_points);
    fill_f3(X, pos, n_points);
    BufferInt ti;
    ti.m_Data.assign(tri_idx, tri_idx + 3 * n_tris);
    SpatialHashSystem shs(P, ti, CPU, make_float3(center[0], center[1], center[2]),
                          make_uint3(size[0], size[1], size[2]),
                          make_float3(cell[0], cell[1], cell[2]));
    shs.InitSH();
    Topology topo;
    fill_tris(topo, n_tris, tri_idx);
    topo.posBuffer = X;
    ContactData cd;
    CCD_SH_Extended(cd, shs, topo, P, thickness);
    long long h = cd.ctxs.GetSize();
    for (long long i = 0; i < h && i < cap; ++i) {
        int s = cd.ctxStartNum.m_Data[i].x;
        for (int j = 0; j < 4; ++j) out_ids[4 * i + j] = cd.ctxIndices.m_Data[s + j];
        out_t[i] = cd.ctxs.m_Data[i].t;
        for (int j = 0; j < 4; ++j) out_w[4 * i + j] = cd.ctxs.m_Data[i].w[j];
        out_n[3 * i] = cd.ctxs.m_Data[i].n.x;
        out_n[3 * i + 1] = cd.ctxs.m_Data[i].n.y;
        out_n[3 * i + 2] = cd.ctxs.m_Data[i].n.z;
    }
    return h;
}

// free CollisionResolveNew (CCD.cpp:1874-1994) on the given contacts
void ref_collision_resolve_new(int n_points, const float *pos, float *prdp,
                               int n_contacts, const int *ids, int iterations,
                               float thickness) {
    Quiet q;
    Topology topo;
    fill_f3(topo.posBuffer, pos, n_points);
    BufferVector3f P;
    fill_f3(P, prdp, n_points);
    ContactData cd;
    for (int c = 0; c < n_contacts; ++c) {
        Contact ct;
        memset(&ct, 0, sizeof(ct));
        ct.type = Contact::VF;
        cd.ctxs.m_Data.push_back(ct);
        cd.ctxStartNum.m_Data.push_back(make_int2(4 * c, 4));
        for (int j = 0; j < 4; ++j) cd.ctxIndices.m_Data.push_back(ids[4 * c + j]);
    }
    int dbg = 0;
    BufferInt vf;
    CollisionResolveNew(topo, P, cd, iterations, thickness, dbg, vf);
    read_f3(P, prdp);
}

// free CollisionResolve (CCD.cpp:2423-2593) with VFResolve (CCD.cpp:2595-2650),
// the older response: two in-place passes over the contacts in order, the
// per-point resolve counters in resolve_times (in and out).  Its debug
// output is silenced; the caches it tries to save go to a D:/ path that
// does not open here, which it skips.
void ref_collision_resolve_old(int n_points, const float *pos, float *prdp, int n_contacts,
                               const int *ids, float thickness, int *resolve_times) {
    Quiet q;
    scrub_stack();
    Topology topo;
    fill_f3(topo.posBuffer, pos, n_points);
    BufferVector3f P;
    fill_f3(P, prdp, n_points);
    ContactData cd;
    for (int c = 0; c < n_contacts; ++c) {
        Contact ct;
        memset(&ct, 0, sizeof(ct));
        ct.type = Contact::VF;
        cd.ctxs.m_Data.push_back(ct);
        cd.ctxStartNum.m_Data.push_back(make_int2(4 * c, 4));
        for (int j = 0; j < 4; ++j) cd.ctxIndices.m_Data.push_back(ids[4 * c + j]);
    }
    int dbg = 0;
    BufferInt vf, rt;
    rt.m_Data.assign(resolve_times, resolve_times + n_points);
    CollisionResolve(topo, P, cd, 2, thickness, dbg, vf, rt);
    read_f3(P, prdp);
    for (int i = 0; i < n_points; ++i) resolve_times[i] = rt.m_Data[i];
}

// free VFResolveTest (CCD.cpp:1996-2032); the reference prints for one
// hard-wired id set, so ids are passed as 0..3.
int ref_vf_resolve_test(const float *x, const float *p, float thickness) {
    Quiet q;
    float3 X[4], P[4];
    for (int j = 0; j < 4; ++j) {
        X[j] = make_float3(x[3 * j], x[3 * j + 1], x[3 * j + 2]);
        P[j] = make_float3(p[3 * j], p[3 * j + 1], p[3 * j + 2]);
    }
    Contact ct;
    memset(&ct, 0, sizeof(ct));
    return VFResolveTest(X[0], X[1], X[2], X[3], P[0], P[1], P[2], P[3], ct, 0, 1, 2, 3,
                         thickness) ? 1 : 0;
}

// free VFResolveNew (CCD.cpp:2034-2090), in place on p[12]
void ref_vf_resolve_new(const float *x, float *p, float thickness) {
    Quiet q;
    float3 X[4], P[4];
    for (int j = 0; j < 4; ++j) {
        X[j] = make_float3(x[3 * j], x[3 * j + 1], x[3 * j + 2]);
        P[j] = make_float3(p[3 * j], p[3 * j + 1], p[3 * j + 2]);
    }
    Contact ct;
    memset(&ct, 0, sizeof(ct));
    VFResolveNew(X[0], X[1], X[2], X[3], P[0], P[1], P[2], P[3], ct, thickness, 0, 1, 2, 3);
    for (int j = 0; j < 4; ++j) {
        p[3 * j] = P[j].x;
        p[3 * j + 1] = P[j].y;
        p[3 * j + 2] = P[j].z;
    }
}


// ---- text caches (P/PBD_cuda.cu:627-640, 660-667, 907-938; P/PBD_Basic.cuh:326-660)

// PBDObject::SaveMeshTopol + SaveConstraint of a scene given as arrays
// (meshTopol triangles as (3t, 3) prims; the buffer names the readers expect)
int ref_save_caches(const char *topol, const char *constr, int n, const float *pos,
                    const float *vel, const float *mass, int nt, const int *tri, float damping,
                    const float *g, int np, const int *prim_list, const int *indices,
                    const int *ctype, const float *rest, const float *stiff, const float *prdp) {
    Quiet q;
    PBDObject obj(damping, make_float3(g[0], g[1], g[2]), CPU);
    fill_f3(obj.meshTopol.posBuffer, pos, n);
    obj.meshTopol.indices.m_Data.assign(tri, tri + 3 * nt);
    obj.meshTopol.primList.m_Data.resize(nt);
    for (int t = 0; t < nt; ++t) obj.meshTopol.primList.m_Data[t] = make_int2(3 * t, 3);
    obj.meshTopol.indices.SetName("Indices");
    obj.meshTopol.posBuffer.SetName("P");
    obj.meshTopol.primList.SetName("primList");
    fill_f3(obj.velBuffer, vel, n);
    obj.massBuffer.m_Data.assign(mass, mass + n);
    fill_topol(obj.constrPBDBuffer.topol, np, prim_list, indices);
    fill_f3(obj.constrPBDBuffer.topol.posBuffer, pos, n);
    obj.constrPBDBuffer.topol.indices.SetName("Indices");
    obj.constrPBDBuffer.topol.posBuffer.SetName("P");
    obj.constrPBDBuffer.topol.primList.SetName("primList");
    fill_f3(obj.constrPBDBuffer.prdPBuffer, prdp, n);
    obj.constrPBDBuffer.restLengthBuffer.m_Data.assign(rest, rest + np);
    obj.constrPBDBuffer.stiffnessBuffer.m_Data.assign(stiff, stiff + np);
    obj.constrPBDBuffer.constraintType.m_Data.assign(ctype, ctype + np);
    obj.SaveMeshTopol(topol);
    obj.SaveConstraint(constr);
    return 0;
}

namespace {
// outs: 0 mesh pos, 1 mesh indices, 2 mesh primList, 3 vel, 4 mass,
// 5 constr indices, 6 constr pos, 7 constr primList, 8 prdP, 9 rest length,
// 10 stiffness, 11 constraint type, 12 damping (1), 13 gravity (3);
// sizes: scalars written per array; returns -1 when an array exceeds cap
int export_obj(PBDObject &o, void **outs, long long cap, long long *sizes) {
    auto f3 = [&](BufferVector3f &b, int k) {
        sizes[k] = 3 * (long long)b.m_Data.size();
        if (sizes[k] > cap) return false;
        read_f3(b, (float *)outs[k]);
        return true;
    };
    auto i1 = [&](BufferInt &b, int k) {
        sizes[k] = (long long)b.m_Data.size();
        if (sizes[k] > cap) return false;
        for (size_t i = 0; i < b.m_Data.size(); ++i) ((int *)outs[k])[i] = b.m_Data[i];
        return true;
    };
    auto i2 = [&](BufferInt2 &b, int k) {
        sizes[k] = 2 * (long long)b.m_Data.size();
        if (sizes[k] > cap) return false;
        for (size_t i = 0; i < b.m_Data.size(); ++i) {
            ((int *)outs[k])[2 * i] = b.m_Data[i].x;
            ((int *)outs[k])[2 * i + 1] = b.m_Data[i].y;
        }
        return true;
    };
    auto f1 = [&](BufferFloat &b, int k) {
        sizes[k] = (long long)b.m_Data.size();
        if (sizes[k] > cap) return false;
        for (size_t i = 0; i < b.m_Data.size(); ++i) ((float *)outs[k])[i] = b.m_Data[i];
        return true;
    };
    bool ok = f3(o.meshTopol.posBuffer, 0) && i1(o.meshTopol.indices, 1) &&
              i2(o.meshTopol.primList, 2) && f3(o.velBuffer, 3) && f1(o.massBuffer, 4) &&
              i1(o.constrPBDBuffer.topol.indices, 5) && f3(o.constrPBDBuffer.topol.posBuffer, 6) &&
              i2(o.constrPBDBuffer.topol.primList, 7) && f3(o.constrPBDBuffer.prdPBuffer, 8) &&
              f1(o.constrPBDBuffer.restLengthBuffer, 9) &&
              f1(o.constrPBDBuffer.stiffnessBuffer, 10) && i1(o.constrPBDBuffer.constraintType, 11);
    ((float *)outs[12])[0] = o.dampingRate;
    ((float *)outs[13])[0] = o.gravity.x;
    ((float *)outs[13])[1] = o.gravity.y;
    ((float *)outs[13])[2] = o.gravity.z;
    return ok ? 0 : -1;
}
}  // namespace

// PBDObject::ContinueSimInit (IO::ReadTopolFromCache + ReadConstraintFromCache)
int ref_read_caches(const char *topol, const char *constr, void **outs, long long cap,
                    long long *sizes) {
    Quiet q;
    PBDObject obj(1.0f, make_float3(0.f, 0.f, 0.f), CPU);
    obj.ContinueSimInit(topol, constr, CPU);
    return export_obj(obj, outs, cap, sizes);
}

// PBDObject::Init(topolFile, distConstrFile) (IO::ReadTopolFromTxt +
// ReadDistConstrFromTxt) on the CPU
int ref_read_txt(const char *topol, const char *dist, float stiffness, void **outs,
                 long long cap, long long *sizes) {
    Quiet q;
    float st[3] = {stiffness, stiffness, stiffness};
    PBDObject obj(1.0f, make_float3(0.f, 0.f, 0.f), CPU);
    obj.SetConstrOption(DISTANCE, st);
    obj.Init(topol, dist);
    return export_obj(obj, outs, cap, sizes);
}
}  // extern "C"

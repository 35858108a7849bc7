// pbd_mesh.cu -- the constraint set of a triangle mesh, built on the device.
//
// The reference builds its constraints on the host: the grid stencil of
// InitDistanceIndices (P/PBD_cuda.cu:19-108) or Houdini caches, and its
// constraint adjacency with std::map (GenePoint2PrimsMap / GenePrim2PrimsMap,
// :155-202; the adjacency is built on the device in pbd_object.cu).  Here the
// constraints of any triangle mesh are derived on the device:
//   * every half-edge -- (t0,t1) of all triangles, then (t1,t2), then (t2,t0)
//     -- gets the key a * n + b of its undirected edge (a < b); a stable LSD
//     radix sort orders the half-edges by key;
//   * the first half-edge of each key is an edge: one distance constraint,
//     rest length |p_a - p_b| in float32 from the rest positions;
//   * a key held by exactly two half-edges is an interior edge: one dihedral
//     bending constraint (e0, e1, wA, wB), wA / wB the vertices opposite the
//     edge in the first / second triangle of the sorted order, oriented so
//     that wing A's triangle lists e0 just before e1; its rest angle is the
//     signed dihedral angle of the rest positions, atan2((nA x nB).E/|E|,
//     nA.nB), in float64, stored as float32.
// Edges and hinges come out in key order.
//
// Compiled with -fmad=false: the float32 rest lengths round every product.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pbd_common.cuh"

namespace pbd {
namespace {

__global__ void k_half_edges(int nt, long long n, const int *__restrict__ tri,
                             unsigned long long *key, int *val) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 3LL * nt) return;
    int slot = (int)(j / nt), t = (int)(j % nt);
    long long a = tri[3LL * t + slot], b = tri[3LL * t + (slot + 1) % 3];
    long long lo = a < b ? a : b, hi = a < b ? b : a;
    key[j] = (unsigned long long)(lo * n + hi);
    val[j] = (int)j;
}

// first[j]: j starts a key run; two[j]: the run that j starts has length 2
__global__ void k_runs(long long m, const unsigned long long *__restrict__ k, int *first,
                       int *two) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    bool f = j == 0 || k[j] != k[j - 1];
    bool t = f && j + 1 < m && k[j + 1] == k[j] && (j + 2 >= m || k[j + 2] != k[j]);
    first[j] = f ? 1 : 0;
    two[j] = t ? 1 : 0;
}

__device__ __forceinline__ float dist32(const float *p, int a, int b) {
    float dx = p[3LL * a] - p[3LL * b], dy = p[3LL * a + 1] - p[3LL * b + 1],
          dz = p[3LL * a + 2] - p[3LL * b + 2];
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

__global__ void k_emit(long long m, int nt, long long n, const unsigned long long *__restrict__ k,
                       const int *__restrict__ v, const int *__restrict__ first,
                       const int *__restrict__ two, const int *__restrict__ eid,
                       const int *__restrict__ hid, const int *__restrict__ tri,
                       const float *__restrict__ rp, int2 *edges, float *elen, int4 *hinges,
                       float *hang) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m || !first[j]) return;
    int a = (int)(k[j] / (unsigned long long)n), b = (int)(k[j] % (unsigned long long)n);
    int e = eid[j];
    edges[e] = make_int2(a, b);
    elen[e] = dist32(rp, a, b);
    if (!two[j]) return;
    // vertex opposite half-edge jj: slot s of triangle t is (t_s, t_{s+1})
    auto opp = [&](int jj) {
        int s = jj / nt, t = jj % nt;
        return tri[3LL * t + (s + 2) % 3];
    };
    int j0 = v[j], j1 = v[j + 1];
    int wa = opp(j0), wb = opp(j1);
    int ta = j0 % nt;
    int q[3] = {tri[3LL * ta], tri[3LL * ta + 1], tri[3LL * ta + 2]};
    int pa = q[0] == a ? 0 : (q[1] == a ? 1 : 2);
    int pb = q[0] == b ? 0 : (q[1] == b ? 1 : 2);
    bool forward = ((pb - pa) % 3 + 3) % 3 == 1;
    int e0 = forward ? a : b, e1 = forward ? b : a;
    int h = hid[j];
    hinges[h] = make_int4(e0, e1, wa, wb);
    // signed dihedral angle of the rest positions, float64
    double P[4][3];
    int ids[4] = {e0, e1, wa, wb};
    for (int i = 0; i < 4; ++i)
        for (int c = 0; c < 3; ++c) P[i][c] = (double)rp[3LL * ids[i] + c];
    double E[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
    double u[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
    double w[3] = {P[2][0] - P[1][0], P[2][1] - P[1][1], P[2][2] - P[1][2]};
    double na[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
    double x[3] = {P[3][0] - P[1][0], P[3][1] - P[1][1], P[3][2] - P[1][2]};
    double y[3] = {P[3][0] - P[0][0], P[3][1] - P[0][1], P[3][2] - P[0][2]};
    double nb[3] = {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
    double el = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
    double cr[3] = {na[1] * nb[2] - na[2] * nb[1], na[2] * nb[0] - na[0] * nb[2],
                    na[0] * nb[1] - na[1] * nb[0]};
    double sn = (cr[0] * E[0] + cr[1] * E[1] + cr[2] * E[2]) / el;
    double cs = na[0] * nb[0] + na[1] * nb[1] + na[2] * nb[2];
    hang[h] = (float)atan2(sn, cs);
}

struct MeshResult {
    std::vector<int2> edges;
    std::vector<float> elen;
    std::vector<int4> hinges;
    std::vector<float> hang;
};

int build(int n_points, const float *rest_pos, int n_tris, const int *tris, MeshResult &res) {
    PBD_CHECK(n_points > 0 && n_tris > 0 && rest_pos && tris, PBD_ERR_ARG, "empty mesh");
    for (long long i = 0; i < 3LL * n_tris; ++i)
        PBD_CHECK(tris[i] >= 0 && tris[i] < n_points, PBD_ERR_ARG,
                  "triangle index %d out of range at %lld", tris[i], i);
    PBD_CHECK(3LL * n_tris < 0x7fffffffLL, PBD_ERR_ARG, "too many triangles");
    cudaStream_t s = nullptr;
    PBD_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{s};
    const long long m = 3LL * n_tris, n = n_points;
    DBuf<int> dtri, v1, v2, first, two, eid, hid, tot;
    DBuf<float> drp, elen, hang;
    DBuf<unsigned long long> k1, k2;
    DBuf<int2> edges;
    DBuf<int4> hinges;
    SortScratch scr;
    PBD_TRY(dtri.upload(tris, (size_t)m, s));
    PBD_TRY(drp.upload(rest_pos, 3 * (size_t)n, s));
    PBD_TRY(k1.alloc(m));
    PBD_TRY(k2.alloc(m));
    PBD_TRY(v1.alloc(m));
    PBD_TRY(v2.alloc(m));
    PBD_TRY(first.alloc(m));
    PBD_TRY(two.alloc(m));
    PBD_TRY(eid.alloc(m));
    PBD_TRY(hid.alloc(m));
    PBD_TRY(tot.alloc(2));
    k_half_edges<<<grid_for(m, 256), 256, 0, s>>>(n_tris, n, dtri.p, k1.p, v1.p);
    PBD_LAUNCH();
    int bits = 1;
    while (bits < 64 && (1ULL << bits) <= (unsigned long long)(n * n)) ++bits;
    bits = (bits + 7) / 8 * 8;
    unsigned long long *sk;
    int *sv;
    PBD_TRY(radix_sort<unsigned long long>(k1.p, v1.p, k2.p, v2.p, m, nullptr, bits, scr, s, &sk,
                                           &sv));
    k_runs<<<grid_for(m, 256), 256, 0, s>>>(m, sk, first.p, two.p);
    PBD_LAUNCH();
    PBD_TRY(exclusive_scan(first.p, eid.p, m, tot.p, s));
    PBD_TRY(exclusive_scan(two.p, hid.p, m, tot.p + 1, s));
    int h_tot[2] = {0, 0};
    PBD_CUDA(cudaMemcpyAsync(h_tot, tot.p, sizeof(h_tot), cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    const int ne = h_tot[0], nh = h_tot[1];
    PBD_TRY(edges.alloc(std::max(ne, 1)));
    PBD_TRY(elen.alloc(std::max(ne, 1)));
    PBD_TRY(hinges.alloc(std::max(nh, 1)));
    PBD_TRY(hang.alloc(std::max(nh, 1)));
    k_emit<<<grid_for(m, 256), 256, 0, s>>>(m, n_tris, n, sk, sv, first.p, two.p, eid.p, hid.p,
                                            dtri.p, drp.p, edges.p, elen.p, hinges.p, hang.p);
    PBD_LAUNCH();
    res.edges.resize(ne);
    res.elen.resize(ne);
    res.hinges.resize(nh);
    res.hang.resize(nh);
    if (ne) {
        PBD_CUDA(cudaMemcpyAsync(res.edges.data(), edges.p, sizeof(int2) * ne, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaMemcpyAsync(res.elen.data(), elen.p, sizeof(float) * ne, cudaMemcpyDeviceToHost, s));
    }
    if (nh) {
        PBD_CUDA(cudaMemcpyAsync(res.hinges.data(), hinges.p, sizeof(int4) * nh, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaMemcpyAsync(res.hang.data(), hang.p, sizeof(float) * nh, cudaMemcpyDeviceToHost, s));
    }
    PBD_CUDA(cudaStreamSynchronize(s));
    return PBD_OK;
}

}  // namespace

// the unique edges (a < b, key order) of a triangle mesh
int mesh_unique_edges(int n_points, int n_tris, const int *tris, std::vector<int2> &edges) {
    std::vector<float> zero(3 * (size_t)n_points, 0.f);
    MeshResult r;
    PBD_TRY(build(n_points, zero.data(), n_tris, tris, r));
    edges.swap(r.edges);
    return PBD_OK;
}

}  // namespace pbd

using namespace pbd;

extern "C" {

int pbd_mesh_constraints(int n_points, const float *rest_pos, int n_tris, const int *tris,
                         long long capacity, int *n_edges, int *n_hinges, int *edges,
                         float *edge_rest, int *hinges, float *hinge_angle) {
    PBD_CHECK(n_edges && n_hinges, PBD_ERR_ARG, "null count pointers");
    MeshResult r;
    PBD_TRY(build(n_points, rest_pos, n_tris, tris, r));
    *n_edges = (int)r.edges.size();
    *n_hinges = (int)r.hinges.size();
    if (!edges && !edge_rest && !hinges && !hinge_angle) return PBD_OK;
    PBD_CHECK((long long)r.edges.size() <= capacity && (long long)r.hinges.size() <= capacity,
              PBD_ERR_OVERFLOW, "%zu edges / %zu hinges exceed the capacity %lld",
              r.edges.size(), r.hinges.size(), capacity);
    for (size_t i = 0; i < r.edges.size(); ++i) {
        if (edges) {
            edges[2 * i] = r.edges[i].x;
            edges[2 * i + 1] = r.edges[i].y;
        }
        if (edge_rest) edge_rest[i] = r.elen[i];
    }
    for (size_t i = 0; i < r.hinges.size(); ++i) {
        if (hinges) {
            hinges[4 * i] = r.hinges[i].x;
            hinges[4 * i + 1] = r.hinges[i].y;
            hinges[4 * i + 2] = r.hinges[i].z;
            hinges[4 * i + 3] = r.hinges[i].w;
        }
        if (hinge_angle) hinge_angle[i] = r.hang[i];
    }
    return PBD_OK;
}

int pbd_object_create_mesh(const pbd_mesh_desc *d, pbd_object **out) {
    PBD_CHECK(d && out && d->pos && d->mass && d->tri_idx, PBD_ERR_ARG, "null argument");
    PBD_CHECK(d->ct_mask & (PBD_DISTANCE | PBD_BENDING), PBD_ERR_ARG,
              "ct_mask selects neither DISTANCE nor BENDING");
    MeshResult r;
    PBD_TRY(build(d->n_points, d->rest_pos ? d->rest_pos : d->pos, d->n_tris, d->tri_idx, r));
    const int nd = (d->ct_mask & PBD_DISTANCE) ? (int)r.edges.size() : 0;
    const int nb = (d->ct_mask & PBD_BENDING) ? (int)r.hinges.size() : 0;
    const int np = nd + nb;
    std::vector<int> pl(2 * (size_t)np), idx(2 * (size_t)nd + 4 * (size_t)nb), ct(np);
    std::vector<float> rl(np, 0.f), st(np), ra(np, 0.f), rp(3 * (size_t)np, 0.f);
    for (int i = 0; i < nd; ++i) {
        pl[2 * i] = 2 * i;
        pl[2 * i + 1] = 2;
        idx[2 * i] = r.edges[i].x;
        idx[2 * i + 1] = r.edges[i].y;
        ct[i] = PBD_DISTANCE;
        rl[i] = r.elen[i];
        st[i] = d->stiffness[0];
    }
    for (int j = 0; j < nb; ++j) {
        int p = nd + j;
        pl[2 * p] = 2 * nd + 4 * j;
        pl[2 * p + 1] = 4;
        idx[2 * nd + 4 * j] = r.hinges[j].x;
        idx[2 * nd + 4 * j + 1] = r.hinges[j].y;
        idx[2 * nd + 4 * j + 2] = r.hinges[j].z;
        idx[2 * nd + 4 * j + 3] = r.hinges[j].w;
        ct[p] = PBD_BENDING;
        st[p] = d->stiffness[1];
        ra[p] = r.hang[j];
    }
    pbd_object_desc od;
    std::memset(&od, 0, sizeof(od));
    od.n_points = d->n_points;
    od.pos = d->pos;
    od.vel = d->vel;
    od.mass = d->mass;
    od.n_tris = d->n_tris;
    od.tri_idx = d->tri_idx;
    od.n_prims = np;
    od.prim_list = pl.data();
    od.indices = idx.data();
    od.constraint_type = ct.data();
    od.rest_length = rl.data();
    od.stiffness = st.data();
    od.rest_angle = ra.data();
    od.rest_pos = rp.data();
    od.point_inst = d->point_inst;
    od.tri_inst = d->tri_inst;
    od.damping_rate = d->damping_rate;
    for (int k = 0; k < 3; ++k) od.gravity[k] = d->gravity[k];
    return pbd_object_create(&od, out);
}

}  // extern "C"

// pbd_collision.cu -- SpatialHashSystem and CollisionSolver on the GPU.
//
// Broadphase (per CCD call, all device-resident so it can sit in a graph):
//   1. per triangle: centroid of its predicted positions, cell
//      floor((c - start)/cell) (SpatialHashSystem.cpp:276-298, 391-399),
//      bucket key (bounded grid: the reference's linear cell id; hashed:
//      Teschner et al. 2003 hash of the cell mod 2^k), swept AABB;
//   2. stable radix sort of (bucket, triangle id) and a bucket -> [start, end)
//      table (the reference's cellStart/cellEnd, reset each update) plus the
//      union of the swept AABBs of each bucket's triangles;
//   3. candidate search (k_point_pairs): one warp per point, one lane per
//      cell of the union of the 27-cell neighbourhoods of the centroid cells
//      of its incident triangles (CCD_SH_Extended, P/CCD.cpp:1541-1586,
//      tests every (point, neighbour) pair; the union holds each distinct
//      pair once); a cell whose bucket AABB is farther than 3.61 h
//      (Euclidean gap) from the point's swept AABB yields nothing; the kept
//      buckets' entries are spread over the lanes (warp prefix sum), each
//      entry checked for its exact cell and for a swept AABB within 3.61 h
//      of the point's, the point's own triangles dropped;
//      found pairs are staged per warp in shared memory and appended with
//      one atomic per batch (warps loop over points, so a batch spans many
//      points);
//   4. distance filter: a pair survives when a lower bound of the
//      point-triangle distance over the step is within the pair's own reach
//      sqrt((2h)^2 + r^2), r = 2h * longest / mean edge (at most 3.61 h).
//      Neither filter can reject a pair ExtendedVFTest would accept.
// Narrowphase: ExtendedVFTest (P/CCD.cpp:1733-1808) with the reference's
// decisions: float triple products (widened to double for the root
// isolation), the double cubic solve (P/CCD.cpp:48-113), the float
// barycentric inside test; the double comparisons are taken in float where
// the float result is provably the same (pbd_ccd.cuh).  One thread per
// candidate evaluates t = 0 and, when the cubic has no root near [0, 1],
// t = 1; the pairs that need the roots are compacted into a list for a
// second kernel, which first drops the pairs whose point provably stays
// outside the grown triangle over the whole step and solves the rest on
// full warps (the FP64 root isolation is slow on this GPU).  Contacts are
// kept in discovery order on the device and sorted by (point, triangle)
// only when copied out.
// Response: per pass every contact computes its four corrections from the
// pass-start positions (VFResolveTest + VFResolveNew, P/CCD.cpp:1996-2090)
// and adds them to per-point sums in 2^-32 m fixed point (integer atomics:
// the sum is exact, so the result does not depend on contact order); each
// point then moves by sum / count.
//
// Compiled with -fmad=false: products round separately as in the reference.
#include <cooperative_groups.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "pbd_common.cuh"
#include "pbd_ccd.cuh"

namespace cg = cooperative_groups;

namespace pbd {
namespace {

constexpr int kMaxInc = 16;     // incident triangles considered per point
constexpr int kPointSlots = 8;  // incident cells kept per point by the hash update

// the slot of every (triangle, corner) among the corner point's first
// kPointSlots incident triangles (the point -> triangle lists are static,
// one entry per corner: a triangle that repeats a point appears once per
// corner, and its i-th appearance in the point's list takes its i-th corner
// holding the point, so every slot in use is written by some corner)
__global__ void k_tri_slots(int n, const int *__restrict__ pt_first,
                            const int *__restrict__ pt_last, const int *__restrict__ pt_tri,
                            const int4 *__restrict__ tri, int *tri_slot) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int f0 = pt_first[v], m = min(pt_last[v] - f0, kPointSlots);
    for (int j = 0; j < m; ++j) {
        const int t = pt_tri[f0 + j];
        int occ = 0;  // earlier appearances of t in this point's list
        for (int i = 0; i < j; ++i) occ += pt_tri[f0 + i] == t;
        const int4 f = tri[t];
        const int c[3] = {f.x, f.y, f.z};
        int k = -1;
        for (int q = 0; q < 3 && k < 0; ++q)
            if (c[q] == v && occ-- == 0) k = q;
        if (k >= 0) tri_slot[3 * (size_t)t + k] = v * kPointSlots + j;
    }
}

// ---------------------------------------------------------------------------
// Clears the buckets the previous update filled: its sorted keys (all nt
// triangles; keys >= nb are the out-of-grid ones) name them.  Also zeroes
// the valid-key count for the update that follows and, when given, `zero`
// (n_zero ints: the detection's counters).
__global__ void k_reset_buckets(const uint32_t *skey, int nt, uint32_t nb, float4 *btab,
                                int *n_valid, int *zero, int n_zero) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        uint32_t k = skey[i];
        if (k < nb) btab[2 * (size_t)k] = make_float4(0.f, 0.f, 0.f, 0.f);  // empty range
    }
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0) *n_valid = 0;
        if (zero && (int)threadIdx.x < n_zero) zero[threadIdx.x] = 0;
    }
}

__global__ void __launch_bounds__(256) k_tri_cells(int nt, GridParams g, float margin,
                                                   const float4 *__restrict__ inst_cell,
                                                   int n_inst_cell,
                                                   const int4 *__restrict__ tri,
                                                   const float4 *__restrict__ x,
                                                   const float4 *__restrict__ p, int4 *tcell,
                                                   float4 *tlo, float4 *thi, uint32_t *key,
                                                   int *id, int *n_valid,
                                                   const int *__restrict__ tri_slot,
                                                   int4 *pt_cell) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = false;
    if (t < nt) {
        int4 f = tri[t];
        v3 a = ld3(p[f.x]), b = ld3(p[f.y]), c = ld3(p[f.z]);
        // centroid (P/SpatialHashSystem.cpp:291-293) and cell (:394-396)
        float cx = (a.x + b.x + c.x) / 3.0f;
        float cy = (a.y + b.y + c.y) / 3.0f;
        float cz = (a.z + b.z + c.z) / 3.0f;
        float3 cell = g.cell;
        if (f.w >= 0 && f.w < n_inst_cell) {
            float4 ic = inst_cell[f.w];
            cell = make_float3(ic.x, ic.y, ic.z);
        }
        int ix = (int)floorf((cx - g.start.x) / cell.x);
        int iy = (int)floorf((cy - g.start.y) / cell.y);
        int iz = (int)floorf((cz - g.start.z) / cell.z);
        valid = g.hashed || !outside(g, ix, iy, iz);
        tcell[t] = make_int4(ix, iy, iz, f.w);
        // the cell in its vertices' slots
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int sl = tri_slot[3 * (size_t)t + k];
            if (sl >= 0) pt_cell[sl] = make_int4(ix, iy, iz, t);
        }
        key[t] = valid ? bucket_of(g, ix, iy, iz, f.w) : g.nb;
        id[t] = t;
        v3 xa = ld3(x[f.x]), xb = ld3(x[f.y]), xc = ld3(x[f.z]);
        if (sliver(a, b, c) || sliver(xa, xb, xc)) {
            tlo[t] = make_float4(-INFINITY, -INFINITY, -INFINITY, 1.f);
            thi[t] = make_float4(INFINITY, INFINITY, INFINITY, 1.f);
        } else {
            float lx = fminf(fminf(fminf(a.x, b.x), fminf(c.x, xa.x)), fminf(xb.x, xc.x));
            float ly = fminf(fminf(fminf(a.y, b.y), fminf(c.y, xa.y)), fminf(xb.y, xc.y));
            float lz = fminf(fminf(fminf(a.z, b.z), fminf(c.z, xa.z)), fminf(xb.z, xc.z));
            float hx = fmaxf(fmaxf(fmaxf(a.x, b.x), fmaxf(c.x, xa.x)), fmaxf(xb.x, xc.x));
            float hy = fmaxf(fmaxf(fmaxf(a.y, b.y), fmaxf(c.y, xa.y)), fmaxf(xb.y, xc.y));
            float hz = fmaxf(fmaxf(fmaxf(a.z, b.z), fmaxf(c.z, xa.z)), fmaxf(xb.z, xc.z));
            tlo[t] = make_float4(lx - margin, ly - margin, lz - margin, 0.f);
            thi[t] = make_float4(hx + margin, hy + margin, hz + margin, 0.f);
        }
    }
    unsigned m = __ballot_sync(0xffffffffu, valid);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(n_valid, __popc(m));
}

__global__ void k_bucket_ranges(const uint32_t *skey, const int *sid, const int *n_valid,
                                const int4 *tcell, const float4 *tlo, const float4 *thi,
                                float4 *btab, float4 *etab) {
    int n = *n_valid;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = skey[i];
        int t = sid[i];
        int4 c = tcell[t];
        etab[3 * (size_t)i] = make_float4(__int_as_float(c.x), __int_as_float(c.y),
                                          __int_as_float(c.z), __int_as_float(t));
        etab[3 * (size_t)i + 1] = tlo[t];
        etab[3 * (size_t)i + 2] = thi[t];
        if (i > 0 && skey[i - 1] == k) continue;
        float4 lo = tlo[sid[i]], hi = thi[sid[i]];
        int e = i + 1;
        for (; e < n && skey[e] == k; ++e) {
            float4 a = tlo[sid[e]], b = thi[sid[e]];
            lo.x = fminf(lo.x, a.x); lo.y = fminf(lo.y, a.y); lo.z = fminf(lo.z, a.z);
            hi.x = fmaxf(hi.x, b.x); hi.y = fmaxf(hi.y, b.y); hi.z = fmaxf(hi.z, b.z);
        }
        btab[2 * (size_t)k] = make_float4(__int_as_float(i), __int_as_float(e), lo.x, lo.y);
        btab[2 * (size_t)k + 1] = make_float4(lo.z, hi.x, hi.y, hi.z);
    }
}

// FindNeighbors (P/SpatialHashSystem.cpp:134-187) for every triangle:
// count (out == nullptr) or fill
__global__ void k_find_neighbors(int nt, GridParams g, const int4 *tcell, const float4 *btab,
                                 const float4 *etab, const int *sid, const int *off, int *cnt,
                                 int *out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int4 c = tcell[t];
    int k = 0, o = out ? off[t] : 0;
    if (g.hashed || !outside(g, c.x, c.y, c.z)) {
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    int nx = c.x + x, ny = c.y + y, nz = c.z + z;
                    if (!g.hashed && outside(g, nx, ny, nz)) continue;
                    float4 b0 = btab[2 * (size_t)bucket_of(g, nx, ny, nz, c.w)];
                    int2 r = make_int2(__float_as_int(b0.x), __float_as_int(b0.y));
                    for (int i = r.x; i < r.y; ++i) {
                        float4 e0 = etab[3 * (size_t)i];
                        int4 sc = make_int4(__float_as_int(e0.x), __float_as_int(e0.y),
                                            __float_as_int(e0.z), __float_as_int(e0.w));
                        if (sc.x != nx || sc.y != ny || sc.z != nz) continue;
                        int id = sc.w;
                        if (id == t) continue;
                        if (out) out[o + k] = id;
                        ++k;
                    }
                }
    }
    if (cnt) cnt[t] = k;
}

// squared Euclidean gap between boxes [pl, ph] and [l, h] (0 when they meet;
// an infinite box meets everything)
__device__ __forceinline__ float box_gap2(float plx, float ply, float plz, float phx, float phy,
                                          float phz, float lx, float ly, float lz, float hx,
                                          float hy, float hz) {
    const float gx = fmaxf(0.f, fmaxf(lx - phx, plx - hx));
    const float gy = fmaxf(0.f, fmaxf(ly - phy, ply - hy));
    const float gz = fmaxf(0.f, fmaxf(lz - phz, plz - hz));
    return (gx * gx + gy * gy) + gz * gz;
}

// Candidate search, one warp per point.  The point's candidate cells are
// the union of the 27-cell neighbourhoods of its incident triangles'
// centroid cells (FindNeighbors around every triangle that holds the point,
// P/SpatialHashSystem.cpp:134-187, as CCD_SH_Extended visits them,
// P/CCD.cpp:1522-1587).  A round takes 32 candidate cells, one per lane; a
// lane keeps its cell when the bucket is non-empty and the bucket's AABB lies
// within the reach margin (Euclidean gap) of the point's swept AABB.  The
// kept buckets' entries are then
// spread over the 32 lanes by a warp prefix sum (lane j of the warp takes
// flat entries j, j+32, ...), so a bucket of any size costs ceil(entries/32)
// coalesced steps; an entry yields a (point, triangle) pair when its cell is
// the lane's cell (the hash may mix cells), its swept AABB lies within the
// margin of the point's and it belongs to the point's instance.
constexpr int kTaskWarps = 8;
constexpr int kPointPairStage = 256;  // pairs staged per warp, appended with one atomic
constexpr unsigned long long kNear3 = 0x0000077707770777ull;  // 3x3x3 corner of a 4x4x4 block
__global__ void __launch_bounds__(32 * kTaskWarps) k_point_pairs(
    int n, GridParams g, float margin, const int *__restrict__ pt_first,
    const int *__restrict__ pt_last, const int *__restrict__ pt_tri,
    const int *__restrict__ point_inst, const int *__restrict__ tri_inst,
    const float4 *__restrict__ x, const float4 *__restrict__ p, const int4 *__restrict__ tcell,
    const float4 *__restrict__ btab, const float4 *__restrict__ etab, int2 *pairs, long long cap,
    int *counters, const int4 *__restrict__ pt_cell) {
    __shared__ int2 stage_all[kTaskWarps][kPointPairStage];
    const int lane = threadIdx.x & 31;
    const int warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    int2 *stage = stage_all[threadIdx.x >> 5];
    int scnt = 0;  // pairs staged by this warp
    for (int v = warp0; v < n; v += nwarps) {
        // one round of independent loads: the point's positions, its
        // incidence range and the slots with its first incident triangles'
        // cells; a point with more incident triangles than slots reads its
        // list and their cells (two more dependent loads)
        const float4 xv = x[v], pv = p[v];
        int f0 = pt_first[v], f1 = pt_last[v];
        const int4 sl = lane < kPointSlots ? pt_cell[(size_t)v * kPointSlots + lane]
                                           : make_int4(0, 0, 0, -1);
        int ninc = f1 - f0;
        if (ninc > kMaxInc) {
            if (lane == 0) atomicOr(counters + 2, 4);
            ninc = kMaxInc;
        }
        const int inst = point_inst ? point_inst[v] : 0;
        int4 mc = make_int4(0, 0, 0, 0);
        bool valid = false;
        int inc_tri = -1;  // this lane's incident triangle
        if (lane < ninc) {
            if (ninc <= kPointSlots) {
                inc_tri = sl.w;
                mc = sl;
            } else {
                inc_tri = pt_tri[f0 + lane];
                mc = tcell[inc_tri];
            }
            valid = g.hashed || !outside(g, mc.x, mc.y, mc.z);
        }
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        if (!vm) continue;
        // box of the valid incident cells
        const int lx = __reduce_min_sync(0xffffffffu, valid ? mc.x : INT_MAX);
        const int ly = __reduce_min_sync(0xffffffffu, valid ? mc.y : INT_MAX);
        const int lz = __reduce_min_sync(0xffffffffu, valid ? mc.z : INT_MAX);
        const int hx = __reduce_max_sync(0xffffffffu, valid ? mc.x : INT_MIN);
        const int hy = __reduce_max_sync(0xffffffffu, valid ? mc.y : INT_MIN);
        const int hz = __reduce_max_sync(0xffffffffu, valid ? mc.z : INT_MIN);
        v3 X0 = ld3(xv), P0 = ld3(pv);
        // the point's swept box; a box within Euclidean distance `margin` of
        // it can hold a hit (the point and the triangle at one time t lie in
        // their swept boxes, and a hit needs them within the reach)
        const float plx = fminf(X0.x, P0.x), phx = fmaxf(X0.x, P0.x);
        const float ply = fminf(X0.y, P0.y), phy = fmaxf(X0.y, P0.y);
        const float plz = fminf(X0.z, P0.z), phz = fmaxf(X0.z, P0.z);
        const float m2 = margin * margin;
        // Incident cells within a 2 x 2 x 2 block (nearly always): the union
        // of their 27-neighbourhoods is a mask over the 4 x 4 x 4 block at
        // (lx - 1, ly - 1, lz - 1), bit x + 4 y + 16 z, OR-reduced over the
        // lanes.  Otherwise each cell of the box is checked against the
        // distinct incident cells.
        const bool compact = hx - lx <= 1 && hy - ly <= 1 && hz - lz <= 1;
        unsigned long long nmask = 0;
        unsigned dm = 0;
        bool single = false;
        int ex = 4, exy = 16, ncell = 64;
        unsigned mex = 0, mexy = 0;
        bool magic = false;
        if (compact) {
            const unsigned long long mine =
                valid ? kNear3 << ((mc.x - lx) + 4 * (mc.y - ly) + 16 * (mc.z - lz)) : 0ull;
            nmask = (unsigned long long)__reduce_or_sync(0xffffffffu, (unsigned)(mine >> 32))
                        << 32 |
                    __reduce_or_sync(0xffffffffu, (unsigned)mine);
        } else {
            // distinct valid incident cells: the lowest lane of each group of
            // lanes holding the same cell
            const unsigned same = __match_any_sync(0xffffffffu, valid ? mc.x : INT_MIN) &
                                  __match_any_sync(0xffffffffu, valid ? mc.y : INT_MIN) &
                                  __match_any_sync(0xffffffffu, valid ? mc.z : INT_MIN);
            dm = __ballot_sync(0xffffffffu, valid && (same & vm & ((1u << lane) - 1u)) == 0u);
            single = __popc(dm) == 1;
            ex = hx - lx + 3;
            exy = ex * (hy - ly + 3);
            ncell = exy * (hz - lz + 3);
            // ci -> (x, y, z) in the box by multiplying with ceil(2^32 / d),
            // exact for ci * d < 2^32 (ex, exy >= 3; ci < ncell); boxes too
            // large for that divide
            magic = (unsigned long long)ncell * (unsigned long long)exy < (1ull << 32);
            mex = 0xffffffffu / (unsigned)ex + 1u;
            mexy = 0xffffffffu / (unsigned)exy + 1u;
        }
        for (int base = 0; base < ncell; base += 32) {
            const int ci = base + lane;
            int cx, cy, cz;
            bool near;
            if (compact) {
                cx = lx - 1 + (ci & 3);
                cy = ly - 1 + ((ci >> 2) & 3);
                cz = lz - 1 + (ci >> 4);
                near = ((nmask >> ci) & 1ull) != 0;
            } else {
                const int qz = magic ? (int)__umulhi((unsigned)ci, mexy) : ci / exy;
                const int rz = ci - qz * exy;
                const int qy = magic ? (int)__umulhi((unsigned)rz, mex) : rz / ex;
                cx = lx - 1 + (rz - qy * ex);
                cy = ly - 1 + qy;
                cz = lz - 1 + qz;
                // within one cell of some valid incident cell (read from the
                // lanes holding the distinct cells; with one cell every box
                // cell is)
                near = single;
                unsigned m = single ? 0u : dm;
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
                    const int sx = __shfl_sync(0xffffffffu, mc.x, src);
                    const int sy = __shfl_sync(0xffffffffu, mc.y, src);
                    const int sz = __shfl_sync(0xffffffffu, mc.z, src);
                    near |= abs(sx - cx) <= 1 && abs(sy - cy) <= 1 && abs(sz - cz) <= 1;
                }
            }
            int cnt = 0, start = 0;
            if (ci < ncell && near && (g.hashed || !outside(g, cx, cy, cz))) {
                const uint32_t b = bucket_of(g, cx, cy, cz, inst);
                // range and box in one sector, loaded together
                const float4 b0 = btab[2 * (size_t)b], b1 = btab[2 * (size_t)b + 1];
                const int rs = __float_as_int(b0.x), re = __float_as_int(b0.y);
                if (rs < re &&
                    box_gap2(plx, ply, plz, phx, phy, phz, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w) <=
                        m2) {
                    cnt = re - rs;
                    start = rs;
                }
            }
            // flat entry index space of these 32 cells' kept buckets
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int excl = incl - cnt;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            for (int f0 = 0; f0 < total; f0 += 32) {
                const int f = f0 + lane;
                // owner: the last lane whose range starts at or before f
                int own = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int cand = own + step;
                    const int e = __shfl_sync(0xffffffffu, excl, cand & 31);
                    if (cand < 32 && e <= f) own = cand;
                }
                const int o_start = __shfl_sync(0xffffffffu, start, own);
                const int o_excl = __shfl_sync(0xffffffffu, excl, own);
                const int ox = __shfl_sync(0xffffffffu, cx, own);
                const int oy = __shfl_sync(0xffffffffu, cy, own);
                const int oz = __shfl_sync(0xffffffffu, cz, own);
                bool hit = false;
                int tri = 0;
                if (f < total) {
                    const int e = o_start + (f - o_excl);
                    // the entry's cell, id and box: 48 contiguous bytes, loaded together
                    const float4 e0 = etab[3 * (size_t)e], tl = etab[3 * (size_t)e + 1],
                                 th = etab[3 * (size_t)e + 2];
                    tri = __float_as_int(e0.w);
                    hit = __float_as_int(e0.x) == ox && __float_as_int(e0.y) == oy &&
                          __float_as_int(e0.z) == oz &&
                          box_gap2(plx, ply, plz, phx, phy, phz, tl.x, tl.y, tl.z, th.x, th.y,
                                   th.z) <= m2 &&
                          (!point_inst || tri_inst[tri] == inst);
                }
                // a triangle of the point itself is no candidate (the point is
                // one of its vertices): matched against the incident list
                if (__any_sync(0xffffffffu, hit))
                    for (int q = 0; q < ninc; ++q)
                        hit &= __shfl_sync(0xffffffffu, inc_tri, q) != tri;
                warp_stage_pair(hit, make_int2(v, tri), stage, kPointPairStage, scnt, lane, pairs,
                                cap, counters + 4, counters + 2, 16);
            }
        }
    }
    if (scnt) warp_flush_pairs(stage, scnt, lane, pairs, cap, counters + 4, counters + 2, 16);
}

// stage 3: one thread per AABB-overlapping pair.  The pair goes on to the
// narrow phase unless the point is a vertex of the triangle or no time of
// the step can pass ExtendedVFTest's two conditions: plane distance < 2h and
// every barycentric coordinate >= -eps, eps = h / mean edge length, at one
// time t.  Those put the point within sqrt((2h)^2 + r^2) of the triangle,
// r = 2h * (longest edge / mean edge) at t (the farthest point of the
// eps-grown triangle from the triangle is a grown corner, eps |2 v_i - v_j -
// v_k| from v_i); that ratio is at most 1.5 at any t, and over the step at
// most the largest end length of an edge (edge vectors move linearly) over
// the mean of the edges' smallest lengths (the distance of the segment
// between an edge's end vectors from 0).  The point-triangle distance is at
// least (d0 + d1 - U) / 2 over the step (d0, d1 at the ends, U the largest
// motion of a triangle corner relative to the point).
__global__ void __launch_bounds__(256) k_dist_filter(const int2 *__restrict__ pairs,
                                                     long long pcap, float th,
                                                     const int4 *__restrict__ tri,
                                                     const float4 *__restrict__ x,
                                                     const float4 *__restrict__ p, int2 *cand,
                                                     long long cap, int *counters) {
    long long n = counters[4];
    if (n > pcap) n = pcap;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int2 c = pairs[i];
        int4 fi = tri[c.y];
        if (fi.x == c.x || fi.y == c.x || fi.z == c.x) continue;
        v3 X0 = ld3(x[c.x]), P0 = ld3(p[c.x]);
        v3 xa = ld3(x[fi.x]), xb = ld3(x[fi.y]), xc = ld3(x[fi.z]);
        v3 pa = ld3(p[fi.x]), pb = ld3(p[fi.y]), pc = ld3(p[fi.z]);
        if (!sliver(xa, xb, xc) && !sliver(pa, pb, pc)) {
            // the pair's reach lies between its values at edge ratio 1 and
            // 1.5 (the ratio computed below is at least 1 and at most 1.5),
            // so only bounds in between need the ratio; rejecting above the
            // largest reach is exactly as safe, and accepting more is always
            // safe (the narrow phase decides)
            const float r15 = 2.f * th * 1.5f, r10 = 2.f * th;
            const float reach_max = sqrtf(4.f * th * th + r15 * r15) * 1.001f + 2e-6f;
            const float reach_min = sqrtf(4.f * th * th + r10 * r10) * 1.001f + 2e-6f;
            v3 D0 = sub3(P0, X0);
            v3 ua = sub3(sub3(pa, xa), D0), ub = sub3(sub3(pb, xb), D0),
               uc = sub3(sub3(pc, xc), D0);
            float U = sqrtf(fmaxf(fmaxf(dot3(ua, ua), dot3(ub, ub)), dot3(uc, uc)));
            float d0 = point_tri_dist(X0, xa, xb, xc);
            if ((d0 - U) * 0.5f > reach_max) continue;  // d1 >= 0 only raises the bound
            float d1 = point_tri_dist(P0, pa, pb, pc);
            const float bound = (d0 + d1 - U) * 0.5f;
            if (bound > reach_max) continue;
            if (bound > reach_min) {
            v3 e0[3] = {sub3(xb, xa), sub3(xc, xb), sub3(xa, xc)};
            v3 e1[3] = {sub3(pb, pa), sub3(pc, pb), sub3(pa, pc)};
            float lmax = 0.f, lsum = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                lmax = fmaxf(lmax, fmaxf(sqrtf(dot3(e0[k], e0[k])), sqrtf(dot3(e1[k], e1[k]))));
                lsum += seg_origin_dist(e0[k], e1[k]);
            }
            float ratio = lsum > 0.f ? fminf(1.5f, lmax / (lsum / 3.f)) : 1.5f;
            float r = 2.f * th * ratio;
            float reach = sqrtf(4.f * th * th + r * r) * 1.001f + 2e-6f;
            if (bound > reach) continue;
            }
        }
        long long slot = agg_inc(counters);
        if (slot < cap)
            cand[slot] = c;
        else
            atomicOr(counters + 2, 1);
    }
}

__device__ __forceinline__ void store_contact(int *counters, long long ccap, int2 c, int4 f,
                                              const VFResult &r, int4 *cids, int *cface,
                                              float4 *ctn, double4 *cw) {
    int slot = agg_inc(counters + 1);
    if (slot >= ccap) {
        atomicOr(counters + 2, 2);
        return;
    }
    cids[slot] = make_int4(c.x, f.x, f.y, f.z);
    cface[slot] = c.y;
    ctn[slot] = make_float4(r.t, r.n.x, r.n.y, r.n.z);
    cw[slot] = make_double4((double)r.w[0], (double)r.w[1], (double)r.w[2], (double)r.w[3]);
}

// narrow phase, common path: t = 0, and t = 1 when the coplanarity cubic has
// no root near [0, 1]; a pair that needs the cubic's roots goes to the hard
// list (counters[3]) so that the FP64 root isolation runs on full warps in
// k_narrow_roots instead of stalling the warps of the common path
// (mode: the narrowphase test, PBD_VFTEST_*; the tests that only look at
// the cubic's roots cannot hit when it has no root near [0, 1])
__device__ __forceinline__ int vf_first_mode(const v3 *X, const v3 *P, float th, int mode,
                                             VFResult &r) {
    if (mode == 0) return extended_vf_first(X, P, th, r);
    if (mode == 3) return vf_dcd_test(P, th, r) ? 1 : 0;
    float a[4];
    vf_coeffs(X, P, a);
    if (!no_root_near_unit(a[0], a[1], a[2], a[3])) return 2;
    if (mode == 4) return vf_dcd_test(P, th, r) ? 1 : 0;
    return 0;
}

__global__ void __launch_bounds__(128) k_narrow(const int2 *__restrict__ cand, long long cap,
                                                int nt, float th,
                                                const int4 *__restrict__ tri,
                                                const float4 *__restrict__ x,
                                                const float4 *__restrict__ p, int *counters,
                                                long long ccap, int4 *cids, int *cface,
                                                float4 *ctn, double4 *cw, int *hard, int mode) {
    long long n = counters[0];
    if (n > cap) n = cap;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int2 c = cand[i];
        int4 f = tri[c.y];
        v3 X[4] = {ld3(x[c.x]), ld3(x[f.x]), ld3(x[f.y]), ld3(x[f.z])};
        v3 P[4] = {ld3(p[c.x]), ld3(p[f.x]), ld3(p[f.y]), ld3(p[f.z])};
        VFResult r;
        int q = vf_first_mode(X, P, th, mode, r);
        if (q == 1) store_contact(counters, ccap, c, f, r, cids, cface, ctn, cw);
        if (q == 2) hard[agg_inc(counters + 3)] = (int)i;  // at most one entry per candidate
    }
}

// narrow phase, hard pairs: no hit when the point stays outside the grown
// triangle over the whole step (nearly all of them), else the cubic's roots
// in [0, 1] and t = 1
__global__ void __launch_bounds__(128) k_narrow_roots(const int2 *__restrict__ cand, float th,
                                                      const int4 *__restrict__ tri,
                                                      const float4 *__restrict__ x,
                                                      const float4 *__restrict__ p,
                                                      int *counters, long long ccap, int4 *cids,
                                                      int *cface, float4 *ctn, double4 *cw,
                                                      const int *__restrict__ hard, int mode) {
    const int n = counters[3];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int2 c = cand[hard[k]];
        int4 f = tri[c.y];
        v3 X[4] = {ld3(x[c.x]), ld3(x[f.x]), ld3(x[f.y]), ld3(x[f.z])};
        v3 P[4] = {ld3(p[c.x]), ld3(p[f.x]), ld3(p[f.y]), ld3(p[f.z])};
        VFResult r;
        bool hit = mode == 0 ? extended_vf_rest(X, P, th, r) : vf_test_mode(X, P, th, mode, r);
        if (hit) store_contact(counters, ccap, c, f, r, cids, cface, ctn, cw);
    }
}

// the predicted positions an overlapped detection reads
__global__ void __launch_bounds__(256) k_copy_points(int n, const float4 *__restrict__ p,
                                                     float4 *__restrict__ q) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = p[i];
}

__global__ void k_clamp_counts(int *counters, long long cap, long long ccap) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (counters[1] > ccap) counters[1] = (int)ccap;
        if (counters[0] > cap) counters[0] = (int)cap;
    }
}

// corrections of one contact (VFResolveTest + VFResolveNew, P/CCD.cpp:1996-2090)
// added to the per-point fixed-point sums
__global__ void __launch_bounds__(128) k_contact_deltas(const int *counters, const int4 *ids,
                                                        const float4 *__restrict__ x,
                                                        const float4 *__restrict__ p, float th,
                                                        int mass_weighted, long long *acc,
                                                        int *acnt) {
    // launched as a programmatic dependent of the sweep's last color phase:
    // nothing is read before that phase has completed; the apply kernel may
    // then launch while the corrections are summed
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    int n = counters[1];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        int4 id = ids[c];
        float4 q0 = x[id.x], q1 = x[id.y], q2 = x[id.z], q3 = x[id.w];
        v3 X0 = ld3(q0), X1 = ld3(q1), X2 = ld3(q2), X3 = ld3(q3);
        v3 P0 = ld3(p[id.x]), P1 = ld3(p[id.y]), P2 = ld3(p[id.z]), P3 = ld3(p[id.w]);
        float wm0 = q0.w, wm1 = q1.w, wm2 = q2.w, wm3 = q3.w;
        v3 e1 = sub3(P2, P1), e2 = sub3(P3, P1);
        v3 pr = cross3(e1, e2);
        float pr2 = dot3(pr, pr);
        bool ok = mass_weighted ? (pr2 > 1e-12f * (dot3(e1, e1) * dot3(e2, e2)))
                                : !((double)pr2 <= 1e-6);
        if (!ok) continue;
        v3 fn = nrm3(cross3(sub3(X2, X1), sub3(X3, X1)));
        bool dir = dot3(sub3(X0, X1), fn) >= 0;  // RelativePos
        v3 pn = nrm3(pr);
        float sg = dir ? 1.0f : -1.0f;
        v3 ns = mul3(pn, sg);
        float gap = (float)((double)dot3(sub3(P0, P1), ns) - 2.0 * (double)th);
        if (!(gap < -1e-6f)) continue;
        v3 p1proj = add3(P1, mul3(mul3(ns, 2.0f), th));
        float depth = (float)((double)dot3(sub3(p1proj, P0), ns) * 0.5);
        v3 w = bary(P0, P1, P2, P3);
        v3 dv, d1, d2, d3;
        if (!mass_weighted) {
            v3 vfix = mul3(ns, depth);
            v3 ffix = mul3(mul3(pn, -sg), depth);
            float sw = w.x * w.x + w.y * w.y + w.z * w.z;
            dv = vfix;
            d1 = div3(mul3(ffix, w.x), sw);
            d2 = div3(mul3(ffix, w.y), sw);
            d3 = div3(mul3(ffix, w.z), sw);
        } else {
            float sw = w.x * w.x + w.y * w.y + w.z * w.z;
            float swm = w.x * w.x * wm1 + w.y * w.y * wm2 + w.z * w.z * wm3;
            float mf = swm / sw;
            float msum = wm0 + mf;
            if (!(msum > 0.0f) || !(sw > 0.0f)) continue;
            float alpha = wm0 / msum;
            float sep = 2.0f * depth;
            dv = mul3(ns, sep * alpha);
            float fs = swm > 0.0f ? -sep * (1.0f - alpha) / swm : 0.0f;
            d1 = mul3(ns, fs * w.x * wm1);
            d2 = mul3(ns, fs * w.y * wm2);
            d3 = mul3(ns, fs * w.z * wm3);
        }
        add_fixed(acc, id.x, dv.x, dv.y, dv.z);
        add_fixed(acc, id.y, d1.x, d1.y, d1.z);
        add_fixed(acc, id.z, d2.x, d2.y, d2.z);
        add_fixed(acc, id.w, d3.x, d3.y, d3.z);
        atomicAdd(acnt + id.x, 1);
        atomicAdd(acnt + id.y, 1);
        atomicAdd(acnt + id.z, 1);
        atomicAdd(acnt + id.w, 1);
    }
}

// every point with a correction: p += sum * 2^-32 / count; sums cleared
__global__ void __launch_bounds__(256) k_apply_deltas(int n, long long *acc, int *acnt,
                                                      float4 *p) {
    asm volatile("griddepcontrol.wait;" ::: "memory");  // every sum is complete
    for (int pt = blockIdx.x * blockDim.x + threadIdx.x; pt < n; pt += gridDim.x * blockDim.x) {
        int cnt = acnt[pt];
        if (cnt <= 0) continue;
        acnt[pt] = 0;
        long long sx = acc[3 * (long long)pt], sy = acc[3 * (long long)pt + 1],
                  sz = acc[3 * (long long)pt + 2];
        acc[3 * (long long)pt] = 0;
        acc[3 * (long long)pt + 1] = 0;
        acc[3 * (long long)pt + 2] = 0;
        float4 P = p[pt];
        double dc = (double)cnt;
        P.x = P.x + (float)((double)sx * (1.0 / 4294967296.0) / dc);
        P.y = P.y + (float)((double)sy * (1.0 / 4294967296.0) / dc);
        P.z = P.z + (float)((double)sz * (1.0 / 4294967296.0) / dc);
        p[pt] = P;
    }
}

// The older response, CollisionResolve + VFResolve (P/CCD.cpp:2423-2650):
// two passes over the contacts in stored order, each applied in place
// before the next is tested, the per-point resolve counters gating the
// crossing case.  The result depends on the order, so one thread walks
// it (the parallel response is k_contact_deltas / k_apply_deltas), in the
// order the contacts are reported: by point, then face triangle.
// sort keys of the contacts: (point, face triangle), the order the
// contacts are reported in
__global__ void k_old_keys(const int *counters, long long ccap, const int4 *ids, const int *face,
                           long long nt, unsigned long long *key, int *val) {
    long long n = counters[1];
    if (n > ccap) n = ccap;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        key[c] = (unsigned long long)ids[c].x * (unsigned long long)nt +
                 (unsigned long long)face[c];
        val[c] = (int)c;
    }
}

__global__ void k_resolve_old(const int *counters, long long ccap, const int4 *ids,
                              const int *order, const float4 *__restrict__ x, float4 *p, int *rt,
                              float th) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    long long n = counters[1];
    if (n > ccap) n = ccap;
    for (int it = 0; it < 2; ++it)
        for (long long k = 0; k < n; ++k) {
            const int4 id = ids[order[k]];
            const int pid[4] = {id.x, id.y, id.z, id.w};
            v3 X[4], P[4];
            float4 q[4];
            for (int j = 0; j < 4; ++j) {
                X[j] = ld3(x[pid[j]]);
                q[j] = p[pid[j]];
                P[j] = ld3(q[j]);
            }
            // skip test of CollisionResolve (P/CCD.cpp:2470-2476, 2537-2539)
            v3 fn = nrm3(cross3(sub3(X[2], X[1]), sub3(X[3], X[1])));
            const bool f_rel = dot3(sub3(X[0], X[1]), fn) >= 0;
            v3 nn = nrm3(cross3(sub3(P[2], P[1]), sub3(P[3], P[1])));
            const bool c_rel = dot3(sub3(P[0], P[1]), nn) >= 0;
            const float distance = point_to_plane(P[0], P[1], P[2], P[3]);
            if (c_rel == f_rel && distance >= 2 * th) continue;
            // VFResolve (P/CCD.cpp:2595-2650)
            v3 n = nrm3(cross3(sub3(P[2], P[1]), sub3(P[3], P[1])));
            const float depth = point_to_plane(P[0], P[1], P[2], P[3]);
            const bool prd_rel = dot3(sub3(P[0], P[1]), n) >= 0;
            float dp = 0.0f;
            v3 w = bary(P[0], P[1], P[2], P[3]);
            if (f_rel == prd_rel && depth < 2 * th) {
                dp = (float)((double)(2 * th - depth) * 0.5);
            } else if (f_rel != prd_rel) {
                VFResult r;
                if (rt[pid[0]] == 0 || rt[pid[1]] == 0 || rt[pid[2]] == 0 || rt[pid[3]] == 0 ||
                    vf_roots_test(X, P, th, false, r))
                    dp = (float)((double)(depth + 2 * th) * 0.5);
            }
            if (dp != 0.0f)
                for (int j = 0; j < 4; ++j) rt[pid[j]] += 1;
            const float sw = w.x * w.x + w.y * w.y + w.z * w.z;
            const v3 mn = mk3(-n.x, -n.y, -n.z);
            const v3 a = f_rel ? n : mn, b = f_rel ? mn : n;
            v3 np0 = add3(P[0], mul3(a, dp));
            v3 np1 = add3(P[1], div3(mul3(mul3(b, dp), w.x), sw));
            v3 np2 = add3(P[2], div3(mul3(mul3(b, dp), w.y), sw));
            v3 np3 = add3(P[3], div3(mul3(mul3(b, dp), w.z), sw));
            p[pid[0]] = make_float4(np0.x, np0.y, np0.z, q[0].w);
            p[pid[1]] = make_float4(np1.x, np1.y, np1.z, q[1].w);
            p[pid[2]] = make_float4(np2.x, np2.y, np2.z, q[2].w);
            p[pid[3]] = make_float4(np3.x, np3.y, np3.z, q[3].w);
        }
}

__global__ void k_vf_batch(int n, const float *x12, const float *p12, const float *th, int mode,
                           int *hit, float *t, double *w, float *nrm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 X[4], P[4];
    for (int j = 0; j < 4; ++j) {
        X[j] = mk3(x12[12 * i + 3 * j], x12[12 * i + 3 * j + 1], x12[12 * i + 3 * j + 2]);
        P[j] = mk3(p12[12 * i + 3 * j], p12[12 * i + 3 * j + 1], p12[12 * i + 3 * j + 2]);
    }
    VFResult r;
    r.t = 0.f;
    r.n = mk3(0.f, 0.f, 0.f);
    r.w[0] = r.w[1] = r.w[2] = r.w[3] = 0.f;
    hit[i] = vf_test_mode(X, P, th[i], mode, r) ? 1 : 0;
    t[i] = r.t;
    for (int k = 0; k < 4; ++k) w[4 * i + k] = (double)r.w[k];
    nrm[3 * i] = r.n.x;
    nrm[3 * i + 1] = r.n.y;
    nrm[3 * i + 2] = r.n.z;
}

int bits_for(long long maxval) {
    int b = 0;
    while (b < 63 && (1LL << b) <= maxval) ++b;
    return b < 1 ? 1 : b;
}
int round8(int b) { return (b + 7) / 8 * 8; }


constexpr int kPersistentBlocks = 8 * kNumSMs;
// the response's contact kernel: grid-stride over the contacts
constexpr int kResponseBlocks = 2 * kNumSMs;
// bucket reset: grid-stride over the previous update's keys
constexpr int kResetBlocks = 2 * kNumSMs;

}  // namespace

// UpdateSH on predicted positions psrc (the object's, or a copy of them),
// enqueued on stream s
static int shs_update_on(pbd_shs *h, cudaStream_t s, const float4 *psrc, int *zero = nullptr,
                         int n_zero = 0) {
    PBD_CHECK(h->initialized, PBD_ERR_STATE, "spatial hash used before InitSH");
    pbd_object *o = h->obj;
    GridParams g = params_of(h);
    if (o->nt == 0) return PBD_OK;
    // clear the ranges of the buckets the previous update filled
    k_reset_buckets<<<kResetBlocks, 256, 0, s>>>(h->skey, o->nt, g.nb, h->btab.p, h->n_valid.p,
                                                 zero, n_zero);
    k_tri_cells<<<grid_for(o->nt, 256), 256, 0, s>>>(o->nt, g, 0.0f, h->inst_cell.p,
                                                     h->n_inst_cell, o->tri.p, o->x.p, psrc,
                                                     h->tcell.p, h->tlo.p, h->thi.p, h->key.p,
                                                     h->id.p, h->n_valid.p, h->tri_slot.p,
                                                     h->pt_cell.p);
    PBD_LAUNCH();
    PBD_TRY(radix_sort<uint32_t>(h->key.p, h->id.p, h->key_alt.p, h->id_alt.p, o->nt, nullptr,
                                 round8(h->key_bits), h->scr, s, &h->skey, &h->sid));
    k_bucket_ranges<<<kPersistentBlocks, 256, 0, s>>>(h->skey, h->sid, h->n_valid.p, h->tcell.p,
                                                      h->tlo.p, h->thi.p, h->btab.p, h->etab.p);
    PBD_LAUNCH();
    return PBD_OK;
}

// UpdateSH on the object's predicted positions
int shs_update(pbd_shs *h) { return shs_update_on(h, h->obj->stream, h->obj->p.p); }

static int colli_alloc(pbd_colli *c) {
    pbd_object *o = c->obj;
    PBD_TRY(c->cand.alloc(c->cand_cap));
    PBD_TRY(c->hard.alloc(c->cand_cap));
    PBD_TRY(c->pairs.alloc(c->task_cap));
    PBD_TRY(c->counters.alloc(16));
    size_t H = (size_t)c->contact_cap;
    PBD_TRY(c->cids.alloc(H));
    PBD_TRY(c->cface.alloc(H));
    PBD_TRY(c->ctn.alloc(H));
    PBD_TRY(c->cw.alloc(H));
    PBD_TRY(c->acc.alloc(3 * (size_t)o->n));
    PBD_TRY(c->acnt.alloc(o->n));
    PBD_CUDA(cudaMemsetAsync(c->acc.p, 0, sizeof(long long) * 3 * (size_t)o->n, o->stream));
    PBD_CUDA(cudaMemsetAsync(c->acnt.p, 0, sizeof(int) * (size_t)o->n, o->stream));
    PBD_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int) * 16, o->stream));
    // overlapped detections (made here, outside any stream capture)
    PBD_TRY(c->psnap.alloc(o->n));
    if (!c->side) {
        int least = 0, greatest = 0;
        PBD_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        PBD_CUDA(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, least));
    }
    if (!c->ev_fork) PBD_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    if (!c->ev_join) PBD_CUDA(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    return PBD_OK;
}

// CCD_SH_Extended on the device from predicted positions psrc, enqueued on
// stream s (buffers already sized); no host synchronisation
static int ccd_detect_on(pbd_colli *c, cudaStream_t s, const float4 *psrc) {
    pbd_object *o = c->obj;
    pbd_shs *h = c->shs;
    if (o->nt == 0) {
        PBD_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int) * 16, s));
        return PBD_OK;
    }
    // the hash update's first kernel also zeroes the 16 counters
    PBD_TRY(shs_update_on(h, s, psrc, c->counters.p, 16));
    GridParams g = params_of(h);
    float th = c->thickness;
    // a hit needs the point within sqrt((2h)^2 + r^2) of the triangle, r =
    // 2h * (longest edge / mean edge) <= 3h (the distance filter's bound),
    // so within 3.606h on every axis: the point's swept box is grown by that
    // with slack (the filter then applies each pair's own reach)
    float margin = 3.61f * th * 1.001f + 2e-6f;

    // warps loop over points, so each warp's staged pairs span many points
    const int pp_blocks = (int)std::min<long long>(grid_for((long long)o->n * 32, 32 * kTaskWarps),
                                                   8 * kNumSMs);
    k_point_pairs<<<pp_blocks, 32 * kTaskWarps, 0, s>>>(
        o->n, g, margin, o->pt_tri_first.p, o->pt_tri_last.p, o->pt_tri.p,
        o->has_inst ? o->point_inst.p : nullptr, o->has_inst ? o->tri_inst.p : nullptr, o->x.p,
        psrc, h->tcell.p, h->btab.p, h->etab.p, c->pairs.p, c->task_cap, c->counters.p,
        h->pt_cell.p);
    PBD_LAUNCH();
    k_dist_filter<<<kPersistentBlocks, 256, 0, s>>>(c->pairs.p, c->task_cap, th, o->tri.p,
                                                    o->x.p, psrc, c->cand.p, c->cand_cap,
                                                    c->counters.p);
    PBD_LAUNCH();
    k_narrow<<<kPersistentBlocks, 128, 0, s>>>(c->cand.p, c->cand_cap, o->nt, th, o->tri.p,
                                               o->x.p, psrc, c->counters.p, c->contact_cap,
                                               c->cids.p, c->cface.p, c->ctn.p, c->cw.p,
                                               c->hard.p, c->vf_test);
    k_narrow_roots<<<kPersistentBlocks, 128, 0, s>>>(c->cand.p, th, o->tri.p, o->x.p, psrc,
                                                     c->counters.p, c->contact_cap, c->cids.p,
                                                     c->cface.p, c->ctn.p, c->cw.p, c->hard.p,
                                                     c->vf_test);
    k_clamp_counts<<<1, 32, 0, s>>>(c->counters.p, c->cand_cap, c->contact_cap);
    PBD_LAUNCH();
    return PBD_OK;
}

static int ccd_prepare(pbd_colli *c) {
    PBD_CHECK(c && c->obj && c->shs, PBD_ERR_STATE, "collision solver needs a target and a hash");
    PBD_CHECK(c->shs->obj == c->obj, PBD_ERR_ARG, "hash and collision solver target differ");
    pbd_object *o = c->obj;
    // (re)size everything for the current target: a first call, a capacity
    // change, or a target with another point count
    if (!c->cand.p || c->sized_n != o->n) {
        PBD_TRY(colli_alloc(c));
        c->sized_n = o->n;
    }
    if (c->ee_on) PBD_TRY(ee_prepare(c));
    return PBD_OK;
}

// CCD_SH_Extended on the device; no host synchronisation
int ccd_detect(pbd_colli *c) {
    PBD_TRY(ccd_prepare(c));
    PBD_TRY(ccd_detect_on(c, c->obj->stream, c->obj->p.p));
    if (c->ee_on) PBD_TRY(ee_detect(c));
    return PBD_OK;
}

int ccd_detect_fork(pbd_colli *c, bool *forked) {
    *forked = false;
    PBD_CHECK(c && c->obj && c->shs, PBD_ERR_STATE, "collision solver needs a target and a hash");
    pbd_object *o = c->obj;
    if (!c->overlap || c->ee_on || !c->cand.p || c->sized_n != o->n || !c->side ||
        o->nt == 0 || c->shs->obj != o)
        return ccd_detect(c);
    cudaStream_t s = o->stream;
    k_copy_points<<<grid_for(o->n, 256), 256, 0, s>>>(o->n, o->p.p, c->psnap.p);
    PBD_LAUNCH();
    PBD_CUDA(cudaEventRecord(c->ev_fork, s));
    PBD_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
    PBD_TRY(ccd_detect_on(c, c->side, c->psnap.p));
    PBD_CUDA(cudaEventRecord(c->ev_join, c->side));
    *forked = true;
    return PBD_OK;
}

int ccd_snapshot(pbd_colli *c, const float4 *src) {
    pbd_object *o = c->obj;
    k_copy_points<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, src, c->psnap.p);
    PBD_LAUNCH();
    return PBD_OK;
}

int ccd_detect_snapshot(pbd_colli *c) {
    PBD_TRY(ccd_prepare(c));
    PBD_TRY(ccd_detect_on(c, c->obj->stream, c->psnap.p));
    if (c->ee_on) PBD_TRY(ee_detect(c));
    return PBD_OK;
}

int ccd_prepare_all(pbd_colli *c) { return ccd_prepare(c); }

int ccd_join(pbd_colli *c) {
    PBD_CUDA(cudaStreamWaitEvent(c->obj->stream, c->ev_join, 0));
    return PBD_OK;
}

int ccd_resolve(pbd_colli *c, int passes) {
    pbd_object *o = c->obj;
    cudaStream_t s = o->stream;
    if (!c->cand.p || o->nt == 0) return PBD_OK;
    PBD_CHECK(c->sized_n == o->n, PBD_ERR_STATE,
              "the target changed since the last CCD pass: detect before resolving");
    // both kernels are programmatic dependents of the kernel before them
    // (their first instruction waits for it), so their launch overlaps it
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cd = {}, ca = {};
    cd.gridDim = dim3(kResponseBlocks);
    cd.blockDim = dim3(128);
    ca.gridDim = dim3(grid_for(o->n, 256));
    ca.blockDim = dim3(256);
    cd.stream = ca.stream = s;
    cd.attrs = ca.attrs = at;
    cd.numAttrs = ca.numAttrs = o->pdl ? 1 : 0;
    for (int k = 0; k < passes; ++k) {
        PBD_CUDA(cudaLaunchKernelEx(&cd, k_contact_deltas, (const int *)c->counters.p,
                                    (const int4 *)c->cids.p, (const float4 *)o->x.p,
                                    (const float4 *)o->p.p, c->thickness,
                                    (int)(c->response == PBD_RESPONSE_MASS_WEIGHTED), c->acc.p,
                                    c->acnt.p));
        if (c->ee_on) PBD_TRY(ee_deltas_launch(c));
        PBD_CUDA(cudaLaunchKernelEx(&ca, k_apply_deltas, o->n, c->acc.p, c->acnt.p, o->p.p));
    }
    return PBD_OK;
}

}  // namespace pbd

using namespace pbd;

extern "C" {

static int shs_alloc(pbd_shs *h) {
    pbd_object *o = h->obj;
    size_t nt = o->nt ? o->nt : 1;
    PBD_TRY(h->tcell.alloc(nt));
    PBD_TRY(h->tlo.alloc(nt));
    PBD_TRY(h->thi.alloc(nt));
    PBD_TRY(h->key.alloc(nt));
    PBD_TRY(h->key_alt.alloc(nt));
    PBD_TRY(h->id.alloc(nt));
    PBD_TRY(h->id_alt.alloc(nt));
    PBD_TRY(h->etab.alloc(3 * nt));
    PBD_TRY(h->n_valid.alloc(1));
    PBD_TRY(h->pt_cell.alloc((size_t)(o->n ? o->n : 1) * kPointSlots));
    PBD_TRY(h->tri_slot.alloc(3 * nt));
    PBD_CUDA(cudaMemsetAsync(h->tri_slot.p, 0xff, sizeof(int) * 3 * nt, o->stream));
    if (o->n && o->nt) {
        k_tri_slots<<<grid_for(o->n, 256), 256, 0, o->stream>>>(
            o->n, o->pt_tri_first.p, o->pt_tri_last.p, o->pt_tri.p, o->tri.p, h->tri_slot.p);
        PBD_LAUNCH();
    }
    PBD_TRY(h->btab.alloc(2 * ((size_t)h->n_buckets + 1)));
    PBD_TRY(radix_reserve(h->scr, (long long)nt, round8(h->key_bits)));
    PBD_CUDA(cudaMemsetAsync(h->btab.p, 0, sizeof(float4) * 2 * (h->n_buckets + 1), o->stream));
    PBD_CUDA(cudaMemsetAsync(h->n_valid.p, 0, sizeof(int), o->stream));
    // no bucket filled yet: the first reset reads keys beyond every bucket
    PBD_CUDA(cudaMemsetAsync(h->key.p, 0xff, sizeof(uint32_t) * nt, o->stream));
    h->skey = h->key.p;
    h->sid = h->id.p;
    return PBD_OK;
}

int pbd_shs_create(pbd_object *obj, const float *center, const int *size, const float *cell,
                   pbd_shs **out) {
    PBD_CHECK(obj && center && size && cell && out, PBD_ERR_ARG, "null argument");
    PBD_CHECK(size[0] > 0 && size[1] > 0 && size[2] > 0, PBD_ERR_ARG, "grid size must be > 0");
    long long ncell = (long long)size[0] * size[1] * size[2];
    PBD_CHECK(ncell < (1LL << 30), PBD_ERR_ARG, "grid has too many cells (%lld)", ncell);
    PBD_CHECK(cell[0] > 0 && cell[1] > 0 && cell[2] > 0, PBD_ERR_ARG, "cell size must be > 0");
    pbd_shs *h = new pbd_shs();
    h->obj = obj;
    for (int k = 0; k < 3; ++k) {
        h->center[k] = center[k];
        h->size[k] = size[k];
        h->cell[k] = cell[k];
    }
    h->n_buckets = (int)ncell;
    h->key_bits = bits_for(ncell);  // keys 0..ncell (ncell = outside)
    *out = h;
    return PBD_OK;
}

int pbd_shs_create_hashed(pbd_object *obj, const float *cell, int log2_table, pbd_shs **out) {
    PBD_CHECK(obj && cell && out, PBD_ERR_ARG, "null argument");
    PBD_CHECK(log2_table >= 4 && log2_table <= 28, PBD_ERR_ARG, "log2_table must be 4..28");
    PBD_CHECK(cell[0] > 0 && cell[1] > 0 && cell[2] > 0, PBD_ERR_ARG, "cell size must be > 0");
    pbd_shs *h = new pbd_shs();
    h->obj = obj;
    h->hashed = true;
    h->log2_table = log2_table;
    for (int k = 0; k < 3; ++k) {
        h->cell[k] = cell[k];
        h->size[k] = 0;
    }
    h->n_buckets = 1 << log2_table;
    h->key_bits = log2_table;
    *out = h;
    return PBD_OK;
}

// The target object is not touched: it may already be gone (a caller's
// finaliser order is not guaranteed); freeing device memory synchronises.
int pbd_shs_destroy(pbd_shs *h) {
    delete h;
    return PBD_OK;
}

int pbd_shs_set_grid_center(pbd_shs *h, const float *c) {
    PBD_CHECK(h && c, PBD_ERR_ARG, "null argument");
    for (int k = 0; k < 3; ++k) h->center[k] = c[k];
    h->initialized = false;
    return PBD_OK;
}

int pbd_shs_set_grid_size(pbd_shs *h, const int *size) {
    PBD_CHECK(h && size && !h->hashed, PBD_ERR_ARG, "bad argument");
    long long ncell = (long long)size[0] * size[1] * size[2];
    PBD_CHECK(size[0] > 0 && size[1] > 0 && size[2] > 0 && ncell < (1LL << 30), PBD_ERR_ARG,
              "bad grid size");
    for (int k = 0; k < 3; ++k) h->size[k] = size[k];
    h->n_buckets = (int)ncell;
    h->key_bits = bits_for(ncell);
    h->initialized = false;
    h->btab.release();
    return PBD_OK;
}

int pbd_shs_set_division(pbd_shs *h, const float *cell) {
    PBD_CHECK(h && cell && cell[0] > 0 && cell[1] > 0 && cell[2] > 0, PBD_ERR_ARG, "bad cell");
    for (int k = 0; k < 3; ++k) h->cell[k] = cell[k];
    h->initialized = false;
    return PBD_OK;
}

int pbd_shs_set_instance_cells(pbd_shs *h, int n, const float *cells3) {
    PBD_CHECK(h && n >= 0 && (n == 0 || cells3), PBD_ERR_ARG, "bad argument");
    PBD_CHECK(n == 0 || h->hashed, PBD_ERR_STATE,
              "per-instance cells need the hashed grid (pbd_shs_create_hashed)");
    std::vector<float4> c(n);
    for (int i = 0; i < n; ++i) {
        PBD_CHECK(cells3[3 * i] > 0 && cells3[3 * i + 1] > 0 && cells3[3 * i + 2] > 0,
                  PBD_ERR_ARG, "cell of instance %d is not positive", i);
        c[i] = make_float4(cells3[3 * i], cells3[3 * i + 1], cells3[3 * i + 2], 0.f);
    }
    if (n) PBD_TRY(h->inst_cell.upload(c.data(), n, h->obj->stream));
    PBD_CUDA(cudaStreamSynchronize(h->obj->stream));
    h->n_inst_cell = n;
    return PBD_OK;
}

int pbd_shs_init(pbd_shs *h) {
    PBD_CHECK(h, PBD_ERR_ARG, "null argument");
    // m_girdStartPos = center - (gridSize * cellSize) / 2 (P/SpatialHashSystem.cpp:91-94)
    for (int k = 0; k < 3; ++k) {
        float shift = ((float)(unsigned)h->size[k] * h->cell[k]) / 2.0f;
        h->start[k] = h->center[k] - shift;
    }
    if (!h->btab.p || h->btab.n < 2 * ((size_t)h->n_buckets + 1)) PBD_TRY(shs_alloc(h));
    h->initialized = true;
    return shs_update(h);
}

int pbd_shs_update(pbd_shs *h) {
    PBD_CHECK(h, PBD_ERR_ARG, "null argument");
    return shs_update(h);
}

int pbd_shs_find_neighbors_all(pbd_shs *h, int *start_num, int *out, long long cap,
                               long long *total) {
    PBD_CHECK(h && total, PBD_ERR_ARG, "null argument");
    PBD_CHECK(h->initialized, PBD_ERR_STATE, "InitSH has not run");
    pbd_object *o = h->obj;
    cudaStream_t s = o->stream;
    int nt = o->nt;
    *total = 0;
    if (!nt) return PBD_OK;
    DBuf<int> cnt, off, tot;
    PBD_TRY(cnt.alloc(nt));
    PBD_TRY(off.alloc(nt));
    PBD_TRY(tot.alloc(1));
    GridParams g = params_of(h);
    k_find_neighbors<<<grid_for(nt, 128), 128, 0, s>>>(nt, g, h->tcell.p, h->btab.p, h->etab.p,
                                                       h->sid, nullptr, cnt.p, nullptr);
    PBD_LAUNCH();
    PBD_TRY(exclusive_scan(cnt.p, off.p, nt, tot.p, s));
    int t = 0;
    PBD_CUDA(cudaMemcpyAsync(&t, tot.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    *total = t;
    if (start_num) {
        std::vector<int> hc(nt), ho(nt);
        PBD_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(int) * nt, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaMemcpyAsync(ho.data(), off.p, sizeof(int) * nt, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaStreamSynchronize(s));
        for (int i = 0; i < nt; ++i) {
            start_num[2 * i] = ho[i];
            start_num[2 * i + 1] = hc[i];
        }
    }
    if (out && t > 0) {
        PBD_CHECK(cap >= t, PBD_ERR_OVERFLOW, "neighbor output needs %d entries", t);
        DBuf<int> dout;
        PBD_TRY(dout.alloc(t));
        k_find_neighbors<<<grid_for(nt, 128), 128, 0, s>>>(nt, g, h->tcell.p, h->btab.p,
                                                           h->etab.p, h->sid, off.p, nullptr,
                                                           dout.p);
        PBD_LAUNCH();
        PBD_CUDA(cudaMemcpyAsync(out, dout.p, sizeof(int) * t, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaStreamSynchronize(s));
    }
    return PBD_OK;
}

int pbd_shs_find_neighbors(pbd_shs *h, int tri, int *out, int cap, int *n) {
    PBD_CHECK(h && n && h->obj && tri >= 0 && tri < h->obj->nt, PBD_ERR_ARG, "bad argument");
    long long total = 0;
    std::vector<int> sn(2 * (size_t)h->obj->nt);
    PBD_TRY(pbd_shs_find_neighbors_all(h, sn.data(), nullptr, 0, &total));
    std::vector<int> all(total > 0 ? total : 1);
    PBD_TRY(pbd_shs_find_neighbors_all(h, nullptr, all.data(), total, &total));
    *n = sn[2 * tri + 1];
    for (int i = 0; i < *n && i < cap && out; ++i) out[i] = all[sn[2 * tri] + i];
    return PBD_OK;
}

int pbd_colli_create(pbd_colli **out) {
    PBD_CHECK(out, PBD_ERR_ARG, "null argument");
    *out = new pbd_colli();
    return PBD_OK;
}

// The target object is not touched (see pbd_shs_destroy).
int pbd_colli_destroy(pbd_colli *c) {
    delete c;
    return PBD_OK;
}

int pbd_colli_set_target(pbd_colli *c, pbd_object *o) {
    if (c) c->ee_n = -1;  // the edge list follows the target
    PBD_CHECK(c && o, PBD_ERR_ARG, "null argument");
    c->obj = o;
    return PBD_OK;
}
int pbd_colli_set_acce_struct(pbd_colli *c, pbd_shs *h) {
    PBD_CHECK(c && h, PBD_ERR_ARG, "null argument");
    c->shs = h;
    return PBD_OK;
}
int pbd_colli_set_thickness(pbd_colli *c, float th) {
    PBD_CHECK(c && th >= 0.f, PBD_ERR_ARG, "bad thickness");
    c->thickness = th;
    return PBD_OK;
}
int pbd_colli_set_iterations(pbd_colli *c, int it) {
    PBD_CHECK(c && it >= 0, PBD_ERR_ARG, "bad iterations");
    c->iterations = it;
    return PBD_OK;
}
int pbd_colli_set_response(pbd_colli *c, int mode) {
    PBD_CHECK(c && (mode == PBD_RESPONSE_REFERENCE || mode == PBD_RESPONSE_MASS_WEIGHTED),
              PBD_ERR_ARG, "bad response mode");
    c->response = mode;
    return PBD_OK;
}
int pbd_colli_set_capacity(pbd_colli *c, long long cand, long long contacts) {
    PBD_CHECK(c && cand > 0 && contacts > 0 && cand < (1LL << 31) && 4 * contacts < (1LL << 31),
              PBD_ERR_ARG, "bad capacity");
    c->cand_cap = cand;
    c->contact_cap = contacts;
    c->task_cap = cand;
    c->cand.release();
    c->cids.release();
    return PBD_OK;
}

int pbd_colli_collision_resolve_old(pbd_colli *c) {
    PBD_CHECK(c && c->obj, PBD_ERR_STATE, "collision solver has no target");
    pbd_object *o = c->obj;
    PBD_CHECK(c->cand.p && c->sized_n == o->n, PBD_ERR_STATE,
              "no detection on the current target: detect before resolving");
    if (!c->resolve_times.p || c->resolve_times.n < (size_t)o->n) {
        PBD_TRY(c->resolve_times.alloc(o->n));
        PBD_CUDA(cudaMemsetAsync(c->resolve_times.p, 0, sizeof(int) * o->n, o->stream));
    }
    // the contacts' reported order (the detection stores them as found)
    const long long cap = c->contact_cap;
    const int bits = round8(bits_for((long long)o->n * (long long)(o->nt > 0 ? o->nt : 1)));
    PBD_TRY(c->old_key.alloc(cap));
    PBD_TRY(c->old_key2.alloc(cap));
    PBD_TRY(c->old_val.alloc(cap));
    PBD_TRY(c->old_val2.alloc(cap));
    PBD_TRY(radix_reserve(c->old_scr, cap, bits));
    cudaStream_t s = o->stream;
    k_old_keys<<<kResponseBlocks, 256, 0, s>>>(c->counters.p, cap, c->cids.p, c->cface.p, o->nt,
                                               c->old_key.p, c->old_val.p);
    PBD_LAUNCH();
    unsigned long long *ko = nullptr;
    int *vo = nullptr;
    PBD_TRY(radix_sort<unsigned long long>(c->old_key.p, c->old_val.p, c->old_key2.p,
                                           c->old_val2.p, cap, c->counters.p + 1, bits,
                                           c->old_scr, s, &ko, &vo));
    k_resolve_old<<<1, 32, 0, s>>>(c->counters.p, cap, c->cids.p, vo, o->x.p, o->p.p,
                                   c->resolve_times.p, c->thickness);
    PBD_LAUNCH();
    return PBD_OK;
}

int pbd_colli_resolve_times(pbd_colli *c, int *out, int reset) {
    PBD_CHECK(c && c->obj, PBD_ERR_STATE, "collision solver has no target");
    pbd_object *o = c->obj;
    if (!c->resolve_times.p || c->resolve_times.n < (size_t)o->n) {
        PBD_TRY(c->resolve_times.alloc(o->n));
        PBD_CUDA(cudaMemsetAsync(c->resolve_times.p, 0, sizeof(int) * o->n, o->stream));
    }
    if (out)
        PBD_CUDA(cudaMemcpyAsync(out, c->resolve_times.p, sizeof(int) * o->n,
                                 cudaMemcpyDeviceToHost, o->stream));
    if (reset) PBD_CUDA(cudaMemsetAsync(c->resolve_times.p, 0, sizeof(int) * o->n, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    return PBD_OK;
}

int pbd_colli_set_vf_test(pbd_colli *c, int mode) {
    PBD_CHECK(c && mode >= PBD_VFTEST_EXTENDED && mode <= PBD_VFTEST_VF, PBD_ERR_ARG,
              "bad vertex-face test");
    c->vf_test = mode;
    return PBD_OK;
}

int pbd_colli_set_overlap(pbd_colli *c, int on) {
    PBD_CHECK(c, PBD_ERR_ARG, "null argument");
    c->overlap = on ? 1 : 0;
    return PBD_OK;
}

int pbd_colli_ccd_sh_extended(pbd_colli *c) {
    PBD_CHECK(c, PBD_ERR_ARG, "null argument");
    PBD_TRY(ccd_detect(c));
    int hc[4] = {0, 0, 0, 0};
    PBD_CUDA(cudaMemcpyAsync(hc, c->counters.p, sizeof(hc), cudaMemcpyDeviceToHost, c->obj->stream));
    PBD_CUDA(cudaStreamSynchronize(c->obj->stream));
    PBD_CHECK(!(hc[2] & 3), PBD_ERR_OVERFLOW,
              "CCD capacity exceeded (flags %d): raise pbd_colli_set_capacity", hc[2]);
    return PBD_OK;
}

int pbd_colli_collision_resolve_new(pbd_colli *c) {
    PBD_CHECK(c && c->obj, PBD_ERR_STATE, "collision solver has no target");
    return ccd_resolve(c, c->iterations);
}

int pbd_colli_get_contacts(pbd_colli *c, int *ids, int *face, float *t, double *w, float *n,
                           long long cap, long long *count) {
    PBD_CHECK(c && count, PBD_ERR_ARG, "null argument");
    *count = 0;
    if (!c->counters.p) return PBD_OK;
    cudaStream_t s = c->obj->stream;
    int hc[4];
    PBD_CUDA(cudaMemcpyAsync(hc, c->counters.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    long long h = hc[1];
    *count = h;
    if (h <= 0 || cap <= 0) return PBD_OK;
    std::vector<int4> hi(h);
    std::vector<int> hf(h);
    std::vector<float4> htn(h);
    std::vector<double4> hw(h);
    PBD_CUDA(cudaMemcpyAsync(hi.data(), c->cids.p, sizeof(int4) * h, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaMemcpyAsync(hf.data(), c->cface.p, sizeof(int) * h, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaMemcpyAsync(htn.data(), c->ctn.p, sizeof(float4) * h, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaMemcpyAsync(hw.data(), c->cw.p, sizeof(double4) * h, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    // order by (point, face triangle)
    std::vector<long long> order(h);
    for (long long i = 0; i < h; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](long long a, long long b) {
        return hi[a].x != hi[b].x ? hi[a].x < hi[b].x : hf[a] < hf[b];
    });
    long long m = std::min(h, cap);
    for (long long k = 0; k < m; ++k) {
        long long i = order[k];
        if (ids) {
            ids[4 * k] = hi[i].x;
            ids[4 * k + 1] = hi[i].y;
            ids[4 * k + 2] = hi[i].z;
            ids[4 * k + 3] = hi[i].w;
        }
        if (face) face[k] = hf[i];
        if (t) t[k] = htn[i].x;
        if (n) {
            n[3 * k] = htn[i].y;
            n[3 * k + 1] = htn[i].z;
            n[3 * k + 2] = htn[i].w;
        }
        if (w) {
            w[4 * k] = hw[i].x;
            w[4 * k + 1] = hw[i].y;
            w[4 * k + 2] = hw[i].z;
            w[4 * k + 3] = hw[i].w;
        }
    }
    return PBD_OK;
}

int pbd_ccd_vf_test_batch(const float *x12, const float *p12, const float *thickness, int n,
                          int *hit, float *t, double *w, float *nrm) {
    return pbd_ccd_vf_test_batch_mode(x12, p12, thickness, n, PBD_VFTEST_EXTENDED, hit, t, w,
                                      nrm);
}

int pbd_ccd_vf_test_batch_mode(const float *x12, const float *p12, const float *thickness,
                               int n, int mode, int *hit, float *t, double *w, float *nrm) {
    PBD_CHECK(x12 && p12 && thickness && hit && t && w && nrm && n >= 0, PBD_ERR_ARG,
              "null argument");
    PBD_CHECK(mode >= PBD_VFTEST_EXTENDED && mode <= PBD_VFTEST_VF, PBD_ERR_ARG,
              "bad vertex-face test %d", mode);
    if (n == 0) return PBD_OK;
    cudaStream_t s = nullptr;
    PBD_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    DBuf<float> dx, dp, dth, dt, dn;
    DBuf<int> dh;
    DBuf<double> dw;
    int r = PBD_OK;
    if ((r = dx.upload(x12, 12 * (size_t)n, s)) || (r = dp.upload(p12, 12 * (size_t)n, s)) ||
        (r = dth.upload(thickness, n, s)) || (r = dh.alloc(n)) || (r = dt.alloc(n)) ||
        (r = dw.alloc(4 * (size_t)n)) || (r = dn.alloc(3 * (size_t)n))) {
        cudaStreamDestroy(s);
        return r;
    }
    k_vf_batch<<<grid_for(n, 128), 128, 0, s>>>(n, dx.p, dp.p, dth.p, mode, dh.p, dt.p, dw.p,
                                                dn.p);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hit, dh.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t, dt.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w, dw.p, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(nrm, dn.p, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    PBD_CUDA(e);
    return PBD_OK;
}

int pbd_colli_get_pairs(pbd_colli *c, int *pairs, long long cap, long long *n) {
    PBD_CHECK(c && n && cap >= 0, PBD_ERR_ARG, "bad argument");
    int cnt = 0;
    if (c->counters.p) {
        PBD_CUDA(cudaMemcpyAsync(&cnt, c->counters.p + 4, sizeof(int), cudaMemcpyDeviceToHost,
                                 c->obj->stream));
        PBD_CUDA(cudaStreamSynchronize(c->obj->stream));
    }
    const long long m = std::min<long long>(cnt, c->task_cap);
    *n = m;
    const long long k = std::min(m, cap);
    if (pairs && k > 0) {
        PBD_CUDA(cudaMemcpyAsync(pairs, c->pairs.p, sizeof(int2) * k, cudaMemcpyDeviceToHost,
                                 c->obj->stream));
        PBD_CUDA(cudaStreamSynchronize(c->obj->stream));
    }
    return PBD_OK;
}

int pbd_colli_stats(pbd_colli *c, long long *cand, long long *contacts, int *overflow) {
    PBD_CHECK(c, PBD_ERR_ARG, "null argument");
    int hc[4] = {0, 0, 0, 0};
    if (c->counters.p) {
        PBD_CUDA(cudaMemcpyAsync(hc, c->counters.p, sizeof(hc), cudaMemcpyDeviceToHost, c->obj->stream));
        PBD_CUDA(cudaStreamSynchronize(c->obj->stream));
    }
    // a radix-sort look-back wait that ran out (never expected) shows as 512
    int st = 0, st_ee = 0;
    if (c->shs) PBD_TRY(radix_status(c->shs->scr, c->obj->stream, &st));
    PBD_TRY(radix_status(c->ee_scr, c->obj->stream, &st_ee));
    if (st || st_ee) hc[2] |= 512;
    if (cand) *cand = hc[0];
    if (contacts) *contacts = hc[1];
    if (overflow) *overflow = hc[2];
    return PBD_OK;
}

}  // extern "C"

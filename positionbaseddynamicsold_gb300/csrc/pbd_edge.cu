// pbd_edge.cu -- edge-edge continuous collision detection and response.
//
// The reference declares the contact kind only (Contact::EE, P/CCD_Basic.h:
// 14; EEResolve is commented out, P/CCD.cpp:925-928, 2589-2592); vertex-face
// CCD alone lets two edges cross without a vertex entering a face.  This path
// is off unless pbd_colli_set_edge_edge turns it on, so the reference's
// step is unchanged by default.
//
// Detection (every CCD pass, all on the device, graph-capturable):
//   1. per mesh edge: the box swept by its two end points over the step,
//      grown by 2 * thickness + slack, and the cells of the hashed grid it
//      overlaps (cell = the spatial hash's); one (bucket, entry) pair per
//      cell, the instance mixed into the bucket like the triangle hash;
//   2. radix sort of the entries by bucket;
//   3. the sorted entries gathered into contiguous records (cell, edge, end
//      points, box); one thread per record pairs it with the later records
//      of its bucket: same cell (the hash may mix cells), no shared point, same
//      instance, overlapping boxes, and the pair is reported only by the cell
//      holding the low corner of the boxes' intersection -- so every pair of
//      edges whose boxes overlap is reported exactly once;
//   4. a pair survives when the lower bound (d0 + d1 - U) / 2 of the
//      distance between the two moving segments over the step (d0, d1 the
//      segment distances at the ends, U the largest relative motion of two
//      end points) stays below the hit distance 2 * thickness;
//   5. one thread per survivor runs the edge-edge test: the coplanarity
//      cubic of ExtendedVFTest (P/CCD.cpp:1740-1743) in FP64, the times 0,
//      its roots in [0, 1] and 1 in ascending order, a hit at the first time
//      the lines of the two edges meet strictly inside both edges closer than
//      2 * thickness.  The side (common normal at t = 0 and the side edge A
//      starts on) is kept with the contact.
// Response: per pass, every contact pushes the closest points of its two
// predicted segments apart along their common normal (oriented like the
// start one) to 2 * thickness on the starting side, split by inverse mass and
// closest-point weights; the corrections join the vertex-face ones in the
// 2^-32 m fixed-point sums, so both kinds form one Jacobi pass.
//
// Compiled with -fmad=false, as the oracle restatement (oracle/pbd_oracle.c,
// orc_ee_test / orc_ee_resolve_deltas) is compiled with -ffp-contract=off.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "pbd_common.cuh"
#include "pbd_ccd.cuh"

namespace pbd {
namespace {

constexpr int kEEMaxCells = 256;      // cells per edge box; more sets overflow bit 32
constexpr int kEEEdgeMask = (1 << 28) - 1;  // entry word: edge | first-cell bits << 28
constexpr int kEEBlocks = 8 * kNumSMs;

// counters slots (pbd_colli::counters) of this path
constexpr int kEntries = 8, kPairs = 9, kCand = 10, kHits = 11;

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// closest points of the lines through a0a1 and b0b1 (Ericson, Real-Time
// Collision Detection, 5.1.8): true when the lines are not near-parallel and
// both parameters lie strictly inside (0, 1); d = A(s) - B(u)
__device__ __forceinline__ bool ee_interior(v3 a0, v3 a1, v3 b0, v3 b1, float &s, float &u,
                                            v3 &d) {
    v3 d1 = sub3(a1, a0), d2 = sub3(b1, b0), r = sub3(a0, b0);
    float a = dot3(d1, d1), e = dot3(d2, d2), b = dot3(d1, d2);
    float c = dot3(d1, r), f = dot3(d2, r);
    float den = a * e - b * b;
    if (!(den > 1e-8f * (a * e))) return false;
    float ss = (b * f - c * e) / den;
    float uu = (a * f - b * c) / den;
    if (!(ss > 0.0f && ss < 1.0f && uu > 0.0f && uu < 1.0f)) return false;
    s = ss;
    u = uu;
    d = sub3(add3(a0, mul3(d1, ss)), add3(b0, mul3(d2, uu)));
    return true;
}

// closest points of the segments (Ericson 5.1.9)
__device__ __forceinline__ void seg_closest(v3 p1, v3 q1, v3 p2, v3 q2, float &s, float &t) {
    v3 d1 = sub3(q1, p1), d2 = sub3(q2, p2), r = sub3(p1, p2);
    float a = dot3(d1, d1), e = dot3(d2, d2), f = dot3(d2, r);
    float ss, tt;
    if (a <= 1e-20f && e <= 1e-20f) {
        ss = 0.0f;
        tt = 0.0f;
    } else if (a <= 1e-20f) {
        ss = 0.0f;
        tt = clamp01(f / e);
    } else {
        float c = dot3(d1, r);
        if (e <= 1e-20f) {
            tt = 0.0f;
            ss = clamp01(-c / a);
        } else {
            float b = dot3(d1, d2), den = a * e - b * b;
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
    s = ss;
    t = tt;
}

__device__ __forceinline__ float seg_dist(v3 a0, v3 a1, v3 b0, v3 b1) {
    float s, u;
    seg_closest(a0, a1, b0, b1, s, u);
    v3 d = sub3(add3(a0, mul3(sub3(a1, a0), s)), add3(b0, mul3(sub3(b1, b0), u)));
    return sqrtf(dot3(d, d));
}

struct EEHit {
    float t, s, u;
    float4 m0;
};

__device__ __forceinline__ bool ee_eval_at(const v3 *X, const v3 *P, float th, double t,
                                           EEHit &h) {
    v3 c0 = lerp_t(X[0], P[0], t), c1 = lerp_t(X[1], P[1], t);
    v3 c2 = lerp_t(X[2], P[2], t), c3 = lerp_t(X[3], P[3], t);
    float s, u;
    v3 d;
    if (!ee_interior(c0, c1, c2, c3, s, u, d)) return false;
    float dist = sqrtf(dot3(d, d));
    if (!plane_close(dist, 2.0f * th)) return false;
    h.t = (float)t;
    h.s = s;
    h.u = u;
    return true;
}

// orc_ee_test with two exact early exits: t = 0 is always the first time
// evaluated, and when the coplanarity cubic provably has no root within
// 1e-3 of [0, 1] only t = 1 remains (the vertex-face test's argument)
__device__ bool ee_test(const v3 *X, const v3 *P, float th, EEHit &h) {
    v3 da = sub3(X[1], X[0]), db = sub3(X[3], X[2]);
    v3 m0 = cross3(da, db);
    if (!(dot3(m0, m0) > 1e-12f * (dot3(da, da) * dot3(db, db)))) return false;
    m0 = nrm3(m0);
    float sg = dot3(sub3(X[0], X[2]), m0) >= 0.0f ? 1.0f : -1.0f;
    h.m0 = make_float4(m0.x, m0.y, m0.z, sg);
    v3 x0 = X[0], v0 = sub3(P[0], x0);
    v3 x1 = sub3(X[1], x0), x2 = sub3(X[2], x0), x3 = sub3(X[3], x0);
    v3 v1 = sub3(sub3(P[1], X[1]), v0), v2 = sub3(sub3(P[2], X[2]), v0),
       v3_ = sub3(sub3(P[3], X[3]), v0);
    const float a0 = stp(x1, x2, x3);
    const float a1 = stp(v1, x2, x3) + stp(x1, v2, x3) + stp(x1, x2, v3_);
    const float a2 = stp(x1, v2, v3_) + stp(v1, x2, v3_) + stp(v1, v2, x3);
    const float a3 = stp(v1, v2, v3_);
    if (ee_eval_at(X, P, th, 0.0, h)) return true;
    if (no_root_near_unit(a0, a1, a2, a3)) return ee_eval_at(X, P, th, 1.0, h);
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
        if (ee_eval_at(X, P, th, t[i], h)) return true;
    }
    return false;
}

// orc_ee_resolve_deltas: P = predicted a0, a1, b0, b1; wm = inverse masses
__device__ __forceinline__ bool ee_deltas(const v3 *P, const float *wm, float4 m0s, float th,
                                          v3 *dl) {
    v3 d1 = sub3(P[1], P[0]), d2 = sub3(P[3], P[2]);
    v3 mp = cross3(d1, d2);
    if (!(dot3(mp, mp) > 1e-12f * (dot3(d1, d1) * dot3(d2, d2)))) return false;
    mp = nrm3(mp);
    if (dot3(mp, mk3(m0s.x, m0s.y, m0s.z)) < 0.0f) mp = mul3(mp, -1.0f);
    float sg = m0s.w;
    float s, u;
    seg_closest(P[0], P[1], P[2], P[3], s, u);
    v3 d = sub3(add3(P[0], mul3(d1, s)), add3(P[2], mul3(d2, u)));
    float g = (float)((double)(sg * dot3(d, mp)) - 2.0 * (double)th);
    if (!(g < -1e-6f)) return false;
    float depth = -g;
    float c[4] = {1.0f - s, s, 1.0f - u, u};
    float den = wm[0] * c[0] * c[0] + wm[1] * c[1] * c[1] + wm[2] * c[2] * c[2] +
                wm[3] * c[3] * c[3];
    if (!(den > 0.0f)) return false;
    float imp = depth / den;
    dl[0] = mul3(mp, sg * c[0] * wm[0] * imp);
    dl[1] = mul3(mp, sg * c[1] * wm[1] * imp);
    dl[2] = mul3(mp, -sg * c[2] * wm[2] * imp);
    dl[3] = mul3(mp, -sg * c[3] * wm[3] * imp);
    return true;
}

__device__ __forceinline__ int cell_of(float v, float start, float cell) {
    return (int)floorf((v - start) / cell);
}

// step 1: boxes and entries
__global__ void __launch_bounds__(256) k_ee_entries(int ne, GridParams g, float grow,
                                                    const float4 *__restrict__ icell, int n_icell,
                                                    const int2 *__restrict__ edges,
                                                    const int *__restrict__ point_inst,
                                                    const float4 *__restrict__ x,
                                                    const float4 *__restrict__ p, float4 *elo,
                                                    float4 *ehi, int4 *ecell, uint32_t *key,
                                                    int *val, long long cap, int *counters) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int2 ed = edges[e];
    float4 xa = x[ed.x], xb = x[ed.y], pa = p[ed.x], pb = p[ed.y];
    float4 lo = make_float4(fminf(fminf(xa.x, xb.x), fminf(pa.x, pb.x)) - grow,
                            fminf(fminf(xa.y, xb.y), fminf(pa.y, pb.y)) - grow,
                            fminf(fminf(xa.z, xb.z), fminf(pa.z, pb.z)) - grow, 0.f);
    float4 hi = make_float4(fmaxf(fmaxf(xa.x, xb.x), fmaxf(pa.x, pb.x)) + grow,
                            fmaxf(fmaxf(xa.y, xb.y), fmaxf(pa.y, pb.y)) + grow,
                            fmaxf(fmaxf(xa.z, xb.z), fmaxf(pa.z, pb.z)) + grow, 0.f);
    elo[e] = lo;
    ehi[e] = hi;
    const int inst = point_inst ? point_inst[ed.x] : 0;
    const float3 cl = inst_cell_of(g, icell, n_icell, inst);
    float ext[6] = {(lo.x - g.start.x) / cl.x, (lo.y - g.start.y) / cl.y,
                    (lo.z - g.start.z) / cl.z, (hi.x - g.start.x) / cl.x,
                    (hi.y - g.start.y) / cl.y, (hi.z - g.start.z) / cl.z};
    for (int k = 0; k < 6; ++k)
        if (!(fabsf(ext[k]) < 1e9f)) {  // non-finite or far outside any grid
            atomicOr(counters + 2, 32);
            return;
        }
    int x0 = cell_of(lo.x, g.start.x, cl.x), x1 = cell_of(hi.x, g.start.x, cl.x);
    int y0 = cell_of(lo.y, g.start.y, cl.y), y1 = cell_of(hi.y, g.start.y, cl.y);
    int z0 = cell_of(lo.z, g.start.z, cl.z), z1 = cell_of(hi.z, g.start.z, cl.z);
    long long nx = x1 - x0 + 1, ny = y1 - y0 + 1, nz = z1 - z0 + 1;
    long long nc = nx * ny * nz;
    if (nc <= 0 || nc > kEEMaxCells) {
        atomicOr(counters + 2, 32);
        return;
    }
    // every slot below cap that the counter hands out is written, so the
    // first min(count, cap) entries are always valid
    long long base = atomicAdd(counters + kEntries, (int)nc);
    if (base + nc > cap) atomicOr(counters + 2, 32);
    int k = 0;
    for (int cz = z0; cz <= z1; ++cz)
        for (int cy = y0; cy <= y1; ++cy)
            for (int cx = x0; cx <= x1; ++cx, ++k) {
                long long q = base + k;
                if (q >= cap) return;
                key[q] = bucket_of(g, cx, cy, cz, inst);
                val[q] = (int)q;
                // bits 28-30: the cell is the box's first along x, y, z
                const int first = (cx == x0) | (cy == y0) << 1 | (cz == z0) << 2;
                ecell[q] = make_int4(cx, cy, cz, e | first << 28);
            }
}

// step 3a: the sorted entries as contiguous records, so that the pairing
// below reads neighbouring words (shared by the lanes of a warp through L1)
// instead of three levels of dependent gathers per pair:
//   r0 = (cell x, cell y, cell z, edge), r1 = (box lo, end point 0),
//   r2 = (box hi, end point 1), rinst = the edge's instance (batches only)
__global__ void __launch_bounds__(256) k_ee_gather(long long cap, const int *__restrict__ sval,
                                                   const int4 *__restrict__ ecell,
                                                   const float4 *__restrict__ elo,
                                                   const float4 *__restrict__ ehi,
                                                   const int2 *__restrict__ edges,
                                                   const int *__restrict__ point_inst, int4 *r0,
                                                   float4 *r1, float4 *r2, int *rinst,
                                                   const int *counters) {
    long long n = counters[kEntries];
    if (n > cap) n = cap;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int4 c = ecell[sval[i]];
        const int e = c.w & kEEEdgeMask;
        const int2 E = edges[e];
        const float4 lo = elo[e], hi = ehi[e];
        r0[i] = c;
        r1[i] = make_float4(lo.x, lo.y, lo.z, __int_as_float(E.x));
        r2[i] = make_float4(hi.x, hi.y, hi.z, __int_as_float(E.y));
        if (point_inst) rinst[i] = point_inst[E.x];
    }
}

// step 3b: pairs within a bucket run.  Work is balanced over a run of m
// records: record a pairs with records (a + d) mod m, d = 1 .. (m - 1) / 2,
// and also d = m / 2 when m is even and a < m / 2 -- every unordered pair
// once, about m / 2 steps per record (the round-robin of a complete graph).
// A warp finds its records' run bounds from ballots of the run heads over
// its 32 records and, for runs crossing its window, over 32-record chunks
// before and after it.  Reported pairs are staged per warp in shared memory
// and appended with one atomic per kEEPairStage pairs (one counter takes
// every pair of the pass).  Reporting rule: the cell of the boxes'
// intersection's low corner is, per axis, the larger of the two boxes' first
// cells (floor((v - start) / cell) is monotone in v), so with both records
// in this cell it is this cell exactly when, on every axis, one of the two
// is its box's first cell there -- the record's three "first" bits.
constexpr int kEEPairStage = 256;
constexpr int kEEPairWarps = 8;

__global__ void __launch_bounds__(32 * kEEPairWarps) k_ee_pairs(
    int cap, const uint32_t *__restrict__ skey, const int4 *__restrict__ r0,
    const float4 *__restrict__ r1, const float4 *__restrict__ r2, const int *__restrict__ rinst,
    int2 *pairs, long long pcap, int *counters) {
    constexpr unsigned kAll = 0xffffffffu;
    __shared__ int2 stage_all[kEEPairWarps][kEEPairStage];
    const int lane = threadIdx.x & 31;
    int2 *stage = stage_all[threadIdx.x >> 5];
    int cnt = 0;
    const int n = min(counters[kEntries], cap);
    const int stride = gridDim.x * blockDim.x;
    for (int w = blockIdx.x * blockDim.x + (threadIdx.x & ~31); w < n; w += stride) {
        const int i = w + lane;
        const bool valid = i < n;
        const unsigned heads =
            __ballot_sync(kAll, valid && (i == 0 || skey[i - 1] != skey[i]));
        // start of the run holding the window's first record
        int s0 = w;
        if (!(heads & 1u)) {
            for (int b = w;; b -= 32) {
                const int q = b - 32 + lane;
                const unsigned hb =
                    __ballot_sync(kAll, q >= 0 && (q == 0 || skey[q - 1] != skey[q]));
                if (hb) {
                    s0 = b - 32 + 31 - __clz(hb);
                    break;
                }
            }
        }
        // end of the run holding the window's last record
        int e31 = n;
        for (int b = w + 32; b < n; b += 32) {
            const int q = b + lane;
            const unsigned hb = __ballot_sync(kAll, q < n && skey[q - 1] != skey[q]);
            if (hb) {
                e31 = b + __ffs(hb) - 1;
                break;
            }
        }
        const unsigned below = heads & (kAll >> (31 - lane));
        const unsigned above = lane == 31 ? 0u : heads & (kAll << (lane + 1));
        const int s = below ? w + 31 - __clz(below) : s0;
        const int e = above ? w + __ffs(above) - 1 : e31;
        const int m = e - s, a = i - s;
        const int steps = valid ? (m - 1) / 2 + ((m & 1) == 0 && a < m / 2) : 0;
        const int max_steps = __reduce_max_sync(kAll, steps);
        if (max_steps == 0) continue;
        int4 ci = make_int4(0, 0, 0, 0);
        float4 lo1 = make_float4(0.f, 0.f, 0.f, 0.f), hi1 = lo1;
        int inst1 = 0;
        if (steps) {
            ci = r0[i];
            lo1 = r1[i];
            hi1 = r2[i];
            if (rinst) inst1 = rinst[i];
        }
        const int e1 = ci.w & kEEEdgeMask, f1 = ci.w >> 28;
        const int a0 = __float_as_int(lo1.w), a1 = __float_as_int(hi1.w);
        int j = i;
        for (int d = 1; d <= max_steps; ++d) {
            bool hit = false;
            int e2 = 0;
            if (d <= steps) {
                if (++j == e) j = s;
                const int4 cj = r0[j];
                if (cj.x == ci.x && cj.y == ci.y && cj.z == ci.z && (f1 | cj.w >> 28) == 7) {
                    const float4 lo2 = r1[j], hi2 = r2[j];
                    const int b0 = __float_as_int(lo2.w), b1 = __float_as_int(hi2.w);
                    hit = !(a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) &&
                          !(lo1.x > hi2.x || lo2.x > hi1.x || lo1.y > hi2.y || lo2.y > hi1.y ||
                            lo1.z > hi2.z || lo2.z > hi1.z) &&
                          (!rinst || rinst[j] == inst1);
                    e2 = cj.w & kEEEdgeMask;
                }
            }
            warp_stage_pair(hit, make_int2(min(e1, e2), max(e1, e2)), stage, kEEPairStage, cnt,
                            lane, pairs, pcap, counters + kPairs, counters + 2, 64);
        }
    }
    if (cnt) warp_flush_pairs(stage, cnt, lane, pairs, pcap, counters + kPairs, counters + 2, 64);
}

// step 4: distance bound over the step
__global__ void __launch_bounds__(256) k_ee_filter(long long pcap, float th,
                                                   const int2 *__restrict__ edges,
                                                   const int2 *__restrict__ pairs,
                                                   const float4 *__restrict__ x,
                                                   const float4 *__restrict__ p, int2 *cand,
                                                   long long ccap, int *counters) {
    long long n = counters[kPairs];
    if (n > pcap) n = pcap;
    const float reach = 2.f * th * 1.001f + 2e-6f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int2 pr = pairs[i];
        const int2 A = edges[pr.x], B = edges[pr.y];
        v3 X[4] = {ld3(x[A.x]), ld3(x[A.y]), ld3(x[B.x]), ld3(x[B.y])};
        v3 P[4] = {ld3(p[A.x]), ld3(p[A.y]), ld3(p[B.x]), ld3(p[B.y])};
        float d0 = seg_dist(X[0], X[1], X[2], X[3]);
        float d1 = seg_dist(P[0], P[1], P[2], P[3]);
        float U = 0.f;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 2; b < 4; ++b) {
                v3 w = sub3(sub3(P[a], X[a]), sub3(P[b], X[b]));
                U = fmaxf(U, sqrtf(dot3(w, w)));
            }
        if ((d0 + d1 - U) * 0.5f > reach) continue;
        const long long slot = agg_inc(counters + kCand);
        if (slot < ccap)
            cand[slot] = pr;
        else
            atomicOr(counters + 2, 128);
    }
}

// step 5: the edge-edge test
__global__ void __launch_bounds__(128) k_ee_narrow(long long ccap, float th,
                                                   const int2 *__restrict__ edges,
                                                   const int2 *__restrict__ cand,
                                                   const float4 *__restrict__ x,
                                                   const float4 *__restrict__ p, int4 *ids,
                                                   float4 *m0, float4 *tsu, int2 *hpair,
                                                   long long hcap, int *counters) {
    long long n = counters[kCand];
    if (n > ccap) n = ccap;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int2 pr = cand[i];
        const int2 A = edges[pr.x], B = edges[pr.y];
        v3 X[4] = {ld3(x[A.x]), ld3(x[A.y]), ld3(x[B.x]), ld3(x[B.y])};
        v3 P[4] = {ld3(p[A.x]), ld3(p[A.y]), ld3(p[B.x]), ld3(p[B.y])};
        EEHit h;
        if (!ee_test(X, P, th, h)) continue;
        const long long slot = agg_inc(counters + kHits);
        if (slot >= hcap) {
            atomicOr(counters + 2, 256);
            continue;
        }
        ids[slot] = make_int4(A.x, A.y, B.x, B.y);
        m0[slot] = h.m0;
        tsu[slot] = make_float4(h.t, h.s, h.u, 0.f);
        hpair[slot] = pr;
    }
}

// response: corrections of every edge-edge contact into the fixed-point sums
__global__ void __launch_bounds__(128) k_ee_deltas(long long hcap, const int4 *__restrict__ ids,
                                                   const float4 *__restrict__ m0,
                                                   const float4 *__restrict__ p, float th,
                                                   long long *acc, int *acnt,
                                                   const int *counters) {
    long long n = counters[kHits];
    if (n > hcap) n = hcap;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        int4 id = ids[c];
        float4 q0 = p[id.x], q1 = p[id.y], q2 = p[id.z], q3 = p[id.w];
        v3 P[4] = {ld3(q0), ld3(q1), ld3(q2), ld3(q3)};
        float wm[4] = {q0.w, q1.w, q2.w, q3.w};
        v3 dl[4];
        if (!ee_deltas(P, wm, m0[c], th, dl)) continue;
        add_fixed(acc, id.x, dl[0].x, dl[0].y, dl[0].z);
        add_fixed(acc, id.y, dl[1].x, dl[1].y, dl[1].z);
        add_fixed(acc, id.z, dl[2].x, dl[2].y, dl[2].z);
        add_fixed(acc, id.w, dl[3].x, dl[3].y, dl[3].z);
        atomicAdd(acnt + id.x, 1);
        atomicAdd(acnt + id.y, 1);
        atomicAdd(acnt + id.z, 1);
        atomicAdd(acnt + id.w, 1);
    }
}

__global__ void k_ee_batch(int n, const float *x12, const float *p12, const float *th, int *hit,
                           float *tsu, float *m0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 X[4], P[4];
    for (int j = 0; j < 4; ++j) {
        X[j] = mk3(x12[12 * i + 3 * j], x12[12 * i + 3 * j + 1], x12[12 * i + 3 * j + 2]);
        P[j] = mk3(p12[12 * i + 3 * j], p12[12 * i + 3 * j + 1], p12[12 * i + 3 * j + 2]);
    }
    EEHit h;
    h.t = h.s = h.u = 0.f;
    h.m0 = make_float4(0.f, 0.f, 0.f, 0.f);
    hit[i] = ee_test(X, P, th[i], h) ? 1 : 0;
    tsu[3 * i] = h.t;
    tsu[3 * i + 1] = h.s;
    tsu[3 * i + 2] = h.u;
    m0[4 * i] = h.m0.x;
    m0[4 * i + 1] = h.m0.y;
    m0[4 * i + 2] = h.m0.z;
    m0[4 * i + 3] = h.m0.w;
}

int pow2_at_least(long long v, int max_log2) {
    int k = 10;
    while (k < max_log2 && (1LL << k) < v) ++k;
    return k;
}

}  // namespace

// unique edges of the object's triangles (pbd_mesh.cu)
int mesh_unique_edges(int n_points, int n_tris, const int *tris, std::vector<int2> &edges);

int ee_prepare(pbd_colli *c) {
    pbd_object *o = c->obj;
    cudaStream_t s = o->stream;
    if (c->ee_n < 0) {
        // the object's unique edges, once
        std::vector<int4> t4(o->nt);
        if (o->nt)
            PBD_CUDA(cudaMemcpyAsync(t4.data(), o->tri.p, sizeof(int4) * o->nt, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaStreamSynchronize(s));
        std::vector<int> tri(3 * (size_t)o->nt);
        for (int i = 0; i < o->nt; ++i) {
            tri[3 * i] = t4[i].x;
            tri[3 * i + 1] = t4[i].y;
            tri[3 * i + 2] = t4[i].z;
        }
        std::vector<int2> e;
        if (o->nt) PBD_TRY(mesh_unique_edges(o->n, o->nt, tri.data(), e));
        PBD_CHECK(e.size() <= (size_t)kEEEdgeMask, PBD_ERR_ARG,
                  "edge-edge CCD: %zu edges, at most %d", e.size(), kEEEdgeMask);
        c->ee_n = (int)e.size();
        PBD_TRY(c->ee_edges.upload(e.data(), std::max<size_t>(e.size(), 1), s));
    }
    const long long ne = std::max(c->ee_n, 1);
    // entries are indexed with 32-bit ints on the device, and the radix sort
    // counts them in 30 bits
    if (!c->ee_entry_cap)
        c->ee_entry_cap = std::min((1LL << 30) - 1, std::max(1LL << 20, 16 * ne));
    const long long ecap = c->ee_entry_cap;
    PBD_TRY(c->ee_lo.alloc(ne));
    PBD_TRY(c->ee_hi.alloc(ne));
    PBD_TRY(c->ee_cell.alloc(ecap));
    PBD_TRY(c->ee_key.alloc(ecap));
    PBD_TRY(c->ee_key2.alloc(ecap));
    PBD_TRY(c->ee_val.alloc(ecap));
    PBD_TRY(c->ee_val2.alloc(ecap));
    PBD_TRY(c->ee_r0.alloc(ecap));
    PBD_TRY(c->ee_r1.alloc(ecap));
    PBD_TRY(c->ee_r2.alloc(ecap));
    if (o->has_inst) PBD_TRY(c->ee_rinst.alloc(ecap));
    PBD_TRY(c->ee_pairs.alloc(c->cand_cap));
    PBD_TRY(c->ee_cand.alloc(c->cand_cap));
    PBD_TRY(c->ee_ids.alloc(c->contact_cap));
    PBD_TRY(c->ee_m0.alloc(c->contact_cap));
    PBD_TRY(c->ee_tsu.alloc(c->contact_cap));
    PBD_TRY(c->ee_hpair.alloc(c->contact_cap));
    c->ee_log2 = pow2_at_least(2 * ecap, 24);
    PBD_TRY(radix_reserve(c->ee_scr, ecap, (c->ee_log2 + 7) / 8 * 8));
    return PBD_OK;
}

int ee_detect(pbd_colli *c) {
    pbd_object *o = c->obj;
    cudaStream_t s = o->stream;
    if (c->ee_n <= 0) return PBD_OK;
    GridParams g = params_of(c->shs);
    g.hashed = 1;
    g.nb = 1u << c->ee_log2;
    const float th = c->thickness;
    const int *pinst = o->has_inst ? o->point_inst.p : nullptr;
    k_ee_entries<<<grid_for(c->ee_n, 256), 256, 0, s>>>(
        c->ee_n, g, 2.f * th * 1.001f + 4e-6f, c->shs->inst_cell.p, c->shs->n_inst_cell,
        c->ee_edges.p, pinst, o->x.p, o->p.p, c->ee_lo.p,
        c->ee_hi.p, c->ee_cell.p, c->ee_key.p, c->ee_val.p, c->ee_entry_cap, c->counters.p);
    PBD_LAUNCH();
    uint32_t *sk;
    int *sv;
    PBD_TRY(radix_sort<uint32_t>(c->ee_key.p, c->ee_val.p, c->ee_key2.p, c->ee_val2.p,
                                 c->ee_entry_cap, c->counters.p + kEntries,
                                 (c->ee_log2 + 7) / 8 * 8, c->ee_scr, s, &sk, &sv));
    k_ee_gather<<<kEEBlocks, 256, 0, s>>>(c->ee_entry_cap, sv, c->ee_cell.p, c->ee_lo.p,
                                          c->ee_hi.p, c->ee_edges.p, pinst, c->ee_r0.p,
                                          c->ee_r1.p, c->ee_r2.p, pinst ? c->ee_rinst.p : nullptr,
                                          c->counters.p);
    PBD_LAUNCH();
    k_ee_pairs<<<kEEBlocks, 32 * kEEPairWarps, 0, s>>>(
        (int)c->ee_entry_cap, sk, c->ee_r0.p, c->ee_r1.p, c->ee_r2.p, pinst ? c->ee_rinst.p : nullptr,
        c->ee_pairs.p, c->cand_cap, c->counters.p);
    PBD_LAUNCH();
    k_ee_filter<<<kEEBlocks, 256, 0, s>>>(c->cand_cap, th, c->ee_edges.p, c->ee_pairs.p, o->x.p,
                                          o->p.p, c->ee_cand.p, c->cand_cap, c->counters.p);
    PBD_LAUNCH();
    k_ee_narrow<<<kEEBlocks, 128, 0, s>>>(c->cand_cap, th, c->ee_edges.p, c->ee_cand.p, o->x.p,
                                          o->p.p, c->ee_ids.p, c->ee_m0.p, c->ee_tsu.p,
                                          c->ee_hpair.p, c->contact_cap, c->counters.p);
    PBD_LAUNCH();
    return PBD_OK;
}

int ee_deltas_launch(pbd_colli *c) {
    pbd_object *o = c->obj;
    if (c->ee_n <= 0) return PBD_OK;
    k_ee_deltas<<<kEEBlocks, 128, 0, o->stream>>>(c->contact_cap, c->ee_ids.p, c->ee_m0.p, o->p.p,
                                                  c->thickness, c->acc.p, c->acnt.p,
                                                  c->counters.p);
    PBD_LAUNCH();
    return PBD_OK;
}

}  // namespace pbd

using namespace pbd;

extern "C" {

int pbd_ee_test_batch(const float *x12, const float *p12, const float *thickness, int n,
                      int *hit, float *tsu, float *m0) {
    PBD_CHECK(n >= 0 && (n == 0 || (x12 && p12 && thickness && hit && tsu && m0)), PBD_ERR_ARG,
              "bad argument");
    if (n == 0) return PBD_OK;
    cudaStream_t s = nullptr;
    PBD_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{s};
    DBuf<float> dx, dp, dt, dtsu, dm;
    DBuf<int> dh;
    PBD_TRY(dx.upload(x12, 12 * (size_t)n, s));
    PBD_TRY(dp.upload(p12, 12 * (size_t)n, s));
    PBD_TRY(dt.upload(thickness, n, s));
    PBD_TRY(dh.alloc(n));
    PBD_TRY(dtsu.alloc(3 * (size_t)n));
    PBD_TRY(dm.alloc(4 * (size_t)n));
    k_ee_batch<<<grid_for(n, 128), 128, 0, s>>>(n, dx.p, dp.p, dt.p, dh.p, dtsu.p, dm.p);
    PBD_LAUNCH();
    PBD_CUDA(cudaMemcpyAsync(hit, dh.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaMemcpyAsync(tsu, dtsu.p, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaMemcpyAsync(m0, dm.p, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    return PBD_OK;
}

int pbd_colli_set_edge_edge(pbd_colli *c, int on) {
    PBD_CHECK(c, PBD_ERR_ARG, "null collision solver");
    PBD_CHECK(!on || c->obj, PBD_ERR_STATE, "set the target before turning edge-edge CCD on");
    c->ee_on = on ? 1 : 0;
    return PBD_OK;
}

int pbd_colli_ee_edges(pbd_colli *c, int *edges, long long cap, int *n) {
    PBD_CHECK(c && c->obj && n, PBD_ERR_ARG, "null argument");
    PBD_TRY(ee_prepare(c));
    *n = c->ee_n;
    if (!edges) return PBD_OK;
    PBD_CHECK(c->ee_n <= cap, PBD_ERR_OVERFLOW, "%d edges exceed the capacity %lld", c->ee_n, cap);
    if (c->ee_n)
        PBD_CUDA(cudaMemcpyAsync(edges, c->ee_edges.p, sizeof(int2) * c->ee_n,
                                 cudaMemcpyDeviceToHost, c->obj->stream));
    PBD_CUDA(cudaStreamSynchronize(c->obj->stream));
    return PBD_OK;
}

int pbd_colli_get_ee_contacts(pbd_colli *c, int *pairs, int *ids, float *tsu, float *m0,
                              long long cap, long long *n) {
    PBD_CHECK(c && c->obj && n, PBD_ERR_ARG, "null argument");
    *n = 0;
    if (!c->ee_on || !c->counters.p || c->ee_n <= 0) return PBD_OK;
    cudaStream_t s = c->obj->stream;
    int hc[16];
    PBD_CUDA(cudaMemcpyAsync(hc, c->counters.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    PBD_CHECK(!(hc[2] & (32 | 64 | 128 | 256)), PBD_ERR_OVERFLOW,
              "edge-edge buffers overflowed (flags 0x%x): raise the capacities", hc[2]);
    long long h = hc[kHits];
    *n = h;
    if (!pairs && !ids && !tsu && !m0) return PBD_OK;
    PBD_CHECK(h <= cap, PBD_ERR_OVERFLOW, "%lld edge-edge contacts exceed the capacity %lld", h, cap);
    std::vector<int2> hp(h);
    std::vector<int4> hi(h);
    std::vector<float4> ht(h), hm(h);
    if (h) {
        PBD_CUDA(cudaMemcpyAsync(hp.data(), c->ee_hpair.p, sizeof(int2) * h, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaMemcpyAsync(hi.data(), c->ee_ids.p, sizeof(int4) * h, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaMemcpyAsync(ht.data(), c->ee_tsu.p, sizeof(float4) * h, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaMemcpyAsync(hm.data(), c->ee_m0.p, sizeof(float4) * h, cudaMemcpyDeviceToHost, s));
        PBD_CUDA(cudaStreamSynchronize(s));
    }
    // discovery order is not deterministic: sort by (edge a, edge b)
    std::vector<long long> ord(h);
    for (long long i = 0; i < h; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](long long a, long long b) {
        return hp[a].x != hp[b].x ? hp[a].x < hp[b].x : hp[a].y < hp[b].y;
    });
    for (long long k = 0; k < h; ++k) {
        long long i = ord[k];
        if (pairs) {
            pairs[2 * k] = hp[i].x;
            pairs[2 * k + 1] = hp[i].y;
        }
        if (ids) {
            ids[4 * k] = hi[i].x;
            ids[4 * k + 1] = hi[i].y;
            ids[4 * k + 2] = hi[i].z;
            ids[4 * k + 3] = hi[i].w;
        }
        if (tsu) {
            tsu[3 * k] = ht[i].x;
            tsu[3 * k + 1] = ht[i].y;
            tsu[3 * k + 2] = ht[i].z;
        }
        if (m0) {
            m0[4 * k] = hm[i].x;
            m0[4 * k + 1] = hm[i].y;
            m0[4 * k + 2] = hm[i].z;
            m0[4 * k + 3] = hm[i].w;
        }
    }
    return PBD_OK;
}

int pbd_colli_ee_stats(pbd_colli *c, long long *entries, long long *pairs, long long *cand,
                       long long *contacts) {
    PBD_CHECK(c, PBD_ERR_ARG, "null collision solver");
    int hc[16] = {0};
    if (c->counters.p && c->obj) {
        PBD_CUDA(cudaMemcpyAsync(hc, c->counters.p, sizeof(hc), cudaMemcpyDeviceToHost,
                                 c->obj->stream));
        PBD_CUDA(cudaStreamSynchronize(c->obj->stream));
    }
    if (entries) *entries = hc[kEntries];
    if (pairs) *pairs = hc[kPairs];
    if (cand) *cand = hc[kCand];
    if (contacts) *contacts = hc[kHits];
    return PBD_OK;
}

}  // extern "C"

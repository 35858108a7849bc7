// pbd_common.cuh -- shared plumbing of libpbd_gb300: error reporting, device
// buffers, launch helpers, and the object / solver / collision structs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "pbd_c.h"

namespace pbd {

void set_error(const char *fmt, ...);

#define PBD_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            ::pbd::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),    \
                             __FILE__, __LINE__);                                       \
            return e_ == cudaErrorMemoryAllocation ? PBD_ERR_OOM : PBD_ERR_CUDA;        \
        }                                                                               \
    } while (0)

#define PBD_CHECK(cond, code, ...)          \
    do {                                    \
        if (!(cond)) {                      \
            ::pbd::set_error(__VA_ARGS__);  \
            return code;                    \
        }                                   \
    } while (0)

#define PBD_TRY(expr)                \
    do {                             \
        int r_ = (expr);             \
        if (r_ != PBD_OK) return r_; \
    } while (0)

// launch-error check after a kernel launch (no synchronisation)
#define PBD_LAUNCH() PBD_CUDA(cudaGetLastError())

constexpr int kNumSMs = 152;

inline int grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffffLL) g = 0x7fffffff;
    return (int)g;
}

// Owning device allocation; sizes in elements.
template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t count) {
        if (count <= n && p) return PBD_OK;
        release();
        size_t bytes = (count ? count : 1) * sizeof(T);
        cudaError_t e = cudaMalloc((void **)&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            set_error("cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? PBD_ERR_OOM : PBD_ERR_CUDA;
        }
        n = count;
        return PBD_OK;
    }
    int upload(const T *h, size_t count, cudaStream_t s) {
        PBD_TRY(alloc(count));
        if (count) PBD_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
        return PBD_OK;
    }
};

// Owning page-locked host allocation (staging of host transfers); sizes in
// elements.
template <class T>
struct HBuf {
    T *p = nullptr;
    size_t n = 0;
    HBuf() = default;
    HBuf(const HBuf &) = delete;
    HBuf &operator=(const HBuf &) = delete;
    ~HBuf() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t count) {
        if (count <= n && p) return PBD_OK;
        release();
        size_t bytes = (count ? count : 1) * sizeof(T);
        cudaError_t e = cudaHostAlloc((void **)&p, bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            p = nullptr;
            set_error("cudaHostAlloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? PBD_ERR_OOM : PBD_ERR_CUDA;
        }
        n = count;
        return PBD_OK;
    }
};


// ---- stable LSD radix sort (8-bit digits) of (key, int value) pairs --------
// Sorts n elements (n read from d_count when non-null, capped by n_cap),
// `bits` low key bits.  Buffers: keys/vals in and alt (same capacity) and a
// scratch (radix_reserve sizes it; radix_sort does when needed, which a
// caller that captures the sort in a graph must have done before).  Returns
// the pointers holding the result.
struct SortScratch {
    DBuf<unsigned> flags;   // look-back words, pass x tile x digit
    DBuf<int> aux;          // digit counts per pass, tile counters, status
};
int radix_reserve(SortScratch &scr, long long n_cap, int bits);
// nonzero when a look-back wait of some earlier sort ran out (never expected)
int radix_status(const SortScratch &scr, cudaStream_t s, int *status);
template <class K>
int radix_sort(K *keys, int *vals, K *keys_alt, int *vals_alt, long long n_cap,
               const int *d_count, int bits, SortScratch &scr, cudaStream_t s,
               K **keys_out, int **vals_out);
// exclusive scan of n ints (single-block, chunked); out may alias in
int exclusive_scan(const int *in, int *out, long long n, int *d_total, cudaStream_t s);

}  // namespace pbd

// ---- handle structs ------------------------------------------------------
struct pbd_object {
    int n = 0, nt = 0, np = 0, n_idx = 0;
    cudaStream_t stream = nullptr;
    float damping = 1.0f;
    float gravity[3] = {0, 0, 0};
    bool has_inst = false;
    // state (w of x and p = massBuffer value)
    pbd::DBuf<float4> x, p, v;
    pbd::DBuf<float> mass;
    std::vector<float> h_mass;              // host copy of massBuffer
    // host transfers of float3 arrays: page-locked staging each way, the
    // device float3 image that the pack / unpack kernels read and write, and
    // an event marking the end of the last upload out of h_in
    pbd::HBuf<float> h_in, h_out;
    pbd::DBuf<float> d3;
    cudaEvent_t in_done = nullptr;
    // meshTopol triangles: (i0, i1, i2, instance)
    pbd::DBuf<int4> tri;
    pbd::DBuf<int> pt_tri_first, pt_tri_last, pt_tri;  // point -> incident triangles
    pbd::DBuf<int> point_inst, tri_inst;
    // constraint buffers by prim id
    pbd::DBuf<int2> prim_list;
    pbd::DBuf<int> indices, ctype;
    pbd::DBuf<float> rest_length, stiffness, rest_angle;
    pbd::DBuf<float4> rest_pos;
    std::vector<int> h_prim_count;          // points per prim (host copy)
    std::vector<int> h_ctype;
    // Prim2PrimsMap
    pbd::DBuf<int2> adj_sn;
    pbd::DBuf<int> adj;
    long long n_adj = 0;
    // coloring
    pbd::DBuf<int> color, prd_color, flag;
    bool colored = false;
    int n_colors = 0;
    pbd::DBuf<int> sorted_color, sorted_prim;   // SortEdgesColors result
    bool sorted = false;
    std::vector<int> h_worksets;                // 2 per color
    // per-color solver records
    pbd::DBuf<int4> drec;                       // i0, i1, rest, stiffness
    pbd::DBuf<int4> bidx;                       // e0, e1, wA, wB
    pbd::DBuf<float2> bpar;                     // rest angle, stiffness
    pbd::DBuf<float4> arec;                     // rest xyz, point id bits
    std::vector<int> h_dseg, h_bseg, h_aseg;    // n_colors+1 starts each
    pbd::DBuf<int> rec_prim;                    // prim of every record, record order
    int n_rec[3] = {0, 0, 0};                   // distance, bending, anchor records
    // stiffness schedule of the projections (PBD_SCHEDULE_*)
    int sched = 0;
    // staging of pbd_object_set_anchor_targets
    pbd::DBuf<int> anc_prim;
    pbd::DBuf<float> anc_t;
    // resident (cluster) form of the sweep: per-color record starts
    // (dseg | bseg | aseg), the distinct stiffness values of the records (at
    // most 8), the cluster sizes whose shared memory holds every point (bit
    // S set for S in 1, 2, 4, 8, 16) and the size in use (0: the largest
    // that fits)
    int cl_state = 0;           // 0 not built, 1 usable, -1 not applicable
    int cl_fit = 0, cl_S = 0, cl_ntab = 0;
    pbd::DBuf<int> cl_seg;
    pbd::DBuf<float> cl_tab;
    // residual
    double res_den = 0.0;
    double res_den_d = 0.0;                 // distance constraints only
    pbd::DBuf<double> res_part;
    pbd::DBuf<double> res_out;
    pbd::SortScratch scr;
    // host copies of the constraint topology (per-point stencils are built
    // from them on first use)
    std::vector<int> h_prim_list, h_indices;
    std::vector<float> h_rest_length;
    // predicted positions right after advect, and the correction the last
    // solved substep applied to them (p_final - p_after_advect, w = 0)
    pbd::DBuf<float4> p0, dprev;
    // prim id of every bending record (record order)
    pbd::DBuf<int> bend_prim;
    // per prim: wrapped dihedral deviation theta - theta0 (bending prims)
    pbd::DBuf<float> theta;
    // per-point stencil of the warm-start features: other points of the
    // first six incident distance constraints, prim ids of the first four
    // incident bending constraints (both by prim id, -1 = none), their rest
    // lengths, the mean incident rest length and the inverse-mass feature
    pbd::DBuf<int4> fnb_a, fnb_b;           // (n0..n3), (n4, n5, h0, h1)
    pbd::DBuf<int2> fnb_c;                  // (h2, h3)
    pbd::DBuf<float4> frest_a, frest_b;     // (r0..r3), (r4, r5, lbar, wrel)
    int n_free = 0;                         // points with nonzero inverse mass
    bool feat_built = false;
    // color phases launched with programmatic dependent launch
    bool pdl = true;
    // threads per block of the per-color launches (set by the autotuner)
    int gs_block = 256;
};

struct pbd_shs {
    pbd_object *obj = nullptr;
    bool hashed = false;
    int log2_table = 0;
    float center[3] = {0, 0, 0};
    int size[3] = {1, 1, 1};
    float cell[3] = {1, 1, 1};
    float start[3] = {0, 0, 0};
    bool initialized = false;
    int n_buckets = 0;
    int key_bits = 0;
    // per triangle (by id)
    pbd::DBuf<int4> tcell;       // cell xyz, valid
    pbd::DBuf<float4> tlo, thi;  // swept AABB of the triangle
    pbd::DBuf<uint32_t> key, key_alt;
    pbd::DBuf<int> id, id_alt;
    uint32_t *skey = nullptr;    // sorted result pointers (into key/key_alt)
    int *sid = nullptr;
    // sorted entries, 3 float4 each (48 contiguous bytes): cell xyz and
    // triangle id as int bits; the swept AABB's low corner; its high corner
    pbd::DBuf<float4> etab;
    // buckets, 2 float4 each (one 32-byte sector): [start, end) in sorted
    // order as int bits, then the union of its triangles' swept AABBs
    // (start, end, lo.x, lo.y), (lo.z, hi.x, hi.y, hi.z)
    pbd::DBuf<float4> btab;
    pbd::DBuf<int> n_valid;
    pbd::SortScratch scr;
    // hashed grid only: a cell size per instance (xyz, w unused), so each
    // batched cloth gets the cells it would get alone; 0 instances = one cell
    pbd::DBuf<float4> inst_cell;
    int n_inst_cell = 0;
    // per point, kPointSlots slots: the cell (xyz) and id (w) of its first
    // incident triangles (the point -> triangle lists' order), rewritten by
    // each update, so the candidate search finds a point's incident cells
    // in one load; tri_slot: per triangle and vertex, that slot (-1 when the
    // vertex has more incident triangles than slots)
    pbd::DBuf<int4> pt_cell;
    pbd::DBuf<int> tri_slot;
};

struct pbd_colli {
    pbd_object *obj = nullptr;
    pbd_shs *shs = nullptr;
    float thickness = 0.0f;
    int iterations = 1;
    int response = PBD_RESPONSE_REFERENCE;
    int vf_test = PBD_VFTEST_EXTENDED;  // narrowphase test of the detection
    long long cand_cap = 1 << 22;
    long long contact_cap = 1 << 20;
    long long task_cap = 1 << 22;
    // candidates (point, triangle)
    pbd::DBuf<int2> pairs;      // AABB-overlapping (point, triangle)
    pbd::DBuf<int2> cand;
    pbd::DBuf<int> counters;    // [0] candidates, [1] contacts, [2] overflow flags, [3] hard
                                // candidates (cubic roots needed), [4] AABB pairs
    pbd::DBuf<int> hard;        // candidate indices that need the cubic's roots
    int sized_n = -1;           // point count the per-point buffers were sized for
    // contacts, in the order the narrow phase found them
    pbd::DBuf<int4> cids;               // i0..i3
    pbd::DBuf<int> cface;
    pbd::DBuf<float4> ctn;              // t, n
    pbd::DBuf<double4> cw;
    // response: per-point 2^-32 m fixed-point sums and counts (kept zero
    // between passes)
    pbd::DBuf<long long> acc;
    pbd::DBuf<int> acnt;
    // the older response's per-point resolve counters (kept across calls)
    // and the sort that puts its contacts in reported order
    pbd::DBuf<int> resolve_times;
    pbd::DBuf<unsigned long long> old_key, old_key2;
    pbd::DBuf<int> old_val, old_val2;
    pbd::SortScratch old_scr;
    // edge-edge CCD (off unless enabled): the object's unique edges (built
    // on first use; -1 = not yet), their grown swept boxes, the edge-cell
    // entries of the edge hash and their sort buffers, the edge pairs,
    // candidates and contacts (ids a0 a1 b0 b1, side m0 + sign, t s u, the
    // edge pair).  counters[8..11]: entries, pairs, candidates, contacts.
    int ee_on = 0;
    int ee_n = -1;
    int ee_log2 = 0;
    long long ee_entry_cap = 0;
    pbd::DBuf<int2> ee_edges;
    pbd::DBuf<float4> ee_lo, ee_hi;
    pbd::DBuf<int4> ee_cell;
    pbd::DBuf<uint32_t> ee_key, ee_key2;
    pbd::DBuf<int> ee_val, ee_val2;
    pbd::DBuf<int4> ee_r0;               // sorted entry records (cell, edge)
    pbd::DBuf<float4> ee_r1, ee_r2;      // (box lo, end 0), (box hi, end 1)
    pbd::DBuf<int> ee_rinst;             // instance of a sorted entry (batches)
    pbd::DBuf<int2> ee_pairs, ee_cand, ee_hpair;
    pbd::DBuf<int4> ee_ids;
    pbd::DBuf<float4> ee_m0, ee_tsu;
    pbd::SortScratch ee_scr;
    // Detection overlapped with the sweep that follows it (the substeps of
    // pbd_solver_step / project_constraint_with_colli): a copy of the
    // predicted positions at the iteration's start, a low-priority side
    // stream the detection runs on, and the fork / join events.  The
    // response after the sweep waits for the join, so the contacts are the
    // ones a detection before the sweep finds.
    int overlap = 1;
    pbd::DBuf<float4> psnap;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    ~pbd_colli() {
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
    }
};

// Device state of the solve-to-residual loop (one per solver).
namespace pbd {
constexpr int kMaxChunk = 32;
struct LoopState {
    double r;             // residual after the last check
    double r_prev;        // residual at the check before
    double r0;            // warm start guard: residual of the advected positions
    double r1;            // warm start guard: residual after the prediction
    int sweeps;           // sweeps of the current substep's solve
    int revert;           // the current substep's prediction was rejected
    int cont;             // loop condition (also set on the graph's handle)
    int pred_used;        // the current substep starts from an accepted prediction
    long long substeps, total_sweeps, reached, reverts;
    float expk[kMaxChunk];  // 1/(sweep+1) of the next chunk's sweeps
};
}  // namespace pbd

struct pbd_warmstart;

struct pbd_solver {
    pbd_object *obj = nullptr;
    pbd_warmstart *ws = nullptr;
    int min_sweeps = 0;   // sweeps that always follow an accepted prediction
    pbd::DBuf<pbd::LoopState> loop;
    // cached graph of pbd_solver_step_to_residual
    cudaGraphExec_t rexec = nullptr;
    float r_dt = 0;
    int r_sub = 0, r_max = 0, r_chunk = 0, r_sig = 0;
    double r_target = 0;
    pbd_colli *r_colli = nullptr;
    long long r_kernels[2] = {0, 0};     // kernels outside / inside one WHILE body
    int gs_path = 0;  // PBD_GS_AUTO / PER_COLOR / CLUSTER
    int sphere_on = 0;
    float sphere_c[3] = {0, 0, 0};
    float sphere_r = 1.0f;
    int ground_on = 0;
    float ground_h = 0.0f;
    // one analytic sphere per instance (cx, cy, cz, r), indexed by point_inst
    pbd::DBuf<float4> inst_spheres;
    int n_inst_spheres = 0;
    // cached graph of pbd_solver_step
    cudaGraphExec_t gexec = nullptr;
    float g_dt = 0;
    int g_sub = 0, g_it = 0;
    pbd_colli *g_colli = nullptr;
    int g_sig = 0;
    long long g_kernels = 0;
};

// Learned warm start: per-point MLP 16 -> 64 -> 64 -> 3 (SiLU), BF16
// operands on the tensor cores, FP32 accumulate; FP32 master parameters
// with Adam moments.
namespace pbd {
constexpr int kWsIn = 16, kWsHid = 64, kWsOut = 3;
// packed FP32 parameters: W1[64][16] (column 15 multiplies the constant
// feature, i.e. it is the first layer's bias), W2[64][64], b2[64],
// W3[3][64], b3[3]
constexpr int kWsOffW1 = 0;
constexpr int kWsOffW2 = kWsOffW1 + kWsHid * kWsIn;
constexpr int kWsOffB2 = kWsOffW2 + kWsHid * kWsHid;
constexpr int kWsOffW3 = kWsOffB2 + kWsHid;
constexpr int kWsOffB3 = kWsOffW3 + kWsOut * kWsHid;
constexpr int kWsParams = kWsOffB3 + kWsOut;
// BF16 operand tiles in the tensor cores' K-major core-matrix layout
// (element offsets into one buffer)
constexpr int kWtW1 = 0;                     // B [64 x 16]
constexpr int kWtW2 = kWtW1 + 64 * 16;       // B [64 x 64]
constexpr int kWtW3 = kWtW2 + 64 * 64;       // B [16 x 64], rows 3..15 zero
constexpr int kWtW3T = kWtW3 + 16 * 64;      // B [64 x 16], columns 3..15 zero
constexpr int kWtW2T = kWtW3T + 64 * 16;     // B [64 x 64]
constexpr int kWtTotal = kWtW2T + 64 * 64;
}  // namespace pbd

struct pbd_warmstart {
    cudaStream_t own = nullptr;          // for calls not tied to an object
    pbd::DBuf<float> params, m, v, grad;
    pbd::DBuf<unsigned short> wtiles;    // BF16 tiles (kWtTotal)
    pbd::DBuf<float> bias;               // b2[64], b3[16] (3..15 zero)
    pbd::DBuf<double> loss;              // [0] sum of squared errors, [1] count
    pbd::DBuf<unsigned short> feat;      // recorded features, BF16 [n x 16]
    pbd::DBuf<float4> tgt;               // training targets (xyz, mask)
    pbd::DBuf<float> scale;              // 16 input scales + output scale
    long long feat_cap = 0;
    long long adam_t = 0;
    pbd::DBuf<int> err;                  // device error flag (tensor-core waits)
};

// internal entry points shared between translation units
namespace pbd {
int ws_prepare(pbd_warmstart *w, pbd_object *o);
int ws_eval_hinges(pbd_object *o, const float4 *pos);
int ws_infer(pbd_warmstart *w, pbd_object *o);
int ws_record(pbd_warmstart *w, pbd_object *o);
int ws_train_on(pbd_warmstart *w, pbd_object *o, float lr, double *loss);
int build_feature_stencil(pbd_object *o);
int launch_advect(pbd_object *o, float dt);
int launch_advect_p0(pbd_object *o, float dt);
int launch_integrate(pbd_object *o, float dt);
int launch_sweeps(pbd_solver *s, int it0, int it1, bool obstacles_inside);
// one sweep whose stiffness exponent 1/(iter+1) is read from device memory
// (the solve-to-residual loop)
int launch_sweep_dev(pbd_solver *s, const float *expk_dev, bool obstacles_inside);
int prepare_gs_path(pbd_solver *s);
// residual partial sums of pos over the distance and/or bending records
// into o->res_part (kResidualParts doubles)
constexpr int kResidualParts = 4 * kNumSMs;
int launch_residual_parts(pbd_object *o, bool dist, bool bend, const float4 *pos);
int launch_obstacles(pbd_solver *s);
int ccd_detect(pbd_colli *c);
// the detection of one iteration started on the side stream from a copy of
// the predicted positions (overlapping the sweep the caller launches next);
// returns PBD_OK with *forked = false when it ran on the object's stream
// instead (overlap off, edge-edge CCD on, or buffers not yet sized)
int ccd_detect_fork(pbd_colli *c, bool *forked);
// the object's stream waits for a forked detection
int ccd_join(pbd_colli *c);
// sizes the collision solver's buffers for its target (outside captures)
int ccd_prepare_all(pbd_colli *c);
// copies positions src into the detection snapshot (c->psnap) on the
// object's stream; ccd_detect_snapshot detects from that snapshot (the
// vertex-face pass; edge-edge CCD, when on, reads the object's positions)
int ccd_snapshot(pbd_colli *c, const float4 *src);
int ccd_detect_snapshot(pbd_colli *c);
int ccd_resolve(pbd_colli *c, int passes);
// priority of the color-phase launches (the greatest the device offers),
// so pending sweep blocks are scheduled before an overlapped detection's
int gs_priority();
// edge-edge CCD (pbd_edge.cu): buffers and edge list, one detection pass,
// the response's corrections into the shared fixed-point sums
int ee_prepare(pbd_colli *c);
int ee_detect(pbd_colli *c);
int ee_deltas_launch(pbd_colli *c);
int shs_update(pbd_shs *h);
}  // namespace pbd

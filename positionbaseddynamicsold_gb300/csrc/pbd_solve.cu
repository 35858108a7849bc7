// pbd_solve.cu -- substeps solved to a residual target instead of a fixed
// iteration count (no counterpart in the reference, whose substeps always
// run `iterations` sweeps: P/PBD_cuda.cu:1308-1435).
//
// Residual: the relative stretch residual sqrt(sum C_d^2) / sqrt(sum l_d^2)
// over the distance constraints (C_d = |p_a - p_b| - l_d), in FP64.  The
// bending constraints are soft (s < 1) and, under the reference's
// iteration-indexed stiffness k = 1 - (1 - s)^(1/(i+1)), have no state of
// zero residual once pins, contacts or gravity oppose them, so they do not
// enter the stopping test.
//
// A substep is: advect; [warm start]; sweeps in chunks of `chunk` until the
// residual is at or below the target or `max_sweeps` would be exceeded;
// [a last CCD detection + response]; record the correction; integrate.  A
// chunk's detection reads the positions its chunk starts from, the first
// one the advected positions (taken before the warm start).
// Sweep i uses the reference's exponent 1/(i+1).  With collisions each chunk
// starts with a CCD detection (the reference detects every 10th iteration,
// P/PBD_cuda.cu:1139-1145: chunk = 10 keeps that cadence) and every sweep is
// followed by the contact response and the analytic obstacles.
//
// Warm start: the advected positions' residual r0 is taken, the network's
// correction is added, and the residual r1 of the result is taken; when
// r1 > r0 the prediction is discarded (positions reset to the advected
// ones) and the substep is solved by the plain sweeps alone.
//
// The loop runs on the device: each check (k_loop_ctl) sets the condition
// of a CUDA graph WHILE node whose body is one chunk, so a captured substep
// needs no host round trip.  The eager form runs the same kernels and reads
// the condition on the host after every chunk.
#include <cmath>
#include <cstring>
#include <vector>

#include "pbd_common.cuh"

namespace pbd {

enum LoopMode { kStartPlain = 0, kGuardR0 = 1, kGuardR1 = 2, kCheck = 3 };

__global__ void k_loop_ctl(int mode, const double *__restrict__ part, int nparts, double sqrt_den,
                           LoopState *__restrict__ L, cudaGraphConditionalHandle h, double target,
                           int max_sweeps, int chunk, int min_sweeps) {
    double s = 0.0;
    for (int k = threadIdx.x; k < nparts; k += 32) s += part[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x != 0) return;
    double r = sqrt_den > 0.0 ? sqrt(s) / sqrt_den : 0.0;
    if (mode == kGuardR0) {
        L->r0 = r;
        return;
    }
    if (mode == kCheck) {
        L->sweeps += chunk;
        L->r_prev = L->r;
        L->r = r;
    } else {
        L->sweeps = 0;
        L->r_prev = INFINITY;
        L->revert = 0;
        if (mode == kGuardR1) {
            L->r1 = r;
            int rev = r > L->r0;
            L->revert = rev;
            L->reverts += rev;
            r = rev ? L->r0 : r;
        }
        L->r = r;
    }
    // an accepted prediction is followed by at least min_sweeps sweeps
    if (mode != kCheck) L->pred_used = mode == kGuardR1 && !L->revert;
    const int need = L->pred_used ? min_sweeps : 0;
    int cont = (L->r > target || L->sweeps < need) && L->sweeps + chunk <= max_sweeps;
    for (int j = 0; j < chunk; ++j) L->expk[j] = (float)(1.0 / (double)(L->sweeps + j + 1));
    if (!cont) {
        L->substeps += 1;
        L->total_sweeps += L->sweeps;
        L->reached += L->r <= target;
    }
    L->cont = cont;
    if (h) cudaGraphSetConditional(h, (unsigned)cont);
}

// reset the positions to the advected ones when the guard rejected the
// prediction
__global__ void __launch_bounds__(256) k_revert(int n, const LoopState *__restrict__ L,
                                                const float4 *__restrict__ p0,
                                                float4 *__restrict__ p) {
    if (!L->revert) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = p0[i];
}

__global__ void __launch_bounds__(256) k_store_correction(int n, const float4 *__restrict__ p,
                                                          const float4 *__restrict__ p0,
                                                          float4 *__restrict__ dprev) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 P = p[i], Q = p0[i];
    dprev[i] = make_float4(P.x - Q.x, P.y - Q.y, P.z - Q.z, 0.f);
}

struct ResArgs {
    double target;
    int max_sweeps, chunk, min_sweeps;
};

static int loop_ctl(pbd_solver *s, int mode, cudaGraphConditionalHandle h, const ResArgs &a) {
    pbd_object *o = s->obj;
    PBD_TRY(launch_residual_parts(o, true, false, o->p.p));
    k_loop_ctl<<<1, 32, 0, o->stream>>>(mode, o->res_part.p, kResidualParts, sqrt(o->res_den_d),
                                        s->loop.p, h, a.target, a.max_sweeps, a.chunk,
                                        a.min_sweeps);
    PBD_LAUNCH();
    return PBD_OK;
}

// one chunk of sweeps followed by the residual check.  With collisions the
// chunk starts with a detection from the snapshot of the positions the
// chunk starts from (the prologue takes the first one from the advected
// positions, before any warm start; each chunk takes the next one), so a
// warm-started and a plain solve of one state detect the same contacts
// first.
static int record_chunk(pbd_solver *s, pbd_colli *c, cudaGraphConditionalHandle h,
                        const ResArgs &a) {
    if (c) PBD_TRY(ccd_detect_snapshot(c));
    for (int j = 0; j < a.chunk; ++j) {
        PBD_TRY(launch_sweep_dev(s, &s->loop.p->expk[j], c == nullptr));
        if (c) {
            PBD_TRY(ccd_resolve(c, c->iterations));
            PBD_TRY(launch_obstacles(s));
        }
    }
    PBD_TRY(loop_ctl(s, kCheck, h, a));
    if (c) PBD_TRY(ccd_snapshot(c, s->obj->p.p));
    return PBD_OK;
}

// warm start of the advected positions o->p0 (= o->p): prediction, guard,
// loop start
static int warm_start(pbd_solver *s, cudaGraphConditionalHandle h, const ResArgs &a) {
    pbd_object *o = s->obj;
    PBD_TRY(ws_eval_hinges(o, o->p0.p));
    PBD_TRY(launch_residual_parts(o, true, false, o->p0.p));
    k_loop_ctl<<<1, 32, 0, o->stream>>>(kGuardR0, o->res_part.p, kResidualParts,
                                        sqrt(o->res_den_d), s->loop.p, h, a.target,
                                        a.max_sweeps, a.chunk, a.min_sweeps);
    PBD_LAUNCH();
    PBD_TRY(ws_infer(s->ws, o));
    PBD_TRY(loop_ctl(s, kGuardR1, h, a));
    k_revert<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, s->loop.p, o->p0.p, o->p.p);
    PBD_LAUNCH();
    return PBD_OK;
}

// advect, warm start or plain start; the loop follows (graph or host)
static int record_prologue(pbd_solver *s, float dt, pbd_colli *c, cudaGraphConditionalHandle h,
                           const ResArgs &a) {
    pbd_object *o = s->obj;
    PBD_TRY(launch_advect_p0(o, dt));
    if (c) PBD_TRY(ccd_snapshot(c, o->p.p));
    if (s->ws) return warm_start(s, h, a);
    return loop_ctl(s, kStartPlain, h, a);
}

static int final_contacts(pbd_solver *s, pbd_colli *c);

static int record_epilogue(pbd_solver *s, float dt, pbd_colli *c) {
    pbd_object *o = s->obj;
    PBD_TRY(final_contacts(s, c));
    k_store_correction<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, o->p.p, o->p0.p,
                                                                   o->dprev.p);
    PBD_LAUNCH();
    return launch_integrate(o, dt);
}

// the loop driven from the host: a chunk while the device says so
static int eager_loop(pbd_solver *s, pbd_colli *c, const ResArgs &a) {
    pbd_object *o = s->obj;
    for (;;) {
        int cont = 0;
        PBD_CUDA(cudaMemcpyAsync(&cont, &s->loop.p->cont, sizeof(int), cudaMemcpyDeviceToHost,
                                 o->stream));
        PBD_CUDA(cudaStreamSynchronize(o->stream));
        if (!cont) break;
        PBD_TRY(record_chunk(s, c, 0, a));
    }
    return PBD_OK;
}

static int eager_substep(pbd_solver *s, float dt, pbd_colli *c, const ResArgs &a) {
    PBD_TRY(record_prologue(s, dt, c, 0, a));
    PBD_TRY(eager_loop(s, c, a));
    return record_epilogue(s, dt, c);
}

static int final_contacts(pbd_solver *s, pbd_colli *c) {
    if (!c) return PBD_OK;
    PBD_TRY(ccd_detect(c));
    PBD_TRY(ccd_resolve(c, c->iterations));
    return launch_obstacles(s);
}

// Captures `substeps` substeps on o->stream (which is capturing); the body of
// each WHILE node is captured on `body`.
static int capture_substeps(pbd_solver *s, float dt, int substeps, pbd_colli *c, const ResArgs &a,
                            cudaStream_t body, std::vector<cudaGraph_t> &bodies) {
    pbd_object *o = s->obj;
    cudaStream_t st = o->stream;
    for (int k = 0; k < substeps; ++k) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t g = nullptr;
        PBD_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
        cudaGraphConditionalHandle h;
        PBD_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
        PBD_TRY(record_prologue(s, dt, c, h, a));
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        PBD_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        PBD_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
        cudaGraph_t bg = cp.conditional.phGraph_out[0];
        bodies.push_back(bg);
        PBD_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                                     cudaStreamSetCaptureDependencies));
        PBD_CUDA(cudaStreamBeginCaptureToGraph(body, bg, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeRelaxed));
        o->stream = body;
        int r = record_chunk(s, c, h, a);
        o->stream = st;
        cudaGraph_t tmp = nullptr;
        cudaError_t e = cudaStreamEndCapture(body, &tmp);
        PBD_TRY(r);
        PBD_CUDA(e);
        PBD_TRY(record_epilogue(s, dt, c));
    }
    return PBD_OK;
}

static int build_graph(pbd_solver *s, float dt, int substeps, pbd_colli *c, const ResArgs &a,
                       cudaGraphExec_t *exec, long long *n_kernels) {
    pbd_object *o = s->obj;
    cudaStream_t st = o->stream;
    cudaStream_t body = nullptr;
    PBD_CUDA(cudaStreamCreateWithFlags(&body, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    int r = PBD_OK;
    std::vector<cudaGraph_t> todo;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        r = capture_substeps(s, dt, substeps, c, a, body, todo);
        e = cudaStreamEndCapture(st, &g);
    }
    cudaStreamDestroy(body);
    if (r != PBD_OK) {
        if (e == cudaSuccess && g) cudaGraphDestroy(g);
        return r;
    }
    PBD_CUDA(e);
    // kernel nodes per pass (the WHILE bodies counted once)
    long long nk = 0, nbody = 0;
    todo.push_back(g);
    for (cudaGraph_t cur : todo) {
        size_t nn = 0;
        cudaGraphGetNodes(cur, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(cur, nodes.data(), &nn);
        for (size_t i = 0; i < nn; ++i) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
                ++(cur == g ? nk : nbody);
        }
    }
    n_kernels[0] = nk;
    n_kernels[1] = todo.size() > 1 ? nbody / (long long)(todo.size() - 1) : 0;
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    PBD_CUDA(e);
    return PBD_OK;
}

static int ensure_ready(pbd_solver *s, pbd_colli *c) {
    pbd_object *o = s->obj;
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "constraints are not color-sorted");
    PBD_CHECK(!c || c->obj == o, PBD_ERR_ARG, "collision solver targets another object");
    if (!s->loop.p) {
        PBD_TRY(s->loop.alloc(1));
        PBD_CUDA(cudaMemsetAsync(s->loop.p, 0, sizeof(LoopState), o->stream));
    }
    PBD_TRY(build_feature_stencil(o));  // p0 / dprev buffers and stencils
    if (c) PBD_TRY(ccd_prepare_all(c));   // the detection snapshot among them
    if (s->ws) PBD_TRY(ws_prepare(s->ws, o));
    PBD_TRY(prepare_gs_path(s));
    return PBD_OK;
}

}  // namespace pbd

using namespace pbd;

extern "C" {

int pbd_solver_set_warmstart(pbd_solver *s, pbd_warmstart *w, int min_sweeps) {
    PBD_CHECK(s && min_sweeps >= 0, PBD_ERR_ARG, "bad argument");
    s->ws = w;
    s->min_sweeps = min_sweeps;
    if (s->rexec) cudaGraphExecDestroy(s->rexec);
    s->rexec = nullptr;
    return PBD_OK;
}

int pbd_solver_step_to_residual(pbd_solver *s, float dt, int substeps, pbd_colli *c,
                                double target, int max_sweeps, int chunk, int use_graph) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(substeps >= 0 && chunk >= 1 && chunk <= kMaxChunk && max_sweeps >= 0, PBD_ERR_ARG,
              "need substeps >= 0, 1 <= chunk <= %d, max_sweeps >= 0", kMaxChunk);
    PBD_TRY(ensure_ready(s, c));
    ResArgs a{target, max_sweeps, chunk, s->min_sweeps};
    pbd_object *o = s->obj;
    if (!use_graph) {
        for (int k = 0; k < substeps; ++k) PBD_TRY(eager_substep(s, dt, c, a));
        return PBD_OK;
    }
    int sig = s->sphere_on * 3 + s->ground_on * 7 +
              (c ? c->response * 11 + c->iterations * 13 + c->ee_on * 101 : 0) +
              (s->n_inst_spheres > 0) * 17 +
              (s->ws != nullptr) * 19 + s->min_sweeps * 29 + (o->pdl ? 23 : 0) +
              s->gs_path * 1009 + o->sched * 7919;
    if (s->rexec && (s->r_dt != dt || s->r_sub != substeps || s->r_colli != c ||
                     s->r_sig != sig || s->r_target != target || s->r_max != max_sweeps ||
                     s->r_chunk != chunk)) {
        cudaGraphExecDestroy(s->rexec);
        s->rexec = nullptr;
    }
    if (!s->rexec) {
        if (c) PBD_TRY(ccd_detect(c));  // sizes every buffer before capture
        PBD_CUDA(cudaStreamSynchronize(o->stream));
        int r = build_graph(s, dt, substeps, c, a, &s->rexec, s->r_kernels);
        if (r != PBD_OK && o->pdl) {
            // retry with plain stream ordering between the color phases
            cudaGetLastError();
            o->pdl = false;
            r = build_graph(s, dt, substeps, c, a, &s->rexec, s->r_kernels);
        }
        PBD_TRY(r);
        s->r_dt = dt;
        s->r_sub = substeps;
        s->r_colli = c;
        s->r_sig = o->pdl ? sig : sig - 23;
        s->r_target = target;
        s->r_max = max_sweeps;
        s->r_chunk = chunk;
    }
    PBD_CUDA(cudaGraphLaunch(s->rexec, o->stream));
    return PBD_OK;
}

int pbd_solver_project_to_residual(pbd_solver *s, pbd_colli *c, double target, int max_sweeps,
                                  int chunk, int *sweeps, double *residual) {
    PBD_CHECK(s && s->obj, PBD_ERR_STATE, "solver has no target");
    PBD_CHECK(chunk >= 1 && chunk <= kMaxChunk && max_sweeps >= 0, PBD_ERR_ARG,
              "need 1 <= chunk <= %d, max_sweeps >= 0", kMaxChunk);
    PBD_TRY(ensure_ready(s, c));
    pbd_object *o = s->obj;
    ResArgs a{target, max_sweeps, chunk, s->min_sweeps};
    PBD_CUDA(cudaMemcpyAsync(o->p0.p, o->p.p, sizeof(float4) * o->n, cudaMemcpyDeviceToDevice,
                             o->stream));
    if (c) PBD_TRY(ccd_snapshot(c, o->p.p));
    PBD_TRY(loop_ctl(s, kStartPlain, 0, a));
    for (;;) {
        int cont = 0;
        PBD_CUDA(cudaMemcpyAsync(&cont, &s->loop.p->cont, sizeof(int), cudaMemcpyDeviceToHost,
                                 o->stream));
        PBD_CUDA(cudaStreamSynchronize(o->stream));
        if (!cont) break;
        PBD_TRY(record_chunk(s, c, 0, a));
    }
    if (c) {
        PBD_TRY(ccd_detect(c));
        PBD_TRY(ccd_resolve(c, c->iterations));
        PBD_TRY(launch_obstacles(s));
    }
    k_store_correction<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, o->p.p, o->p0.p,
                                                                   o->dprev.p);
    PBD_LAUNCH();
    LoopState L;
    PBD_CUDA(cudaMemcpyAsync(&L, s->loop.p, sizeof(L), cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    if (sweeps) *sweeps = L.sweeps;
    if (residual) *residual = L.r;
    return PBD_OK;
}

int pbd_solver_train_substep(pbd_solver *s, pbd_warmstart *w, float dt, pbd_colli *c,
                             double target, int max_sweeps, int chunk, float lr, int on_policy,
                             double *loss) {
    PBD_CHECK(s && s->obj && w, PBD_ERR_ARG, "null argument");
    PBD_CHECK(chunk >= 1 && chunk <= kMaxChunk && max_sweeps >= 0, PBD_ERR_ARG,
              "need 1 <= chunk <= %d, max_sweeps >= 0", kMaxChunk);
    PBD_TRY(ensure_ready(s, c));
    PBD_TRY(ws_prepare(w, s->obj));
    pbd_object *o = s->obj;
    ResArgs a{target, max_sweeps, chunk, s->min_sweeps};
    // the plain solve of the advected state gives the target
    PBD_TRY(launch_advect_p0(o, dt));
    if (c) PBD_TRY(ccd_snapshot(c, o->p.p));
    PBD_TRY(ws_record(w, o));
    PBD_TRY(loop_ctl(s, kStartPlain, 0, a));
    PBD_TRY(eager_loop(s, c, a));
    PBD_TRY(final_contacts(s, c));
    PBD_TRY(ws_train_on(w, o, lr, loss));
    if (on_policy) {
        // the trajectory continues from the warm-started solve of the same state
        PBD_CUDA(cudaMemcpyAsync(o->p.p, o->p0.p, sizeof(float4) * o->n, cudaMemcpyDeviceToDevice,
                                 o->stream));
        if (c) PBD_TRY(ccd_snapshot(c, o->p.p));
        pbd_warmstart *keep = s->ws;
        s->ws = w;
        int r = warm_start(s, 0, a);
        s->ws = keep;
        PBD_TRY(r);
        PBD_TRY(eager_loop(s, c, a));
        PBD_TRY(final_contacts(s, c));
    }
    k_store_correction<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, o->p.p, o->p0.p,
                                                                   o->dprev.p);
    PBD_LAUNCH();
    PBD_TRY(launch_integrate(o, dt));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    return PBD_OK;
}

int pbd_solver_solve_stats(pbd_solver *s, pbd_solve_stats *st, int reset) {
    PBD_CHECK(s && s->obj && st, PBD_ERR_ARG, "null argument");
    memset(st, 0, sizeof(*st));
    if (!s->loop.p) return PBD_OK;
    LoopState L;
    cudaStream_t q = s->obj->stream;
    PBD_CUDA(cudaMemcpyAsync(&L, s->loop.p, sizeof(L), cudaMemcpyDeviceToHost, q));
    PBD_CUDA(cudaStreamSynchronize(q));
    st->substeps = L.substeps;
    st->sweeps = L.total_sweeps;
    st->reached = L.reached;
    st->reverts = L.reverts;
    st->last_residual = L.r;
    st->last_sweeps = L.sweeps;
    st->last_r0 = L.r0;
    st->last_r1 = L.r1;
    if (reset) {
        L.substeps = L.total_sweeps = L.reached = L.reverts = 0;
        PBD_CUDA(cudaMemcpyAsync(s->loop.p, &L, sizeof(L), cudaMemcpyHostToDevice, q));
        PBD_CUDA(cudaStreamSynchronize(q));
    }
    return PBD_OK;
}

int pbd_solver_residual_graph_kernels(pbd_solver *s, long long *n_outer, long long *n_body) {
    PBD_CHECK(s && n_outer && n_body, PBD_ERR_ARG, "null argument");
    *n_outer = s->rexec ? s->r_kernels[0] : 0;
    *n_body = s->rexec ? s->r_kernels[1] : 0;
    return PBD_OK;
}

int pbd_constraints_residual_stretch(pbd_object *o, double *res) {
    PBD_CHECK(o && res, PBD_ERR_ARG, "null argument");
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "SortEdgesColors has not run");
    PBD_TRY(launch_residual_parts(o, true, false, o->p.p));
    std::vector<double> h(kResidualParts);
    PBD_CUDA(cudaMemcpyAsync(h.data(), o->res_part.p, sizeof(double) * kResidualParts,
                             cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    double num = 0.0;
    for (double v : h) num += v;
    *res = o->res_den_d > 0.0 ? sqrt(num) / sqrt(o->res_den_d) : 0.0;
    return PBD_OK;
}

}  // extern "C"

// pbd_noalloc.cu -- the relative constraint residual without device
// allocation.
//
// pbd_constraints_residual (pbd_object.cu) reduces through per-block partial
// sums held in buffers the object allocated.  Some callers own all device
// memory themselves and cannot let a library call cudaMalloc: a host engine
// that carves every buffer out of one arena it reserved at start-up, code
// running between the allocation phase and a CUDA graph capture, or a process
// that runs under a hard device-memory budget.  For them this file computes
// the same residual from device buffers the caller passes in, and keeps its
// partial sums in a fixed file-scope __device__ array instead of allocating.
//
// Every GPU that loads the library holds that array (1 MiB) until the process
// exits.  Calls share it: two calls whose kernels overlap on the GPU (on
// different streams, or from different host threads) race on it and give
// wrong results; serialise them.  Each call writes every slot it then reads,
// except the out-of-range flag, which it clears first.
#include <mutex>

#include "pbd_common.cuh"

namespace {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = 1 << 16;

// [2*b] numerator, [2*b+1] denominator of block b
static __device__ __align__(256) double g_residual_scratch[2 * kMaxBlocks + 32];

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// one thread per constraint: distance first, then bending
__global__ void __launch_bounds__(kBlock) k_residual_parts(
    const float4 *__restrict__ p, int n_points, const int2 *__restrict__ didx,
    const float *__restrict__ rest, int nd, const int4 *__restrict__ bidx,
    const float *__restrict__ rest_angle, const float *__restrict__ hinge_rest, int nb,
    double *parts, int *bad) {
    __shared__ double sn[kBlock / 32], sd[kBlock / 32];
    int t = blockIdx.x * kBlock + threadIdx.x;
    double num = 0.0, den = 0.0;
    if (t < nd) {
        int2 e = didx[t];
        if (e.x >= 0 && e.x < n_points && e.y >= 0 && e.y < n_points) {
            float4 a = p[e.x], b = p[e.y];
            double dx = (double)a.x - b.x, dy = (double)a.y - b.y, dz = (double)a.z - b.z;
            double l = rest[t];
            double c = sqrt(dx * dx + dy * dy + dz * dz) - l;
            num = c * c;
            den = l * l;
        } else {
            atomicOr(bad, 1);
        }
    } else if (t < nd + nb) {
        int j = t - nd;
        int4 r = bidx[j];
        if (r.x >= 0 && r.x < n_points && r.y >= 0 && r.y < n_points && r.z >= 0 &&
            r.z < n_points && r.w >= 0 && r.w < n_points) {
            float4 q0 = p[r.x], q1 = p[r.y], q2 = p[r.z], q3 = p[r.w];
            double E[3] = {(double)q1.x - q0.x, (double)q1.y - q0.y, (double)q1.z - q0.z};
            double A0[3] = {(double)q2.x - q0.x, (double)q2.y - q0.y, (double)q2.z - q0.z};
            double A1[3] = {(double)q2.x - q1.x, (double)q2.y - q1.y, (double)q2.z - q1.z};
            double B1[3] = {(double)q3.x - q1.x, (double)q3.y - q1.y, (double)q3.z - q1.z};
            double B0[3] = {(double)q3.x - q0.x, (double)q3.y - q0.y, (double)q3.z - q0.z};
            double na[3] = {A0[1] * A1[2] - A0[2] * A1[1], A0[2] * A1[0] - A0[0] * A1[2],
                            A0[0] * A1[1] - A0[1] * A1[0]};
            double nbv[3] = {B1[1] * B0[2] - B1[2] * B0[1], B1[2] * B0[0] - B1[0] * B0[2],
                             B1[0] * B0[1] - B1[1] * B0[0]};
            double cx[3] = {na[1] * nbv[2] - na[2] * nbv[1], na[2] * nbv[0] - na[0] * nbv[2],
                            na[0] * nbv[1] - na[1] * nbv[0]};
            double el = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
            double th = el > 0.0 ? atan2((cx[0] * E[0] + cx[1] * E[1] + cx[2] * E[2]) / el,
                                         na[0] * nbv[0] + na[1] * nbv[1] + na[2] * nbv[2])
                                 : 0.0;
            double c = th - (double)rest_angle[j];
            if (c > 3.141592653589793) c -= 6.283185307179586;
            if (c < -3.141592653589793) c += 6.283185307179586;
            double lr = hinge_rest[j];
            num = (c * el) * (c * el);
            den = lr * lr;
        } else {
            atomicOr(bad, 1);
        }
    }
    num = wsum(num);
    den = wsum(den);
    if ((threadIdx.x & 31) == 0) {
        sn[threadIdx.x >> 5] = num;
        sd[threadIdx.x >> 5] = den;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kBlock / 32; ++w) {
            a += sn[w];
            b += sd[w];
        }
        parts[2 * blockIdx.x] = a;
        parts[2 * blockIdx.x + 1] = b;
    }
}

// fixed-order sum of the block partials; out = {residual, num, den}
__global__ void __launch_bounds__(1024) k_residual_final(const double *parts, int nblocks,
                                                         const int *bad, double *out) {
    __shared__ double sn[32], sd[32];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += 1024) {
        a += parts[2 * i];
        b += parts[2 * i + 1];
    }
    a = wsum(a);
    b = wsum(b);
    if ((threadIdx.x & 31) == 0) {
        sn[threadIdx.x >> 5] = a;
        sd[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < 32; ++w) {
            x += sn[w];
            y += sd[w];
        }
        double r = y > 0.0 ? sqrt(x) / sqrt(y) : 0.0;
        if (*bad) r = __longlong_as_double(0x7ff8000000000000LL);  // NaN: an index was out of range
        out[0] = r;
        out[1] = x;
        out[2] = y;
    }
}

std::mutex g_setup_mu;
constexpr int kMaxDevices = 64;

// The array's address belongs to the module loaded in one CUDA context.
// After cudaDeviceReset (or with another context current) the module is
// loaded again, possibly elsewhere, so the cached address is keyed by the
// context's unique id and looked up again when that id changes.
struct ScratchSlot {
    unsigned long long ctx_id;
    double *ptr;
};
ScratchSlot g_slot[kMaxDevices] = {};

typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
bool g_ctx_fns_tried = false;

// id of the current context (0 when it cannot be read: then the address is
// looked up on every call)
unsigned long long current_context_id() {
    if (!g_ctx_fns_tried) {
        g_ctx_fns_tried = true;
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_current = (CtxGetCurrentFn)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_id = (CtxGetIdFn)f;
        cudaGetLastError();
    }
    if (!g_ctx_current || !g_ctx_id) return 0;
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&ctx) != 0 || !ctx || g_ctx_id(ctx, &id) != 0) return 0;
    return id;
}

// device address of the scratch array in the current device's context
int scratch_address(double **out) {
    int dev = 0;
    PBD_CUDA(cudaGetDevice(&dev));
    PBD_CHECK(dev >= 0 && dev < kMaxDevices, PBD_ERR_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_setup_mu);
    unsigned long long id = current_context_id();
    if (!g_slot[dev].ptr || id == 0 || g_slot[dev].ctx_id != id) {
        void *p = nullptr;
        PBD_CUDA(cudaGetSymbolAddress(&p, g_residual_scratch));
        // the lookup made the device's context current if it was not yet
        if (id == 0) id = current_context_id();
        g_slot[dev].ptr = (double *)p;
        g_slot[dev].ctx_id = id;
    }
    *out = g_slot[dev].ptr;
    return PBD_OK;
}

}  // namespace

extern "C" int pbd_residual_noalloc(const float *d_pos4, int n_points, const int *d_dist_idx,
                                    const float *d_rest_length, int n_dist,
                                    const int *d_bend_idx, const float *d_rest_angle,
                                    const float *d_hinge_rest, int n_bend, double *d_out,
                                    void *stream) {
    PBD_CHECK(d_pos4 && d_out && n_points > 0 && n_dist >= 0 && n_bend >= 0, PBD_ERR_ARG,
              "pbd_residual_noalloc: bad argument");
    PBD_CHECK(n_dist == 0 || (d_dist_idx && d_rest_length), PBD_ERR_ARG,
              "pbd_residual_noalloc: distance buffers missing");
    PBD_CHECK(n_bend == 0 || (d_bend_idx && d_rest_angle && d_hinge_rest), PBD_ERR_ARG,
              "pbd_residual_noalloc: bending buffers missing");
    PBD_CHECK(((uintptr_t)d_pos4 & 15) == 0 && ((uintptr_t)d_dist_idx & 7) == 0 &&
                  ((uintptr_t)d_bend_idx & 15) == 0 && ((uintptr_t)d_out & 7) == 0,
              PBD_ERR_ARG, "pbd_residual_noalloc: positions and bending ids need 16-byte, "
                           "distance ids and the output 8-byte alignment");
    long long total = (long long)n_dist + n_bend;
    PBD_CHECK(total <= (long long)kMaxBlocks * kBlock, PBD_ERR_ARG,
              "pbd_residual_noalloc: %lld constraints exceed the maximum of %d",
              total, kMaxBlocks * kBlock);
    double *scratch = nullptr;
    PBD_TRY(scratch_address(&scratch));
    int *bad = (int *)(scratch + 2 * kMaxBlocks);
    cudaStream_t s = (cudaStream_t)stream;
    PBD_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
    int nblocks = (int)((total + kBlock - 1) / kBlock);
    if (nblocks < 1) nblocks = 1;
    k_residual_parts<<<nblocks, kBlock, 0, s>>>((const float4 *)d_pos4, n_points,
                                                (const int2 *)d_dist_idx, d_rest_length, n_dist,
                                                (const int4 *)d_bend_idx, d_rest_angle,
                                                d_hinge_rest, n_bend, scratch, bad);
    k_residual_final<<<1, 1024, 0, s>>>(scratch, nblocks, bad, d_out);
    PBD_LAUNCH();
    return PBD_OK;
}

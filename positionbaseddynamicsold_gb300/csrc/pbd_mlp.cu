// pbd_mlp.cu -- learned warm start: a per-point MLP that predicts the
// correction the colored Gauss-Seidel solve will apply to the advected
// positions, so that fewer sweeps reach the residual target.
//
// Network: 16 features -> 64 -> 64 -> 3, SiLU on both hidden layers.
// Features of point i (all dimensionless):
//   0..5   strain (|p_i - p_j| - l)/l of the first six incident distance
//          constraints (by prim id; 0 where the point has fewer)
//   6..8   previous substep's correction / lbar (lbar = mean incident rest
//          length)
//   9      inverse-mass share w_i / (w_i + mean_j w_j) over distance
//          neighbours
//   10     pinned flag (w_i == 0)
//   11..14 dihedral deviation theta - theta0 of the first four incident
//          bending constraints (by prim id)
//   15     constant 1 (the first layer's bias)
// Features 0..14 are multiplied by per-feature scales before they enter the
// network; its output y (3) is the correction / (lbar * output scale).
// Pinned points get no correction.
//
// The three GEMMs of a tile of 128 points run on the 5th-generation tensor
// cores: tcgen05.mma kind::f16 with BF16 operands in shared memory (K-major
// core-matrix layout, no swizzle), FP32 accumulators in tensor memory,
// read back with tcgen05.ld; one elected thread issues the MMAs and
// tcgen05.commit signals an mbarrier.  Thread t of the 128-thread block
// owns point (tile*128 + t), which is row t of every M=128 GEMM and TMEM
// lane t, so the epilogues (bias, SiLU, BF16 packing) need no shuffles.
//
// Training (k_mlp_train) runs the forward pass, the backward pass and the
// weight gradients of a tile on the tensor cores as well:
//   dH2 = dY W3, dH1 = dZ2 W2 (M=128 GEMMs over the tile's points) and
//   [dW3^T | dW2] = [H2^T ; dZ2^T] [dY^T ; H1^T]^T, dW1 = dZ1^T X
// (K = the tile's 128 points), the latter accumulated in TMEM over all the
// tiles a block processes and added to the global gradient once.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "pbd_common.cuh"

namespace pbd {

// ---------------------------------------------------------------------------
// tcgen05 / mbarrier helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor, no swizzle: start address, leading byte
// offset (distance between core matrices along K), stride byte offset
// (distance between 8-row groups), descriptor version 1 at bit 46.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D F32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N>>3 at bit 17, M>>4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
        : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for the mbarrier phase `parity` to complete; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int i = 0; i < (1 << 20); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

template <int NCOLS>
__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     slot_saddr),
                 "n"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
template <int NCOLS>
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "n"(NCOLS)
                 : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// ---------------------------------------------------------------------------
// operand layout: K-major, no swizzle.  A core matrix is 8 rows x 16 bytes
// (8 BF16 along K) stored as 128 contiguous bytes; core matrices adjacent
// along K are 128 B apart (LBO), 8-row groups are K*16 B apart (SBO).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int cm_off(int row, int col, int K) {
    return (row >> 3) * (K * 8) + (col >> 3) * 64 + (row & 7) * 8 + (col & 7);
}
// descriptor of a [rows x K] tile at k-step s (16 columns per MMA)
__device__ __forceinline__ uint64_t tile_desc(const unsigned short *tile, int K, int s) {
    return sdesc(smem_u32(tile) + 256u * (uint32_t)s, 128u, (uint32_t)K * 16u);
}

__device__ __forceinline__ unsigned short f2bf(float f) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    return (uint32_t)f2bf(a) | ((uint32_t)f2bf(b) << 16);
}
// write 8 consecutive K values of one row (one 16-byte store)
__device__ __forceinline__ void st_row8(unsigned short *tile, int row, int col0, int K,
                                        const float *v) {
    uint4 q = make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]),
                         pack2(v[6], v[7]));
    *reinterpret_cast<uint4 *>(tile + cm_off(row, col0, K)) = q;
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// ---------------------------------------------------------------------------
// features
// ---------------------------------------------------------------------------
struct FeatArgs {
    const float4 *pos;      // positions the features are taken at (advected)
    const float4 *dprev;    // previous substep's correction (may be null)
    const int4 *fa, *fb;
    const int2 *fc;
    const float4 *ra, *rb;
    const float *theta;     // per prim
    const float *scale;     // 16 input scales (15th unused) + the output scale
};

__device__ __forceinline__ float strain(float4 P, const float4 *pos, int j, float l) {
    if (j < 0 || !(l > 0.f)) return 0.f;
    float4 Q = pos[j];
    float dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
    return (sqrtf(dx * dx + dy * dy + dz * dz) - l) / l;
}
__device__ __forceinline__ float hinge(const float *theta, int h) { return h >= 0 ? theta[h] : 0.f; }

// features of point i; returns lbar (0 for a point without distance
// constraints) and the pinned flag through P.w == 0
__device__ __forceinline__ float point_features(const FeatArgs &a, int i, float *f, float4 &P) {
    P = a.pos[i];
    int4 na = a.fa[i], nb = a.fb[i];
    int2 nc = a.fc[i];
    float4 ra = a.ra[i], rb = a.rb[i];
    f[0] = strain(P, a.pos, na.x, ra.x);
    f[1] = strain(P, a.pos, na.y, ra.y);
    f[2] = strain(P, a.pos, na.z, ra.z);
    f[3] = strain(P, a.pos, na.w, ra.w);
    f[4] = strain(P, a.pos, nb.x, rb.x);
    f[5] = strain(P, a.pos, nb.y, rb.y);
    float lbar = rb.z;
    float inv = lbar > 0.f ? 1.f / lbar : 0.f;
    float4 d = a.dprev ? a.dprev[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    f[6] = d.x * inv;
    f[7] = d.y * inv;
    f[8] = d.z * inv;
    f[9] = rb.w;
    f[10] = P.w == 0.f ? 1.f : 0.f;
    f[11] = hinge(a.theta, nb.z);
    f[12] = hinge(a.theta, nb.w);
    f[13] = hinge(a.theta, nc.x);
    f[14] = hinge(a.theta, nc.y);
#pragma unroll
    for (int k = 0; k < 15; ++k) f[k] *= a.scale[k];
    f[15] = 1.f;
    return lbar;
}

// wrapped dihedral deviation theta - theta0 of every bending record, stored
// by prim id (same float arithmetic as the projection's constraint value)
__global__ void __launch_bounds__(256) k_eval_hinges(int nb, const int4 *__restrict__ bidx,
                                                     const float2 *__restrict__ bpar,
                                                     const int *__restrict__ bend_prim,
                                                     const float4 *__restrict__ p,
                                                     float *__restrict__ theta) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb) return;
    int4 r = bidx[t];
    float4 Q0 = p[r.x], Q1 = p[r.y], Q2 = p[r.z], Q3 = p[r.w];
    float Ex = Q1.x - Q0.x, Ey = Q1.y - Q0.y, Ez = Q1.z - Q0.z;
    float ax = Q2.x - Q0.x, ay = Q2.y - Q0.y, az = Q2.z - Q0.z;
    float bx = Q2.x - Q1.x, by = Q2.y - Q1.y, bz = Q2.z - Q1.z;
    float nax = ay * bz - az * by, nay = az * bx - ax * bz, naz = ax * by - ay * bx;
    float cx = Q3.x - Q1.x, cy = Q3.y - Q1.y, cz = Q3.z - Q1.z;
    float dx = Q3.x - Q0.x, dy = Q3.y - Q0.y, dz = Q3.z - Q0.z;
    float nbx = cy * dz - cz * dy, nby = cz * dx - cx * dz, nbz = cx * dy - cy * dx;
    float el = sqrtf(Ex * Ex + Ey * Ey + Ez * Ez);
    float c = 0.f;
    if (el > 0.f) {
        float sx = nay * nbz - naz * nby, sy = naz * nbx - nax * nbz, sz = nax * nby - nay * nbx;
        float sn = (sx * Ex + sy * Ey + sz * Ez) / el;
        float cs = nax * nbx + nay * nby + naz * nbz;
        c = atan2f(sn, cs) - bpar[t].x;
        if (c > 3.14159265f) c -= 6.28318531f;
        if (c < -3.14159265f) c += 6.28318531f;
    }
    theta[bend_prim[t]] = c;
}

// features of every point as BF16 rows of 16 (training records)
__global__ void __launch_bounds__(256) k_features(int n, FeatArgs a,
                                                  unsigned short *__restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float f[16];
    float4 P;
    point_features(a, i, f, P);
    uint4 *o = reinterpret_cast<uint4 *>(out + 16 * (size_t)i);
    o[0] = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
    o[1] = make_uint4(pack2(f[8], f[9]), pack2(f[10], f[11]), pack2(f[12], f[13]),
                      pack2(f[14], f[15]));
}

}  // namespace pbd

namespace pbd {

constexpr int kTile = 128;  // points per tile = GEMM M = TMEM lanes

// ---------------------------------------------------------------------------
// inference: p = p0 + lbar * MLP(features(p0)) for every free point
// ---------------------------------------------------------------------------
struct InferSmem {
    unsigned short w1[64 * 16];   // B tiles, same order as kWtW1..kWtW3
    unsigned short w2[64 * 64];
    unsigned short w3[16 * 64];
    unsigned short x[kTile * 16];   // A tiles
    unsigned short h[kTile * 64];   // H1, then (after layer 2 has read it) H2
    float b2[64], b3[16];
    unsigned long long mbar;
    uint32_t tslot;
};
// TMEM columns [0,64) hold Z1, then Z2, then Y: each is read out completely
// before the next GEMM writes there
constexpr int kInferCols = 64;
// dynamic shared memory requested per block: at most six blocks per SM (228
// KB of shared memory), whose 6 x 64 TMEM columns always fit in 512
constexpr int kInferSmem = 36 * 1024;
constexpr int kInferBlocksPerSM = 6;
static_assert(sizeof(InferSmem) + 1024 <= kInferSmem, "inference smem");

__device__ __forceinline__ void copy_u4(void *dst, const void *src, int bytes, int tid, int nthr) {
    const uint4 *s = reinterpret_cast<const uint4 *>(src);
    uint4 *d = reinterpret_cast<uint4 *>(dst);
    for (int k = tid; k < bytes / 16; k += nthr) d[k] = s[k];
}

__device__ __forceinline__ unsigned char *align1024(unsigned char *p) {
    return reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(p) + 1023) &
                                             ~(uintptr_t)1023);
}

// Elected-thread MMA chain: D (tmem column dcol) = sum_s A_s B_s^T
__device__ __forceinline__ void issue_gemm(uint32_t tbase, int dcol, const unsigned short *a,
                                           int ka, const unsigned short *b, int kb, int ksteps,
                                           uint32_t idesc, bool accumulate_first) {
    for (int s = 0; s < ksteps; ++s)
        mma_bf16(tbase + (uint32_t)dcol, tile_desc(a, ka, s), tile_desc(b, kb, s), idesc,
                 (accumulate_first || s > 0) ? 1u : 0u);
}

// RAW = false: features of the points from fa, p = p0 + correction.
// RAW = true: BF16 feature rows from xin (column 15 forced to 1), network
// outputs (with b3) to yout.
template <bool RAW>
__global__ void __launch_bounds__(kTile, 1) k_mlp_infer(int n, FeatArgs fa, float4 *__restrict__ p,
                                                        const unsigned short *__restrict__ xin,
                                                        float4 *__restrict__ yout,
                                                        const unsigned short *__restrict__ wt,
                                                        const float *__restrict__ bias,
                                                        int *__restrict__ err) {
    extern __shared__ unsigned char smraw[];
    InferSmem &S = *reinterpret_cast<InferSmem *>(align1024(smraw));
    const int tid = threadIdx.x, warp = tid >> 5;
    copy_u4(S.w1, wt + kWtW1, (64 * 16 + 64 * 64 + 16 * 64) * 2, tid, kTile);
    if (tid < 64) S.b2[tid] = bias[tid];
    if (tid < 16) S.b3[tid] = bias[64 + tid];
    if (tid == 0) mbar_init(smem_u32(&S.mbar), 1);
    if (warp == 0) tmem_alloc<kInferCols>(smem_u32(&S.tslot));
    fence_proxy_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = S.tslot;
    const uint32_t lane = tb + ((uint32_t)(warp * 32) << 16);
    const uint32_t mbar = smem_u32(&S.mbar);
    const uint32_t id64 = idesc_bf16(kTile, 64), id16 = idesc_bf16(kTile, 16);
    uint32_t phase = 0;
    bool ok = true;
    const int ntiles = (n + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * kTile + tid;
        const bool valid = i < n;
        float f[16];
        float4 P = make_float4(0.f, 0.f, 0.f, 0.f);
        float lbar = 0.f;
        if (valid && RAW) {
            const uint4 *xr = reinterpret_cast<const uint4 *>(xin + 16 * (size_t)i);
            uint4 q0 = xr[0], q1 = xr[1];
            uint32_t u[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                f[2 * k] = __uint_as_float(u[k] << 16);
                f[2 * k + 1] = __uint_as_float(u[k] & 0xffff0000u);
            }
            f[15] = 1.f;
        } else if (valid) {
            lbar = point_features(fa, i, f, P);
        } else {
#pragma unroll
            for (int k = 0; k < 16; ++k) f[k] = 0.f;
        }
        st_row8(S.x, tid, 0, 16, f);
        st_row8(S.x, tid, 8, 16, f + 8);
        fence_proxy_async();
        fence_before_sync();
        __syncthreads();
        // layer 1
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 0, S.x, 16, S.w1, 16, 1, id64, false);
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) break;
        fence_after_sync();
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float z[16];
            tmem_ld16(lane + 16 * c, z);
#pragma unroll
            for (int k = 0; k < 16; ++k) z[k] = silu(z[k]);
            st_row8(S.h, tid, 16 * c, 64, z);
            st_row8(S.h, tid, 16 * c + 8, 64, z + 8);
        }
        fence_proxy_async();
        fence_before_sync();
        __syncthreads();
        // layer 2
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 0, S.h, 64, S.w2, 64, 4, id64, false);
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) break;
        fence_after_sync();
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float z[16];
            tmem_ld16(lane + 16 * c, z);
#pragma unroll
            for (int k = 0; k < 16; ++k) z[k] = silu(z[k] + S.b2[16 * c + k]);
            st_row8(S.h, tid, 16 * c, 64, z);
            st_row8(S.h, tid, 16 * c + 8, 64, z + 8);
        }
        fence_proxy_async();
        fence_before_sync();
        __syncthreads();
        // layer 3
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 0, S.h, 64, S.w3, 64, 4, id16, false);
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) break;
        fence_after_sync();
        float y[16];
        tmem_ld16(lane, y);
        if (RAW) {
            if (valid) yout[i] = make_float4(y[0] + S.b3[0], y[1] + S.b3[1], y[2] + S.b3[2], 0.f);
        } else if (valid && P.w != 0.f && lbar > 0.f) {
            const float os = fa.scale[16] * lbar;
            float dx = (y[0] + S.b3[0]) * os, dy = (y[1] + S.b3[1]) * os,
                  dz = (y[2] + S.b3[2]) * os;
            p[i] = make_float4(P.x + dx, P.y + dy, P.z + dz, P.w);
        }
        fence_before_sync();
    }
    if (!ok) {
        if (tid == 0) {
            atomicExch(err, 1);
            mbar_wait(mbar, phase);  // let an MMA still in flight finish
        }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0) tmem_dealloc<kInferCols>(tb);
}

}  // namespace pbd

namespace pbd {

// ---------------------------------------------------------------------------
// training: loss = 1/2 * inv_count * sum over masked points of |y - t|^2;
// the gradient of every parameter is added to grad, the loss to loss[0]
// ---------------------------------------------------------------------------
constexpr int kGaRows = 192;  // H2^T (0..63), dZ2^T (64..127), dZ1^T (128..191)
constexpr int kGbRows = 80;   // dY^T (0..15), H1^T (16..79)
struct TrainSmem {
    unsigned short w[kWtTotal];     // w1, w2, w3, w3t, w2t
    unsigned short x[kTile * 16];
    unsigned short h1[kTile * 64];
    unsigned short h2[kTile * 64];
    unsigned short dy[kTile * 16];
    unsigned short dz2[kTile * 64];
    unsigned short ga[kGaRows * kTile];
    unsigned short gb[kGbRows * kTile];
    unsigned short xt[16 * kTile];
    float b2[64], b3[16];
    float db3[4];
    double lsum;
    unsigned long long mbar;
    uint32_t tslot;
};
// TMEM columns: Z1 [0,64) Z2 [64,128) Y [128,144) dH2 [160,224) dH1 [224,288)
// G1 [288,368) G2 [384,400); the whole 512 columns, one block per SM
constexpr int kTrainCols = 512;
constexpr int kTrainSmem = (int)sizeof(TrainSmem) + 1024;
static_assert(kTrainSmem > 116 * 1024 && kTrainSmem <= 227 * 1024, "training smem");

#define PBD_MLP_BARRIER() \
    fence_proxy_async();  \
    fence_before_sync();  \
    __syncthreads();
#define PBD_MLP_WAIT()                      \
    ok = mbar_wait(mbar, phase);            \
    phase ^= 1;                             \
    if (!__syncthreads_and(ok)) break;      \
    fence_after_sync();

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kTile, 1) k_mlp_train(
    int n, const unsigned short *__restrict__ X, const float4 *__restrict__ T, float inv_count,
    const unsigned short *__restrict__ wt, const float *__restrict__ bias, float *__restrict__ grad,
    double *__restrict__ loss, int *__restrict__ err) {
    extern __shared__ unsigned char smraw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(align1024(smraw));
    const int tid = threadIdx.x, warp = tid >> 5;
    copy_u4(S.w, wt, kWtTotal * 2, tid, kTile);
    if (tid < 64) S.b2[tid] = bias[tid];
    if (tid < 16) S.b3[tid] = bias[64 + tid];
    if (tid < 4) S.db3[tid] = 0.f;
    if (tid == 0) {
        S.lsum = 0.0;
        mbar_init(smem_u32(&S.mbar), 1);
    }
    if (warp == 0) tmem_alloc<kTrainCols>(smem_u32(&S.tslot));
    fence_proxy_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = S.tslot;
    const uint32_t lane = tb + ((uint32_t)(warp * 32) << 16);
    const uint32_t mbar = smem_u32(&S.mbar);
    const uint32_t id64 = idesc_bf16(kTile, 64), id16 = idesc_bf16(kTile, 16),
                   id80 = idesc_bf16(kTile, 80);
    uint32_t phase = 0;
    bool ok = true;
    int done = 0;
    double lacc = 0.0;
    const int ntiles = (n + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * kTile + tid;
        const bool valid = i < n;
        float f[16];
        float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid) {
            const uint4 *xr = reinterpret_cast<const uint4 *>(X + 16 * (size_t)i);
            uint4 q0 = xr[0], q1 = xr[1];
            uint32_t u[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                f[2 * k] = __uint_as_float(u[k] << 16);
                f[2 * k + 1] = __uint_as_float(u[k] & 0xffff0000u);
            }
            f[15] = 1.f;  // the constant feature
            t = T[i];
        } else {
#pragma unroll
            for (int k = 0; k < 16; ++k) f[k] = 0.f;
        }
        st_row8(S.x, tid, 0, 16, f);
        st_row8(S.x, tid, 8, 16, f + 8);
#pragma unroll
        for (int k = 0; k < 16; ++k) S.xt[cm_off(k, tid, kTile)] = f2bf(f[k]);
        PBD_MLP_BARRIER();
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 0, S.x, 16, S.w + kWtW1, 16, 1, id64, false);
            mma_commit(mbar);
        }
        PBD_MLP_WAIT();
        // H1 = silu(Z1)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float z[16];
            tmem_ld16(lane + 16 * c, z);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                z[k] = silu(z[k]);
                S.gb[cm_off(16 + 16 * c + k, tid, kTile)] = f2bf(z[k]);
            }
            st_row8(S.h1, tid, 16 * c, 64, z);
            st_row8(S.h1, tid, 16 * c + 8, 64, z + 8);
        }
        PBD_MLP_BARRIER();
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 64, S.h1, 64, S.w + kWtW2, 64, 4, id64, false);
            mma_commit(mbar);
        }
        PBD_MLP_WAIT();
        // H2 = silu(Z2 + b2)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float z[16];
            tmem_ld16(lane + 64 + 16 * c, z);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                z[k] = silu(z[k] + S.b2[16 * c + k]);
                S.ga[cm_off(16 * c + k, tid, kTile)] = f2bf(z[k]);
            }
            st_row8(S.h2, tid, 16 * c, 64, z);
            st_row8(S.h2, tid, 16 * c + 8, 64, z + 8);
        }
        PBD_MLP_BARRIER();
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 128, S.h2, 64, S.w + kWtW3, 64, 4, id16, false);
            mma_commit(mbar);
        }
        PBD_MLP_WAIT();
        // dY = mask * (y - t) * inv_count
        {
            float y[16], d[16];
            tmem_ld16(lane + 128, y);
            bool use = valid && t.w != 0.f;
            float e0 = use ? y[0] + S.b3[0] - t.x : 0.f;
            float e1 = use ? y[1] + S.b3[1] - t.y : 0.f;
            float e2 = use ? y[2] + S.b3[2] - t.z : 0.f;
            lacc += (double)e0 * e0 + (double)e1 * e1 + (double)e2 * e2;
#pragma unroll
            for (int k = 0; k < 16; ++k) d[k] = 0.f;
            d[0] = e0 * inv_count;
            d[1] = e1 * inv_count;
            d[2] = e2 * inv_count;
            st_row8(S.dy, tid, 0, 16, d);
            st_row8(S.dy, tid, 8, 16, d + 8);
#pragma unroll
            for (int k = 0; k < 16; ++k) S.gb[cm_off(k, tid, kTile)] = f2bf(d[k]);
            float s0 = warp_sum_f(d[0]), s1 = warp_sum_f(d[1]), s2 = warp_sum_f(d[2]);
            if ((tid & 31) == 0) {
                atomicAdd(&S.db3[0], s0);
                atomicAdd(&S.db3[1], s1);
                atomicAdd(&S.db3[2], s2);
            }
        }
        PBD_MLP_BARRIER();
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 160, S.dy, 16, S.w + kWtW3T, 16, 1, id64, false);
            mma_commit(mbar);
        }
        PBD_MLP_WAIT();
        // dZ2 = dH2 * silu'(Z2 + b2)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float g[16], z[16];
            tmem_ld16(lane + 160 + 16 * c, g);
            tmem_ld16(lane + 64 + 16 * c, z);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                g[k] *= dsilu(z[k] + S.b2[16 * c + k]);
                S.ga[cm_off(64 + 16 * c + k, tid, kTile)] = f2bf(g[k]);
            }
            st_row8(S.dz2, tid, 16 * c, 64, g);
            st_row8(S.dz2, tid, 16 * c + 8, 64, g + 8);
        }
        PBD_MLP_BARRIER();
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 224, S.dz2, 64, S.w + kWtW2T, 64, 4, id64, false);
            mma_commit(mbar);
        }
        PBD_MLP_WAIT();
        // dZ1 = dH1 * silu'(Z1)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float g[16], z[16];
            tmem_ld16(lane + 224 + 16 * c, g);
            tmem_ld16(lane + 16 * c, z);
#pragma unroll
            for (int k = 0; k < 16; ++k)
                S.ga[cm_off(128 + 16 * c + k, tid, kTile)] = f2bf(g[k] * dsilu(z[k]));
        }
        PBD_MLP_BARRIER();
        // weight gradients over the tile's points, accumulated in TMEM
        if (tid == 0) {
            fence_after_sync();
            issue_gemm(tb, 288, S.ga, kTile, S.gb, kTile, 8, id80, done > 0);
            issue_gemm(tb, 384, S.ga + 64 * kTile, kTile, S.xt, kTile, 8, id16, done > 0);
            mma_commit(mbar);
        }
        PBD_MLP_WAIT();
        ++done;
    }
    if (ok && done > 0) {
        // G1 rows 0..63: dW3^T (cols 0..2); rows 64..127: dW2 (cols 16..79).
        // G2 rows 0..63: column 15 = sum of dZ2 = db2; rows 64..127: dW1.
        float v[16];
        if (warp < 2) {
            const int h = tid;
            tmem_ld16(lane + 288, v);
            for (int o = 0; o < kWsOut; ++o) atomicAdd(&grad[kWsOffW3 + o * 64 + h], v[o]);
            tmem_ld16(lane + 384, v);
            atomicAdd(&grad[kWsOffB2 + h], v[15]);
        } else {
            const int h = tid - 64;
            for (int c = 0; c < 4; ++c) {
                tmem_ld16(lane + 288 + 16 + 16 * c, v);
                for (int k = 0; k < 16; ++k) atomicAdd(&grad[kWsOffW2 + h * 64 + 16 * c + k], v[k]);
            }
            tmem_ld16(lane + 384, v);
            for (int k = 0; k < 16; ++k) atomicAdd(&grad[kWsOffW1 + h * 16 + k], v[k]);
        }
    }
    double ls = lacc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
    if ((tid & 31) == 0) atomicAdd(&S.lsum, ls);
    if (!ok && tid == 0) {
        atomicExch(err, 1);
        mbar_wait(mbar, phase);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (ok && done > 0 && tid < kWsOut) atomicAdd(&grad[kWsOffB3 + tid], S.db3[tid]);
    if (tid == 0) atomicAdd(loss, S.lsum);
    if (warp == 0) tmem_dealloc<kTrainCols>(tb);
}

#undef PBD_MLP_BARRIER
#undef PBD_MLP_WAIT

}  // namespace pbd

namespace pbd {

// FP32 master parameters -> BF16 operand tiles and FP32 biases
__global__ void k_pack_weights(const float *__restrict__ P, unsigned short *__restrict__ wt,
                               float *__restrict__ bias) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 64 * 16) {
        int h = t / 16, k = t % 16;
        wt[kWtW1 + cm_off(h, k, 16)] = f2bf(P[kWsOffW1 + t]);
    }
    if (t < 64 * 64) {
        int r = t / 64, c = t % 64;
        unsigned short w = f2bf(P[kWsOffW2 + t]);
        wt[kWtW2 + cm_off(r, c, 64)] = w;
        wt[kWtW2T + cm_off(c, r, 64)] = w;
    }
    if (t < 16 * 64) {
        int o = t / 64, h = t % 64;
        unsigned short w = f2bf(o < kWsOut ? P[kWsOffW3 + o * 64 + h] : 0.f);
        wt[kWtW3 + cm_off(o, h, 64)] = w;
        wt[kWtW3T + cm_off(h, o, 16)] = w;
    }
    if (t < 64) bias[t] = P[kWsOffB2 + t];
    if (t < 16) bias[64 + t] = t < kWsOut ? P[kWsOffB3 + t] : 0.f;
}

// Adam (Kingma & Ba 2015) with bias correction; clears the gradient
__global__ void k_adam(int n, float *__restrict__ P, float *__restrict__ m, float *__restrict__ v,
                       float *__restrict__ g, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    g[i] = 0.f;
}

// training targets of a solved substep: t = (p - p0)/lbar, w = 1 for free
// points with distance constraints, 0 otherwise
__global__ void k_targets(int n, const float4 *__restrict__ p, const float4 *__restrict__ p0,
                          const float4 *__restrict__ rb, const float *__restrict__ scale,
                          float4 *__restrict__ T) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 P = p[i], Q = p0[i];
    float lbar = rb[i].z;
    bool use = Q.w != 0.f && lbar > 0.f;
    float inv = use ? 1.f / (lbar * scale[16]) : 0.f;
    T[i] = make_float4((P.x - Q.x) * inv, (P.y - Q.y) * inv, (P.z - Q.z) * inv, use ? 1.f : 0.f);
}

// correction of the solved substep: dprev = p - p0
__global__ void k_store_delta(int n, const float4 *__restrict__ p, const float4 *__restrict__ p0,
                              float4 *__restrict__ dprev) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 P = p[i], Q = p0[i];
    dprev[i] = make_float4(P.x - Q.x, P.y - Q.y, P.z - Q.z, 0.f);
}

static unsigned short host_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return (unsigned short)(u >> 16);  // inf / nan
    u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even
    return (unsigned short)(u >> 16);
}

// per-point feature stencils from the host copy of the constraint topology
int build_feature_stencil(pbd_object *o) {
    if (o->feat_built) return PBD_OK;
    PBD_CHECK(o->sorted, PBD_ERR_STATE, "constraints are not color-sorted");
    const int n = o->n;
    std::vector<int4> fa(n, make_int4(-1, -1, -1, -1)), fb(n, make_int4(-1, -1, -1, -1));
    std::vector<int2> fc(n, make_int2(-1, -1));
    std::vector<float4> ra(n, make_float4(0, 0, 0, 0)), rb(n, make_float4(0, 0, 0, 0));
    std::vector<int> nd(n, 0), nh(n, 0);
    std::vector<double> lsum(n, 0.0), wsum(n, 0.0);
    std::vector<int> lcnt(n, 0);
    auto set_nb = [&](int i, int slot, int j, float l) {
        int *a = slot < 4 ? &fa[i].x : &fb[i].x;
        float *r = slot < 4 ? &ra[i].x : &rb[i].x;
        a[slot & 3] = j;
        r[slot & 3] = l;
    };
    auto set_h = [&](int i, int slot, int prim) {
        if (slot == 0) fb[i].z = prim;
        else if (slot == 1) fb[i].w = prim;
        else if (slot == 2) fc[i].x = prim;
        else fc[i].y = prim;
    };
    for (int p = 0; p < o->np; ++p) {
        const int *ix = o->h_indices.data() + o->h_prim_list[2 * p];
        if (o->h_ctype[p] == PBD_DISTANCE) {
            float l = o->h_rest_length[p];
            for (int e = 0; e < 2; ++e) {
                int i = ix[e], j = ix[1 - e];
                if (nd[i] < 6) set_nb(i, nd[i], j, l);
                ++nd[i];
                lsum[i] += l;
                wsum[i] += o->h_mass[j];
                ++lcnt[i];
            }
        } else if (o->h_ctype[p] == PBD_BENDING) {
            for (int e = 0; e < 4; ++e) {
                int i = ix[e];
                if (nh[i] < 4) set_h(i, nh[i], p);
                ++nh[i];
            }
        }
    }
    int nfree = 0;
    for (int i = 0; i < n; ++i) {
        float w = o->h_mass[i];
        float lbar = lcnt[i] ? (float)(lsum[i] / lcnt[i]) : 0.f;
        float wm = lcnt[i] ? (float)(wsum[i] / lcnt[i]) : 0.f;
        rb[i].z = lbar;
        rb[i].w = (w + wm) > 0.f ? w / (w + wm) : 0.f;
        if (w != 0.f && lbar > 0.f) ++nfree;
    }
    cudaStream_t s = o->stream;
    PBD_TRY(o->fnb_a.upload(fa.data(), n, s));
    PBD_TRY(o->fnb_b.upload(fb.data(), n, s));
    PBD_TRY(o->fnb_c.upload(fc.data(), n, s));
    PBD_TRY(o->frest_a.upload(ra.data(), n, s));
    PBD_TRY(o->frest_b.upload(rb.data(), n, s));
    PBD_TRY(o->theta.alloc(o->np > 0 ? o->np : 1));
    PBD_CUDA(cudaMemsetAsync(o->theta.p, 0, sizeof(float) * (o->np > 0 ? o->np : 1), s));
    if (!o->p0.p) PBD_TRY(o->p0.alloc(n));
    if (!o->dprev.p) {
        PBD_TRY(o->dprev.alloc(n));
        PBD_CUDA(cudaMemsetAsync(o->dprev.p, 0, sizeof(float4) * n, s));
    }
    PBD_CUDA(cudaStreamSynchronize(s));
    o->n_free = nfree;
    o->feat_built = true;
    return PBD_OK;
}

static FeatArgs feat_args(pbd_object *o, const float4 *pos, const pbd_warmstart *w) {
    FeatArgs a;
    a.scale = w->scale.p;
    a.pos = pos;
    a.dprev = o->dprev.p;
    a.fa = o->fnb_a.p;
    a.fb = o->fnb_b.p;
    a.fc = o->fnb_c.p;
    a.ra = o->frest_a.p;
    a.rb = o->frest_b.p;
    a.theta = o->theta.p;
    return a;
}

int ws_eval_hinges(pbd_object *o, const float4 *pos) {
    int nb = o->h_bseg.empty() ? 0 : o->h_bseg.back();
    if (!nb) return PBD_OK;
    k_eval_hinges<<<grid_for(nb, 256), 256, 0, o->stream>>>(nb, o->bidx.p, o->bpar.p,
                                                            o->bend_prim.p, pos, o->theta.p);
    PBD_LAUNCH();
    return PBD_OK;
}

static int infer_grid(long long n) {
    long long tiles = (n + kTile - 1) / kTile;
    return (int)std::max(1LL, std::min(tiles, (long long)kInferBlocksPerSM * kNumSMs));
}
static int train_grid(long long n) {
    long long tiles = (n + kTile - 1) / kTile;
    return (int)std::max(1LL, std::min(tiles, (long long)kNumSMs));
}

static int set_smem_attrs() {
    static int done = 0;
    if (done) return PBD_OK;
    PBD_CUDA(cudaFuncSetAttribute(k_mlp_infer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kInferSmem));
    PBD_CUDA(cudaFuncSetAttribute(k_mlp_infer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kInferSmem));
    PBD_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kTrainSmem));
    done = 1;
    return PBD_OK;
}

int ws_prepare(pbd_warmstart *w, pbd_object *o) {
    PBD_CHECK(w && o, PBD_ERR_ARG, "null argument");
    PBD_TRY(build_feature_stencil(o));
    PBD_TRY(set_smem_attrs());
    return PBD_OK;
}

// p = p0 + lbar * MLP(features(p0)) on the object's stream; hinges at p0
// must have been evaluated into o->theta
int ws_infer(pbd_warmstart *w, pbd_object *o) {
    k_mlp_infer<false><<<infer_grid(o->n), kTile, kInferSmem, o->stream>>>(
        o->n, feat_args(o, o->p0.p, w), o->p.p, nullptr, nullptr, w->wtiles.p, w->bias.p,
        w->err.p);
    PBD_LAUNCH();
    return PBD_OK;
}

static int pack(pbd_warmstart *w, cudaStream_t s) {
    k_pack_weights<<<16, 256, 0, s>>>(w->params.p, w->wtiles.p, w->bias.p);
    PBD_LAUNCH();
    return PBD_OK;
}

// features of the object's advected positions o->p0 into w->feat
int ws_record(pbd_warmstart *w, pbd_object *o) {
    PBD_TRY(ws_prepare(w, o));
    PBD_TRY(ws_eval_hinges(o, o->p0.p));
    if (w->feat_cap < o->n) {
        PBD_TRY(w->feat.alloc(16 * (size_t)o->n));
        w->feat_cap = o->n;
    }
    k_features<<<grid_for(o->n, 256), 256, 0, o->stream>>>(o->n, feat_args(o, o->p0.p, w),
                                                            w->feat.p);
    PBD_LAUNCH();
    return PBD_OK;
}

static int train_pass(pbd_warmstart *w, const unsigned short *dx, const float4 *dt, int n,
                      int n_used, cudaStream_t s, double *loss_out);
static int adam_step(pbd_warmstart *w, cudaStream_t s, float lr, float b1, float b2, float eps);

// one Adam step on (w->feat, (o->p - o->p0) / lbar) over the object's points
int ws_train_on(pbd_warmstart *w, pbd_object *o, float lr, double *loss) {
    cudaStream_t s = o->stream;
    PBD_TRY(w->tgt.alloc(o->n));
    k_targets<<<grid_for(o->n, 256), 256, 0, s>>>(o->n, o->p.p, o->p0.p, o->frest_b.p,
                                                  w->scale.p, w->tgt.p);
    PBD_LAUNCH();
    PBD_TRY(train_pass(w, w->feat.p, w->tgt.p, o->n, o->n_free, s, loss));
    return adam_step(w, s, lr, 0.9f, 0.999f, 1e-8f);
}

static int check_err(pbd_warmstart *w, cudaStream_t s) {
    int e = 0;
    PBD_CUDA(cudaMemcpyAsync(&e, w->err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    PBD_CHECK(e == 0, PBD_ERR_TIMEOUT, "tensor-core wait timed out in the warm-start network");
    return PBD_OK;
}

}  // namespace pbd

using namespace pbd;

extern "C" {

int pbd_warmstart_num_params(void) { return kWsParams; }

int pbd_warmstart_create(pbd_warmstart **out) {
    PBD_CHECK(out, PBD_ERR_ARG, "null argument");
    *out = nullptr;
    pbd_warmstart *w = new pbd_warmstart();
    auto fail = [&](int r) {
        pbd_warmstart_destroy(w);
        return r;
    };
    if (cudaStreamCreateWithFlags(&w->own, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed: %s", cudaGetErrorString(cudaGetLastError()));
        delete w;
        return PBD_ERR_CUDA;
    }
    int r;
    if ((r = w->params.alloc(kWsParams)) || (r = w->m.alloc(kWsParams)) ||
        (r = w->v.alloc(kWsParams)) || (r = w->grad.alloc(kWsParams)) ||
        (r = w->wtiles.alloc(kWtTotal)) || (r = w->bias.alloc(80)) || (r = w->loss.alloc(2)) ||
        (r = w->err.alloc(1)) || (r = w->scale.alloc(17)))
        return fail(r);
    {
        std::vector<float> ones(17, 1.f);
        if ((r = w->scale.upload(ones.data(), 17, w->own))) return fail(r);
    }
    cudaStream_t s = w->own;
    if (cudaMemsetAsync(w->params.p, 0, sizeof(float) * kWsParams, s) ||
        cudaMemsetAsync(w->m.p, 0, sizeof(float) * kWsParams, s) ||
        cudaMemsetAsync(w->v.p, 0, sizeof(float) * kWsParams, s) ||
        cudaMemsetAsync(w->grad.p, 0, sizeof(float) * kWsParams, s) ||
        cudaMemsetAsync(w->wtiles.p, 0, sizeof(unsigned short) * kWtTotal, s) ||
        cudaMemsetAsync(w->err.p, 0, sizeof(int), s) || cudaStreamSynchronize(s)) {
        set_error("warm start init failed: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(PBD_ERR_CUDA);
    }
    if ((r = pack(w, s)) || (r = set_smem_attrs())) return fail(r);
    *out = w;
    return PBD_OK;
}

int pbd_warmstart_destroy(pbd_warmstart *w) {
    if (!w) return PBD_OK;
    if (w->own) cudaStreamSynchronize(w->own);
    cudaStream_t s = w->own;
    delete w;
    if (s) cudaStreamDestroy(s);
    return PBD_OK;
}

int pbd_warmstart_set_params(pbd_warmstart *w, const float *params, int n) {
    PBD_CHECK(w && params, PBD_ERR_ARG, "null argument");
    PBD_CHECK(n == kWsParams, PBD_ERR_ARG, "expected %d parameters, got %d", kWsParams, n);
    cudaStream_t s = w->own;
    PBD_CUDA(cudaMemcpyAsync(w->params.p, params, sizeof(float) * kWsParams, cudaMemcpyHostToDevice, s));
    PBD_CUDA(cudaMemsetAsync(w->m.p, 0, sizeof(float) * kWsParams, s));
    PBD_CUDA(cudaMemsetAsync(w->v.p, 0, sizeof(float) * kWsParams, s));
    PBD_CUDA(cudaMemsetAsync(w->grad.p, 0, sizeof(float) * kWsParams, s));
    w->adam_t = 0;
    PBD_TRY(pack(w, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    return PBD_OK;
}

int pbd_warmstart_set_scales(pbd_warmstart *w, const float *scales, int n) {
    PBD_CHECK(w && scales && n == 17, PBD_ERR_ARG, "expected 17 scales");
    for (int k = 0; k < 17; ++k)
        PBD_CHECK(std::isfinite(scales[k]) && scales[k] > 0.f, PBD_ERR_ARG,
                  "scale %d must be finite and > 0", k);
    PBD_TRY(w->scale.upload(scales, 17, w->own));
    PBD_CUDA(cudaStreamSynchronize(w->own));
    return PBD_OK;
}

int pbd_warmstart_get_scales(pbd_warmstart *w, float *scales, int n) {
    PBD_CHECK(w && scales && n == 17, PBD_ERR_ARG, "expected 17 scales");
    PBD_CUDA(cudaStreamSynchronize(w->own));
    PBD_CUDA(cudaMemcpy(scales, w->scale.p, sizeof(float) * 17, cudaMemcpyDeviceToHost));
    return PBD_OK;
}

int pbd_warmstart_get_params(pbd_warmstart *w, float *params, int n) {
    PBD_CHECK(w && params, PBD_ERR_ARG, "null argument");
    PBD_CHECK(n == kWsParams, PBD_ERR_ARG, "expected %d parameters, got %d", kWsParams, n);
    PBD_CUDA(cudaStreamSynchronize(w->own));
    PBD_CUDA(cudaMemcpy(params, w->params.p, sizeof(float) * kWsParams, cudaMemcpyDeviceToHost));
    return PBD_OK;
}

static int upload_rows(pbd_warmstart *w, const float *x, int n, DBuf<unsigned short> &dst) {
    std::vector<unsigned short> h(16 * (size_t)n);
    for (size_t k = 0; k < h.size(); ++k) h[k] = host_bf16(x[k]);
    return dst.upload(h.data(), h.size(), w->own);
}

int pbd_warmstart_forward(pbd_warmstart *w, const float *x, int n, float *y) {
    PBD_CHECK(w && x && y && n > 0, PBD_ERR_ARG, "bad argument");
    DBuf<unsigned short> dx;
    DBuf<float4> dy;
    PBD_TRY(upload_rows(w, x, n, dx));
    PBD_TRY(dy.alloc(n));
    cudaStream_t s = w->own;
    k_mlp_infer<true><<<infer_grid(n), kTile, kInferSmem, s>>>(n, FeatArgs{}, nullptr, dx.p, dy.p,
                                                               w->wtiles.p, w->bias.p, w->err.p);
    PBD_LAUNCH();
    std::vector<float4> h(n);
    PBD_CUDA(cudaMemcpyAsync(h.data(), dy.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, s));
    PBD_TRY(check_err(w, s));
    for (int i = 0; i < n; ++i) {
        y[3 * i] = h[i].x;
        y[3 * i + 1] = h[i].y;
        y[3 * i + 2] = h[i].z;
    }
    return PBD_OK;
}

// one training pass over n rows already on the device; gradient added to
// w->grad, loss (1/2 * mean over used rows of |y - t|^2) to *loss_out
}  // extern "C"

namespace pbd {
static int train_pass(pbd_warmstart *w, const unsigned short *dx, const float4 *dt, int n,
                      int n_used, cudaStream_t s, double *loss_out) {
    float inv = n_used > 0 ? 1.f / (float)n_used : 0.f;
    PBD_CUDA(cudaMemsetAsync(w->loss.p, 0, sizeof(double) * 2, s));
    k_mlp_train<<<train_grid(n), kTile, kTrainSmem, s>>>(n, dx, dt, inv, w->wtiles.p, w->bias.p,
                                                          w->grad.p, w->loss.p, w->err.p);
    PBD_LAUNCH();
    if (loss_out) {
        double l = 0.0;
        PBD_CUDA(cudaMemcpyAsync(&l, w->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
        PBD_TRY(check_err(w, s));
        *loss_out = n_used > 0 ? 0.5 * l / n_used : 0.0;
    }
    return PBD_OK;
}

}  // namespace pbd

extern "C" {

int pbd_warmstart_gradients(pbd_warmstart *w, const float *x, const float *t, const float *mask,
                            int n, float *grad, double *loss) {
    PBD_CHECK(w && x && t && grad && n > 0, PBD_ERR_ARG, "bad argument");
    cudaStream_t s = w->own;
    DBuf<unsigned short> dx;
    DBuf<float4> dtg;
    PBD_TRY(upload_rows(w, x, n, dx));
    std::vector<float4> ht(n);
    int used = 0;
    for (int i = 0; i < n; ++i) {
        float mk = mask ? (mask[i] != 0.f ? 1.f : 0.f) : 1.f;
        used += mk != 0.f;
        ht[i] = make_float4(t[3 * i], t[3 * i + 1], t[3 * i + 2], mk);
    }
    PBD_TRY(dtg.upload(ht.data(), n, s));
    PBD_CUDA(cudaMemsetAsync(w->grad.p, 0, sizeof(float) * kWsParams, s));
    double l = 0.0;
    PBD_TRY(train_pass(w, dx.p, dtg.p, n, used, s, &l));
    PBD_CUDA(cudaMemcpyAsync(grad, w->grad.p, sizeof(float) * kWsParams, cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaMemsetAsync(w->grad.p, 0, sizeof(float) * kWsParams, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = l;
    return PBD_OK;
}

}  // extern "C"

namespace pbd {
static int adam_step(pbd_warmstart *w, cudaStream_t s, float lr, float b1, float b2, float eps) {
    ++w->adam_t;
    float c1 = (float)(1.0 / (1.0 - pow((double)b1, (double)w->adam_t)));
    float c2 = (float)(1.0 / (1.0 - pow((double)b2, (double)w->adam_t)));
    k_adam<<<grid_for(kWsParams, 256), 256, 0, s>>>(kWsParams, w->params.p, w->m.p, w->v.p,
                                                    w->grad.p, lr, b1, b2, eps, c1, c2);
    PBD_LAUNCH();
    return pack(w, s);
}

}  // namespace pbd

extern "C" {

int pbd_warmstart_adam(pbd_warmstart *w, float lr, float beta1, float beta2, float eps) {
    PBD_CHECK(w && lr >= 0.f, PBD_ERR_ARG, "bad argument");
    PBD_TRY(adam_step(w, w->own, lr, beta1, beta2, eps));
    PBD_CUDA(cudaStreamSynchronize(w->own));
    return PBD_OK;
}

int pbd_warmstart_set_gradient(pbd_warmstart *w, const float *grad, int n) {
    PBD_CHECK(w && grad && n == kWsParams, PBD_ERR_ARG, "bad argument");
    PBD_CUDA(cudaMemcpyAsync(w->grad.p, grad, sizeof(float) * n, cudaMemcpyHostToDevice, w->own));
    PBD_CUDA(cudaStreamSynchronize(w->own));
    return PBD_OK;
}

int pbd_warmstart_record(pbd_warmstart *w, pbd_object *o) {
    PBD_CHECK(w && o, PBD_ERR_ARG, "null argument");
    PBD_TRY(ws_prepare(w, o));
    cudaStream_t s = o->stream;
    PBD_CUDA(cudaMemcpyAsync(o->p0.p, o->p.p, sizeof(float4) * o->n, cudaMemcpyDeviceToDevice, s));
    PBD_TRY(ws_eval_hinges(o, o->p0.p));
    if (w->feat_cap < o->n) {
        PBD_TRY(w->feat.alloc(16 * (size_t)o->n));
        w->feat_cap = o->n;
    }
    k_features<<<grid_for(o->n, 256), 256, 0, s>>>(o->n, feat_args(o, o->p0.p, w), w->feat.p);
    PBD_LAUNCH();
    return PBD_OK;
}

int pbd_warmstart_train_step(pbd_warmstart *w, pbd_object *o, float lr, double *loss) {
    PBD_CHECK(w && o, PBD_ERR_ARG, "null argument");
    PBD_CHECK(o->feat_built && w->feat_cap >= o->n, PBD_ERR_STATE,
              "pbd_warmstart_record has not run on this object");
    cudaStream_t s = o->stream;
    PBD_TRY(w->tgt.alloc(o->n));
    k_targets<<<grid_for(o->n, 256), 256, 0, s>>>(o->n, o->p.p, o->p0.p, o->frest_b.p,
                                                  w->scale.p, w->tgt.p);
    PBD_LAUNCH();
    PBD_TRY(train_pass(w, w->feat.p, w->tgt.p, o->n, o->n_free, s, loss));
    PBD_TRY(adam_step(w, s, lr, 0.9f, 0.999f, 1e-8f));
    k_store_delta<<<grid_for(o->n, 256), 256, 0, s>>>(o->n, o->p.p, o->p0.p, o->dprev.p);
    PBD_LAUNCH();
    PBD_CUDA(cudaStreamSynchronize(s));
    return PBD_OK;
}

int pbd_warmstart_predict(pbd_warmstart *w, pbd_object *o) {
    PBD_CHECK(w && o, PBD_ERR_ARG, "null argument");
    PBD_TRY(ws_prepare(w, o));
    cudaStream_t s = o->stream;
    PBD_CUDA(cudaMemcpyAsync(o->p0.p, o->p.p, sizeof(float4) * o->n, cudaMemcpyDeviceToDevice, s));
    PBD_TRY(ws_eval_hinges(o, o->p0.p));
    PBD_TRY(ws_infer(w, o));
    return check_err(w, s);
}

int pbd_warmstart_features(pbd_warmstart *w, pbd_object *o, float *x) {
    PBD_CHECK(w && o && x, PBD_ERR_ARG, "null argument");
    PBD_TRY(ws_prepare(w, o));
    cudaStream_t s = o->stream;
    DBuf<unsigned short> f;
    PBD_TRY(f.alloc(16 * (size_t)o->n));
    PBD_TRY(ws_eval_hinges(o, o->p.p));
    k_features<<<grid_for(o->n, 256), 256, 0, s>>>(o->n, feat_args(o, o->p.p, w), f.p);
    PBD_LAUNCH();
    std::vector<unsigned short> h(16 * (size_t)o->n);
    PBD_CUDA(cudaMemcpyAsync(h.data(), f.p, sizeof(unsigned short) * h.size(), cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    for (size_t k = 0; k < h.size(); ++k) {
        uint32_t u = (uint32_t)h[k] << 16;
        memcpy(&x[k], &u, 4);
    }
    return PBD_OK;
}

int pbd_object_set_correction(pbd_object *o, const float *d) {
    PBD_CHECK(o && d, PBD_ERR_ARG, "null argument");
    if (!o->dprev.p) PBD_TRY(o->dprev.alloc(o->n));
    std::vector<float4> h(o->n);
    for (int i = 0; i < o->n; ++i) h[i] = make_float4(d[3 * i], d[3 * i + 1], d[3 * i + 2], 0.f);
    PBD_CUDA(cudaMemcpyAsync(o->dprev.p, h.data(), sizeof(float4) * o->n, cudaMemcpyHostToDevice, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    return PBD_OK;
}

int pbd_object_get_correction(pbd_object *o, float *d) {
    PBD_CHECK(o && d, PBD_ERR_ARG, "null argument");
    PBD_CHECK(o->dprev.p, PBD_ERR_STATE, "no correction recorded yet");
    std::vector<float4> h(o->n);
    PBD_CUDA(cudaMemcpyAsync(h.data(), o->dprev.p, sizeof(float4) * o->n, cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    for (int i = 0; i < o->n; ++i) {
        d[3 * i] = h[i].x;
        d[3 * i + 1] = h[i].y;
        d[3 * i + 2] = h[i].z;
    }
    return PBD_OK;
}

}  // extern "C"

// pbd_sort.cu -- stable LSD radix sort and exclusive scan used by the
// coloring sort (SortEdgesColors), the broadphase (triangles by cell bucket)
// and the contact ordering.
//
// One-sweep LSD radix sort with 8-bit digits (after Adinets & Merrill,
// "Onesweep: A Faster Least Significant Digit Radix Sort for GPUs", 2022):
// one kernel counts the digits of every pass in a single read of the keys;
// then one kernel per pass, whose blocks take 2048-key tiles in order from a
// counter, rank their keys stably inside the tile (warp match-any per
// 32-key round, warps in order), publish their per-digit tile counts and
// find the counts of all earlier tiles by decoupled look-back over the
// published words (count | status: aggregate, or inclusive prefix), then
// scatter.  A tile only waits for tiles taken before it by blocks already
// running, so every wait ends; each poll loop is still bounded and, should
// it run out, sets a sticky status word.  The element count may live on the
// device (d_count) so a sort can sit inside a CUDA graph whose sizes are only
// known on the GPU.
#include <algorithm>

#include "pbd_common.cuh"

namespace pbd {

namespace {
constexpr int kBlock = 256;
constexpr int kItems = 8;
constexpr int kTile = kBlock * kItems;
constexpr int kMaxPasses = 8;                 // 64-bit keys
constexpr unsigned kAggregate = 1u << 30, kPrefix = 2u << 30, kCountMask = (1u << 30) - 1u;
constexpr int kMaxPolls = 1 << 20;

__device__ __forceinline__ long long count_of(long long n_cap, const int *d_count) {
    if (!d_count) return n_cap;
    long long c = *d_count;
    return c < n_cap ? c : n_cap;
}

// A look-back word holds its count itself and guards no other data, so
// relaxed device-scope accesses suffice, and several loads can be in flight.
__device__ __forceinline__ void st_word(unsigned *p, unsigned v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_word(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
constexpr int kLookBatch = 8;  // earlier tiles' words loaded together

// digit counts of every pass (ghist[pass][digit], zeroed before), and the
// look-back words of the tiles this sort will use cleared
template <class K>
__global__ void __launch_bounds__(kBlock) k_digit_hist(const K *__restrict__ keys, long long n_cap,
                                                       const int *d_count, int npass,
                                                       long long ntiles_cap, int *ghist,
                                                       unsigned *flags) {
    __shared__ int h[kMaxPasses][256];
    for (int i = threadIdx.x; i < kMaxPasses * 256; i += kBlock) (&h[0][0])[i] = 0;
    __syncthreads();
    const long long n = count_of(n_cap, d_count);
    const long long stride = (long long)gridDim.x * kBlock;
    for (long long i = (long long)blockIdx.x * kBlock + threadIdx.x; i < n; i += stride) {
        const K k = keys[i];
        for (int q = 0; q < npass; ++q) atomicAdd(&h[q][(int)((k >> (8 * q)) & 255)], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npass * 256; i += kBlock) {
        const int v = (&h[0][0])[i];
        if (v) atomicAdd(ghist + i, v);
    }
    const long long ntiles = (n + kTile - 1) / kTile;
    for (int q = 0; q < npass; ++q)
        for (long long i = (long long)blockIdx.x * kBlock + threadIdx.x; i < ntiles * 256;
             i += stride)
            flags[(long long)q * ntiles_cap * 256 + i] = 0u;
}

// block-wide exclusive scan of one value per thread (blockDim multiple of 32)
__device__ __forceinline__ int block_exclusive(int x, int *warp_sums, int &total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int inc = x;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += y;
    }
    if (lane == 31) warp_sums[w] = inc;
    __syncthreads();
    if (w == 0) {
        int s = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, off);
            if (lane >= off) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    int excl = inc - x + (w > 0 ? warp_sums[w - 1] : 0);
    total = warp_sums[nw - 1];
    __syncthreads();
    return excl;
}

// one pass: ranks inside the tile, look-back for the earlier tiles' counts,
// scatter
template <class K>
__global__ void __launch_bounds__(kBlock) k_onesweep(
    const K *__restrict__ kin, const int *__restrict__ vin, K *__restrict__ kout,
    int *__restrict__ vout, long long n_cap, const int *d_count, int pass, long long ntiles_cap,
    const int *__restrict__ ghist, int *tile_ctr, unsigned *flags, int *status) {
    __shared__ int wh[kBlock / 32][256];
    __shared__ int boff[256];
    __shared__ int ws[32];
    __shared__ int tile_s;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int shift = 8 * pass;
    if (tid == 0) tile_s = atomicAdd(tile_ctr + pass, 1);
    for (int i = tid; i < (kBlock / 32) * 256; i += kBlock) (&wh[0][0])[i] = 0;
    __syncthreads();
    const long long n = count_of(n_cap, d_count);
    const int tile = tile_s;
    const long long tile0 = (long long)tile * kTile;
    if (tile0 >= n) return;
    const long long base = tile0 + (long long)w * (32 * kItems);
    K k[kItems];
    int v[kItems], d[kItems], r[kItems];
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        long long i = base + j * 32 + lane;
        if (i < n) {
            k[j] = kin[i];
            v[j] = vin[i];
            d[j] = (int)((k[j] >> shift) & 255);
        } else {
            d[j] = 256;
        }
    }
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        unsigned peers = __match_any_sync(0xffffffffu, d[j]);
        int before = __popc(peers & ((1u << lane) - 1u));
        int cnt = d[j] < 256 ? wh[w][d[j]] : 0;
        __syncwarp();
        if (d[j] < 256 && before == 0) wh[w][d[j]] += __popc(peers);
        __syncwarp();
        r[j] = cnt + before;
    }
    __syncthreads();
    // digit tid: warp offsets inside the tile, and the tile's count
    int c = 0;
#pragma unroll
    for (int ww = 0; ww < kBlock / 32; ++ww) {
        int t = wh[ww][tid];
        wh[ww][tid] = c;
        c += t;
    }
    const unsigned *col = flags + (long long)pass * ntiles_cap * 256 + tid;  // digit tid
    unsigned *mine = flags + ((long long)pass * ntiles_cap + tile) * 256 + tid;
    int excl = 0;
    if (tile == 0) {
        st_word(mine, kPrefix | (unsigned)c);
    } else {
        st_word(mine, kAggregate | (unsigned)c);
        // earlier tiles, nearest first, kLookBatch words per round trip,
        // until an inclusive prefix
        bool done = false;
        for (int pt = tile - 1; pt >= 0 && !done; pt -= kLookBatch) {
            unsigned fv[kLookBatch];
#pragma unroll
            for (int b = 0; b < kLookBatch; ++b)
                fv[b] = pt - b >= 0 ? ld_word(col + (long long)(pt - b) * 256) : 0u;
#pragma unroll
            for (int b = 0; b < kLookBatch; ++b) {
                if (done || pt - b < 0) break;
                unsigned v = fv[b];
                for (int polls = 0; !(v & ~kCountMask) && polls < kMaxPolls; ++polls)
                    v = ld_word(col + (long long)(pt - b) * 256);
                if (!(v & ~kCountMask)) {
                    atomicOr(status, 1);
                    done = true;
                    break;
                }
                excl += (int)(v & kCountMask);
                if (v & kPrefix) done = true;
            }
        }
        st_word(mine, kPrefix | (unsigned)(excl + c));
    }
    int tot;
    const int gbase = block_exclusive(ghist[pass * 256 + tid], ws, tot);
    boff[tid] = gbase + excl;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        if (d[j] < 256) {
            int pos = boff[d[j]] + wh[w][d[j]] + r[j];
            kout[pos] = k[j];
            vout[pos] = v[j];
        }
    }
}

// chunked single-block exclusive scan
__global__ void __launch_bounds__(1024) k_scan_single(const int *in, int *out, long long n,
                                                      int *total) {
    __shared__ int ws[32];
    int carry = 0;
    for (long long b0 = 0; b0 < n; b0 += 4096) {
        long long i0 = b0 + (long long)threadIdx.x * 4;
        int v[4];
        int local = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = (i0 + k < n) ? in[i0 + k] : 0;
            local += v[k];
        }
        int tot;
        int e = block_exclusive(local, ws, tot) + carry;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i0 + k < n) out[i0 + k] = e;
            e += v[k];
        }
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}
}  // namespace

int radix_reserve(SortScratch &scr, long long n_cap, int bits) {
    const int npass = (bits + 7) / 8;
    PBD_CHECK(npass <= kMaxPasses && n_cap < (1LL << 30), PBD_ERR_ARG,
              "radix sort of %lld keys with %d bits", n_cap, bits);
    const long long ntiles = std::max(1LL, (n_cap + kTile - 1) / kTile);
    PBD_TRY(scr.flags.alloc((size_t)std::max(npass, 1) * ntiles * 256));
    // ghist (kMaxPasses x 256), tile counters (kMaxPasses), status (1)
    if (!scr.aux.p) {
        PBD_TRY(scr.aux.alloc(kMaxPasses * 256 + kMaxPasses + 1));
        PBD_CUDA(cudaMemset(scr.aux.p, 0, sizeof(int) * scr.aux.n));
    }
    return PBD_OK;
}

int radix_status(const SortScratch &scr, cudaStream_t s, int *status) {
    *status = 0;
    if (!scr.aux.p) return PBD_OK;
    PBD_CUDA(cudaMemcpyAsync(status, scr.aux.p + kMaxPasses * 256 + kMaxPasses, sizeof(int),
                             cudaMemcpyDeviceToHost, s));
    PBD_CUDA(cudaStreamSynchronize(s));
    return PBD_OK;
}

template <class K>
int radix_sort(K *keys, int *vals, K *keys_alt, int *vals_alt, long long n_cap,
               const int *d_count, int bits, SortScratch &scr, cudaStream_t s, K **keys_out,
               int **vals_out) {
    *keys_out = keys;
    *vals_out = vals;
    if (n_cap <= 0 || bits <= 0) return PBD_OK;
    PBD_TRY(radix_reserve(scr, n_cap, bits));
    const int npass = (bits + 7) / 8;
    const long long ntiles = (n_cap + kTile - 1) / kTile;
    int *ghist = scr.aux.p, *tile_ctr = scr.aux.p + kMaxPasses * 256;
    int *status = tile_ctr + kMaxPasses;
    PBD_CUDA(cudaMemsetAsync(ghist, 0, sizeof(int) * (kMaxPasses * 256 + kMaxPasses), s));
    const int hblocks = (int)std::min<long long>(ntiles, 4 * kNumSMs);
    k_digit_hist<K><<<hblocks, kBlock, 0, s>>>(keys, n_cap, d_count, npass, ntiles, ghist,
                                               scr.flags.p);
    PBD_LAUNCH();
    K *ki = keys, *kb = keys_alt;
    int *vi = vals, *vb = vals_alt;
    for (int q = 0; q < npass; ++q) {
        k_onesweep<K><<<(int)ntiles, kBlock, 0, s>>>(ki, vi, kb, vb, n_cap, d_count, q, ntiles,
                                                      ghist, tile_ctr, scr.flags.p, status);
        PBD_LAUNCH();
        K *tk = ki; ki = kb; kb = tk;
        int *tv = vi; vi = vb; vb = tv;
    }
    *keys_out = ki;
    *vals_out = vi;
    return PBD_OK;
}

template int radix_sort<uint32_t>(uint32_t *, int *, uint32_t *, int *, long long, const int *,
                                  int, SortScratch &, cudaStream_t, uint32_t **, int **);
template int radix_sort<unsigned long long>(unsigned long long *, int *, unsigned long long *,
                                            int *, long long, const int *, int, SortScratch &,
                                            cudaStream_t, unsigned long long **, int **);

int exclusive_scan(const int *in, int *out, long long n, int *d_total, cudaStream_t s) {
    if (n <= 0) {
        if (d_total) PBD_CUDA(cudaMemsetAsync(d_total, 0, sizeof(int), s));
        return PBD_OK;
    }
    k_scan_single<<<1, 1024, 0, s>>>(in, out, n, d_total);
    PBD_LAUNCH();
    return PBD_OK;
}

}  // namespace pbd

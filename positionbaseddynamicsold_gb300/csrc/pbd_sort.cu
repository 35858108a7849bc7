// pbd_sort.cu -- stable LSD radix sort and exclusive scan used by the
// coloring sort (SortEdgesColors), the broadphase (triangles by cell bucket)
// and the contact ordering.
//
// Per 8-bit digit pass: an upsweep counts digits per 2048-key tile, 256
// blocks scan one digit's tile counts each, one block turns the digit totals
// into bases, and the downsweep ranks keys stably inside the tile (warp
// match-any per 32-key round, warps in order) and scatters.  The element
// count may live on the device (d_count) so passes can sit inside a CUDA
// graph whose sizes are only known on the GPU.
#include "pbd_common.cuh"

namespace pbd {

namespace {
constexpr int kBlock = 256;
constexpr int kItems = 8;
constexpr int kTile = kBlock * kItems;

__device__ __forceinline__ long long count_of(long long n_cap, const int *d_count) {
    if (!d_count) return n_cap;
    long long c = *d_count;
    return c < n_cap ? c : n_cap;
}

template <class K>
__global__ void __launch_bounds__(kBlock) k_upsweep(const K *__restrict__ keys, long long n_cap,
                                                    const int *d_count, int shift, int nblocks,
                                                    int *__restrict__ hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    long long n = count_of(n_cap, d_count);
    long long base = (long long)blockIdx.x * kTile;
    if (base < n) {
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            long long i = base + j * kBlock + threadIdx.x;
            if (i < n) atomicAdd(&h[(int)((keys[i] >> shift) & 255)], 1);
        }
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
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

// one block per digit: exclusive scan of that digit's counts over the
// active tiles, in place; the digit's total goes to totals[d]
__global__ void __launch_bounds__(kBlock) k_digit_scan(int *hist, int nblocks, long long n_cap,
                                                       const int *d_count, int *totals) {
    __shared__ int ws[32];
    long long n = count_of(n_cap, d_count);
    int nb = (int)((n + kTile - 1) / kTile);
    int *row = hist + (long long)blockIdx.x * nblocks;
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += kBlock) {
        int b = b0 + threadIdx.x;
        int x = b < nb ? row[b] : 0;
        int tot;
        int e = block_exclusive(x, ws, tot);
        if (b < nb) row[b] = e + carry;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kBlock) k_digit_base(int *totals) {
    __shared__ int ws[32];
    int tot;
    int e = block_exclusive(totals[threadIdx.x], ws, tot);
    totals[threadIdx.x] = e;
}

template <class K>
__global__ void __launch_bounds__(kBlock) k_downsweep(const K *__restrict__ kin,
                                                      const int *__restrict__ vin,
                                                      K *__restrict__ kout, int *__restrict__ vout,
                                                      long long n_cap, const int *d_count,
                                                      int shift, int nblocks,
                                                      const int *__restrict__ hist,
                                                      const int *__restrict__ base_of_digit) {
    __shared__ int wh[kBlock / 32][256];
    __shared__ int boff[256];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    long long n = count_of(n_cap, d_count);
    long long tile0 = (long long)blockIdx.x * kTile;
    if (tile0 >= n) return;
    for (int i = tid; i < (kBlock / 32) * 256; i += kBlock) (&wh[0][0])[i] = 0;
    boff[tid] = base_of_digit[tid] + hist[tid * nblocks + blockIdx.x];
    __syncthreads();
    long long base = tile0 + (long long)w * (32 * kItems);
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
    {
        int acc = 0;
#pragma unroll
        for (int ww = 0; ww < kBlock / 32; ++ww) {
            int t = wh[ww][tid];
            wh[ww][tid] = acc;
            acc += t;
        }
    }
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

int radix_hist_size(long long n_cap) {
    long long nb = (n_cap + kTile - 1) / kTile;
    if (nb < 1) nb = 1;
    return (int)(256 * nb);
}

template <class K>
int radix_sort(K *keys, int *vals, K *keys_alt, int *vals_alt, long long n_cap,
               const int *d_count, int bits, SortScratch &scr, cudaStream_t s, K **keys_out,
               int **vals_out) {
    *keys_out = keys;
    *vals_out = vals;
    if (n_cap <= 0 || bits <= 0) return PBD_OK;
    int nblocks = (int)((n_cap + kTile - 1) / kTile);
    PBD_TRY(scr.hist.alloc((size_t)256 * nblocks));
    PBD_TRY(scr.carry.alloc(256));
    K *ki = keys, *kb = keys_alt;
    int *vi = vals, *vb = vals_alt;
    for (int shift = 0; shift < bits; shift += 8) {
        k_upsweep<K><<<nblocks, kBlock, 0, s>>>(ki, n_cap, d_count, shift, nblocks, scr.hist.p);
        k_digit_scan<<<256, kBlock, 0, s>>>(scr.hist.p, nblocks, n_cap, d_count, scr.carry.p);
        k_digit_base<<<1, kBlock, 0, s>>>(scr.carry.p);
        k_downsweep<K><<<nblocks, kBlock, 0, s>>>(ki, vi, kb, vb, n_cap, d_count, shift, nblocks,
                                                  scr.hist.p, scr.carry.p);
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

// Device-wide scan and stable LSD radix sort (see prims.cuh).
#include "prims.cuh"

#include "common.cuh"

namespace sbp {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanChunk = kScanThreads * kScanItems;  // 2048

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per tile
constexpr int kWarps = kSortThreads / 32;

thread_local int64_t g_launches = 0;

// Block-wide exclusive scan of one int per thread; returns the block total.
__device__ __forceinline__ int block_exclusive_scan(int x, int* warp_tot, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int v = lane < nw ? warp_tot[lane] : 0;
        int vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(SBP_FULL_MASK, vi, o);
            if (lane >= o) vi += y;
        }
        if (lane < nw) warp_tot[lane] = vi - v;
        if (lane == nw - 1) *total = vi;
    }
    __syncthreads();
    const int res = incl - x + warp_tot[wid];
    __syncthreads();
    return res;
}

__global__ void k_scan_reduce(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ partials) {
    const int64_t base = (int64_t)blockIdx.x * kScanChunk;
    int s = 0;
    for (int i = threadIdx.x; i < kScanChunk; i += kScanThreads) {
        const int64_t j = base + i;
        if (j < n) s += in[j];
    }
    s = warp_sum_i(s);
    __shared__ int ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += ws[w];
        partials[blockIdx.x] = t;
    }
}

// Single block: exclusive scan of partials[0..np) in place; total to *d_total.
__global__ void k_scan_partials(int32_t* __restrict__ partials, int64_t np, int32_t* __restrict__ d_total) {
    __shared__ int warp_tot[32];
    __shared__ int total;
    int carry = 0;
    for (int64_t base = 0; base < np; base += blockDim.x) {
        const int64_t j = base + threadIdx.x;
        const int x = j < np ? partials[j] : 0;
        const int ex = block_exclusive_scan(x, warp_tot, &total);
        if (j < np) partials[j] = carry + ex;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && d_total) *d_total = carry;
}

__global__ void k_scan_down(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                            const int32_t* __restrict__ partials, bool inclusive) {
    __shared__ int buf[kScanChunk];
    __shared__ int warp_tot[32];
    __shared__ int total;
    const int64_t base = (int64_t)blockIdx.x * kScanChunk;
    for (int i = threadIdx.x; i < kScanChunk; i += kScanThreads) {
        const int64_t j = base + i;
        buf[i] = j < n ? in[j] : 0;
    }
    __syncthreads();
    int loc[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        loc[k] = buf[threadIdx.x * kScanItems + k];
        s += loc[k];
    }
    int ex = block_exclusive_scan(s, warp_tot, &total) + partials[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int v = loc[k];
        buf[threadIdx.x * kScanItems + k] = inclusive ? ex + v : ex;
        ex += v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kScanChunk; i += kScanThreads) {
        const int64_t j = base + i;
        if (j < n) out[j] = buf[i];
    }
}

__global__ void k_radix_hist(const uint64_t* __restrict__ keys, int64_t n, int shift, int32_t* __restrict__ hist,
                             int64_t num_tiles) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += kSortThreads) {
        const int64_t j = base + i;
        if (j < n) atomicAdd(&h[(int)((keys[j] >> shift) & 0xff)], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * num_tiles + blockIdx.x] = h[threadIdx.x];
}

template <bool kVals>
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint64_t* __restrict__ keys,
                                                                const int32_t* __restrict__ vals, int64_t n,
                                                                int shift, const int32_t* __restrict__ offsets,
                                                                int64_t num_tiles, uint64_t* __restrict__ okeys,
                                                                int32_t* __restrict__ ovals) {
    __shared__ int wcnt[kWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * 256; i += kSortThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile + (int64_t)w * (32 * kSortItems);
    uint64_t k[kSortItems];
    int32_t v[kSortItems];
    int d[kSortItems];
    int rank[kSortItems];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const int64_t idx = base + j * 32 + lane;
        const bool valid = idx < n;
        k[j] = valid ? keys[idx] : 0ull;
        if (kVals) v[j] = valid ? vals[idx] : 0;
        d[j] = valid ? (int)((k[j] >> shift) & 0xff) : 256;
        const unsigned peers = __match_any_sync(SBP_FULL_MASK, d[j]);
        const int leader = __ffs(peers) - 1;
        int cur = 0;
        if (d[j] < 256) cur = wcnt[w][d[j]];
        rank[j] = cur + __popc(peers & lt);
        __syncwarp();
        if (lane == leader && d[j] < 256) wcnt[w][d[j]] = cur + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const int dig = threadIdx.x;  // 256 threads, one digit each
        int run = 0;
#pragma unroll
        for (int ww = 0; ww < kWarps; ++ww) {
            const int c = wcnt[ww][dig];
            wcnt[ww][dig] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        if (d[j] < 256) {
            const int64_t pos = (int64_t)offsets[(int64_t)d[j] * num_tiles + blockIdx.x] + wcnt[w][d[j]] + rank[j];
            okeys[pos] = k[j];
            if (kVals) ovals[pos] = v[j];
        }
    }
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace

int64_t prims_launch_count() { return g_launches; }

size_t scan_temp_bytes(int64_t n) {
    const int64_t nb = ceil_div(n > 0 ? n : 1, kScanChunk);
    return (size_t)(nb + 64) * sizeof(int32_t);
}

void scan_i32(const int32_t* in, int32_t* out, int64_t n, bool inclusive, int32_t* d_total, void* temp,
              cudaStream_t st) {
    if (n <= 0) {
        if (d_total) cudaMemsetAsync(d_total, 0, sizeof(int32_t), st);
        return;
    }
    const int64_t nb = ceil_div(n, kScanChunk);
    int32_t* partials = static_cast<int32_t*>(temp);
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, partials);
    k_scan_partials<<<1, 1024, 0, st>>>(partials, nb, d_total);
    k_scan_down<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, partials, inclusive);
    g_launches += 3;
}

size_t radix_temp_bytes(int64_t n) {
    const int64_t tiles = ceil_div(n > 0 ? n : 1, kSortTile);
    const int64_t hist = 256 * tiles;
    return (size_t)hist * sizeof(int32_t) + scan_temp_bytes(hist) + 256;
}

void radix_sort_u64(uint64_t* keys, uint64_t* keys_alt, int32_t* vals, int32_t* vals_alt, int64_t n, int end_bit,
                    void* temp, cudaStream_t st) {
    if (n <= 1 || end_bit <= 0) return;
    const int64_t tiles = ceil_div(n, kSortTile);
    const int64_t hist_n = 256 * tiles;
    int32_t* hist = static_cast<int32_t*>(temp);
    void* scan_tmp = reinterpret_cast<char*>(temp) + ((hist_n * sizeof(int32_t) + 255) / 256) * 256;
    uint64_t* src_k = keys;
    uint64_t* dst_k = keys_alt;
    int32_t* src_v = vals;
    int32_t* dst_v = vals_alt;
    int passes = 0;
    for (int shift = 0; shift < end_bit; shift += 8, ++passes) {
        k_radix_hist<<<(unsigned)tiles, kSortThreads, 0, st>>>(src_k, n, shift, hist, tiles);
        scan_i32(hist, hist, hist_n, false, nullptr, scan_tmp, st);
        if (vals)
            k_radix_scatter<true><<<(unsigned)tiles, kSortThreads, 0, st>>>(src_k, src_v, n, shift, hist, tiles,
                                                                            dst_k, dst_v);
        else
            k_radix_scatter<false><<<(unsigned)tiles, kSortThreads, 0, st>>>(src_k, nullptr, n, shift, hist,
                                                                             tiles, dst_k, nullptr);
        g_launches += 2;
        uint64_t* tk = src_k;
        src_k = dst_k;
        dst_k = tk;
        int32_t* tv = src_v;
        src_v = dst_v;
        dst_v = tv;
    }
    if (passes & 1) {
        cudaMemcpyAsync(keys, keys_alt, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
        if (vals) cudaMemcpyAsync(vals, vals_alt, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    }
}

}  // namespace sbp

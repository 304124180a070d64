// Degree-corrected nonparametric terms on the device (args.degreecorrected; reference
// include/entropy.hpp:117-133, src/entropy.cpp:617-764, :994-1110).
//
// With degree correction the nonparametric description length gains
//   * get_deg_entropy: -lgamma(k_in + 1) - lgamma(k_out + 1) per vertex, k the sizes of
//     its neighbour lists (self-loops in both);
//   * get_deg_dl_dist: per block log_q(d_out, size) + log_q(d_in, size), minus
//     lgamma(count + 1) over the block's in-degree (directed only) and out-degree
//     histograms, plus lgamma(size + 1) twice (once when undirected),
// and a vertex move's delta gains get_delta_deg_dl, the change of those per-block terms
// for the vertex's two blocks.  (The vterm's change to lgamma of the block degrees is in
// np.cuh.)  The histograms are those of Blockmodel's constructor for the current
// assignment (blockmodel.cpp:209-235), counted here into two open-addressing tables keyed
// by (block, degree).  log_q -- the Szekeres asymptotic of the number of partitions of n
// into at most k parts, through the dilogarithm -- is computed in double per term and
// rounded to 2^-24 like every other nonparametric term, so sums stay exact and order-free.
//
// Bound: evaluation only (the description length and vertex-move deltas of a blockmodel);
// one pass over the vertices to count, one over the table slots and blocks to sum.
#include <cmath>
#include <new>
#include <stdexcept>
#include <vector>

#include "kernels.cuh"
#include "np.cuh"

namespace sbp {

namespace {

constexpr int kDcT = 256;
constexpr double kFixD = 16777216.0;  // 2^24

// Li2(z) = sum z^k / k^2 for 0 <= z <= 1/2; Euler's reflection
// Li2(z) = pi^2/6 - log(z) log(1 - z) - Li2(1 - z) above; Li2(1) = pi^2/6.
__device__ double li2_series(double z) {
    double sum = 0.0, p = z;
    for (int k = 1; k <= 200; ++k) {
        const double t = p / ((double)k * (double)k);
        sum += t;
        if (t <= 1e-18 * sum) break;
        p *= z;
    }
    return sum;
}
__device__ double dc_li2(double z) {
    const double pi2_6 = 1.6449340668482264;  // pi^2 / 6
    if (z >= 1.0) return pi2_6;
    if (z > 0.5) return pi2_6 - log(z) * log1p(-z) - li2_series(1.0 - z);
    return li2_series(z);
}
// get_v (entropy.cpp:677-686): v = u sqrt(spence(e^-v)) iterated to within 1e-8, with
// spence(x) = Li2(1 - x) and 1 - e^-v formed as -expm1(-v).
__device__ double dc_get_v(double u) {
    double v = u, delta = 1.0;
    for (int it = 0; delta > 1e-8 && it < 100000; ++it) {
        const double nv = u * sqrt(dc_li2(-expm1(-v)));
        delta = fabs(nv - v);
        v = nv;
    }
    return v;
}
// fastlbinom (entropy.hpp:144-148) in double.
__device__ double dc_lbinom(long long N, long long k) {
    if (N == 0 || k == 0 || k > N) return 0.0;
    return (lgamma((double)(N + 1)) - lgamma((double)(k + 1))) - lgamma((double)(N - k + 1));
}
// log_q (entropy.cpp:688-707).
__device__ double dc_log_q(long long n, long long k) {
    if (n <= 0 || k < 1) return 0.0;
    if (k > n) k = n;
    if ((double)k < pow((double)n, 0.25)) return dc_lbinom(n - 1, k - 1) - lgamma((double)(k + 1));
    const double u = (double)k / sqrt((double)n);
    const double v = dc_get_v(u);
    const double lf = log(v) - log1p(-exp(-v) * (1 + u * u / 2)) / 2 - log(2.0) * 3 / 2. - log(u) -
                      log(3.141592653589793);
    const double gg = 2 * v / u - u * log1p(-exp(-v));
    return lf - log((double)n) + sqrt((double)n) * gg;
}
__device__ __forceinline__ long long dc_fix(double x) { return llrint(x * kFixD); }

__device__ __forceinline__ int32_t dc_kout(const DevGraph& g, int32_t v) {
    return __ldg(g.out_off + v + 1) - __ldg(g.out_off + v);
}
// in-neighbour list size with self-loops (the graph keeps them apart)
__device__ __forceinline__ int32_t dc_kin(const DevGraph& g, int32_t v) {
    return __ldg(g.inns_off + v + 1) - __ldg(g.inns_off + v) + __ldg(g.selfcnt + v);
}

__device__ __forceinline__ uint32_t dc_hash(uint64_t key, uint32_t mask) {
    key ^= key >> 31;
    key *= 0x9e3779b97f4a7c15ull;
    key ^= key >> 29;
    return (uint32_t)key & mask;
}
// (block, degree) -> table key; 0 marks an empty slot
__device__ __forceinline__ uint64_t dc_key(int32_t b, int32_t k) {
    return ((uint64_t)(uint32_t)(b + 1) << 32) | (uint32_t)k;
}
__device__ void dc_insert(uint64_t* keys, int32_t* cnt, uint32_t mask, uint64_t key) {
    uint32_t s = dc_hash(key, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS((unsigned long long*)(keys + s), 0ull, (unsigned long long)key);
        if (prev == 0ull || prev == key) {
            atomicAdd(cnt + s, 1);
            return;
        }
        s = (s + 1) & mask;
    }
}
__device__ int32_t dc_lookup(const uint64_t* keys, const int32_t* cnt, uint32_t mask, uint64_t key) {
    uint32_t s = dc_hash(key, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint64_t k = keys[s];
        if (k == key) return cnt[s];
        if (k == 0) return 0;
        s = (s + 1) & mask;
    }
    return 0;
}

struct DcTables {
    uint64_t* in_keys;
    int32_t* in_cnt;
    uint64_t* out_keys;
    int32_t* out_cnt;
    uint32_t mask;
};

__global__ void k_dc_count(DevGraph g, DevBM bm, DcTables t) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < g.N; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = bm.asg[v];
        dc_insert(t.in_keys, t.in_cnt, t.mask, dc_key(b, dc_kin(g, (int32_t)v)));
        dc_insert(t.out_keys, t.out_cnt, t.mask, dc_key(b, dc_kout(g, (int32_t)v)));
    }
}

__device__ __forceinline__ void dc_block_add(unsigned long long* out, long long acc) {
    acc = warp_sum_ll(acc);
    __shared__ long long ws[kDcT / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int i = 0; i < kDcT / 32; ++i) s += ws[i];
        atomicAdd(out, (unsigned long long)s);
    }
}

// The degree-corrected additions to the description length, in units of 2^-24: the
// vertices' degree entropies, each block's log_q and size terms, and the histogram terms.
__global__ void __launch_bounds__(kDcT) k_dc_mdl(DevGraph g, DevBM bm, DcTables t, unsigned long long* out) {
    long long acc = 0;
    const int64_t slots = (int64_t)t.mask + 1;
    const int64_t n = max(max((int64_t)g.N, (int64_t)bm.B), slots);
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        if (j < g.N) acc -= np_lg(g, dc_kin(g, (int32_t)j)) + np_lg(g, dc_kout(g, (int32_t)j));
        if (j < bm.B) {
            const int32_t size = bm.sizes[j];
            acc += dc_fix(dc_log_q(bm.d_out[j], size)) + dc_fix(dc_log_q(bm.d_in[j], size));
            acc += (g.np_und ? 1 : 2) * np_lg(g, size);
        }
        if (j < slots) {
            if (!g.np_und && t.in_keys[j] != 0) acc -= np_lg(g, t.in_cnt[j]);
            if (t.out_keys[j] != 0) acc -= np_lg(g, t.out_cnt[j]);
        }
    }
    dc_block_add(out, acc);
}

// get_delta_deg_dl_dist_change (entropy.cpp:994-1070): a vertex with degrees (kin, kout)
// leaving (diff = -1) or joining (+1) block b, in units of 2^-24.
__device__ long long dc_change(const DevGraph& g, const DevBM& bm, const DcTables& t, int32_t b, int32_t kin,
                               int32_t kout, int diff) {
    const long long total = bm.sizes[b], ep = bm.d_out[b], em = bm.d_in[b];
    long long d = 0;
    if (!g.np_und) {
        const int32_t nd = dc_lookup(t.in_keys, t.in_cnt, t.mask, dc_key(b, kin));
        d -= np_lg(g, nd + diff) - np_lg(g, nd);
    }
    const int32_t nd = dc_lookup(t.out_keys, t.out_cnt, t.mask, dc_key(b, kout));
    d -= np_lg(g, nd + diff) - np_lg(g, nd);
    d += dc_fix(dc_log_q(em + diff * kin, total + diff)) - dc_fix(dc_log_q(em, total));
    d += dc_fix(dc_log_q(ep + diff * kout, total + diff)) - dc_fix(dc_log_q(ep, total));
    d += (g.np_und ? 1 : 2) * (np_lg(g, total + diff) - np_lg(g, total));
    return d;
}

// Adds get_delta_deg_dl (entropy.cpp:1072-1109) to each vertex move's delta.
__global__ void k_dc_vertex(DevGraph g, DevBM bm, DcTables t, const int32_t* __restrict__ vs,
                            const int32_t* __restrict__ ss, int64_t n, long long* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = vs[i], s = ss[i], r = bm.asg[v];
        if (r == s) continue;
        const int32_t kin = dc_kin(g, v), kout = dc_kout(g, v);
        out[i] += dc_change(g, bm, t, r, kin, kout, -1) + dc_change(g, bm, t, s, kin, kout, +1);
    }
}

unsigned dc_grid(int64_t n) {
    int64_t b = (n + kDcT - 1) / kDcT;
    if (b < 1) b = 1;
    if (b > (int64_t)device_sms() * 16) b = (int64_t)device_sms() * 16;
    return (unsigned)b;
}

// The histogram tables of the current assignment, on stream-ordered temporaries.
DcTables dc_tables(const DevGraph& g, const DevBM& bm, std::vector<void*>& tmp, cudaStream_t st) {
    uint64_t cap = 1;
    while (cap < 2 * (uint64_t)g.N + 2) cap <<= 1;
    DcTables t{};
    t.mask = (uint32_t)(cap - 1);
    void* p[4] = {nullptr, nullptr, nullptr, nullptr};
    const size_t bytes[4] = {cap * 8, cap * 4, cap * 8, cap * 4};
    for (int i = 0; i < 4; ++i) {  // the caller frees tmp, also when this throws
        if (cudaMallocAsync(&p[i], bytes[i], st) != cudaSuccess) {
            cudaGetLastError();
            throw std::bad_alloc();
        }
        tmp.push_back(p[i]);
        if (cudaMemsetAsync(p[i], 0, bytes[i], st) != cudaSuccess)
            throw std::runtime_error("degree histogram tables: cudaMemsetAsync failed");
    }
    t.in_keys = static_cast<uint64_t*>(p[0]);
    t.in_cnt = static_cast<int32_t*>(p[1]);
    t.out_keys = static_cast<uint64_t*>(p[2]);
    t.out_cnt = static_cast<int32_t*>(p[3]);
    k_dc_count<<<dc_grid(g.N), kDcT, 0, st>>>(g, bm, t);
    count_launches(1);
    return t;
}

void dc_free(std::vector<void*>& tmp, cudaStream_t st) {
    for (void* q : tmp) cudaFreeAsync(q, st);
    tmp.clear();
}

}  // namespace

void launch_dc_mdl(const DevGraph& g, const DevBM& bm, unsigned long long* acc, cudaStream_t st) {
    std::vector<void*> tmp;
    try {
        const DcTables t = dc_tables(g, bm, tmp, st);
        const int64_t n = std::max<int64_t>(std::max<int64_t>(g.N, bm.B), (int64_t)t.mask + 1);
        k_dc_mdl<<<dc_grid(n), kDcT, 0, st>>>(g, bm, t, acc);
        count_launches(1);
    } catch (...) {
        dc_free(tmp, st);
        throw;
    }
    dc_free(tmp, st);
}

void launch_dc_vertex_deltas(const DevGraph& g, const DevBM& bm, const int32_t* v, const int32_t* s, int64_t n,
                             long long* out, cudaStream_t st) {
    if (n <= 0) return;
    std::vector<void*> tmp;
    try {
        const DcTables t = dc_tables(g, bm, tmp, st);
        k_dc_vertex<<<dc_grid(n), kDcT, 0, st>>>(g, bm, t, v, s, n, out);
        count_launches(1);
    } catch (...) {
        dc_free(tmp, st);
        throw;
    }
    dc_free(tmp, st);
}

}  // namespace sbp

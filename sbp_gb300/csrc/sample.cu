// Sampling and extension on the device (reference src/sample.cpp, src/main.cpp:98-140):
// choose a vertex sample, cut the sampled subgraph out of the graph, and extend a
// partition of the sample back to every vertex.
//
//  * max_degree (sample.cpp:255-270): a stable descending sort of the vertex degrees, as
//    one 64-bit radix sort of (~degree, vertex).
//  * random (:272-284): the canonical shuffle (domain 6) of the vertex ids.
//  * degree_product (:28-49): the edges in source order sorted stably by descending
//    degree product; the reference walks them, numbering each endpoint at its first
//    appearance, and stops after the edge at which the count reaches the target.  Here
//    every vertex gets the position of its first appearance (an atomic minimum over the
//    sorted edges), the vertices are ordered by it, and the cut is the edge holding the
//    target-th first appearance.
//  * detach (:12-26): vertices of degree above 1, numbered in id order by a scan.
//  * from_vertices (:240-253): the out-CSR slots whose two endpoints are sampled, in CSR
//    order (by source id, each source's neighbours in order), compacted by a scan.
//  * extend (:159-199): the reference assigns the unsampled vertices one at a time in id
//    order, each to the block most of its already-assigned neighbours are in.  A vertex's
//    result depends only on its neighbours of smaller id that were unsampled, so the
//    vertices are assigned in waves: a vertex is ready once none of those is pending, and
//    two ready vertices are never neighbours.  Ties go to the smallest block (the
//    reference iterates a hash map); a vertex without assigned neighbours draws its block
//    from the canonical stream (domain 7).
//  * expansion_snowball and degree_product_snowball (:51-157) grow the sample one vertex at
//    a time from a frontier; they run on the host over a copy of the adjacency, with the
//    k-th random draw of a run taken from the canonical stream (domain 11).
//  * reattach (:365-405) for the detached vertices (degree 0 or 1): a vertex with an
//    assigned neighbour takes its block; a vertex whose one neighbour is detached as well
//    shares the block drawn for the smaller of the two (domain 10).
#include <climits>
#include <queue>
#include <set>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "delta.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace sbp {

// Philox4x32-10 on the host, the same stream as the device's philox4x32_10.
void philox_host(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint64_t seed, uint32_t w[4]) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0;
        c1 = (uint32_t)p1;
        c2 = n2;
        c3 = (uint32_t)p0;
    }
    w[0] = c0;
    w[1] = c1;
    w[2] = c2;
    w[3] = c3;
}

// Out-lists in input order; in-lists with each self-loop as the vertex itself.
HostAdjacency host_adjacency(const DevGraph& g, cudaStream_t st) {
    const int64_t N = g.N, E = g.E;
    HostAdjacency a;
    std::vector<int32_t> inns_off(N + 1), self(N), inns;
    a.out_off.resize(N + 1);
    a.out_nbr.resize(E);
    cudaMemcpyAsync(a.out_off.data(), g.out_off, (N + 1) * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(inns_off.data(), g.inns_off, (N + 1) * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(self.data(), g.selfcnt, N * 4, cudaMemcpyDeviceToHost, st);
    if (E) cudaMemcpyAsync(a.out_nbr.data(), g.out_nbr, E * 4, cudaMemcpyDeviceToHost, st);
    host_wait(st);
    inns.resize(inns_off[N]);
    if (!inns.empty()) cudaMemcpyAsync(inns.data(), g.inns_nbr, inns.size() * 4, cudaMemcpyDeviceToHost, st);
    host_wait(st);
    a.in_off.assign(N + 1, 0);
    for (int64_t v = 0; v < N; ++v) a.in_off[v + 1] = a.in_off[v] + (inns_off[v + 1] - inns_off[v]) + self[v];
    a.in_nbr.resize(a.in_off[N]);
    a.deg.resize(N);
    for (int64_t v = 0; v < N; ++v) {
        int32_t o = a.in_off[v];
        for (int32_t j = inns_off[v]; j < inns_off[v + 1]; ++j) a.in_nbr[o++] = inns[j];
        for (int32_t j = 0; j < self[v]; ++j) a.in_nbr[o++] = (int32_t)v;
        a.deg[v] = (a.out_off[v + 1] - a.out_off[v]) + (a.in_off[v + 1] - a.in_off[v]) - (self[v] > 0 ? 1 : 0);
    }
    return a;
}

namespace {

enum : uint32_t { DOM_SAMPLE = 6, DOM_EXTEND = 7 };

unsigned grid_of(int64_t n, int per = 256) {
    int64_t b = (n + per - 1) / per;
    if (b < 1) b = 1;
    if (b > (int64_t)device_sms() * 16) b = (int64_t)device_sms() * 16;
    return (unsigned)b;
}

// Graph::degrees (graph.cpp:24-31): out + in - (has a self-loop).
__device__ __forceinline__ int32_t vertex_degree(const DevGraph& g, int32_t v) {
    const int32_t self = __ldg(g.selfcnt + v);
    return (__ldg(g.out_off + v + 1) - __ldg(g.out_off + v)) + (__ldg(g.inns_off + v + 1) - __ldg(g.inns_off + v)) +
           self - (self > 0 ? 1 : 0);
}

__global__ void k_degree_keys(DevGraph g, uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.N; v += gridDim.x * blockDim.x) {
        keys[v] = ((uint64_t)(0xffffffffu - (uint32_t)vertex_degree(g, v)) << 32) | (uint32_t)v;
        vals[v] = v;
    }
}

// mapping[order[i]] = i for i < n.
__global__ void k_number(const int32_t* __restrict__ order, int64_t n, int32_t* __restrict__ mapping) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        mapping[order[i]] = (int32_t)i;
}

__global__ void k_edge_info_keys(DevGraph g, uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.E; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t info = (uint64_t)vertex_degree(g, __ldg(g.esrc + e)) * (uint64_t)vertex_degree(g, __ldg(g.out_nbr + e));
        keys[e] = ~info;  // ascending ~info = descending info; the sort is stable
        vals[e] = (int32_t)e;
    }
}

__global__ void k_first_seen(DevGraph g, const int32_t* __restrict__ sorted_edges, int32_t* __restrict__ first) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < g.E; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t e = sorted_edges[i];
        atomicMin(first + __ldg(g.esrc + e), (int32_t)(2 * i));
        atomicMin(first + __ldg(g.out_nbr + e), (int32_t)(2 * i + 1));
    }
}

__global__ void k_first_keys(const int32_t* __restrict__ first, int32_t N, uint64_t* __restrict__ keys,
                             int32_t* __restrict__ vals) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
        keys[v] = ((uint64_t)(uint32_t)first[v] << 32) | (uint32_t)v;
        vals[v] = v;
    }
}

// Vertices whose first appearance is at most `cut`, numbered in order of appearance
// (keys sorted ascending by (first, vertex)).
__global__ void k_number_first(const uint64_t* __restrict__ keys, const int32_t* __restrict__ vals, int32_t N,
                               uint32_t cut, int32_t* __restrict__ mapping) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        if ((uint32_t)(keys[i] >> 32) <= cut) mapping[vals[i]] = i;
}

// Number of sorted keys whose first appearance is at most `cut`.
__global__ void k_count_upto(const uint64_t* __restrict__ keys, int32_t N, uint32_t cut, int32_t* __restrict__ n) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        if ((uint32_t)(keys[i] >> 32) <= cut) atomicMax(n, i + 1);
}

__global__ void k_degree_flags(DevGraph g, int32_t* __restrict__ flags) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.N; v += gridDim.x * blockDim.x)
        flags[v] = vertex_degree(g, v) > 1 ? 1 : 0;
}

__global__ void k_number_flagged(const int32_t* __restrict__ flags, const int32_t* __restrict__ pos, int32_t N,
                                 int32_t* __restrict__ mapping) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x)
        mapping[v] = flags[v] ? pos[v] : -1;
}

__global__ void k_sub_flags(DevGraph g, const int32_t* __restrict__ mapping, int32_t* __restrict__ flags) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.E; e += (int64_t)gridDim.x * blockDim.x)
        flags[e] = (mapping[__ldg(g.esrc + e)] >= 0 && mapping[__ldg(g.out_nbr + e)] >= 0) ? 1 : 0;
}

__global__ void k_sub_edges(DevGraph g, const int32_t* __restrict__ mapping, const int32_t* __restrict__ flags,
                            const int32_t* __restrict__ pos, int32_t* __restrict__ src, int32_t* __restrict__ dst) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.E; e += (int64_t)gridDim.x * blockDim.x)
        if (flags[e]) {
            src[pos[e]] = mapping[__ldg(g.esrc + e)];
            dst[pos[e]] = mapping[__ldg(g.out_nbr + e)];
        }
}

// ---- extend
__global__ void k_extend_init(const int32_t* __restrict__ mapping, const int32_t* __restrict__ sample_asg, int32_t N,
                              int32_t* __restrict__ asg, int32_t* __restrict__ pending, int32_t* __restrict__ npending) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
        const int32_t m = mapping[v];
        asg[v] = m >= 0 ? sample_asg[m] : -1;
        if (m < 0) pending[atomicAdd(npending, 1)] = v;
    }
}

// Splits the pending list into the vertices that can be assigned now and the rest.
__global__ void k_extend_ready(DevGraph g, const int32_t* __restrict__ asg, const int32_t* __restrict__ pending,
                               int32_t np, int32_t* __restrict__ ready, int32_t* __restrict__ nready,
                               int32_t* __restrict__ rest, int32_t* __restrict__ nrest) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int32_t v = pending[i];
        bool ok = true;
        for (int32_t j = __ldg(g.out_off + v); ok && j < __ldg(g.out_off + v + 1); ++j) {
            const int32_t u = __ldg(g.out_nbr + j);
            ok = !(u < v && asg[u] < 0);
        }
        for (int32_t j = __ldg(g.inns_off + v); ok && j < __ldg(g.inns_off + v + 1); ++j) {
            const int32_t u = __ldg(g.inns_nbr + j);
            ok = !(u < v && asg[u] < 0);
        }
        if (ok) ready[atomicAdd(nready, 1)] = v;
        else rest[atomicAdd(nrest, 1)] = v;
    }
}

// One CTA per ready vertex: counts of its assigned neighbours' blocks in a shared hash,
// then the block with the largest count (smallest id among equals).
__global__ void k_extend_assign(DevGraph g, int32_t* __restrict__ asg, const int32_t* __restrict__ ready, int32_t nr,
                                int32_t B, uint64_t seed, int log2cap) {
    extern __shared__ int32_t sh[];
    const int cap = 1 << log2cap;
    int32_t* hk = sh;
    int32_t* hc = sh + cap;
    __shared__ unsigned long long best;
    for (int32_t i = blockIdx.x; i < nr; i += gridDim.x) {
        const int32_t v = ready[i];
        for (int j = threadIdx.x; j < cap; j += blockDim.x) {
            hk[j] = -1;
            hc[j] = 0;
        }
        if (threadIdx.x == 0) best = 0ull;
        __syncthreads();
        for (int32_t j = __ldg(g.out_off + v) + threadIdx.x; j < __ldg(g.out_off + v + 1); j += blockDim.x) {
            const int32_t b = asg[__ldg(g.out_nbr + j)];
            if (b >= 0) hinsert(hk, hc, log2cap, b);
        }
        for (int32_t j = __ldg(g.inns_off + v) + threadIdx.x; j < __ldg(g.inns_off + v + 1); j += blockDim.x) {
            const int32_t b = asg[__ldg(g.inns_nbr + j)];
            if (b >= 0) hinsert(hk, hc, log2cap, b);
        }
        __syncthreads();
        // pack (count, ~block): the maximum has the largest count, then the smallest block
        for (int j = threadIdx.x; j < cap; j += blockDim.x)
            if (hk[j] >= 0)
                atomicMax(&best, ((unsigned long long)(uint32_t)hc[j] << 32) | (uint32_t)(0x7fffffff - hk[j]));
        __syncthreads();
        if (threadIdx.x == 0) {
            int32_t b;
            if (best == 0ull) {
                uint32_t w[4];
                philox4x32_10((uint32_t)v, 0u, 0u, DOM_EXTEND, seed, w);
                b = (int32_t)u32_below(w[0], (uint32_t)B);
            } else {
                b = 0x7fffffff - (int32_t)(uint32_t)(best & 0xffffffffull);
            }
            asg[v] = b;
        }
        __syncthreads();
    }
}

// ---- the snowball samplers: serial frontier processes, run on the host over a copy of
// the adjacency (as the reference runs them serially)

enum : uint32_t { DOM_SNOWBALL = 11 };

// common::random_integer(lo, hi) as the k-th draw of a run.
struct SnowballRng {
    uint64_t seed;
    uint32_t k = 0;
    int64_t operator()(int64_t lo, int64_t hi) {
        uint32_t w[4];
        philox_host(k++, 0, 0, DOM_SNOWBALL, seed, w);
        const unsigned __int128 x = ((unsigned __int128)(((uint64_t)w[0] << 32) | w[1])) * (uint64_t)(hi - lo + 1);
        return lo + (int64_t)(uint64_t)(x >> 64);
    }
};

// sample::expansion_snowball (sample.cpp:125-157; es_add_vertex :103-117,
// es_update_contribution :119-130).
int64_t expansion_snowball(const HostAdjacency& a, int64_t N, int64_t target, uint64_t seed,
                           std::vector<int32_t>& mapping) {
    SnowballRng rng{seed};
    std::vector<int64_t> contribution(N, 0);
    std::vector<char> in_hood(N, 0);
    std::set<int64_t> hood;
    int64_t contribution_sum = 0, n = 0;
    auto update = [&](int64_t x) {
        for (int32_t j = a.out_off[x]; j < a.out_off[x + 1]; ++j) {
            const int32_t y = a.out_nbr[j];
            if (in_hood[y] || mapping[y] >= 0) continue;
            contribution[x]++;
            contribution_sum++;
        }
        for (int32_t j = a.in_off[x]; j < a.in_off[x + 1]; ++j) {
            const int32_t y = a.in_nbr[j];
            if (contribution[y] > 0) {
                contribution[y]--;
                contribution_sum--;
            }
        }
    };
    auto add = [&](int64_t x) {
        mapping[x] = (int32_t)n++;
        for (int32_t j = a.out_off[x]; j < a.out_off[x + 1]; ++j) {
            const int32_t y = a.out_nbr[j];
            if (in_hood[y] || mapping[y] >= 0) continue;
            hood.insert(y);
            in_hood[y] = 1;
            if (contribution[y] > 0) continue;
            update(y);
        }
        hood.erase(x);
        in_hood[x] = 0;
    };
    add(rng(0, N - 1));
    while (n < target) {
        if (hood.empty()) {
            int64_t x;
            do x = rng(0, N - 1);
            while (mapping[x] >= 0);
            add(x);
        } else if (contribution_sum == 0) {
            auto it = hood.begin();
            std::advance(it, rng(0, (int64_t)hood.size() - 1));
            add(*it);
        } else {
            int64_t best = 0;  // utils::argmax: the first largest contribution
            for (int64_t x = 1; x < N; ++x)
                if (contribution[x] > contribution[best]) best = x;
            add(best);
        }
    }
    return n;
}

// sample::degree_product_snowball (sample.cpp:51-101): the frontier edge of the largest
// degree product first (ties: the earliest pushed).
int64_t degree_product_snowball(const HostAdjacency& a, int64_t N, int64_t target, uint64_t seed,
                                std::vector<int32_t>& mapping) {
    SnowballRng rng{seed};
    std::priority_queue<std::tuple<int64_t, int64_t, int32_t, int32_t>> frontier;
    int64_t pushes = 0, n = 0;
    auto add = [&](int64_t x) {
        mapping[x] = (int32_t)n++;
        for (int32_t j = a.out_off[x]; j < a.out_off[x + 1]; ++j) {
            const int32_t y = a.out_nbr[j];
            if (mapping[y] != -1) continue;
            frontier.push({(int64_t)a.deg[x] * a.deg[y], -(pushes++), (int32_t)x, y});
        }
        for (int32_t j = a.in_off[x]; j < a.in_off[x + 1]; ++j) {
            const int32_t y = a.in_nbr[j];
            if (mapping[y] != -1) continue;
            frontier.push({(int64_t)a.deg[y] * a.deg[x], -(pushes++), y, (int32_t)x});
        }
    };
    add(rng(0, N - 1));
    while (n < target) {
        if (frontier.empty()) {
            int64_t x;
            do x = rng(0, N - 1);
            while (mapping[x] >= 0);
            add(x);
            if (frontier.empty()) continue;
        }
        const auto next = frontier.top();
        frontier.pop();
        if (mapping[std::get<2>(next)] == -1) add(std::get<2>(next));
        if (mapping[std::get<3>(next)] == -1) add(std::get<3>(next));
    }
    return n;
}

enum : uint32_t { DOM_REATTACH = 10 };

// sample::reattach for vertices of degree 0 or 1 (the complement of detach).  flags a
// vertex of larger degree in *bad.
__global__ void k_reattach(DevGraph g, const int32_t* __restrict__ mapping, const int32_t* __restrict__ sample_asg,
                           int32_t B, uint64_t seed, int32_t* __restrict__ asg, int32_t* __restrict__ bad) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.N; v += gridDim.x * blockDim.x) {
        if (mapping[v] >= 0) {
            asg[v] = sample_asg[mapping[v]];
            continue;
        }
        if (vertex_degree(g, v) > 1) {
            atomicAdd(bad, 1);
            continue;
        }
        // the one neighbour other than v itself, if any
        int32_t u = -1;
        for (int32_t j = __ldg(g.out_off + v); j < __ldg(g.out_off + v + 1); ++j)
            if (__ldg(g.out_nbr + j) != v) u = __ldg(g.out_nbr + j);
        for (int32_t j = __ldg(g.inns_off + v); j < __ldg(g.inns_off + v + 1); ++j) u = __ldg(g.inns_nbr + j);
        int32_t b;
        if (u >= 0 && mapping[u] >= 0) {
            b = sample_asg[mapping[u]];
        } else {  // alone, or paired with another detached vertex: the smaller one's draw
            const int32_t x = (u >= 0 && u < v) ? u : v;
            uint32_t w[4];
            philox4x32_10((uint32_t)x, 0u, 0u, DOM_REATTACH, seed, w);
            b = (int32_t)u32_below(w[0], (uint32_t)B);
        }
        asg[v] = b;
    }
}

template <class T>
T* talloc(std::vector<void*>& tmp, size_t n, cudaStream_t st) {
    void* p = nullptr;
    if (cudaMallocAsync(&p, (n ? n : 1) * sizeof(T), st) != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error("device allocation failed");
    }
    tmp.push_back(p);
    return static_cast<T*>(p);
}

void free_tmp(std::vector<void*>& tmp, cudaStream_t st) {
    for (void* p : tmp) cudaFreeAsync(p, st);
    tmp.clear();
}

int32_t read_i32(const int32_t* d, cudaStream_t st) {
    int32_t* h = static_cast<int32_t*>(host_scratch());
    cudaMemcpyAsync(h, d, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    host_wait(st);
    return *h;
}

}  // namespace

int64_t sample_vertices(const DevGraph& g, int alg, double samplesize, uint64_t seed, int32_t* mapping, Work& w,
                        cudaStream_t st) {
    const int64_t N = g.N, E = g.E;
    const int64_t target = (int64_t)(samplesize * (double)N);  // long(args.samplesize * double(N))
    cudaMemsetAsync(mapping, 0xff, N * sizeof(int32_t), st);
    std::vector<void*> tmp;
    int64_t n = 0;
    try {
        if (alg == 0) {  // max_degree
            k_degree_keys<<<grid_of(N), 256, 0, st>>>(g, w.keys, w.vals);
            radix_sort_u64(w.keys, w.keys_alt, w.vals, w.vals_alt, N, 64, w.temp, st);
            n = std::min(std::max<int64_t>(target, 0), N);
            k_number<<<grid_of(n), 256, 0, st>>>(w.vals, n, mapping);
            count_launches(2);
        } else if (alg == 1) {  // random
            int32_t* order = talloc<int32_t>(tmp, N, st);
            int32_t* base = talloc<int32_t>(tmp, N, st);
            std::vector<int32_t> iota(N);
            for (int64_t v = 0; v < N; ++v) iota[v] = (int32_t)v;
            cudaMemcpyAsync(base, iota.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice, st);
            shuffle(base, (int32_t)N, seed, 0, 0, DOM_SAMPLE, order, w, st);
            n = std::min(std::max<int64_t>(target, 0), N);
            k_number<<<grid_of(n), 256, 0, st>>>(order, n, mapping);
            count_launches(1);
            host_wait(st);
        } else if (alg == 2) {  // degree_product
            if (E == 0) return 0;
            if (E >= (1ll << 30)) throw std::invalid_argument("degree_product sampling supports E < 2^30");
            k_edge_info_keys<<<grid_of(E), 256, 0, st>>>(g, w.keys, w.vals);
            radix_sort_u64(w.keys, w.keys_alt, w.vals, w.vals_alt, E, 64, w.temp, st);
            int32_t* first = talloc<int32_t>(tmp, N, st);
            cudaMemsetAsync(first, 0x7f, N * sizeof(int32_t), st);
            k_first_seen<<<grid_of(E), 256, 0, st>>>(g, w.vals, first);
            k_first_keys<<<grid_of(N), 256, 0, st>>>(first, (int32_t)N, w.keys, w.vals);
            radix_sort_u64(w.keys, w.keys_alt, w.vals, w.vals_alt, N, 64, w.temp, st);
            count_launches(4);
            // the vertex of the target-th first appearance fixes the last edge walked
            uint32_t cut;
            uint64_t* hk = static_cast<uint64_t*>(host_scratch());
            if (target <= 0) {
                cut = 1u;  // the reference walks at least the first edge
            } else {
                cudaMemcpyAsync(hk, w.keys + std::min<int64_t>(target, N) - 1, sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                st);
                host_wait(st);
                const uint32_t p = (uint32_t)(*hk >> 32);
                cut = p == 0x7f7f7f7fu ? 0x7f7f7f7eu : ((p >> 1) << 1) + 1;  // fewer vertices with edges: all of them
            }
            k_number_first<<<grid_of(N), 256, 0, st>>>(w.keys, w.vals, (int32_t)N, cut, mapping);
            int32_t* cnt = talloc<int32_t>(tmp, 1, st);
            cudaMemsetAsync(cnt, 0, sizeof(int32_t), st);
            k_count_upto<<<grid_of(N), 256, 0, st>>>(w.keys, (int32_t)N, cut, cnt);
            count_launches(2);
            n = read_i32(cnt, st);
        } else if (alg == 3) {  // detach
            int32_t* flags = talloc<int32_t>(tmp, N, st);
            int32_t* pos = talloc<int32_t>(tmp, N, st);
            int32_t* total = talloc<int32_t>(tmp, 1, st);
            k_degree_flags<<<grid_of(N), 256, 0, st>>>(g, flags);
            scan_i32(flags, pos, N, false, total, w.temp, st);
            k_number_flagged<<<grid_of(N), 256, 0, st>>>(flags, pos, (int32_t)N, mapping);
            count_launches(2);
            n = read_i32(total, st);
        } else if (alg == 4 || alg == 5) {  // expansion_snowball, degree_product_snowball
            const HostAdjacency a = host_adjacency(g, st);
            std::vector<int32_t> m(N, -1);
            const int64_t t = std::min(std::max<int64_t>(target, 1), N);
            n = alg == 4 ? expansion_snowball(a, N, t, seed, m) : degree_product_snowball(a, N, t, seed, m);
            cudaMemcpyAsync(mapping, m.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice, st);
            host_wait(st);
        } else {
            throw std::invalid_argument("unknown sampling algorithm");
        }
    } catch (...) {
        host_wait(st);
        free_tmp(tmp, st);
        throw;
    }
    host_wait(st);
    free_tmp(tmp, st);
    return n;
}

void subgraph_edges(const DevGraph& g, const int32_t* mapping, int32_t** d_src, int32_t** d_dst, int64_t* E_out,
                    Work& w, cudaStream_t st) {
    *d_src = *d_dst = nullptr;
    *E_out = 0;
    if (g.E == 0) return;
    std::vector<void*> tmp;
    int32_t* flags = talloc<int32_t>(tmp, g.E, st);
    int32_t* pos = talloc<int32_t>(tmp, g.E, st);
    int32_t* total = talloc<int32_t>(tmp, 1, st);
    k_sub_flags<<<grid_of(g.E), 256, 0, st>>>(g, mapping, flags);
    scan_i32(flags, pos, g.E, false, total, w.temp, st);
    const int32_t E2 = read_i32(total, st);
    std::vector<void*> out;
    *d_src = talloc<int32_t>(out, E2, st);
    *d_dst = talloc<int32_t>(out, E2, st);
    k_sub_edges<<<grid_of(g.E), 256, 0, st>>>(g, mapping, flags, pos, *d_src, *d_dst);
    count_launches(2);
    *E_out = E2;
    host_wait(st);
    free_tmp(tmp, st);
}

void extend_assignment(const DevGraph& g, const int32_t* mapping, const int32_t* sample_asg, int32_t B,
                       int32_t max_k, uint64_t seed, int32_t* asg, cudaStream_t st) {
    const int64_t N = g.N;
    int log2cap = ceil_log2((uint64_t)(2 * (max_k > 16 ? max_k : 16)));
    if (log2cap > 14) throw std::invalid_argument("vertex degree above 8192");
    std::vector<void*> tmp;
    int32_t* lists = talloc<int32_t>(tmp, 3 * N, st);
    int32_t* counts = talloc<int32_t>(tmp, 4, st);
    int32_t* pending = lists;
    int32_t* ready = lists + N;
    int32_t* rest = lists + 2 * N;
    cudaMemsetAsync(counts, 0, 4 * sizeof(int32_t), st);
    k_extend_init<<<grid_of(N), 256, 0, st>>>(mapping, sample_asg, (int32_t)N, asg, pending, counts);
    count_launches(1);
    int32_t np = read_i32(counts, st);
    const size_t smem = (size_t)2 * sizeof(int32_t) << log2cap;
    allow_max_dynamic_smem((const void*)k_extend_assign);
    int rounds = 0;
    while (np > 0) {
        if (++rounds > N + 1) {  // every round assigns at least the smallest pending vertex
            free_tmp(tmp, st);
            throw std::runtime_error("extend made no progress");
        }
        cudaMemsetAsync(counts + 1, 0, 2 * sizeof(int32_t), st);
        k_extend_ready<<<grid_of(np), 256, 0, st>>>(g, asg, pending, np, ready, counts + 1, rest, counts + 2);
        int32_t* h = static_cast<int32_t*>(host_scratch());
        cudaMemcpyAsync(h, counts + 1, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        host_wait(st);
        const int32_t nr = h[0], nrest = h[1];
        k_extend_assign<<<grid_of(nr, 1), 128, smem, st>>>(g, asg, ready, nr, B, seed, log2cap);
        count_launches(2);
        std::swap(pending, rest);
        np = nrest;
    }
    host_wait(st);
    free_tmp(tmp, st);
}

void reattach_assignment(const DevGraph& g, const int32_t* mapping, const int32_t* sample_asg, int32_t B, uint64_t seed,
                         int32_t* asg, cudaStream_t st) {
    std::vector<void*> tmp;
    int32_t* bad = talloc<int32_t>(tmp, 1, st);
    cudaMemsetAsync(bad, 0, sizeof(int32_t), st);
    k_reattach<<<grid_of(g.N), 256, 0, st>>>(g, mapping, sample_asg, B, seed, asg, bad);
    count_launches(1);
    const int32_t nbad = read_i32(bad, st);
    free_tmp(tmp, st);
    if (nbad) throw std::invalid_argument("reattach: an unsampled vertex has degree above 1");
}

}  // namespace sbp

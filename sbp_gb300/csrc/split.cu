// Top-down cluster splits on the device (reference divisive::split_communities,
// src/top_down_sbp.cpp:472-530, with propose_random_split :248-260): every cluster of
// at least 0.001 N vertices gets 10 random two-way splits, each scored by the
// nonparametric description length of the split cluster's subgraph.
//
// All clusters and proposals are counted in one pass over the vertices and one over the
// edges: a vertex's 10 sides are bits of one mask (drawn from the canonical stream), and
// each edge inside a cluster adds to one of the four cells of each proposal's 2 x 2
// blockmatrix.  The host turns the counts into description lengths, picks the best split
// of each cluster and the clusters to split; one more pass moves side-1 vertices into
// their new blocks.
//
// The snowball splits grow one or two sets from seed vertices, a serial frontier process
// per cluster and proposal; they run on the host over the clusters' subgraphs, ordered
// sets standing in for the reference's hash maps (ascending vertex order), and their sides
// go to the same edge-counting pass.
#include <algorithm>
#include <map>
#include <set>
#include <utility>

#include "kernels.cuh"

namespace sbp {

namespace {

enum : uint32_t { DOM_SPLIT_SIZE = 8, DOM_SPLIT_SIDE = 9 };
constexpr int kProposals = 10;  // NUM_AGG_PROPOSALS_PER_BLOCK (top_down_sbp.hpp:28)

unsigned grid_of(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > (int64_t)device_sms() * 16) b = (int64_t)device_sms() * 16;
    return (unsigned)b;
}

// Per (cluster, proposal): the size of side 0 (or -1 when the cluster is not split); per
// cluster whether it is split at all (at least 0.001 N vertices).
__global__ void k_split_sizes(const int32_t* __restrict__ sizes, int32_t B, int32_t N, uint64_t seed, uint32_t step,
                              long long* __restrict__ split_size, int32_t* __restrict__ eligible) {
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < B * kProposals; k += gridDim.x * blockDim.x) {
        const int32_t c = k / kProposals, i = k % kProposals;
        const long long n = sizes[c];
        const bool elig = !((double)n < 0.001 * (double)N);
        if (i == 0) eligible[c] = elig ? 1 : 0;
        long long sz = -1;
        if (elig && n >= 2) {
            const long long lo = (long long)((double)n * 0.2), hi = (long long)((double)n * 0.8);
            uint32_t w[4];
            philox4x32_10((uint32_t)c, (uint32_t)i, step, DOM_SPLIT_SIZE, seed, w);
            sz = lo + (long long)u64_below(w[0], w[1], (uint64_t)(hi - lo + 1));
        } else if (elig) {
            sz = n;  // a cluster of one vertex keeps it on side 0
        }
        split_size[k] = sz;
    }
}

__global__ void k_split_vertices(const int32_t* __restrict__ asg, const int32_t* __restrict__ sizes, int32_t N,
                                 uint64_t seed, uint32_t step, const long long* __restrict__ split_size,
                                 const int32_t* __restrict__ eligible, uint16_t* __restrict__ mask,
                                 int32_t* __restrict__ n1) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
        const int32_t c = asg[v];
        uint32_t m = 0;
        const long long n = sizes[c];
        if (eligible[c] && n >= 2) {
            for (int i = 0; i < kProposals; ++i) {
                uint32_t w[4];
                philox4x32_10((uint32_t)v, (uint32_t)i, step, DOM_SPLIT_SIDE, seed, w);
                const uint64_t sz = (uint64_t)split_size[c * kProposals + i];
                if ((uint64_t)w[0] * (uint64_t)n >= (sz << 32)) {
                    m |= 1u << i;
                    atomicAdd(n1 + c * kProposals + i, 1);
                }
            }
        }
        mask[v] = (uint16_t)m;
    }
}

__global__ void k_split_edges(DevGraph g, const int32_t* __restrict__ asg, const int32_t* __restrict__ eligible,
                              const uint16_t* __restrict__ mask, int32_t* __restrict__ cells,
                              unsigned long long* __restrict__ ecount) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.E; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = __ldg(g.esrc + e), v = __ldg(g.out_nbr + e);
        const int32_t c = asg[u];
        if (c != asg[v] || !eligible[c]) continue;
        atomicAdd(ecount + c, 1ull);
        const uint32_t mu = mask[u], mv = mask[v];
        for (int i = 0; i < kProposals; ++i)
            atomicAdd(cells + ((int64_t)c * kProposals + i) * 4 + 2 * ((mu >> i) & 1u) + ((mv >> i) & 1u), 1);
    }
}

__global__ void k_split_apply(int32_t* __restrict__ asg, int32_t N, const uint16_t* __restrict__ mask,
                              const int32_t* __restrict__ new_block, const int32_t* __restrict__ proposal) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
        const int32_t c = asg[v];
        const int32_t nb = new_block[c];
        if (nb >= 0 && ((mask[v] >> proposal[c]) & 1u)) asg[v] = nb;
    }
}

}  // namespace

void split_count(const DevGraph& g, const DevBM& bm, uint64_t seed, uint32_t step, SplitBuffers& b, cudaStream_t st) {
    const int32_t B = bm.B;
    cudaMemsetAsync(b.n1, 0, sizeof(int32_t) * (size_t)B * kProposals, st);
    cudaMemsetAsync(b.cells, 0, sizeof(int32_t) * (size_t)B * kProposals * 4, st);
    cudaMemsetAsync(b.ecount, 0, sizeof(unsigned long long) * (size_t)B, st);
    k_split_sizes<<<grid_of((int64_t)B * kProposals), 256, 0, st>>>(bm.sizes, B, g.N, seed, step, b.split_size,
                                                                  b.eligible);
    k_split_vertices<<<grid_of(g.N), 256, 0, st>>>(bm.asg, bm.sizes, g.N, seed, step, b.split_size, b.eligible, b.mask,
                                                   b.n1);
    k_split_edges<<<grid_of(g.E), 256, 0, st>>>(g, bm.asg, b.eligible, b.mask, b.cells, b.ecount);
    count_launches(3);
}

void split_apply(const DevGraph& g, DevBM& bm, const SplitBuffers& b, cudaStream_t st) {
    k_split_apply<<<grid_of(g.N), 256, 0, st>>>(bm.asg, g.N, b.mask, b.new_block, b.proposal);
    count_launches(1);
}

void split_count_edges(const DevGraph& g, const DevBM& bm, SplitBuffers& b, cudaStream_t st) {
    const int32_t B = bm.B;
    cudaMemsetAsync(b.cells, 0, sizeof(int32_t) * (size_t)B * kProposals * 4, st);
    cudaMemsetAsync(b.ecount, 0, sizeof(unsigned long long) * (size_t)B, st);
    k_split_edges<<<grid_of(g.E), 256, 0, st>>>(g, bm.asg, b.eligible, b.mask, b.cells, b.ecount);
    count_launches(1);
}

namespace {

enum : uint32_t { DOM_SPLIT_SNOWBALL = 12 };

// A cluster's subgraph: local ids in vertex order; neighbours = out then in (Graph::neighbors).
struct ClusterLists {
    int64_t n = 0;
    std::vector<std::vector<int32_t>> nbrs;
    std::vector<int64_t> deg;
};

// common::random_integer for the k-th draw of proposal `proposal` of `cluster`.
struct SplitDraws {
    uint64_t seed;
    uint32_t cluster, proposal, step, k = 0;
    uint32_t word() {
        uint32_t w[4];
        philox_host(cluster, proposal | (k++ << 8), step, DOM_SPLIT_SNOWBALL, seed, w);
        return w[0];
    }
    int64_t operator()(int64_t lo, int64_t hi) {
        uint32_t w[4];
        philox_host(cluster, proposal | (k++ << 8), step, DOM_SPLIT_SNOWBALL, seed, w);
        const unsigned __int128 x = ((unsigned __int128)(((uint64_t)w[0] << 32) | w[1])) * (uint64_t)(hi - lo + 1);
        return lo + (int64_t)(uint64_t)(x >> 64);
    }
};

// split_init (top_down_sbp.cpp:532-583) with a stable descending degree ranking; the
// degree-weighted draw uses the top max(n / 10, 2) vertices.
std::pair<int64_t, int64_t> seeds_of(const ClusterLists& c, int init, SplitDraws& d) {
    const int64_t n = c.n;
    if (init == 0 || n < 10) {
        const int64_t x = d(0, n - 1);
        int64_t y = d(0, n - 1);
        while (y == x) y = d(0, n - 1);
        return {x, y};
    }
    std::vector<int64_t> rank(n);
    for (int64_t x = 0; x < n; ++x) rank[x] = x;
    std::stable_sort(rank.begin(), rank.end(), [&](int64_t p, int64_t q) { return c.deg[p] > c.deg[q]; });
    if (init == 2) return {rank[0], rank[1]};
    const int64_t m = std::max<int64_t>(n / 10, 2);
    const int64_t x = d(0, m - 1);
    int64_t y = d(0, m - 1);
    while (y == x) y = d(0, m - 1);
    return {rank[x], rank[y]};
}

// propose_snowball_split (:313-363).
std::vector<int8_t> two_snowballs(const ClusterLists& c, int init, SplitDraws& d) {
    const int64_t n = c.n;
    std::vector<int8_t> side(n, -1);
    std::set<int64_t> rest;
    for (int64_t x = 0; x < n; ++x) rest.insert(x);
    std::set<int64_t> front[2];
    const auto s0 = seeds_of(c, init, d);
    const int64_t seed_v[2] = {s0.first, s0.second};
    for (int id = 0; id < 2; ++id) {
        side[seed_v[id]] = (int8_t)id;
        rest.erase(seed_v[id]);
    }
    for (int id = 0; id < 2; ++id)
        for (int32_t y : c.nbrs[seed_v[id]])
            if (side[y] == -1) front[id].insert(y);
    const int64_t size = d((int64_t)((double)n * 0.2), (int64_t)((double)n * 0.8));
    while (!rest.empty()) {
        const int id = (uint64_t)d.word() * (uint64_t)n < ((uint64_t)size << 32) ? 0 : 1;
        const int64_t x = front[id].empty() ? *rest.begin() : *front[id].begin();
        side[x] = (int8_t)id;
        rest.erase(x);
        front[0].erase(x);
        front[1].erase(x);
        for (int32_t y : c.nbrs[x])
            if (side[y] == -1) front[id].insert(y);
    }
    return side;
}

// propose_single_snowball_split (:382-426); the map lookup that tests membership adds the
// vertex to the map's count, as in the reference.
std::vector<int8_t> one_snowball(const ClusterLists& c, int init, SplitDraws& d) {
    const int64_t n = c.n;
    std::vector<int8_t> side(n, 0);
    std::map<int64_t, bool> seen, front, next;
    const int64_t s0 = seeds_of(c, init, d).first;
    side[s0] = 1;
    seen[s0] = true;
    for (int32_t y : c.nbrs[s0])
        if (side[y] != 1) front[y] = true;
    const uint64_t target = (uint64_t)d((int64_t)((double)n * 0.2), (int64_t)((double)n * 0.8));
    while (seen.size() < target) {
        if (front.empty() && next.empty()) break;
        for (const auto& e : front) {
            const int64_t x = e.first;
            if (!seen[x]) {
                side[x] = 1;
                seen[x] = true;
                for (int32_t y : c.nbrs[x])
                    if (side[y] != 1) next[y] = true;
            }
            if (seen.size() >= target) break;
        }
        front = std::move(next);
        next.clear();
    }
    return side;
}

// propose_connectivity_snowball_split (:262-311).
std::vector<int8_t> connected_snowballs(const ClusterLists& c, int init, SplitDraws& d) {
    const int64_t n = c.n;
    std::vector<int8_t> side(n, -1);
    std::set<int64_t> rest;
    for (int64_t x = 0; x < n; ++x) rest.insert(x);
    std::map<int64_t, bool> front, next;
    const auto s0 = seeds_of(c, init, d);
    const int64_t seed_v[2] = {s0.first, s0.second};
    for (int id = 0; id < 2; ++id) {
        side[seed_v[id]] = (int8_t)id;
        rest.erase(seed_v[id]);
    }
    for (int id = 0; id < 2; ++id)
        for (int32_t y : c.nbrs[seed_v[id]])
            if (side[y] == -1) front[y] = true;
    auto take = [&](int64_t x) {
        int to0 = 0, to1 = 0;
        for (int32_t y : c.nbrs[x]) {
            to0 += side[y] == 0;
            to1 += side[y] == 1;
            if (side[y] == -1) next[y] = true;
        }
        side[x] = to1 > to0 ? 1 : 0;
        rest.erase(x);
        front[x] = false;
    };
    while (!rest.empty()) {
        if (front.empty()) {
            take(*rest.begin());
            continue;
        }
        for (const auto& e : front) take(e.first);
        front = std::move(next);
        next.clear();
    }
    return side;
}

}  // namespace

void snowball_split_masks(const HostAdjacency& a, const std::vector<int32_t>& asg, const std::vector<int32_t>& sizes,
                          const std::vector<int32_t>& eligible, int32_t B, int split, int init, uint64_t seed,
                          uint32_t step, std::vector<uint16_t>& mask, std::vector<int32_t>& n1) {
    const int64_t N = (int64_t)asg.size();
    mask.assign(N, 0);
    n1.assign((size_t)B * kProposals, 0);
    std::vector<std::vector<int32_t>> members(B);
    for (int64_t v = 0; v < N; ++v)
        if (eligible[asg[v]] && sizes[asg[v]] >= 2) members[asg[v]].push_back((int32_t)v);
    std::vector<int32_t> local(N, -1);
    for (int32_t cl = 0; cl < B; ++cl) {
        const std::vector<int32_t>& mem = members[cl];
        if (mem.empty()) continue;
        ClusterLists c;
        c.n = (int64_t)mem.size();
        for (int64_t x = 0; x < c.n; ++x) local[mem[x]] = (int32_t)x;
        std::vector<std::vector<int32_t>> out(c.n), in(c.n);
        std::vector<char> self(c.n, 0);
        for (int32_t u : mem)
            for (int32_t j = a.out_off[u]; j < a.out_off[u + 1]; ++j) {
                const int32_t v = a.out_nbr[j];
                if (local[v] < 0) continue;
                out[local[u]].push_back(local[v]);
                in[local[v]].push_back(local[u]);
                if (u == v) self[local[u]] = 1;
            }
        c.nbrs.resize(c.n);
        c.deg.resize(c.n);
        for (int64_t x = 0; x < c.n; ++x) {
            c.nbrs[x] = out[x];
            c.nbrs[x].insert(c.nbrs[x].end(), in[x].begin(), in[x].end());
            c.deg[x] = (int64_t)out[x].size() + (int64_t)in[x].size() - self[x];
        }
        for (int i = 0; i < kProposals; ++i) {
            SplitDraws d{seed, (uint32_t)cl, (uint32_t)i, step};
            const std::vector<int8_t> side =
                split == 1 ? two_snowballs(c, init, d) : split == 2 ? one_snowball(c, init, d) : connected_snowballs(c, init, d);
            for (int64_t x = 0; x < c.n; ++x)
                if (side[x] == 1) {
                    mask[mem[x]] |= (uint16_t)(1u << i);
                    n1[(size_t)cl * kProposals + i]++;
                }
        }
        for (int32_t u : mem) local[u] = -1;
    }
}

}  // namespace sbp

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
#include "kernels.cuh"

namespace sbp {

namespace {

enum : uint32_t { DOM_SPLIT_SIZE = 8, DOM_SPLIT_SIDE = 9 };
constexpr int kProposals = 10;  // NUM_AGG_PROPOSALS_PER_BLOCK (top_down_sbp.hpp:28)

unsigned grid_of(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152 * 16) b = 152 * 16;
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

}  // namespace sbp

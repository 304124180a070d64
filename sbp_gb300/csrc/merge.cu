// Block-merge pass (reference src/block_merge.cpp:178-228).
//
//  * k_merge_propose: one warp per block, NUM_AGG_PROPOSALS_PER_BLOCK = 10 proposals
//    (block_merge.hpp:23), duplicates skipped (propose_merge_sparse :251-285), each
//    scored by block_merge_delta_mdl over the static CSR/CSC in O(|row r| + |col r|).
//  * carry_out_best_merges_advanced (:40-117): the queue is the stable radix sort of the
//    proposals by (delta, block); the carry-out itself is in carry.cu.  Block
//    relabelling (block_map, update_block_assignment, build_mapping) is a union-find
//    followed by a dense relabel in ascending root order.
//  * Blockmodel::carry_out_best_merges (src/blockmodel/blockmodel.cpp:55-122) for
//    --approximate: sorted order, translate() chains, no recomputation.
#include <cfloat>
#include <climits>

#include <stdexcept>

#include "chain.cuh"
#include "delta.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace sbp {

namespace {

constexpr int kMergeWarps = 8;

inline unsigned grid_cap(int64_t n, int64_t per, int64_t cap) {
    int64_t b = (n + per - 1) / per;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

template <bool kNP>
__global__ void __launch_bounds__(256) k_merge_propose(DevGraph g, DevBM bm, uint64_t seed, uint32_t step,
                                                       int32_t* __restrict__ best, double* __restrict__ best_dS,
                                                       DevFlags* flags) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long evaluated = 0;
    const int32_t nonempty = kNP ? *bm.nonempty : 0;
    for (int32_t r = blockIdx.x * kMergeWarps + wid; r < bm.B; r += gridDim.x * kMergeWarps) {
        long long bestq = LLONG_MAX;
        int32_t bests = -1;
        int32_t past[10];
        int np = 0;
#pragma unroll 1
        for (int i = 0; i < 10; ++i) {
            uint32_t w[4];
            philox4x32_10((uint32_t)r, 0u, step, DOM_MERGE | ((uint32_t)i << 8), seed, w);
            const int32_t s = sample_merge_proposal(bm, r, w);
            if (s < 0 || s >= bm.B) {
                if (lane == 0) atomicOr(&flags->err, ERR_SELECT);
                continue;
            }
            bool dup = false;
            for (int j = 0; j < np; ++j) dup |= past[j] == s;
            if (dup) continue;
            past[np++] = s;
            const long long dS = kNP ? np_merge_delta_csr<32>(g, bm, r, s, nonempty, nullptr)
                                     : merge_delta_fixed_csr<32>(g, bm, r, s, nullptr);
            ++evaluated;
            if (bests < 0 || dS < bestq) {
                bestq = dS;
                bests = s;
            }
        }
        if (lane == 0) {
            best[r] = bests;
            best_dS[r] = bests < 0 ? DBL_MAX : fixed_to_double(bestq);
        }
    }
    if (lane == 0) atomicAdd(&flags->counters[6], evaluated);
}

// Sort keys of the best deltas: each is an exact multiple of 2^-24 (a block without a
// proposal has DBL_MAX), turned into its int64 count of 2^-24 units with the sign bit
// flipped, so ascending unsigned order is ascending delta order.
__global__ void k_merge_keys(const double* __restrict__ dS, int32_t B, uint64_t* __restrict__ keys,
                             int32_t* __restrict__ vals) {
    for (int32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        const double d = dS[b];
        const long long q = d == DBL_MAX ? LLONG_MAX : __double2ll_rn(d * 16777216.0);
        keys[b] = (uint64_t)q ^ 0x8000000000000000ull;
        vals[b] = b;
    }
}

__global__ void k_iota(int32_t* p, int32_t n) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

__global__ void k_carry_approx(const int32_t* __restrict__ sorted_blk, int32_t nq, const int32_t* __restrict__ best,
                               int32_t* block_map, long long num_to_merge, int32_t* out_merged) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long merged = 0;
    int32_t counter = 0;
    while (merged < num_to_merge && counter < nq) {
        const int32_t from = sorted_blk[counter++];
        int32_t b = best[from];
        while (block_map[b] != b) b = block_map[b];  // translate (blockmodel.cpp:75-85)
        if (b != from) {
            block_map[from] = b;
            ++merged;
        }
    }
    *out_merged = (int32_t)merged;
}

__global__ void k_roots(int32_t* parent, int32_t B, int32_t* __restrict__ root) {
    for (int32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        int32_t x = b;
        while (parent[x] != x) x = parent[x];
        root[b] = x;
    }
}

__global__ void k_mark_used(const int32_t* __restrict__ asg, int32_t N, const int32_t* __restrict__ root,
                            int32_t* __restrict__ used) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) used[root[asg[v]]] = 1;
}

__global__ void k_relabel(int32_t* __restrict__ asg, int32_t N, const int32_t* __restrict__ root,
                          const int32_t* __restrict__ mapping) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x)
        asg[v] = mapping[root[asg[v]]];
}

}  // namespace

void merge_propose(const DevGraph& g, const DevBM& bm, uint64_t seed, uint32_t step, Work& w, cudaStream_t st,
                   bool np) {
    if (np && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    if (np)
        k_merge_propose<true><<<grid_cap(bm.B, kMergeWarps, device_sms() * 8), 256, 0, st>>>(g, bm, seed, step, w.best,
                                                                                    w.best_dS, w.flags_dev);
    else
        k_merge_propose<false><<<grid_cap(bm.B, kMergeWarps, device_sms() * 8), 256, 0, st>>>(g, bm, seed, step, w.best,
                                                                                     w.best_dS, w.flags_dev);
    count_launches(1);
}

void carry_out(const DevGraph& g, DevBM& bm, int64_t num_to_merge, int approximate, Work& w, cudaStream_t st,
               bool np, bool cluster) {
    const int32_t B = bm.B;
    // queue order: stable sort of (delta, block)
    k_merge_keys<<<grid_cap(B, 256, device_sms() * 16), 256, 0, st>>>(w.best_dS, B, w.keys, w.vals);
    radix_sort_u64(w.keys, w.keys_alt, w.vals, w.vals_alt, B, 64, w.temp, st);
    k_iota<<<grid_cap(B, 256, device_sms() * 16), 256, 0, st>>>(w.parent, B);
    count_launches(2);
    int32_t* d_merged = w.d_scalar + 1;
    if (approximate) {
        k_carry_approx<<<1, 32, 0, st>>>(w.vals, B, w.best, w.parent, num_to_merge, d_merged);
    } else if (cluster) {
        carry_out_cluster(g, bm, num_to_merge, w, st, np);
    } else {
        carry_out_exact(g, bm, num_to_merge, w, st, np);
    }
    count_launches(1);
    // union-find roots -> dense labels in ascending root order (build_mapping)
    k_roots<<<grid_cap(B, 256, device_sms() * 16), 256, 0, st>>>(w.parent, B, w.root);
    cudaMemsetAsync(w.used, 0, sizeof(int32_t) * B, st);
    k_mark_used<<<grid_cap(g.N, 256, device_sms() * 16), 256, 0, st>>>(bm.asg, g.N, w.root, w.used);
    scan_i32(w.used, w.used, B, false, w.d_scalar + 2, w.temp, st);
    k_relabel<<<grid_cap(g.N, 256, device_sms() * 16), 256, 0, st>>>(bm.asg, g.N, w.root, w.used);
    count_launches(3);
}

}  // namespace sbp

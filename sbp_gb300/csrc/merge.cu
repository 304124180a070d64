// Block-merge pass (reference src/block_merge.cpp:178-228).
//
//  * k_merge_propose: one warp per block, NUM_AGG_PROPOSALS_PER_BLOCK = 10 proposals
//    (block_merge.hpp:23), duplicates skipped (propose_merge_sparse :251-285), each
//    scored by block_merge_delta_mdl over the static CSR/CSC in O(|row r| + |col r|).
//  * carry_out_best_merges_advanced (:40-117): one CTA pops merges in (delta, block)
//    order -- the initial queue is the stable radix sort of the proposals, re-queued
//    entries go to a binary heap -- recomputes each delta against the current
//    blockmatrix (DevChain) and either re-queues or merges.  Block relabelling
//    (block_map, update_block_assignment, build_mapping) is a union-find followed by a
//    dense relabel in ascending root order.
//  * Blockmodel::carry_out_best_merges (src/blockmodel/blockmodel.cpp:55-122) for
//    --approximate: sorted order, translate() chains, no recomputation.
#include <cfloat>
#include <climits>

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

__global__ void __launch_bounds__(256) k_merge_propose(DevGraph g, DevBM bm, uint64_t seed, uint32_t step,
                                                       int32_t* __restrict__ best, double* __restrict__ best_dS,
                                                       DevFlags* flags) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long evaluated = 0;
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
            const long long dS = merge_delta_fixed_csr<32>(g, bm, r, s, nullptr);
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

// Order keys of doubles: ascending unsigned order == ascending double order.
__global__ void k_merge_keys(const double* __restrict__ dS, int32_t B, uint64_t* __restrict__ keys,
                             int32_t* __restrict__ vals) {
    for (int32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        const uint64_t u = (uint64_t)__double_as_longlong(dS[b]);
        keys[b] = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
        vals[b] = b;
    }
}

__global__ void k_iota(int32_t* p, int32_t n) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

__device__ __forceinline__ bool qless(double a, int32_t ab, double b, int32_t bb) {
    return a < b || (a == b && ab < bb);
}

__device__ __forceinline__ int32_t uf_find(int32_t* parent, int32_t x) {
    while (true) {
        const int32_t p = parent[x];
        if (p == x) return x;
        const int32_t gp = parent[p];
        parent[x] = gp;
        x = gp;
    }
}

// entropy::block_merge_delta_mdl over the current (chain) blockmatrix.
// Warp-synchronous: launched with one warp (the carry-out kernel).
__device__ long long merge_delta_fixed_chain(const DevGraph& g, const DevBM& bm, const DevChain& ch, int32_t r,
                                             int32_t s) {
    const LogTab Lq{g.Lq, g.E + 1};
    const int32_t dout_r = bm.d_out[r], din_r = bm.d_in[r], dout_s = bm.d_out[s], din_s = bm.d_in[s];
    const int32_t dout_s2 = dout_s + dout_r, din_s2 = din_s + din_r;
    long long acc = 0, sRow = 0, sCol = 0;
    chain_for_each(bm.row_col, bm.row_off[r], bm.row_off[r + 1], ch.row_head[r], ch, [&](int32_t c) {
        const int32_t m = chain_get(ch, r, c);
        if (m == 0) return;
        const int32_t dinc = bm.d_in[c];
        acc += ce_fixed(Lq, m, dinc, dout_r);
        if (c != r && c != s) {
            const int32_t Msc = chain_get(ch, s, c);
            acc += ce_fixed(Lq, Msc, dinc, dout_s) - ce_fixed(Lq, Msc + m, dinc, dout_s2);
            sRow += Msc;
        }
    });
    chain_for_each(bm.col_row, bm.col_off[r], bm.col_off[r + 1], ch.col_head[r], ch, [&](int32_t x) {
        if (x == r) return;
        const int32_t m = chain_get(ch, x, r);
        if (m == 0) return;
        const int32_t doutx = bm.d_out[x];
        acc += ce_fixed(Lq, m, din_r, doutx);
        if (x != s) {
            const int32_t Mxs = chain_get(ch, x, s);
            acc += ce_fixed(Lq, Mxs, din_s, doutx) - ce_fixed(Lq, Mxs + m, din_s2, doutx);
            sCol += Mxs;
        }
    });
    acc = warp_sum_ll(acc);
    sRow = warp_sum_ll(sRow);
    sCol = warp_sum_ll(sCol);
    const int32_t Mrr = chain_get(ch, r, r), Mrs = chain_get(ch, r, s), Msr = chain_get(ch, s, r),
                  Mss = chain_get(ch, s, s);
    const int32_t dss = Mrr + Mrs + Msr;
    long long tot = acc;
    if (dss > 0) tot += ce_fixed(Lq, Mss, din_s, dout_s) - ce_fixed(Lq, Mss + dss, din_s2, dout_s2);
    else tot += ce_delta(Lq, Mss, din_s, dout_s, din_s2, dout_s2);
    tot += ((long long)dout_s - Msr - Mss - sRow) * (Lx(Lq, dout_s2) - Lx(Lq, dout_s));
    tot += ((long long)din_s - Mrs - Mss - sCol) * (Lx(Lq, din_s2) - Lx(Lq, din_s));
    return tot;
}

enum : int { ACT_STOP = 0, ACT_SKIP = 1, ACT_EVAL = 2, ACT_REQUEUE = 3, ACT_MERGE = 4 };

// Re-queued merges live in a 32-ary min-heap in global memory ordered by (delta, block),
// operated by warp 0: a pop reads the 32 children of a node with one coalesced load and
// takes their minimum with shuffles, so its depth is log32(n).
__device__ __forceinline__ void warp_min(double& d, int32_t& b, int32_t& pos) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double d2 = __shfl_xor_sync(SBP_FULL_MASK, d, o);
        const int32_t b2 = __shfl_xor_sync(SBP_FULL_MASK, b, o);
        const int32_t p2 = __shfl_xor_sync(SBP_FULL_MASK, pos, o);
        if (qless(d2, b2, d, b)) {
            d = d2;
            b = b2;
            pos = p2;
        }
    }
}

__device__ __forceinline__ void heap_pop(double* hd, int32_t* hb, int32_t& n) {
    const int lane = threadIdx.x & 31;
    --n;
    const double kd = hd[n];
    const int32_t kb = hb[n];
    int32_t i = 0;
    while (true) {
        const int32_t c = 32 * i + 1 + lane;
        double cd = INFINITY;
        int32_t cb = INT_MAX, cp = -1;
        if (c < n) {
            cd = hd[c];
            cb = hb[c];
            cp = c;
        }
        warp_min(cd, cb, cp);
        if (cp < 0 || !qless(cd, cb, kd, kb)) break;
        if (lane == 0) {
            hd[i] = cd;
            hb[i] = cb;
        }
        __syncwarp();
        i = cp;
    }
    if (lane == 0 && n > 0) {
        hd[i] = kd;
        hb[i] = kb;
    }
    __syncwarp();
}

__device__ __forceinline__ void heap_push(double* hd, int32_t* hb, int32_t& n, double d, int32_t b) {
    int32_t i = n++;
    while (i > 0) {
        const int32_t p = (i - 1) >> 5;
        if (!qless(d, b, hd[p], hb[p])) break;
        hd[i] = hd[p];
        hb[i] = hb[p];
        i = p;
    }
    hd[i] = d;
    hb[i] = b;
}

// One warp: every step is warp-synchronous, so there are no block barriers on the
// sequential path.  Lanes stride over the rows and columns being merged.
__global__ void __launch_bounds__(32, 1) k_carry_out(
    DevGraph g, DevBM bm, DevChain ch, const int32_t* __restrict__ sorted_blk, int32_t nq,
    const int32_t* __restrict__ best, const double* __restrict__ best_dS, double* heap_dS, int32_t* heap_blk,
    int32_t* parent, long long num_to_merge, int32_t* stage_row, int32_t* stage_col, int stage_cap,
    int32_t* out_merged, DevFlags* flags) {
    __shared__ int32_t s_to, s_nrt, s_nct, s_p0, s_p1;
    const int lane = threadIdx.x;
    int32_t cursor = 0, heap_n = 0;  // identical in every lane
    long long merged = 0;            // identical in every lane
    while (merged < num_to_merge && (cursor < nq || heap_n > 0)) {
        __syncwarp();  // shared scalars of the previous step have been read by every lane
        // pop the smallest (delta, block) of the sorted proposals and the re-queued heap
        bool from_heap;
        if (cursor < nq && heap_n > 0) {
            const int32_t a = sorted_blk[cursor];
            from_heap = qless(heap_dS[0], heap_blk[0], best_dS[a], a);
        } else {
            from_heap = heap_n > 0;
        }
        int32_t from;
        if (from_heap) {
            from = heap_blk[0];
            __syncwarp();
            heap_pop(heap_dS, heap_blk, heap_n);
        } else {
            from = sorted_blk[cursor++];
        }
        if (lane == 0) s_to = uf_find(parent, best[from]);
        __syncwarp();
        const int32_t to = s_to;
        if (to == from) continue;  // block_merge.cpp:63 (already in the same block)
        const long long dq = merge_delta_fixed_chain(g, bm, ch, from, to);
        const double actual = fixed_to_double(dq);
        if (cursor < nq || heap_n > 0) {
            double top;
            if (cursor < nq && heap_n > 0) {
                const int32_t a = sorted_blk[cursor];
                top = qless(heap_dS[0], heap_blk[0], best_dS[a], a) ? heap_dS[0] : best_dS[a];
            } else if (cursor < nq) {
                top = best_dS[sorted_blk[cursor]];
            } else {
                top = heap_dS[0];
            }
            if (actual > top) {  // block_merge.cpp:79: put it back with its actual delta
                __syncwarp();
                if (lane == 0) heap_push(heap_dS, heap_blk, heap_n, actual, from);
                heap_n = __shfl_sync(SBP_FULL_MASK, heap_n, 0);
                __syncwarp();
                continue;
            }
        }
        // Blockmodel::merge_block (blockmodel.cpp:337-363): move row / column `from` into
        // `to`.  New keys of row `to` and column `to` are staged for bulk appends; each other
        // list receiving a key is touched by one lane.
        if (lane == 0) {
            s_nrt = 0;
            s_nct = 0;
        }
        __syncwarp();
        chain_for_each(bm.row_col, bm.row_off[from], bm.row_off[from + 1], ch.row_head[from], ch, [&](int32_t c) {
            const int32_t m = chain_get(ch, from, c);
            if (m == 0) return;
            chain_add(ch, from, c, -m, flags);
            const int32_t c2 = (c == from || c == to) ? to : c;
            if (chain_add(ch, to, c2, m, flags)) {
                stage(stage_row, &s_nrt, stage_cap, c2, flags);
                if (c2 == to) stage(stage_col, &s_nct, stage_cap, to, flags);
                else list_push1(ch.col_head, ch, c2, to, flags);
            }
        });
        chain_for_each(bm.col_row, bm.col_off[from], bm.col_off[from + 1], ch.col_head[from], ch, [&](int32_t x) {
            if (x == from) return;
            const int32_t m = chain_get(ch, x, from);
            if (m == 0) return;
            chain_add(ch, x, from, -m, flags);
            const int32_t x2 = x == to ? to : x;
            if (chain_add(ch, x2, to, m, flags)) {
                stage(stage_col, &s_nct, stage_cap, x2, flags);
                if (x2 == to) stage(stage_row, &s_nrt, stage_cap, to, flags);
                else list_push1(ch.row_head, ch, x2, to, flags);
            }
        });
        __syncwarp();
        {
            const int nr = min(s_nrt, stage_cap), nc = min(s_nct, stage_cap);
            if (lane == 0) s_p0 = nr > 0 ? list_reserve(ch.row_head, ch, to, nr, flags) : -1;
            if (lane == 1) s_p1 = nc > 0 ? list_reserve(ch.col_head, ch, to, nc, flags) : -1;
            __syncwarp();
            const int32_t p0 = s_p0, p1 = s_p1;
            if (p0 >= 0)
                for (int i = lane; i < nr; i += 32) ch.pool[p0 + i] = stage_row[i];
            if (p1 >= 0)
                for (int i = lane; i < nc; i += 32) ch.pool[p1 + i] = stage_col[i];
        }
        if (lane == 0) {
            bm.d_out[to] += bm.d_out[from];
            bm.d_in[to] += bm.d_in[from];
            bm.d_out[from] = 0;
            bm.d_in[from] = 0;
            bm.d_tot[from] = 0;
            bm.d_tot[to] = bm.d_out[to] + bm.d_in[to] - chain_get(ch, to, to);
            bm.sizes[to] += bm.sizes[from];
            bm.sizes[from] = 0;
            parent[from] = to;
        }
        ++merged;
        __syncwarp();
    }
    if (lane == 0) *out_merged = (int32_t)merged;
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

void merge_propose(const DevGraph& g, const DevBM& bm, uint64_t seed, uint32_t step, Work& w, cudaStream_t st) {
    k_merge_propose<<<grid_cap(bm.B, kMergeWarps, 152 * 8), 256, 0, st>>>(g, bm, seed, step, w.best, w.best_dS,
                                                                          w.flags_dev);
    count_launches(1);
}

void carry_out(const DevGraph& g, DevBM& bm, int64_t num_to_merge, int approximate, Work& w, cudaStream_t st) {
    const int32_t B = bm.B;
    // queue order: stable sort of (delta, block)
    k_merge_keys<<<grid_cap(B, 256, 152 * 16), 256, 0, st>>>(w.best_dS, B, w.keys, w.vals);
    radix_sort_u64(w.keys, w.keys_alt, w.vals, w.vals_alt, B, 64, w.temp, st);
    k_iota<<<grid_cap(B, 256, 152 * 16), 256, 0, st>>>(w.parent, B);
    count_launches(2);
    int32_t* d_merged = w.d_scalar + 1;
    if (approximate) {
        k_carry_approx<<<1, 32, 0, st>>>(w.vals, B, w.best, w.parent, num_to_merge, d_merged);
    } else {
        chain_init(bm, w, (uint64_t)2 * (uint64_t)bm.nnz, st);
        k_carry_out<<<1, 32, 0, st>>>(g, bm, w.chain, w.vals, B, w.best, w.best_dS, w.heap_dS, w.heap_blk,
                                                 w.parent, num_to_merge, w.list_small, w.list_big, 2 * g.N,
                                                 d_merged, w.flags_dev);
    }
    count_launches(1);
    // union-find roots -> dense labels in ascending root order (build_mapping)
    k_roots<<<grid_cap(B, 256, 152 * 16), 256, 0, st>>>(w.parent, B, w.root);
    cudaMemsetAsync(w.used, 0, sizeof(int32_t) * B, st);
    k_mark_used<<<grid_cap(g.N, 256, 152 * 16), 256, 0, st>>>(bm.asg, g.N, w.root, w.used);
    scan_i32(w.used, w.used, B, false, w.d_scalar + 2, w.temp, st);
    k_relabel<<<grid_cap(g.N, 256, 152 * 16), 256, 0, st>>>(bm.asg, g.N, w.root, w.used);
    count_launches(3);
}

}  // namespace sbp

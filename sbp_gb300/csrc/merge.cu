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
__device__ long long merge_delta_fixed_chain(const DevGraph& g, const DevBM& bm, const DevChain& ch, int32_t r,
                                             int32_t s, long long* red) {
    typedef Group<kChainThreads> G;
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
    acc = G::sum(acc, red);
    sRow = G::sum(sRow, red);
    sCol = G::sum(sCol, red);
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

__global__ void __launch_bounds__(kChainThreads, 1) k_carry_out(
    DevGraph g, DevBM bm, DevChain ch, const int32_t* __restrict__ sorted_blk, int32_t nq,
    const int32_t* __restrict__ best, const double* __restrict__ best_dS, double* heap_dS, int32_t* heap_blk,
    int32_t* parent, long long num_to_merge, int32_t* new_rows, int32_t* new_cols, int new_cap,
    int32_t* out_merged, DevFlags* flags) {
    __shared__ long long red[32];
    __shared__ int32_t s_from, s_to, s_action, s_newn;
    const int tid = threadIdx.x;
    int32_t cursor = 0, heap_n = 0;  // owned by thread 0
    long long merged = 0;
    while (true) {
        if (tid == 0) {
            int action = ACT_STOP;
            if (merged < num_to_merge && (cursor < nq || heap_n > 0)) {
                int32_t blk;
                bool from_heap = false;
                if (cursor < nq && heap_n > 0) {
                    const int32_t a = sorted_blk[cursor];
                    from_heap = qless(heap_dS[0], heap_blk[0], best_dS[a], a);
                } else {
                    from_heap = heap_n > 0;
                }
                if (from_heap) {
                    blk = heap_blk[0];
                    // pop: move the last element to the root and sift down
                    --heap_n;
                    const double kd = heap_dS[heap_n];
                    const int32_t kb = heap_blk[heap_n];
                    int32_t i = 0;
                    while (true) {
                        const int32_t l = 2 * i + 1;
                        if (l >= heap_n) break;
                        int32_t c = l;
                        if (l + 1 < heap_n && qless(heap_dS[l + 1], heap_blk[l + 1], heap_dS[l], heap_blk[l])) c = l + 1;
                        if (!qless(heap_dS[c], heap_blk[c], kd, kb)) break;
                        heap_dS[i] = heap_dS[c];
                        heap_blk[i] = heap_blk[c];
                        i = c;
                    }
                    if (heap_n > 0) {
                        heap_dS[i] = kd;
                        heap_blk[i] = kb;
                    }
                } else {
                    blk = sorted_blk[cursor++];
                }
                const int32_t to = uf_find(parent, best[blk]);
                s_from = blk;
                s_to = to;
                action = (to == blk) ? ACT_SKIP : ACT_EVAL;
            }
            s_action = action;
        }
        __syncthreads();
        const int action = s_action;
        if (action == ACT_STOP) break;
        if (action == ACT_SKIP) {
            __syncthreads();
            continue;
        }
        const int32_t from = s_from, to = s_to;
        const long long dq = merge_delta_fixed_chain(g, bm, ch, from, to, red);
        if (tid == 0) {
            const double actual = fixed_to_double(dq);
            bool requeue = false;
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
                requeue = actual > top;  // block_merge.cpp:79
            }
            if (requeue) {
                int32_t i = heap_n++;
                while (i > 0) {
                    const int32_t p = (i - 1) >> 1;
                    if (!qless(actual, from, heap_dS[p], heap_blk[p])) break;
                    heap_dS[i] = heap_dS[p];
                    heap_blk[i] = heap_blk[p];
                    i = p;
                }
                heap_dS[i] = actual;
                heap_blk[i] = from;
                s_action = ACT_REQUEUE;
            } else {
                s_action = ACT_MERGE;
                s_newn = 0;
            }
        }
        __syncthreads();
        if (s_action == ACT_REQUEUE) {
            __syncthreads();
            continue;
        }
        // Blockmodel::merge_block (blockmodel.cpp:337-363): move row / column `from` into `to`.
        chain_for_each(bm.row_col, bm.row_off[from], bm.row_off[from + 1], ch.row_head[from], ch, [&](int32_t c) {
            const int32_t m = chain_get(ch, from, c);
            if (m == 0) return;
            chain_add(ch, from, c, -m, new_rows, new_cols, &s_newn, new_cap, flags);
            chain_add(ch, to, (c == from || c == to) ? to : c, m, new_rows, new_cols, &s_newn, new_cap, flags);
        });
        chain_for_each(bm.col_row, bm.col_off[from], bm.col_off[from + 1], ch.col_head[from], ch, [&](int32_t x) {
            if (x == from) return;
            const int32_t m = chain_get(ch, x, from);
            if (m == 0) return;
            chain_add(ch, x, from, -m, new_rows, new_cols, &s_newn, new_cap, flags);
            chain_add(ch, x, to, m, new_rows, new_cols, &s_newn, new_cap, flags);
        });
        __syncthreads();
        append_new_keys(ch, new_rows, new_cols, min(s_newn, new_cap), flags);
        if (tid == 0) {
            bm.d_out[to] += bm.d_out[from];
            bm.d_in[to] += bm.d_in[from];
            bm.d_out[from] = 0;
            bm.d_in[from] = 0;
            bm.d_tot[from] = 0;
            bm.d_tot[to] = bm.d_out[to] + bm.d_in[to] - chain_get(ch, to, to);
            bm.sizes[to] += bm.sizes[from];
            bm.sizes[from] = 0;
            parent[from] = to;
            ++merged;
        }
        __syncthreads();
    }
    if (tid == 0) *out_merged = (int32_t)merged;
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
        k_carry_out<<<1, kChainThreads, 0, st>>>(g, bm, w.chain, w.vals, B, w.best, w.best_dS, w.heap_dS, w.heap_blk,
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

// MCMC vertex-move sweep kernels.
//
// Asynchronous Gibbs (reference src/finetune.cpp:34-107, 563-646 low-degree part):
//   1. k_gibbs_small / k_gibbs_big: every vertex of the batch proposes against the same
//      snapshot (propose_gibbs_move_v3 + eval_vertex_move_v3, :871-901, :447-462): one
//      warp per vertex (k <= 128, shared-memory block hash per warp) or one CTA per
//      vertex for larger degrees.
//   2. apply in vertex-id order with the block-size-1 rule of
//      Blockmodel::move_vertex(VertexMove_v3) (src/blockmodel/blockmodel.cpp:437-443).
//      A move can only be refused when every member of its block leaves and it is the
//      last one (largest id); it is then refused unless an earlier accepted move entered
//      the block.  k_apply_* resolve this exactly in parallel (dependencies between
//      "last leavers" are resolved by a fixed point over a short list).
//   3. the caller rebuilds the blockmatrix from the new assignment (the serial
//      incremental apply ends in the same state).
// Hybrid MCMC sequential phase (:589-594): k_mh_chain, one CTA that walks the shuffled
// high-degree vertices and applies every accepted move before the next proposal.
#include <stdexcept>

#include "chain.cuh"
#include "delta.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace sbp {

namespace {

constexpr int kSmallLog2 = 8;  // 256-slot hash per warp: k <= 128
constexpr int kGibbsWarps = 8;

inline unsigned grid_cap(int64_t n, int64_t per, int64_t cap) {
    int64_t b = (n + per - 1) / per;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

__global__ void k_split_by_degree(DevGraph g, const int32_t* __restrict__ list, int32_t n, int32_t small_k,
                                  int32_t* __restrict__ out_small, int32_t* __restrict__ out_big,
                                  int32_t* __restrict__ counts) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t v = list[i];
        const int32_t k = (__ldg(g.out_off + v + 1) - __ldg(g.out_off + v)) +
                          (__ldg(g.inns_off + v + 1) - __ldg(g.inns_off + v));
        if (k <= small_k) out_small[atomicAdd(counts, 1)] = v;
        else out_big[atomicAdd(counts + 1, 1)] = v;
    }
}

// kMode: ACC_GREEDY (the default configuration, compiled without the Hastings
// correction), ACC_HASTINGS or ACC_NP (nonparametric delta, no correction).
template <int kThreads, int kMode>
__device__ __forceinline__ int32_t gibbs_one(const DevGraph& g, const DevBM& bm, int32_t v, uint64_t seed,
                                             uint32_t iter, uint32_t step, int32_t* hk, int32_t* hO, int32_t* hI,
                                             int log2cap, long long (*red)[8], DevFlags* flags) {
    const int32_t r = bm.asg[v];
    uint32_t w[4];
    philox4x32_10((uint32_t)v, iter, step, DOM_GIBBS, seed, w);
    const int32_t s = sample_vertex_proposal(g, bm, v, r, w);
    if (s < 0) {
        if (Group<kThreads>::rank() == 0) atomicOr(&flags->err, ERR_SELECT);
        return -1;
    }
    if (s == r) return -1;
    if constexpr (kMode == ACC_NP) {
        const long long dS = vertex_delta_fixed<kThreads, CsrAcc, true>(g, bm.asg, bm.d_out, bm.d_in, CsrAcc{bm}, v, r,
                                                                        s, hk, hO, hI, log2cap, red, bm.sizes,
                                                                        *bm.nonempty);
        return accept_move(dS, 1.0, false, w[3]) ? s : -1;
    }
    const long long dS =
        vertex_delta_fixed<kThreads>(g, bm.asg, bm.d_out, bm.d_in, CsrAcc{bm}, v, r, s, hk, hO, hI, log2cap, red);
    if (kMode == ACC_GREEDY) return dS < 0 ? s : -1;  // finetune::accept with greedy (finetune.cpp:22-25)
    double H = 1.0;
    const int32_t o0 = __ldg(g.out_off + v), i0 = __ldg(g.inns_off + v);
    const int32_t kout = __ldg(g.out_off + v + 1) - o0, kin = __ldg(g.inns_off + v + 1) - i0;
    if (kout + kin > 0)
        H = hastings_fixed<kThreads>(CsrAcc{bm}, [&](int32_t b) { return bm.d_tot[b]; }, bm.d_out, bm.d_in, bm.B, r,
                                     s, kout, kin, __ldg(g.selfcnt + v), hk, hO, hI, log2cap, red);
    return accept_move(dS, H, false, w[3]) ? s : -1;  // finetune::accept (finetune.cpp:26-31)
}

template <int kMode>
__global__ void __launch_bounds__(256) k_gibbs_small(DevGraph g, DevBM bm, const int32_t* __restrict__ list,
                                                     const int32_t* __restrict__ d_n, uint64_t seed, uint32_t iter,
                                                     uint32_t step, int32_t* __restrict__ moves, DevFlags* flags) {
    __shared__ int32_t hk[kGibbsWarps][1 << kSmallLog2];
    __shared__ int32_t hO[kGibbsWarps][1 << kSmallLog2];
    __shared__ int32_t hI[kGibbsWarps][1 << kSmallLog2];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int32_t n = *d_n;
    unsigned long long edges = 0, accepted = 0;
    for (int32_t i = blockIdx.x * kGibbsWarps + wid; i < n; i += gridDim.x * kGibbsWarps) {
        const int32_t v = list[i];
        const int32_t mv = gibbs_one<32, kMode>(g, bm, v, seed, iter, step, hk[wid], hO[wid], hI[wid], kSmallLog2,
                                                  nullptr, flags);
        if (lane == 0) {
            moves[v] = mv;
            edges += (__ldg(g.out_off + v + 1) - __ldg(g.out_off + v)) + (__ldg(g.inns_off + v + 1) - __ldg(g.inns_off + v));
            accepted += mv >= 0;
        }
    }
    if (lane == 0) {
        atomicAdd(&flags->counters[3], edges);
        atomicAdd(&flags->counters[1], accepted);
    }
}

template <int kMode>
__global__ void __launch_bounds__(256) k_gibbs_big(DevGraph g, DevBM bm, const int32_t* __restrict__ list,
                                                   const int32_t* __restrict__ d_n, uint64_t seed, uint32_t iter,
                                                   uint32_t step, int log2cap, int32_t* __restrict__ moves,
                                                   DevFlags* flags) {
    extern __shared__ int32_t dyn[];
    __shared__ long long red[32][8];
    const int cap = 1 << log2cap;
    const int32_t n = *d_n;
    for (int32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const int32_t v = list[i];
        const int32_t k = (__ldg(g.out_off + v + 1) - __ldg(g.out_off + v)) + (__ldg(g.inns_off + v + 1) - __ldg(g.inns_off + v));
        int32_t mv = -1;
        if (2 * k > cap) {
            if (threadIdx.x == 0) atomicOr(&flags->err, ERR_DEGREE);
        } else {
            mv = gibbs_one<256, kMode>(g, bm, v, seed, iter, step, dyn, dyn + cap, dyn + 2 * cap, log2cap, red, flags);
        }
        if (threadIdx.x == 0) {
            moves[v] = mv;
            atomicAdd(&flags->counters[3], (unsigned long long)k);
            if (mv >= 0) atomicAdd(&flags->counters[1], 1ull);
        }
        __syncthreads();
    }
}

// ---- apply with the block-size-1 rule
__global__ void k_apply_count(const int32_t* __restrict__ list, int32_t n, const int32_t* __restrict__ asg,
                              const int32_t* __restrict__ moves, int32_t* __restrict__ m_out, int32_t* __restrict__ last) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t v = list[i];
        if (moves[v] < 0) continue;
        const int32_t q = asg[v];
        atomicAdd(m_out + q, 1);
        atomicMax(last + q, v);
    }
}

__global__ void k_apply_saved(const int32_t* __restrict__ list, int32_t n, const int32_t* __restrict__ asg,
                              const int32_t* __restrict__ moves, const int32_t* __restrict__ sizes,
                              const int32_t* __restrict__ m_out, const int32_t* __restrict__ last,
                              int32_t* __restrict__ acc, int32_t* __restrict__ dep, int32_t* __restrict__ ndep) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t v = list[i];
        const int32_t t = moves[v];
        if (t < 0) continue;
        if (m_out[t] != sizes[t] || v >= last[t]) continue;  // t not at risk, or v arrives too late
        const int32_t q = asg[v];
        const bool v_last = m_out[q] == sizes[q] && last[q] == v;
        if (!v_last) {
            acc[t] = 1;  // a certainly accepted move enters t before its last leaver
        } else {
            const int32_t p = atomicAdd(ndep, 1);
            dep[2 * p] = q;
            dep[2 * p + 1] = t;
        }
    }
}

__global__ void k_resolve(const int32_t* __restrict__ dep, const int32_t* __restrict__ ndep, int32_t* acc,
                          DevFlags* flags) {
    __shared__ int changed;
    const int32_t n = *ndep;
    for (int32_t round = 0; round <= n; ++round) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const int32_t q = dep[2 * i], t = dep[2 * i + 1];
            if (((volatile int32_t*)acc)[q] && !((volatile int32_t*)acc)[t]) {
                acc[t] = 1;
                changed = 1;
            }
        }
        __syncthreads();
        if (!changed) return;
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicOr(&flags->err, ERR_STATE);
}

__global__ void k_apply_commit(const int32_t* __restrict__ list, int32_t n, int32_t* __restrict__ asg,
                               const int32_t* __restrict__ moves, const int32_t* __restrict__ sizes,
                               const int32_t* __restrict__ m_out, const int32_t* __restrict__ last,
                               const int32_t* __restrict__ acc, DevFlags* flags) {
    unsigned long long applied = 0;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t v = list[i];
        const int32_t t = moves[v];
        if (t < 0) continue;
        const int32_t q = asg[v];
        if (m_out[q] == sizes[q] && last[q] == v && !acc[q]) continue;  // would empty block q
        asg[v] = t;
        ++applied;
    }
    applied = (unsigned long long)warp_sum_ll((long long)applied);
    if ((threadIdx.x & 31) == 0 && applied) atomicAdd(&flags->counters[2], applied);
}

// ---- hybrid MH chain (one CTA)
__global__ void __launch_bounds__(kChainThreads, 1) k_mh_chain(DevGraph g, DevBM bm, DevChain ch,
                                                               const int32_t* __restrict__ order, int32_t n,
                                                               uint64_t seed, uint32_t iter, uint32_t step,
                                                               int log2cap, int nbits, DevFlags* flags) {
    extern __shared__ int32_t dyn[];
    __shared__ long long red[32][8];
    __shared__ int32_t hist[1024];
    __shared__ int s_bucket;
    __shared__ long long s_t;
    __shared__ int32_t s_v, s_r, s_go, s_nrs, s_ncs, s_p0, s_p1, s_Or, s_Ir, s_Os, s_Is, s_cnt;
    const int cap = 1 << log2cap;
    int32_t* hk = dyn;
    int32_t* hO = dyn + cap;
    int32_t* hI = dyn + 2 * cap;
    const int gcap = (3 * cap) / 2;
    int32_t* gkeys = dyn;
    int32_t* gvals = dyn + gcap;
    const int ncap = cap + 8;
    int32_t* nrows = dyn + 3 * cap;
    int32_t* ncols = nrows + ncap;
    const int tid = threadIdx.x;
    unsigned long long edges = 0, moved = 0;
    long long dsum = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (tid == 0) {
            const int32_t v = order[i];
            const int32_t r = bm.asg[v];
            s_v = v;
            s_r = r;
            s_go = bm.sizes[r] == 1 ? 0 : 1;  // propose_move: a singleton block never moves (finetune.cpp:845)
        }
        __syncthreads();
        const int32_t v = s_v, r = s_r;
        const int32_t o0 = __ldg(g.out_off + v), o1 = __ldg(g.out_off + v + 1);
        const int32_t i0 = __ldg(g.inns_off + v), i1 = __ldg(g.inns_off + v + 1);
        const int32_t kout = o1 - o0, kin = i1 - i0, k = kout + kin;
        edges += k;
        if (!s_go) {
            __syncthreads();
            continue;
        }
        if (2 * k > cap) {
            if (tid == 0) atomicOr(&flags->err, ERR_DEGREE);
            __syncthreads();
            continue;
        }
        uint32_t w[4];
        philox4x32_10((uint32_t)v, iter, step, DOM_MH, seed, w);
        int32_t s;
        if (k == 0) {
            s = random_block(r, bm.B, w[1]);
        } else {
            const int32_t idx = (int32_t)u32_below(w[0], (uint32_t)k);
            const int32_t nbr = idx < kout ? __ldg(g.out_nbr + o0 + idx) : __ldg(g.inns_nbr + i0 + idx - kout);
            const int32_t nb = ((volatile int32_t*)bm.asg)[nbr];
            const long long R = ((volatile int32_t*)bm.d_out)[nb];
            const long long C = (long long)((volatile int32_t*)bm.d_in)[nb] - chain_get(ch, nb, nb);
            long long t = (long long)u64_below(w[1], w[2], (uint64_t)(R + C));
            const bool in_row = t < R;
            if (!in_row) t -= R;
            if (tid == 0) s_cnt = 0;
            __syncthreads();
            auto gather = [&](int32_t key) {
                const int32_t val = in_row ? chain_get(ch, nb, key) : chain_get(ch, key, nb);
                if (val == 0 || (!in_row && key == nb)) return;
                const int p = atomicAdd(&s_cnt, 1);
                if (p < gcap) {
                    gkeys[p] = key;
                    gvals[p] = val;
                }
            };
            if (in_row) chain_for_each(bm.row_col, bm.row_off[nb], bm.row_off[nb + 1], ch.row_head[nb], ch, gather);
            else chain_for_each(bm.col_row, bm.col_off[nb], bm.col_off[nb + 1], ch.col_head[nb], ch, gather);
            __syncthreads();
            const int cnt = s_cnt;
            if (cnt > gcap) {
                if (tid == 0) atomicOr(&flags->err, ERR_DEGREE);
                __syncthreads();
                continue;
            }
            s = cta_radix_select(gkeys, gvals, cnt, t, nbits, -1, -1, hist, &s_bucket, &s_t);
            if (s < 0) {
                if (tid == 0) atomicOr(&flags->err, ERR_SELECT);
                __syncthreads();
                continue;
            }
        }
        if (s == r) {
            __syncthreads();
            continue;
        }
        const long long dS = vertex_delta_fixed<kChainThreads>(g, bm.asg, bm.d_out, bm.d_in, ChainAcc{ch}, v, r, s, hk,
                                                              hO, hI, log2cap, red);
        if (!(dS < 0)) {
            __syncthreads();
            continue;
        }
        // Blockmodel::move_vertex(Vertex, Delta, proposal) (blockmodel.cpp:408-435).  New
        // keys of row s / column s are staged and appended in bulk; every other list is
        // appended by the thread that owns its block.
        if (tid == 0) {
            s_nrs = 0;
            s_ncs = 0;
            s_Or = s_Ir = s_Os = s_Is = 0;
        }
        __syncthreads();
        for (int j = tid; j < cap; j += kChainThreads) {
            const int32_t b = hk[j];
            if (b < 0) continue;
            const int32_t O = hO[j], I = hI[j];
            if (b == r) {
                s_Or = O;
                s_Ir = I;
                continue;
            }
            if (b == s) {
                s_Os = O;
                s_Is = I;
                continue;
            }
            if (O) {
                chain_add(ch, r, b, -O, flags);
                if (chain_add(ch, s, b, O, flags)) {
                    stage(nrows, &s_nrs, ncap, b, flags);
                    list_push1(ch.col_head, ch, b, s, flags);
                }
            }
            if (I) {
                chain_add(ch, b, r, -I, flags);
                if (chain_add(ch, b, s, I, flags)) {
                    list_push1(ch.row_head, ch, b, s, flags);
                    stage(ncols, &s_ncs, ncap, b, flags);
                }
            }
        }
        __syncthreads();
        const int32_t L = __ldg(g.selfcnt + v);
        if (tid == 0) {
            if (chain_add(ch, r, r, -s_Or - s_Ir - L, flags)) {
                list_push1(ch.row_head, ch, r, r, flags);
                list_push1(ch.col_head, ch, r, r, flags);
            }
            if (chain_add(ch, r, s, s_Ir - s_Os, flags)) {
                list_push1(ch.row_head, ch, r, s, flags);
                stage(ncols, &s_ncs, ncap, r, flags);
            }
            if (chain_add(ch, s, r, s_Or - s_Is, flags)) {
                stage(nrows, &s_nrs, ncap, r, flags);
                list_push1(ch.col_head, ch, r, s, flags);
            }
            if (chain_add(ch, s, s, s_Os + s_Is + L, flags)) {
                stage(nrows, &s_nrs, ncap, s, flags);
                stage(ncols, &s_ncs, ncap, s, flags);
            }
        }
        __syncthreads();
        {
            const int nr = min(s_nrs, ncap), nc = min(s_ncs, ncap);
            if (tid == 0) s_p0 = nr > 0 ? list_reserve(ch.row_head, ch, s, nr, flags) : -1;
            if (tid == 32) s_p1 = nc > 0 ? list_reserve(ch.col_head, ch, s, nc, flags) : -1;
            __syncthreads();
            if (s_p0 >= 0)
                for (int i = tid; i < nr; i += kChainThreads) ch.pool[s_p0 + i] = nrows[i];
            if (s_p1 >= 0)
                for (int i = tid; i < nc; i += kChainThreads) ch.pool[s_p1 + i] = ncols[i];
        }
        if (tid == 0) {
            const int32_t selfw = L > 0 ? 1 : 0;
            bm.d_out[r] -= kout;
            bm.d_out[s] += kout;
            bm.d_in[r] -= (kin + selfw);
            bm.d_in[s] += (kin + selfw);
            bm.d_tot[r] = bm.d_out[r] + bm.d_in[r] - chain_get(ch, r, r);
            bm.d_tot[s] = bm.d_out[s] + bm.d_in[s] - chain_get(ch, s, s);
            bm.sizes[r] -= 1;
            bm.sizes[s] += 1;
            bm.asg[v] = s;
            moved++;
            dsum += dS;
        }
        __syncthreads();
    }
    if (tid == 0) {
        atomicAdd(&flags->counters[4], edges);
        atomicAdd(&flags->counters[5], moved);
        atomicAdd(&flags->counters[7], (unsigned long long)dsum);
    }
}

__global__ void k_shuffle_keys(const int32_t* __restrict__ base, int32_t n, uint64_t seed, uint32_t iter,
                               uint32_t step, uint32_t dom, uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t w[4];
        philox4x32_10((uint32_t)i, iter, step, dom, seed, w);
        keys[i] = ((uint64_t)w[0] << 32) | (uint32_t)i;
        vals[i] = base[i];
    }
}

}  // namespace

template <int kMode>
void gibbs_launch(const DevGraph& g, const DevBM& bm, int32_t n, int32_t max_k, const int32_t* counts, uint64_t seed,
                  uint32_t iter, uint32_t step, Work& w, cudaStream_t st) {
    k_gibbs_small<kMode><<<grid_cap(n, kGibbsWarps, device_sms() * 8), 256, 0, st>>>(g, bm, w.list_small, counts, seed, iter,
                                                                            step, w.moves, w.flags_dev);
    count_launches(1);
    if (max_k > (1 << (kSmallLog2 - 1))) {
        int log2cap = ceil_log2((uint64_t)(2 * max_k));
        if (log2cap > 14) log2cap = 14;
        const size_t smem = (size_t)(3 * sizeof(int32_t)) << log2cap;
        allow_max_dynamic_smem((const void*)k_gibbs_big<kMode>);
        k_gibbs_big<kMode><<<device_sms() * 2, 256, smem, st>>>(g, bm, w.list_big, counts + 1, seed, iter, step, log2cap,
                                                       w.moves, w.flags_dev);
        count_launches(1);
    }
}

void gibbs_propose(const DevGraph& g, const DevBM& bm, const int32_t* vlist, int32_t n, int32_t max_k, uint64_t seed,
                   uint32_t iter, uint32_t step, int mode, Work& w, cudaStream_t st) {
    if (n <= 0) return;
    if (mode == ACC_NP && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    int32_t* counts = w.d_scalar + 6;  // [6], [7]
    cudaMemsetAsync(counts, 0, 2 * sizeof(int32_t), st);
    k_split_by_degree<<<grid_cap(n, 256, device_sms() * 16), 256, 0, st>>>(g, vlist, n, 1 << (kSmallLog2 - 1), w.list_small,
                                                                  w.list_big, counts);
    count_launches(1);
    if (mode == ACC_NP) gibbs_launch<ACC_NP>(g, bm, n, max_k, counts, seed, iter, step, w, st);
    else if (mode == ACC_HASTINGS) gibbs_launch<ACC_HASTINGS>(g, bm, n, max_k, counts, seed, iter, step, w, st);
    else gibbs_launch<ACC_GREEDY>(g, bm, n, max_k, counts, seed, iter, step, w, st);
}

void gibbs_apply(const DevBM& bm, const int32_t* vlist, int32_t n, Work& w, cudaStream_t st) {
    if (n <= 0) return;
    int32_t* ndep = w.d_scalar + 3;
    cudaMemsetAsync(w.m_out, 0, sizeof(int32_t) * bm.B, st);
    cudaMemsetAsync(w.last, 0xff, sizeof(int32_t) * bm.B, st);
    cudaMemsetAsync(w.acc, 0, sizeof(int32_t) * bm.B, st);
    cudaMemsetAsync(ndep, 0, sizeof(int32_t), st);
    const unsigned grid = grid_cap(n, 256, device_sms() * 16);
    k_apply_count<<<grid, 256, 0, st>>>(vlist, n, bm.asg, w.moves, w.m_out, w.last);
    k_apply_saved<<<grid, 256, 0, st>>>(vlist, n, bm.asg, w.moves, bm.sizes, w.m_out, w.last, w.acc, w.dep, ndep);
    k_resolve<<<1, 1024, 0, st>>>(w.dep, ndep, w.acc, w.flags_dev);
    k_apply_commit<<<grid, 256, 0, st>>>(vlist, n, bm.asg, w.moves, bm.sizes, w.m_out, w.last, w.acc, w.flags_dev);
    count_launches(4);
}

void mh_chain(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, int32_t max_k, uint64_t seed,
              uint32_t iter, uint32_t step, int greedy, Work& w, cudaStream_t st) {
    if (n <= 0) return;
    int log2cap = ceil_log2((uint64_t)(2 * (max_k > 64 ? max_k : 64)));
    if (log2cap > 13) log2cap = 13;
    const size_t smem = (size_t)(3 * sizeof(int32_t) << log2cap) + 2 * sizeof(int32_t) * ((1 << log2cap) + 8);
    allow_max_dynamic_smem((const void*)k_mh_chain);
    const int nbits = ceil_log2((uint64_t)(bm.B > 1 ? bm.B : 2));
    k_mh_chain<<<1, kChainThreads, smem, st>>>(g, bm, w.chain, order, n, seed, iter, step, log2cap, nbits, w.flags_dev);
    count_launches(1);
    (void)greedy;
}

void shuffle(const int32_t* base, int32_t n, uint64_t seed, uint32_t iter, uint32_t step, uint32_t dom,
             int32_t* order, Work& w, cudaStream_t st) {
    if (n <= 0) return;
    k_shuffle_keys<<<grid_cap(n, 256, device_sms() * 16), 256, 0, st>>>(base, n, seed, iter, step, dom, w.keys, w.vals);
    radix_sort_u64(w.keys, w.keys_alt, w.vals, w.vals_alt, n, 64, w.temp, st);
    cudaMemcpyAsync(order, w.vals, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st);
    count_launches(1);
}

}  // namespace sbp

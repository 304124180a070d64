// Sequential Metropolis-Hastings chain of hybrid MCMC (reference src/finetune.cpp:589-594;
// propose_move :842-869, move_vertex :822-840, Blockmodel::move_vertex(Vertex, Delta,
// proposal) src/blockmodel/blockmodel.cpp:408-435), evaluated in windows.
//
// The chain visits vertices in order and applies each accepted move before the next
// proposal.  A proposal and its delta read only
//   * the blocks of the vertex's neighbours, r = its block, s = the proposal, nb = the
//     block of the sampled neighbour,
//   * cells of rows / columns r and s (and of nb, for the sampler), block degrees and
//     sizes of those blocks,
// so a move u: a -> b can change the outcome of a later vertex v only if a or b lies in
// T(v) = {r, s, nb} + v's neighbour blocks, or nb(v) lies in T(u) (u's neighbours in
// block nb shift counts of row / column nb between columns / rows a and b).  Each round
// therefore evaluates the next W vertices of the order at once (one warp each) against
// the same state; the replay takes them in order and stops before the first vertex
// that an earlier accepted move of the round may have changed (one ballot: that vertex is
// the first with a conflict bit, since the bits name accepted earlier entries only); the
// accepted moves are then applied together (every update is an addition, so their order
// does not matter).
// The result equals the one-vertex-at-a-time chain exactly.
//
// Nonparametric entropy (kNP): a delta also reads the sizes of r and s (covered by T(v))
// and, when the move would empty r or fill s, the number of non-empty blocks; an accepted
// move that changes that number therefore also ends the round before every later entry
// whose delta read it.
//
// Cell counts: B x B dense in shared memory (B <= kWinSharedMax) or dense M and its
// transpose in global memory (leading dimension a multiple of 4); degrees and sizes in
// shared memory unless B is large.  Each warp's neighbour hash lives in shared memory (up
// to 512 slots) or, for vertices of degree above 256, in a per-warp global region.  Only
// the assignment is written back; the caller rebuilds afterwards.
#include <climits>
#include <stdexcept>

#include "window.cuh"

namespace sbp {

namespace {

// kMode 0: cells, degrees and sizes in shared memory; 1: cells dense in global memory,
// degrees and sizes in shared memory; 2: all of them in global memory (large B).
template <int kMode, bool kNP>
__global__ void __launch_bounds__(kWinMaxWarps * 32, 1)
    k_mh_window(DevGraph g, DevBM bm, const int32_t* __restrict__ order, int32_t n, uint64_t seed, uint32_t iter,
                uint32_t step, GlobalCells gc, int32_t ld, int log2cap, int nwarps, bool greedy, int32_t* ghash,
                DevFlags* flags) {
    constexpr bool kShared = kMode == 0;
    constexpr bool kGlobalDeg = kMode == 2;
    extern __shared__ int32_t sm[];
    const int32_t B = bm.B;
    const int cap = 1 << log2cap;
    int32_t* dout = kGlobalDeg ? bm.d_out : sm;
    int32_t* din = kGlobalDeg ? bm.d_in : dout + B;
    int32_t* size = kGlobalDeg ? bm.sizes : din + B;
    int32_t* hash = kGlobalDeg ? sm : size + B;  // nwarps x (keys, out counts, in counts, items) x 512
    int32_t* lq = hash + (4 << kSmemHashL2) * nwarps;  // the first kLqCache log-table entries
    int32_t* M = lq + kLqCache;                        // shared cells (kShared): B rows of ld
    // a vertex's hash: shared memory up to 2^kSmemHashL2 slots, else the warp's global region
    // Each warp's hash: keys, out counts, in counts and the list of taken slots, at a fixed
    // stride (2^kSmemHashL2 in shared memory, 2^kGlobalHashL2 in the global region) so that
    // a slot keeps its place whatever the size of the hash that used it last.
    auto hash_of = [&](int w, int l2) {
        return l2 <= kSmemHashL2 ? hash + (4 << kSmemHashL2) * w : ghash + ((int64_t)4 << kGlobalHashL2) * w;
    };
    __shared__ WinResult res[kWinMaxWarps];
    __shared__ int32_t s_consumed, s_acc_mask, s_ne;
    __shared__ uint32_t s_conf[kWinMaxWarps];
    __shared__ int32_t s_dirty[kWinMaxWarps];   // slots of the shared hash left by the last one
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nt = nwarps * 32;
    (void)cap;

    for (int i = tid; i < kLqCache; i += nt) lq[i] = __ldg(g.Lq + min(i, g.E + 1));
    // the shared hashes start clean and are kept clean through their slot lists
    for (int i = tid; i < nwarps << (kSmemHashL2 + 2); i += nt) {
        const int part = (i >> kSmemHashL2) & 3;
        if (part < 3) hash[i] = part == 0 ? -1 : 0;
    }
    if (tid < kWinMaxWarps) s_dirty[tid] = 0;
    if (tid == 0) s_ne = kNP ? *bm.nonempty : 0;
    if (kShared) {
        for (int i = tid; i < B * ld; i += nt) M[i] = 0;
        __syncthreads();
        for (int32_t j = tid; j < bm.nnz; j += nt) M[bm.row_of[j] * ld + bm.row_col[j]] = bm.row_cnt[j];
    }
    if (!kGlobalDeg) {
        for (int b = tid; b < B; b += nt) {
            dout[b] = bm.d_out[b];
            din[b] = bm.d_in[b];
            size[b] = bm.sizes[b];
        }
    }
    __syncthreads();
    const SharedCells sc{M, ld};

    unsigned long long edges = 0, moved = 0, rounds = 0;
    long long dsum = 0;
    int32_t it0 = 0, next_pos = -1, next_v = -1;
    int guard = 0;
    while (it0 < n && guard++ < (1 << 30)) {
        const int wn = min(nwarps, n - it0);
        // ---- evaluate the next wn vertices against the current state, one warp each
        if (wid < wn) {
            WinResult c;
            c.v = next_pos == it0 + wid ? next_v : order[it0 + wid];
            c.r = __ldcg(bm.asg + c.v);
            c.s = -1;
            c.nb = -1;
            c.dS = 0;
            c.dB = 0;
            c.ni = 0;
            const int32_t o0 = __ldg(g.out_off + c.v), o1 = __ldg(g.out_off + c.v + 1);
            const int32_t i0 = __ldg(g.inns_off + c.v), i1 = __ldg(g.inns_off + c.v + 1);
            c.kout = o1 - o0;
            c.kin = i1 - i0;
            c.k = c.kout + c.kin;
            c.L = __ldg(g.selfcnt + c.v);
            c.l2 = hash_log2(c.k, log2cap);
            c.status = ST_SKIP;
            const bool in_smem = c.l2 <= kSmemHashL2;
            const int32_t hs = in_smem ? 1 << kSmemHashL2 : 1 << kGlobalHashL2;
            int32_t* hk = hash_of(wid, c.l2);
            int32_t* hO = hk + hs;
            int32_t* hI = hO + hs;
            int32_t* items = hI + hs;
            if (size[c.r] != 1) {  // a singleton block never moves (finetune.cpp:845)
                uint32_t w[4];
                philox4x32_10((uint32_t)c.v, iter, step, DOM_MH, seed, w);
                // a clean hash: the shared one through the slot list of its last use, the
                // global one (vertices of degree above 256) in full
                if (in_smem) {
                    const int32_t nd = s_dirty[wid];
                    for (int j = lane; j < nd; j += 32) {
                        const int32_t sl = items[j];
                        hk[sl] = -1;
                        hO[sl] = 0;
                        hI[sl] = 0;
                    }
                } else {
                    for (int i = lane; i < (1 << c.l2); i += 32) {
                        hk[i] = -1;
                        hO[i] = 0;
                        hI[i] = 0;
                    }
                }
                __syncwarp();
                // the neighbour blocks first; the proposal's sampled neighbour is among them
                const int32_t idx = c.k > 0 ? (int32_t)u32_below(w[0], (uint32_t)c.k) : -1;
                // (the shared hash through pointers the compiler sees are shared: its inserts
                // are then shared-memory atomics)
                // the sampler's first reads (cell (nb, nb), nb's degrees and the first group
                // of tile sums of its row and column), issued before the hash inserts
                int32_t p_dnn = 0, p_R = 0, p_din = 0, p_tr[8], p_tc[8];
                auto on_nb = [&](int32_t nb) {
                    if (kShared || nb < 0) return;
                    p_dnn = gc.row_get(nb, nb);
                    p_R = dout[nb];
                    p_din = din[nb];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int32_t tile = 8 * lane + j;
                        p_tr[j] = tile < gc.nt ? __ldcg(gc.TS + (int64_t)nb * gc.nt + tile) : 0;
                        p_tc[j] = tile < gc.nt ? __ldcg(gc.TST + (int64_t)nb * gc.nt + tile) : 0;
                    }
                };
                int32_t* sh = hash + (4 << kSmemHashL2) * wid;
                const int32_t nbg =
                    in_smem ? warp_gather(g, bm.asg, c.v, c.r, o0, c.kout, i0, c.k, idx, sh, sh + (1 << kSmemHashL2),
                                          sh + (2 << kSmemHashL2), c.l2, sh + (3 << kSmemHashL2), c.ni, on_nb)
                            : warp_gather(g, bm.asg, c.v, c.r, o0, c.kout, i0, c.k, idx, hk, hO, hI, c.l2, items, c.ni,
                                          on_nb);
                if (in_smem && lane == 0) s_dirty[wid] = c.ni;
                int32_t s;
                if (c.k == 0) {
                    s = random_block(c.r, B, w[1]);
                } else {
                    // common::propose_new_block: uniform neighbour, then a multinomial over
                    // nb's row (ascending column) followed by its column without the diagonal
                    const int32_t nb = nbg;
                    c.nb = nb;
                    const int32_t dnn = kShared ? sc.row_get(nb, nb) : p_dnn;
                    const long long R = kShared ? dout[nb] : p_R, C = (long long)(kShared ? din[nb] : p_din) - dnn;
                    long long t = (long long)u64_below(w[1], w[2], (uint64_t)(R + C));
                    if (t < R) {
                        s = kShared ? warp_select(B, t, [&](int32_t i) { return sc.row_get(nb, i); })
                                    : warp_select_tiles(gc.M + (int64_t)nb * ld, gc.TS + (int64_t)nb * gc.nt, B,
                                                        gc.nt, t, -1, 0, p_tr);
                    } else {
                        t -= R;
                        s = kShared ? warp_select(B, t, [&](int32_t i) { return i == nb ? 0 : sc.row_get(i, nb); })
                                    : warp_select_tiles(gc.MT + (int64_t)nb * ld, gc.TST + (int64_t)nb * gc.nt, B,
                                                        gc.nt, t, nb, dnn, p_tc);
                    }
                }
                if (s < 0) {
                    if (lane == 0) atomicOr(&flags->err, ERR_SELECT);
                    c.status = ST_SKIP;
                } else if (s == c.r) {
                    c.status = ST_NOMOVE;
                } else {
                    c.s = s;
                    if constexpr (kNP) c.dB = np_count_change(size[c.r], size[s], 1);
                    c.dS = kShared ? warp_delta<SharedCells, kNP>(g, dout, din, sc, c.r, s, c.kout, c.kin, c.L, hk, hO,
                                                                  hI, items, c.ni, lq, size, s_ne)
                                   : warp_delta<GlobalCells, kNP>(g, dout, din, gc, c.r, s, c.kout, c.kin, c.L, hk, hO,
                                                                  hI, items, c.ni, lq, size, s_ne);
                    double H = 1.0;
                    if (!kNP && !greedy && c.k > 0) {  // entropy::hastings_correction (entropy.cpp:497-561)
                        H = kShared ? hastings_fixed<32>(sc, [&](int32_t b) { return dout[b] + din[b] - sc.row_get(b, b); },
                                                         dout, din, B, c.r, s, c.kout, c.kin, c.L, hk, hO, hI, c.l2,
                                                         nullptr)
                                    : hastings_fixed<32>(gc, [&](int32_t b) { return dout[b] + din[b] - gc.row_get(b, b); },
                                                         dout, din, B, c.r, s, c.kout, c.kin, c.L, hk, hO, hI, c.l2,
                                                         nullptr);
                    }
                    // finetune::accept (finetune.cpp:22-32)
                    c.status = accept_move(c.dS, H, greedy && !kNP, w[3]) ? ST_ACCEPT : ST_REJECT;
                }
            }
            if (lane == 0) res[wid] = c;
        }
        // bit u of s_conf[j]: an accepted move of window entry u would change entry j
        if (tid < kWinMaxWarps) s_conf[tid] = 0u;
        __syncthreads();
        if (tid < wn * wn) {
            const int u = tid / wn, j = tid % wn;
            if (u < j && res[u].status == ST_ACCEPT) {
                const WinResult& cj = res[j];
                const WinResult& cu = res[u];
                const int32_t* hj = hash_of(j, cj.l2);
                if (in_touched(cj, hj, cu.r) || in_touched(cj, hj, cu.s) ||
                    (cj.nb >= 0 && in_touched(cu, hash_of(u, cu.l2), cj.nb)) ||
                    (kNP && cu.dB != 0 && cj.dB != 0 && cj.status >= ST_REJECT))
                    atomicOr(&s_conf[j], 1u << u);
            }
        }
        __syncthreads();
        // ---- replay in order; stop before the first vertex an accepted move may change.
        // s_conf[j] holds accepted entries before j only, and every entry before the stop
        // is taken, so the stop is the first entry with a conflict bit: one ballot.
        if (wid == 0) {
            const unsigned stop = __ballot_sync(SBP_FULL_MASK, lane < wn && s_conf[lane] != 0u);
            const int consumed = stop ? __ffs(stop) - 1 : wn;
            const bool taken = lane < consumed;
            const bool acc = taken && res[lane].status == ST_ACCEPT;
            const unsigned acc_mask = __ballot_sync(SBP_FULL_MASK, acc);
            const int32_t k_sum = warp_sum_i(taken ? res[lane].k : 0);
            const long long d_sum = warp_sum_ll(acc ? res[lane].dS : 0ll);
            const int32_t dB_sum = warp_sum_i(acc ? res[lane].dB : 0);
            if (lane == 0) {
                edges += (unsigned long long)k_sum;
                moved += (unsigned long long)__popc(acc_mask);
                dsum += d_sum;
                s_ne += dB_sum;  // blockmodel.cpp:429-430
                s_consumed = consumed;
                s_acc_mask = (int32_t)acc_mask;
                ++rounds;
            }
        }
        __syncthreads();
        // the vertex this warp evaluates next, loaded while the moves are applied
        next_pos = it0 + s_consumed + wid;
        if (wid < nwarps && next_pos < n) next_v = __ldg(order + next_pos);
        else next_pos = -1;
        // ---- apply the accepted moves (Blockmodel::move_vertex, blockmodel.cpp:408-435)
        if (wid < wn && ((s_acc_mask >> wid) & 1)) {
            const WinResult c = res[wid];
            const int32_t r = c.r, s = c.s;
            const int32_t hs = c.l2 <= kSmemHashL2 ? 1 << kSmemHashL2 : 1 << kGlobalHashL2;
            const int32_t* hk = hash_of(wid, c.l2);
            const int32_t* hO = hk + hs;
            const int32_t* hI = hO + hs;
            const int32_t* items = hI + hs;
            for (int j = lane; j < c.ni; j += 32) {
                const int i = items[j];
                const int32_t b = hk[i];
                if (b == r || b == s) continue;
                const int32_t O = hO[i], I = hI[i];
                if (kShared) {
                    if (O) {
                        atomicAdd(M + r * ld + b, -O);
                        atomicAdd(M + s * ld + b, O);
                    }
                    if (I) {
                        atomicAdd(M + b * ld + r, -I);
                        atomicAdd(M + b * ld + s, I);
                    }
                } else {
                    if (O) {
                        gc.add(r, b, -O);
                        gc.add(s, b, O);
                    }
                    if (I) {
                        gc.add(b, r, -I);
                        gc.add(b, s, I);
                    }
                }
            }
            if (lane == 0) {
                const int32_t Or = hash_get(hk, hO, c.l2, r), Ir = hash_get(hk, hI, c.l2, r);
                const int32_t Os = hash_get(hk, hO, c.l2, s), Is = hash_get(hk, hI, c.l2, s);
                const int32_t L = c.L, selfw = L > 0 ? 1 : 0;
                const int32_t drr = -Or - Ir - L, drs = Ir - Os, dsr = Or - Is, dss = Os + Is + L;
                if (kShared) {
                    atomicAdd(M + r * ld + r, drr);
                    atomicAdd(M + r * ld + s, drs);
                    atomicAdd(M + s * ld + r, dsr);
                    atomicAdd(M + s * ld + s, dss);
                } else {
                    gc.add(r, r, drr);
                    gc.add(r, s, drs);
                    gc.add(s, r, dsr);
                    gc.add(s, s, dss);
                }
                atomicAdd(dout + r, -c.kout);
                atomicAdd(dout + s, c.kout);
                atomicAdd(din + r, -(c.kin + selfw));
                atomicAdd(din + s, c.kin + selfw);
                atomicAdd(size + r, -1);
                atomicAdd(size + s, 1);
                bm.asg[c.v] = s;
            }
        }
        it0 += s_consumed;
        __syncthreads();
    }
    if (tid == 0) {
        atomicAdd(&flags->counters[4], edges);
        atomicAdd(&flags->counters[5], moved);
        atomicAdd(&flags->counters[7], (unsigned long long)dsum);
        atomicAdd(&flags->counters[8], rounds);
    }
}

constexpr size_t kWinSmemBudget = 220 * 1024;

size_t window_smem(int32_t B, int mode, int log2cap, int nwarps) {
    (void)log2cap;
    const size_t deg = mode == 2 ? 0 : 3 * (size_t)B;
    const size_t cells = mode == 0 ? (size_t)B * ((size_t)B + 1) : 0;
    return sizeof(int32_t) * (deg + ((size_t)nwarps << (kSmemHashL2 + 2)) + kLqCache + cells);
}

}  // namespace

uint64_t mh_window_cells(int32_t B) {
    const uint64_t ld = ((uint64_t)B + 3) & ~3ull, nt = ((uint64_t)B + 127) >> 7;
    return 2 * (uint64_t)B * ld + 2 * (uint64_t)B * nt;
}

bool mh_window_plan(int32_t B, int32_t max_k, const Work& w, WindowPlan* p) {
    const int l = ceil_log2((uint64_t)(2 * (max_k > 16 ? max_k : 16)));
    if (l > kGlobalHashL2 || (l > kSmemHashL2 && !w.win_hash)) return false;
    p->log2cap = l;
    if (B <= kWinSharedMax) {
        p->mode = 0;
        p->ld = B + 1;
    } else {
        if (!w.cells || mh_window_cells(B) > w.cells_elems) return false;
        p->ld = ((int64_t)B + 3) & ~3ll;
        p->mode = window_smem(B, 1, l, kWinMaxWarps) <= kWinSmemBudget ? 1 : 2;
    }
    int nw = kWinMaxWarps;
    while (nw > 0 && window_smem(B, p->mode, l, nw) > kWinSmemBudget) --nw;
    p->nw = nw;
    return nw >= 2;
}

template <int kMode>
void launch_window(bool np, const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, const WindowPlan& p,
                   uint64_t seed, uint32_t iter, uint32_t step, bool greedy, const GlobalCells& gc, size_t smem,
                   Work& w, cudaStream_t st) {
    auto k = np ? k_mh_window<kMode, true> : k_mh_window<kMode, false>;
    allow_max_dynamic_smem((const void*)k);
    k<<<1, 32 * p.nw, smem, st>>>(g, bm, order, n, seed, iter, step, gc, (int32_t)p.ld, p.log2cap, p.nw, greedy,
                                  w.win_hash, w.flags_dev);
}

void mh_chain_window(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, const WindowPlan& p,
                     uint64_t seed, uint32_t iter, uint32_t step, int mode, Work& w, cudaStream_t st) {
    if (n <= 0) return;
    if (mode == ACC_NP && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    const size_t smem = window_smem(bm.B, p.mode, p.log2cap, p.nw);
    const bool np = mode == ACC_NP, greedy = mode == ACC_GREEDY;
    if (p.mode == 0) {
        launch_window<0>(np, g, bm, order, n, p, seed, iter, step, greedy, GlobalCells{}, smem, w, st);
        count_launches(1);
        return;
    }
    const int64_t B = bm.B, nt = (B + 127) >> 7;
    GlobalCells gc;
    gc.ld = p.ld;
    gc.nt = (int32_t)nt;
    gc.M = w.cells;
    gc.MT = gc.M + B * p.ld;
    gc.TS = gc.MT + B * p.ld;
    gc.TST = gc.TS + B * nt;
    window_fill(bm, gc, st);
    if (p.mode == 1) launch_window<1>(np, g, bm, order, n, p, seed, iter, step, greedy, gc, smem, w, st);
    else launch_window<2>(np, g, bm, order, n, p, seed, iter, step, greedy, gc, smem, w, st);
    count_launches(2);
}

}  // namespace sbp

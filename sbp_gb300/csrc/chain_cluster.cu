// Sequential Metropolis-Hastings chain of hybrid MCMC (reference src/finetune.cpp:589-594;
// propose_move :842-869, move_vertex :822-840, Blockmodel::move_vertex(Vertex, Delta,
// proposal) src/blockmodel/blockmodel.cpp:408-435) evaluated in windows spread over a
// thread-block cluster, for blockmodels with many blocks.
//
// The window rule is the one of chain_window.cu: the next W vertices of the order are
// evaluated against one state, and the round takes them in order up to the first vertex
// that an accepted move of an earlier entry may have changed (a move u: a -> b changes v
// only if a or b lies in T(v) = {r, s, nb} + v's neighbour blocks, or nb(v) lies in T(u)).
// With many blocks such conflicts are rare, so the window is wide: every CTA of the
// cluster (one per SM) evaluates 16 entries, one warp each, W = 16 x cluster size.  The
// cluster's distributed shared memory carries the rest of the round:
//   1. each warp evaluates its entry (gather of the neighbour blocks into its shared hash,
//      the proposal's multinomial draw, delta, acceptance) and publishes the result;
//   2. cluster barrier; each CTA copies the window's results, tests its own entries
//      against every accepted earlier entry (reading the hashes of entries of other CTAs
//      through distributed shared memory) and records its first conflicted entry;
//   3. cluster barrier; the round stops at the smallest of those, and each CTA applies
//      its accepted entries before the stop (every update is an atomic addition, so the
//      order of the round's moves does not matter);
//   4. cluster barrier; the next round starts after the stop.
// The barriers are the hardware cluster barrier (no spinning on memory).  The result equals
// the one-vertex-at-a-time chain exactly.
//
// Cells: dense M and its transpose in global memory with row tile sums (GlobalCells) while
// they fit the dense budget, else the chain hash (HashCells): exact counts under
// open-addressing keys and per-row / per-column key lists.  A multinomial draw over a
// hashed row copies the row's keys and counts to the warp's scratch and selects by 5-bit
// digits of the key (ascending key order, the canonical order of the draw).  Degrees and
// sizes are read and updated in global memory; the caller rebuilds afterwards.
#include <cooperative_groups.h>

#include <stdexcept>
#include <type_traits>

#include "chain.cuh"
#include "window.cuh"

namespace cg = cooperative_groups;

namespace sbp {

namespace {

constexpr int kClWarps = 16;          // window entries per CTA
constexpr int kClMaxCluster = 16;
constexpr int kScratchCap = 4096;     // keys of a hashed row copied for a draw (per warp)

// Cell counts in the chain hash.  A new key is appended to its row's and column's key
// lists; lists receive keys from several CTAs at once (list_push1_shared).
struct HashCells {
    DevChain ch;
    __device__ __forceinline__ int32_t row_get(int32_t r, int32_t c) const { return chain_get(ch, r, c); }
    __device__ __forceinline__ int32_t col_get(int32_t c, int32_t r) const { return chain_get(ch, r, c); }
    __device__ __forceinline__ void add(int32_t r, int32_t c, int32_t d, DevFlags* flags) const {
        if (d == 0) return;
        bool ins;
        const int32_t slot = chain_slot(ch, r, c, &ins, flags);
        if (slot < 0) return;
        atomicAdd(slot_val(ch, slot), d);
        if (ins) {
            list_push1_shared(ch.row_head, ch, r, c, flags);
            list_push1_shared(ch.col_head, ch, c, r, flags);
        }
    }
};

__device__ __forceinline__ void cells_add(const GlobalCells& gc, int32_t r, int32_t c, int32_t d, DevFlags*) {
    gc.add(r, c, d);
}
__device__ __forceinline__ void cells_add(const HashCells& hc, int32_t r, int32_t c, int32_t d, DevFlags* flags) {
    hc.add(r, c, d, flags);
}

// Entry at cumulative unit t, in ascending key order, over one chain list (snapshot
// segment seg[lo, hi) and the chunks from head) weighted by the current counts get(key),
// key `skip` left out; one warp.  Keys and weights go to the warp's scratch (sk, sw; cap
// entries), then each 5-bit digit of the key, from the top, is chosen by a 32-bin weighted
// histogram.  Returns -1 when t is out of range or the list exceeds the scratch.
template <class Get>
__device__ int32_t warp_select_list(const int32_t* __restrict__ seg, int32_t lo, int32_t hi, int32_t head,
                                    const DevChain& ch, long long t, int32_t skip, int nbits, int32_t* sk, int32_t* sw,
                                    int32_t* bins, Get get, DevFlags* flags) {
    const int lane = threadIdx.x & 31;
    const int32_t nseg = hi - lo;
    int32_t m = 0;
    if (nseg <= kScratchCap) {
        for (int32_t j = lane; j < nseg; j += 32) {
            const int32_t key = __ldg(seg + lo + j);
            sk[j] = key;
            sw[j] = key == skip ? 0 : get(key);
        }
        m = nseg;
    } else {
        m = kScratchCap + 1;
    }
    int32_t c = head;
    int guard = 0;
    while (c >= 0 && m <= kScratchCap && guard++ < (1 << 24)) {
        const int32_t cnt = min(((volatile int32_t*)ch.pool)[c + 1], ((volatile int32_t*)ch.pool)[c + 2]);
        if (m + cnt > kScratchCap) {
            m = kScratchCap + 1;
            break;
        }
        for (int32_t i = lane; i < cnt; i += 32) {
            const int32_t key = ((volatile int32_t*)ch.pool)[c + 3 + i];
            sk[m + i] = key;
            sw[m + i] = key == skip ? 0 : get(key);
        }
        m += cnt;
        c = ((volatile int32_t*)ch.pool)[c];
    }
    if (m > kScratchCap) {
        if (lane == 0) atomicOr(&flags->err, ERR_DEGREE);
        return -1;
    }
    __syncwarp();
    const int passes = (nbits + 4) / 5;
    int32_t prefix = 0;
    for (int p = passes - 1; p >= 0; --p) {
        const int shift = 5 * p;
        bins[lane] = 0;
        __syncwarp();
        for (int32_t j = lane; j < m; j += 32) {
            const int32_t key = sk[j];
            if (shift + 5 < 31 && (key >> (shift + 5)) != prefix) continue;
            const int32_t wt = sw[j];
            if (wt) atomicAdd(bins + ((key >> shift) & 31), wt);
        }
        __syncwarp();
        const long long x = bins[lane];
        long long incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
            if (lane >= o) incl += y;
        }
        const unsigned hit = __ballot_sync(SBP_FULL_MASK, incl > t);
        if (!hit) return -1;
        const int d = __ffs(hit) - 1;
        t -= __shfl_sync(SBP_FULL_MASK, incl - x, d);
        prefix = (prefix << 5) | d;
        __syncwarp();
    }
    return prefix;
}

template <class Cells, bool kNP>
__global__ void __launch_bounds__(kClWarps * 32, 1)
    k_mh_cluster(DevGraph g, DevBM bm, const int32_t* __restrict__ order, int32_t n, uint64_t seed, uint32_t iter,
                 uint32_t step, Cells cells, int log2cap, int nbits, bool greedy, int32_t* ghash, int32_t* scratch,
                 DevFlags* flags) {
    constexpr bool kHash = std::is_same<Cells, HashCells>::value;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int cs = (int)cluster.num_blocks();
    const int W = cs * kClWarps;
    extern __shared__ int32_t sm[];
    int32_t* hash = sm;                                     // kClWarps x (keys, out, in, items) x 512
    int32_t* lq = hash + (4 << kSmemHashL2) * kClWarps;     // the first kLqCache log-table entries
    WinResult* all = reinterpret_cast<WinResult*>(lq + kLqCache);  // the window's results
    __shared__ WinResult res[kClWarps];
    __shared__ int32_t s_dirty[kClWarps];
    __shared__ int32_t s_bins[kClWarps][32];
    __shared__ int32_t s_stop, s_ne;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int32_t B = bm.B;
    // warp w of CTA q: its global hash region (vertices of degree above 256) and scratch
    auto ghash_of = [&](int q, int w) { return ghash + ((int64_t)4 << kGlobalHashL2) * (q * kClWarps + w); };
    auto shash_of = [&](int w) { return hash + (4 << kSmemHashL2) * w; };

    for (int i = tid; i < kLqCache; i += blockDim.x) lq[i] = __ldg(g.Lq + min(i, g.E + 1));
    for (int i = tid; i < kClWarps << (kSmemHashL2 + 2); i += blockDim.x) {
        const int part = (i >> kSmemHashL2) & 3;
        if (part < 3) hash[i] = part == 0 ? -1 : 0;
    }
    if (tid < kClWarps) s_dirty[tid] = 0;
    if (tid == 0) s_ne = kNP ? *bm.nonempty : 0;
    int32_t* sk = scratch + (int64_t)2 * kScratchCap * (rank * kClWarps + wid);
    int32_t* sw = sk + kScratchCap;
    __syncthreads();

    unsigned long long edges = 0, moved = 0, rounds = 0;
    long long dsum = 0;
    int32_t it0 = 0;
    int guard = 0;
    // entries evaluated per round: doubled while rounds are taken whole, else twice the last
    // round's take (a round waits on its slowest evaluation, so entries past the likely stop
    // cost time); the same value on every CTA
    int wa = W;
    while (it0 < n && guard++ < (1 << 30)) {
        const int wn = min(wa, n - it0);
        const int j = rank * kClWarps + wid;  // this warp's window entry
        // ---- 1. evaluate
        if (j < wn) {
            WinResult c;
            c.v = __ldg(order + it0 + j);
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
            int32_t* hk = in_smem ? shash_of(wid) : ghash_of(rank, wid);
            int32_t* hO = hk + hs;
            int32_t* hI = hO + hs;
            int32_t* items = hI + hs;
            if (__ldcg(bm.sizes + c.r) != 1) {  // a singleton block never moves (finetune.cpp:845)
                uint32_t w[4];
                philox4x32_10((uint32_t)c.v, iter, step, DOM_MH, seed, w);
                if (in_smem) {
                    const int32_t nd = s_dirty[wid];
                    for (int q = lane; q < nd; q += 32) {
                        const int32_t sl = items[q];
                        hk[sl] = -1;
                        hO[sl] = 0;
                        hI[sl] = 0;
                    }
                } else {
                    for (int q = lane; q < (1 << c.l2); q += 32) {
                        hk[q] = -1;
                        hO[q] = 0;
                        hI[q] = 0;
                    }
                }
                __syncwarp();
                const int32_t idx = c.k > 0 ? (int32_t)u32_below(w[0], (uint32_t)c.k) : -1;
                int32_t p_dnn = 0, p_R = 0, p_din = 0, p_tr[8], p_tc[8];
                auto on_nb = [&](int32_t nb) {
                    if (nb < 0) return;
                    p_dnn = cells.row_get(nb, nb);
                    p_R = __ldcg(bm.d_out + nb);
                    p_din = __ldcg(bm.d_in + nb);
                    if constexpr (!kHash) {
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const int32_t tile = 8 * lane + q;
                            p_tr[q] = tile < cells.nt ? __ldcg(cells.TS + (int64_t)nb * cells.nt + tile) : 0;
                            p_tc[q] = tile < cells.nt ? __ldcg(cells.TST + (int64_t)nb * cells.nt + tile) : 0;
                        }
                    }
                };
                int32_t* sh = shash_of(wid);
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
                    const long long R = p_R, C = (long long)p_din - p_dnn;
                    long long t = (long long)u64_below(w[1], w[2], (uint64_t)(R + C));
                    if constexpr (kHash) {
                        const DevChain& ch = cells.ch;
                        if (t < R) {
                            s = warp_select_list(bm.row_col, bm.row_off[nb], bm.row_off[nb + 1],
                                                 ((volatile int32_t*)ch.row_head)[nb], ch, t, -1, nbits, sk, sw,
                                                 s_bins[wid], [&](int32_t key) { return chain_get(ch, nb, key); },
                                                 flags);
                        } else {
                            s = warp_select_list(bm.col_row, bm.col_off[nb], bm.col_off[nb + 1],
                                                 ((volatile int32_t*)ch.col_head)[nb], ch, t - R, nb, nbits, sk, sw,
                                                 s_bins[wid], [&](int32_t key) { return chain_get(ch, key, nb); },
                                                 flags);
                        }
                    } else {
                        if (t < R) {
                            s = warp_select_tiles(cells.M + (int64_t)nb * cells.ld, cells.TS + (int64_t)nb * cells.nt,
                                                  B, cells.nt, t, -1, 0, p_tr);
                        } else {
                            s = warp_select_tiles(cells.MT + (int64_t)nb * cells.ld,
                                                  cells.TST + (int64_t)nb * cells.nt, B, cells.nt, t - R, nb, p_dnn,
                                                  p_tc);
                        }
                    }
                }
                if (s < 0) {
                    if (lane == 0) atomicOr(&flags->err, ERR_SELECT);
                    c.status = ST_SKIP;
                } else if (s == c.r) {
                    c.status = ST_NOMOVE;
                } else {
                    c.s = s;
                    if constexpr (kNP) c.dB = np_count_change(__ldcg(bm.sizes + c.r), __ldcg(bm.sizes + s), 1);
                    c.dS = warp_delta<Cells, kNP>(g, bm.d_out, bm.d_in, cells, c.r, s, c.kout, c.kin, c.L, hk, hO, hI,
                                                  items, c.ni, lq, bm.sizes, s_ne);
                    double H = 1.0;
                    if (!kNP && !greedy && c.k > 0) {  // entropy::hastings_correction (entropy.cpp:497-561)
                        H = hastings_fixed<32>(
                            cells, [&](int32_t b) { return bm.d_out[b] + bm.d_in[b] - cells.row_get(b, b); },
                            bm.d_out, bm.d_in, B, c.r, s, c.kout, c.kin, c.L, hk, hO, hI, c.l2, nullptr);
                    }
                    // finetune::accept (finetune.cpp:22-32)
                    c.status = accept_move(c.dS, H, greedy && !kNP, w[3]) ? ST_ACCEPT : ST_REJECT;
                }
            }
            if (lane == 0) res[wid] = c;
        }
        cluster.sync();
        // ---- 2. the window's results, and the conflicts of this CTA's entries
        for (int i = tid; i < wn; i += blockDim.x)
            all[i] = *cluster.map_shared_rank(&res[i % kClWarps], i / kClWarps);
        if (tid == 0) s_stop = W;
        __syncthreads();
        for (int q = tid; q < kClWarps * wn; q += blockDim.x) {
            const int jj = rank * kClWarps + q / wn, u = q % wn;
            if (jj >= wn || u >= jj || all[u].status != ST_ACCEPT) continue;
            const WinResult& cj = all[jj];
            const WinResult& cu = all[u];
            const int32_t* hj = cj.l2 <= kSmemHashL2 ? shash_of(jj % kClWarps) : ghash_of(rank, jj % kClWarps);
            const int32_t* hu = cu.l2 <= kSmemHashL2
                                    ? cluster.map_shared_rank(shash_of(u % kClWarps), u / kClWarps)
                                    : ghash_of(u / kClWarps, u % kClWarps);
            if (in_touched(cj, hj, cu.r) || in_touched(cj, hj, cu.s) ||
                (cj.nb >= 0 && in_touched(cu, hu, cj.nb)) ||
                (kNP && cu.dB != 0 && cj.dB != 0 && cj.status >= ST_REJECT))
                atomicMin(&s_stop, jj);
        }
        cluster.sync();
        // ---- 3. the stop, then this CTA's accepted moves before it
        int stop = wn;
        for (int q = 0; q < cs; ++q) stop = min(stop, *cluster.map_shared_rank(&s_stop, q));
        if (j < stop && res[wid].status == ST_ACCEPT) {  // Blockmodel::move_vertex (blockmodel.cpp:408-435)
            const WinResult c = res[wid];
            const int32_t r = c.r, s = c.s;
            const bool in_smem = c.l2 <= kSmemHashL2;
            const int32_t hs = in_smem ? 1 << kSmemHashL2 : 1 << kGlobalHashL2;
            const int32_t* hk = in_smem ? shash_of(wid) : ghash_of(rank, wid);
            const int32_t* hO = hk + hs;
            const int32_t* hI = hO + hs;
            const int32_t* items = hI + hs;
            for (int q = lane; q < c.ni; q += 32) {
                const int i = items[q];
                const int32_t b = hk[i];
                if (b == r || b == s) continue;
                const int32_t O = hO[i], I = hI[i];
                if (O) {
                    cells_add(cells, r, b, -O, flags);
                    cells_add(cells, s, b, O, flags);
                }
                if (I) {
                    cells_add(cells, b, r, -I, flags);
                    cells_add(cells, b, s, I, flags);
                }
            }
            if (lane == 0) {
                const int32_t Or = hash_get(hk, hO, c.l2, r), Ir = hash_get(hk, hI, c.l2, r);
                const int32_t Os = hash_get(hk, hO, c.l2, s), Is = hash_get(hk, hI, c.l2, s);
                const int32_t L = c.L, selfw = L > 0 ? 1 : 0;
                cells_add(cells, r, r, -Or - Ir - L, flags);
                cells_add(cells, r, s, Ir - Os, flags);
                cells_add(cells, s, r, Or - Is, flags);
                cells_add(cells, s, s, Os + Is + L, flags);
                atomicAdd(bm.d_out + r, -c.kout);
                atomicAdd(bm.d_out + s, c.kout);
                atomicAdd(bm.d_in + r, -(c.kin + selfw));
                atomicAdd(bm.d_in + s, c.kin + selfw);
                atomicAdd(bm.sizes + r, -1);
                atomicAdd(bm.sizes + s, 1);
                bm.asg[c.v] = s;
            }
        }
        if (wid == 0) {
            int32_t k_sum = 0, acc = 0, dB_sum = 0;
            long long d_sum = 0;
            for (int i = lane; i < stop; i += 32) {
                k_sum += all[i].k;
                if (all[i].status == ST_ACCEPT) {
                    ++acc;
                    d_sum += all[i].dS;
                    dB_sum += all[i].dB;
                }
            }
            k_sum = warp_sum_i(k_sum);
            acc = warp_sum_i(acc);
            d_sum = warp_sum_ll(d_sum);
            dB_sum = warp_sum_i(dB_sum);
            if (lane == 0) {
                s_ne += dB_sum;  // blockmodel.cpp:429-430
                if (rank == 0) {
                    edges += (unsigned long long)k_sum;
                    moved += (unsigned long long)acc;
                    dsum += d_sum;
                    ++rounds;
                }
            }
        }
        it0 += stop;
        wa = stop >= wn ? min(W, 2 * wa) : min(W, max(2 * kClWarps, (2 * stop + kClWarps - 1) / kClWarps * kClWarps));
        cluster.sync();
    }
    if (rank == 0 && tid == 0) {
        atomicAdd(&flags->counters[4], edges);
        atomicAdd(&flags->counters[5], moved);
        atomicAdd(&flags->counters[7], (unsigned long long)dsum);
        atomicAdd(&flags->counters[8], rounds);
    }
}

size_t cluster_smem(int cs) {
    return sizeof(int32_t) * (((size_t)kClWarps << (kSmemHashL2 + 2)) + kLqCache) +
           sizeof(WinResult) * (size_t)kClWarps * cs;
}

// Largest cluster (16, else 8, else 4) whose CTAs the device can hold at once.
template <class K>
int pick_cluster(K kernel, size_t smem) {
    static int cached = -1;
    if (cached > 0) return cached;
    cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int cs = kClMaxCluster; cs >= 4; cs /= 2) {
        cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cluster_smem(cs));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(kClWarps * 32);
        cfg.dynamicSmemBytes = cluster_smem(cs);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, (const void*)kernel, &cfg) == cudaSuccess && nc >= 1) {
            cached = cs;
            return cs;
        }
        cudaGetLastError();
    }
    cached = 0;
    return 0;
}

template <class Cells, bool kNP>
void launch_cluster(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, uint64_t seed, uint32_t iter,
                    uint32_t step, const Cells& cells, int log2cap, bool greedy, Work& w, int cs, cudaStream_t st) {
    auto kernel = k_mh_cluster<Cells, kNP>;
    const size_t smem = cluster_smem(cs);
    cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kClWarps * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const int nbits = ceil_log2((uint64_t)(bm.B > 1 ? bm.B : 2));
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, g, bm, order, n, seed, iter, step, cells, log2cap, nbits,
                                             greedy, w.cl_hash, w.cl_scratch, w.flags_dev);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cluster chain launch: ") + cudaGetErrorString(e));
}

}  // namespace

int mh_cluster_size() { return pick_cluster(k_mh_cluster<HashCells, false>, cluster_smem(kClMaxCluster)); }

size_t mh_cluster_hash_ints(int cs) { return (size_t)cs * kClWarps * ((size_t)4 << kGlobalHashL2); }
size_t mh_cluster_scratch_ints(int cs) { return (size_t)cs * kClWarps * 2 * kScratchCap; }

void mh_chain_cluster(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, int32_t max_k, bool hashed,
                      uint64_t seed, uint32_t iter, uint32_t step, int mode, Work& w, cudaStream_t st) {
    if (n <= 0) return;
    if (mode == ACC_NP && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    const int cs = mh_cluster_size();
    if (cs <= 0 || !w.cl_hash || !w.cl_scratch) throw std::logic_error("cluster chain buffers missing");
    const int log2cap = ceil_log2((uint64_t)(2 * (max_k > 16 ? max_k : 16)));
    if (log2cap > kGlobalHashL2) throw std::logic_error("cluster chain: vertex degree above the hash limit");
    const bool np = mode == ACC_NP, greedy = mode == ACC_GREEDY;
    if (hashed) {
        const HashCells hc{w.chain};
        if (np) launch_cluster<HashCells, true>(g, bm, order, n, seed, iter, step, hc, log2cap, greedy, w, cs, st);
        else launch_cluster<HashCells, false>(g, bm, order, n, seed, iter, step, hc, log2cap, greedy, w, cs, st);
        count_launches(1);
        return;
    }
    const int64_t B = bm.B, nt = (B + 127) >> 7, ld = (B + 3) & ~3ll;
    GlobalCells gc;
    gc.ld = ld;
    gc.nt = (int32_t)nt;
    gc.M = w.cells;
    gc.MT = gc.M + B * ld;
    gc.TS = gc.MT + B * ld;
    gc.TST = gc.TS + B * nt;
    window_fill(bm, gc, st);
    if (np) launch_cluster<GlobalCells, true>(g, bm, order, n, seed, iter, step, gc, log2cap, greedy, w, cs, st);
    else launch_cluster<GlobalCells, false>(g, bm, order, n, seed, iter, step, gc, log2cap, greedy, w, cs, st);
    count_launches(1);
}

}  // namespace sbp

// Exact block-merge carry-out (block_merge::carry_out_best_merges_advanced, reference
// src/block_merge.cpp:40-117) on a thread-block cluster, for blockmodels with many blocks.
//
// The round structure is the one of carry.cu (the W smallest live queue entries are
// re-scored against one state, the reference's pop / put-back / merge rule is replayed over
// those values up to the first entry whose value a merge of the round has changed, and the
// round's merges are applied together), with a window of 16 entries per CTA of the cluster
// (up to 256) so that the many independent merges of a large blockmodel are found in few
// rounds.  CTA 0 keeps the queue and replays the rule; the cluster's distributed shared
// memory and hardware barriers carry the rest:
//   1. CTA 0 selects the candidates (the W smallest entries of the sorted proposals, the
//      global put-back runs and its shared put-back buffer) and the bound (the next entry);
//   2. each warp re-scores one candidate and publishes its block in a per-block array;
//   3. each warp finds the candidates a merge of its own would change: a candidate's value
//      reads the cells of its block's row and column and the degrees of their keys, and x
//      is a key of block a's row exactly when a is a key of x's column, so walking the row
//      and column key lists of the merge's two blocks and looking each key up in the
//      per-block array finds them (a key whose cell has dropped to zero only adds a
//      conflict that need not be one);
//   4. CTA 0 collects the values and those sets and replays the rule on one warp: runs of
//      candidates that merge (or are skipped) without a put-back and that no earlier merge
//      of the run changes are taken 32 at a time with ballots, every other pop under the
//      full rule on one lane (a merge marks the candidates it changes; popping a marked
//      candidate or put-back entry ends the round); the round's put-backs are then folded
//      into CTA 0's buffer;
//   5. the round's merges (disjoint rows, columns and targets, by the conflict rule) are
//      applied by all CTAs at once.
// Merges, their order and every put-back delta equal those of the one-at-a-time loop; ties
// of equal delta pop in ascending block order.
#include <cooperative_groups.h>

#include <algorithm>
#include <stdexcept>

#include "carry.cuh"

namespace cg = cooperative_groups;

namespace sbp {

namespace {

constexpr int kCcWarps = 16;
constexpr int kCcThreads = kCcWarps * 32;
constexpr int kCcMaxCluster = 16;
constexpr int kCcMaxW = kCcWarps * kCcMaxCluster;  // candidates per round
constexpr int kCcWords = kCcMaxW / 32;              // words of a conflict mask
constexpr int kCcQS = 4096;                         // CTA 0's sorted put-back buffer
constexpr int kCcStage = 1 << 15;                   // staged new keys per merge and list
constexpr int kCcQCap = 2 * kCcMaxW;                // the replay's put-back list
constexpr int kCcBigKeys = 512;                     // keys above which the whole CTA scores a candidate

// Shared memory of every CTA (dynamic); the queue parts are used by CTA 0 only.
struct CcShared {
    long long s_dS[2][kCcQS];
    int32_t s_blk[2][kCcQS];
    long long hs_dS[3][kCcMaxW + 1];
    int32_t hs_blk[3][kCcMaxW + 1];
    long long c_dS[kCcMaxW];
    int32_t c_blk[kCcMaxW];
    int32_t c_src[kCcMaxW];
    int32_t c_to[kCcMaxW];
    long long c_act[kCcMaxW];
    int32_t c_count[kCcMaxW];
    uint32_t inv[kCcMaxW][kCcWords];  // bit j of inv[i]: a merge of candidate i changes j's value
    int32_t m_from[kCcMaxW], m_to[kCcMaxW];
    int32_t a_rank[kCcMaxW];    // greedy replay: rank of each candidate by (recomputed delta, block)
    long long a_d[kCcMaxW];     // ... and the candidates in that order
    int32_t a_b[kCcMaxW], a_c[kCcMaxW];
    long long h_d[kCcQCap];  // the round's put-back entries, sorted, live in [qh, qh + nq)
    int32_t h_b[kCcQCap], h_c[kCcQCap];
    uint32_t smask[kCcWords];  // candidates whose value a merge of the round has changed
    // this CTA's own candidates
    int32_t my_to[kCcWarps];
    long long my_act[kCcWarps];
    int32_t my_count[kCcWarps];
    uint32_t my_inv[kCcWarps][kCcWords];
    int32_t big[kCcWarps];  // this CTA's candidates left to the whole CTA (by warp)
    int32_t nbig;
    long long big_acc;
    // new keys of the row / column of each merge's target, staged, then appended in bulk
    int32_t st_n[kCcWarps / 2][2];
    int32_t st_slot[kCcWarps / 2][2];
    long long b_dS, merged, rounds;
    int32_t b_blk;
    int32_t p, q, nR, rsel, ns, ssel, ne;
    int32_t ncand, has_bound, done, nm, cS, nq, qh;
};

template <class Cells, bool kNP>
__global__ void __launch_bounds__(kCcThreads, 1) k_carry_cluster(
    DevGraph g, DevBM bm, DevChain ch, Cells cells, const uint64_t* __restrict__ pkeys,
    const int32_t* __restrict__ pblk, int32_t nP, const int32_t* __restrict__ best, long long* r0_dS, int32_t* r0_blk,
    long long* r1_dS, int32_t* r1_blk, int32_t* parent, long long num_to_merge, int32_t* cand_of, int32_t* stage_buf,
    int32_t* out_merged, DevFlags* flags) {
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank(), cs = (int)cluster.num_blocks();
    const int W = kCcWarps * cs;
    extern __shared__ __align__(16) unsigned char cc_raw[];
    CcShared& sh = *reinterpret_cast<CcShared*>(cc_raw);
    CcShared& ctl = *cluster.map_shared_rank(&sh, 0);  // CTA 0's queue and round results
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool controller = rank == 0;
    if (controller && tid == 0) {
        sh.p = sh.q = sh.nR = sh.rsel = sh.ns = sh.ssel = 0;
        sh.merged = 0;
        sh.rounds = 0;
        sh.ne = kNP ? *bm.nonempty : 0;
    }
    const long long max_rounds = 64ll * (nP + 1) + 4096;
    unsigned long long keys_seen = 0, evals = 0;
    cluster.sync();
    while (true) {
        // ---- 1. CTA 0: stop test, the candidates and the bound
        if (controller) {
            if (tid == 0) {
                sh.done = sh.merged >= num_to_merge;
                if (!sh.done && sh.rounds >= max_rounds) {
                    atomicOr(&flags->err, ERR_STATE);
                    sh.done = 1;
                }
            }
            __syncthreads();
            if (!sh.done) {
                const int p = sh.p, q = sh.q, nR = sh.nR, ns = sh.ns, ssel = sh.ssel;
                const long long* rdS = sh.rsel ? r1_dS : r0_dS;
                const int32_t* rb = sh.rsel ? r1_blk : r0_blk;
                const int n0 = max(0, min(W + 1, nP - p)), n1 = max(0, min(W + 1, nR - q)), n2 = min(W + 1, ns);
                for (int k = tid; k < n0; k += kCcThreads) {
                    sh.hs_dS[0][k] = key_to_fixed(pkeys[p + k]);
                    sh.hs_blk[0][k] = pblk[p + k];
                }
                for (int k = tid; k < n1; k += kCcThreads) {
                    sh.hs_dS[1][k] = rdS[q + k];
                    sh.hs_blk[1][k] = rb[q + k];
                }
                for (int k = tid; k < n2; k += kCcThreads) {
                    sh.hs_dS[2][k] = sh.s_dS[ssel][k];
                    sh.hs_blk[2][k] = sh.s_blk[ssel][k];
                }
                __syncthreads();
                const int n[3] = {n0, n1, n2};
                for (int e = tid; e < n0 + n1 + n2; e += kCcThreads) {
                    const int src = e < n0 ? 0 : (e < n0 + n1 ? 1 : 2);
                    const int k = e - (src == 0 ? 0 : (src == 1 ? n0 : n0 + n1));
                    const long long d = sh.hs_dS[src][k];
                    const int32_t b = sh.hs_blk[src][k];
                    int r = k;
                    for (int o = 0; o < 3; ++o)
                        if (o != src) r += count_before(sh.hs_dS[o], sh.hs_blk[o], n[o], d, b);
                    if (r < W) {
                        sh.c_dS[r] = d;
                        sh.c_blk[r] = b;
                        sh.c_src[r] = src;
                    } else if (r == W) {
                        sh.b_dS = d;
                        sh.b_blk = b;
                    }
                }
                if (tid == 0) {
                    const int tot = n0 + n1 + n2;
                    sh.ncand = min(W, tot);
                    sh.has_bound = tot > W;
                    if (sh.ncand == 0) sh.done = 1;
                }
            }
        }
        cluster.sync();
        if (ctl.done) break;
        const int ncand = ctl.ncand;
        // ---- 2. re-score the candidates; publish their blocks in cand_of.  Each warp takes
        // one candidate; a candidate whose row and column lists are long is left to the whole
        // CTA afterwards, so that no round waits on one warp walking a hub block's lists.
        for (int i = tid; i < kCcWarps * kCcWords; i += kCcThreads) (&sh.my_inv[0][0])[i] = 0u;
        if (tid == 0) sh.nbig = 0;
        __syncthreads();
        const int j = rank * kCcWarps + warp;
        if (j < ncand) {
            const int32_t from = ctl.c_blk[j];
            int32_t to = 0, len = 0;
            if (lane == 0) {
                const int32_t b = best[from];
                to = (b < 0 || b >= bm.B) ? from : uf_find(parent, b);
                cand_of[from] = j;
                len = (bm.row_off[from + 1] - bm.row_off[from]) + (bm.col_off[from + 1] - bm.col_off[from]) +
                      list_chunk_keys(ch.row_head[from], ch) + list_chunk_keys(ch.col_head[from], ch);
            }
            to = __shfl_sync(SBP_FULL_MASK, to, 0);
            len = __shfl_sync(SBP_FULL_MASK, len, 0);
            long long part = 0;
            // nonparametric: zero when either block is empty (entropy.cpp:1203-1204)
            const bool counted = !kNP || (to != from && bm.sizes[from] != 0 && bm.sizes[to] != 0);
            const bool scored = to != from && counted;
            if (scored && len > kCcBigKeys) {
                if (lane == 0) sh.big[atomicAdd(&sh.nbig, 1)] = warp;
            } else if (scored) {
                part = merge_delta_part<Cells, kNP>(g, bm, ch, cells, from, to, lane, 32, true, [](int32_t) {},
                                                    keys_seen);
                if (lane == 0) ++evals;
            }
            if (lane == 0) {
                sh.my_to[warp] = to;
                sh.my_act[warp] = part;
                sh.my_count[warp] = kNP && counted;
            }
        }
        __syncthreads();
        for (int q = 0; q < sh.nbig; ++q) {
            const int w = sh.big[q];
            const int32_t from = ctl.c_blk[rank * kCcWarps + w], to = sh.my_to[w];
            if (tid == 0) sh.big_acc = 0;
            __syncthreads();
            const long long part = merge_delta_part<Cells, kNP>(g, bm, ch, cells, from, to, tid, kCcThreads, warp == 0,
                                                                [](int32_t) {}, keys_seen);
            if (lane == 0) atomicAdd(reinterpret_cast<unsigned long long*>(&sh.big_acc), (unsigned long long)part);
            __syncthreads();
            if (tid == 0) {
                sh.my_act[w] = sh.big_acc;
                ++evals;
            }
        }
        cluster.sync();
        // ---- 3. the candidates a merge of this one (a -> b) would change: those whose value
        // reads a cell of row / column a or b or a degree of a or b -- their block is a or b,
        // their target is a or b, or their block is a key of the row or column of a or b
        // (cell (x, a) is non-zero only if x is listed in column a, and so on)
        for (int k = tid; k < ncand; k += kCcThreads)
            sh.c_to[k] = cluster.map_shared_rank(&sh, k / kCcWarps)->my_to[k % kCcWarps];
        __syncthreads();
        if (j < ncand) {
            const int32_t a = ctl.c_blk[j], b = sh.my_to[warp];
            uint32_t* inv = sh.my_inv[warp];
            auto mark = [&](int32_t x) {
                const int32_t r = __ldcg(cand_of + x);
                if (r >= 0 && r != j && r < ncand) atomicOr(inv + (r >> 5), 1u << (r & 31));
            };
            if (lane == 0) {
                mark(a);
                mark(b);
            }
            for (int k = lane; k < ncand; k += 32) {
                const int32_t t = sh.c_to[k];
                if (k != j && (t == a || t == b)) atomicOr(inv + (k >> 5), 1u << (k & 31));
            }
            list_for_each(bm.row_col, bm.row_off[a], bm.row_off[a + 1], ch.row_head[a], ch, lane, 32, mark);
            list_for_each(bm.col_row, bm.col_off[a], bm.col_off[a + 1], ch.col_head[a], ch, lane, 32, mark);
            if (b != a) {
                list_for_each(bm.row_col, bm.row_off[b], bm.row_off[b + 1], ch.row_head[b], ch, lane, 32, mark);
                list_for_each(bm.col_row, bm.col_off[b], bm.col_off[b + 1], ch.col_head[b], ch, lane, 32, mark);
            }
        }
        cluster.sync();
        // ---- 4. CTA 0: collect, replay the queue rule (block_merge.cpp:54-95), fold put-backs
        if (controller) {
            for (int k = tid; k < ncand; k += kCcThreads) {
                const CcShared& o = *cluster.map_shared_rank(&sh, k / kCcWarps);
                sh.c_act[k] = o.my_act[k % kCcWarps];
                sh.c_count[k] = o.my_count[k % kCcWarps];
            }
            for (int e = tid; e < ncand * kCcWords; e += kCcThreads) {
                const int k = e / kCcWords, w = e % kCcWords;
                sh.inv[k][w] = cluster.map_shared_rank(&sh, k / kCcWarps)->my_inv[k % kCcWarps][w];
            }
            if (tid < kCcWords) sh.smask[tid] = 0u;
            __syncthreads();
            if constexpr (!kNP) {
                // Greedy entropy: an entry put back in this round carries its recomputed delta,
                // which is known for every candidate, so the put-back entries are kept as a set
                // of ranks in the candidates' (recomputed delta, block) order: a 256-bit mask
                // whose lowest set bit is the list's head.  The ranks first, in parallel.
                for (int c = tid; c < ncand; c += kCcThreads) {
                    const long long d = sh.c_act[c];
                    const int32_t b = sh.c_blk[c];
                    int r = 0;
                    for (int k = 0; k < ncand; ++k) r += qless(sh.c_act[k], sh.c_blk[k], d, b);
                    sh.a_rank[c] = r;
                    sh.a_d[r] = d;
                    sh.a_b[r] = b;
                    sh.a_c[r] = c;
                }
                // The replay runs first in parallel, as far as it provably agrees with the
                // sequential rule: candidate i (thread i) merges when its recomputed delta is at
                // most the next key -- the next candidate's or the bound -- and is put back
                // otherwise, unless it already shares its target's block.  That decision leaves
                // out the put-back list, so it holds while no entry put back earlier in the round
                // would pop before candidate i or lower the value it is compared with; P is the
                // first candidate where that fails.  The pass also ends at the first candidate S
                // that an earlier merge of the round made stale (the prefix OR of the merges'
                // conflict sets) and after the merge that completes the pass (L).  The
                // sequential loop below takes over at P when P comes first.
                __shared__ uint32_t sp_or[kCcMaxW / 32][kCcWords];
                __shared__ long long sp_md[kCcMaxW / 32];
                __shared__ int32_t sp_mb[kCcMaxW / 32], sp_cnt[kCcMaxW / 32];
                __shared__ uint32_t sp_stl[kCcWords], sp_pend[kCcWords];
                __shared__ int32_t sp_P, sp_S, sp_L, sp_nm, sp_c[3];
                if (tid < kCcWords) sp_stl[tid] = sp_pend[tid] = 0u;
                if (tid == 0) {
                    sp_P = ncand;
                    sp_S = ncand;
                    sp_L = sh.merged < num_to_merge ? INT_MAX : 0;  // after the merge that completes the pass
                    sp_nm = 0;
                    sp_c[0] = sp_c[1] = sp_c[2] = 0;
                }
                __syncthreads();  // the ranks too
                const bool lead = tid < kCcMaxW;  // thread i < 256 takes candidate i
                const int ci0 = tid;
                bool x_same = false, x_pb = false, x_mg = false;
                long long x_key = 0, x_T0 = LLONG_MAX, x_exd = LLONG_MAX;
                int32_t x_kb = 0, x_exb = INT_MAX;
                int x_before = 0;
                uint32_t x_ex = 0u;  // word `warp` of the prefix OR before this candidate
                if (lead) {
                    const bool hc = ci0 < ncand;
                    const long long act = hc ? sh.c_act[ci0] : 0;
                    x_key = hc ? sh.c_dS[ci0] : 0;
                    x_kb = hc ? sh.c_blk[ci0] : 0;
                    const bool hc2 = ci0 + 1 < ncand;
                    x_T0 = sh.has_bound ? sh.b_dS : LLONG_MAX;
                    if (hc2) x_T0 = min(x_T0, sh.c_dS[ci0 + 1]);
                    x_same = hc && sh.c_to[ci0] == x_kb;
                    x_pb = hc && !x_same && (hc2 || sh.has_bound) && act > x_T0;
                    x_mg = hc && !x_same && !x_pb;
                    // in-warp prefix minimum, in (delta, block) order, of the entries put back
                    long long md = x_pb ? act : LLONG_MAX;
                    int32_t mb = x_pb ? x_kb : INT_MAX;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const long long od = __shfl_up_sync(SBP_FULL_MASK, md, o);
                        const int32_t ob = __shfl_up_sync(SBP_FULL_MASK, mb, o);
                        if (lane >= o && qless(od, ob, md, mb)) {
                            md = od;
                            mb = ob;
                        }
                    }
                    x_exd = __shfl_up_sync(SBP_FULL_MASK, md, 1);
                    x_exb = __shfl_up_sync(SBP_FULL_MASK, mb, 1);
                    if (lane == 0) {
                        x_exd = LLONG_MAX;
                        x_exb = INT_MAX;
                    }
                    // in-warp prefix OR of the merges' conflict sets, and the merges before
#pragma unroll
                    for (int w = 0; w < kCcWords; ++w) {
                        uint32_t v = x_mg ? sh.inv[ci0][w] : 0u;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const uint32_t y = __shfl_up_sync(SBP_FULL_MASK, v, o);
                            if (lane >= o) v |= y;
                        }
                        const uint32_t e = __shfl_up_sync(SBP_FULL_MASK, v, 1);
                        if (w == warp) x_ex = lane == 0 ? 0u : e;
                        if (lane == 31) sp_or[warp][w] = v;
                    }
                    const unsigned mgm = __ballot_sync(SBP_FULL_MASK, x_mg);
                    x_before = __popc(mgm & lanemask_lt());
                    if (lane == 31) {
                        sp_md[warp] = md;
                        sp_mb[warp] = mb;
                        sp_cnt[warp] = __popc(mgm);
                    }
                }
                __syncthreads();
                if (lead && ci0 < ncand) {
                    // add the warps before this one
                    long long qd = x_exd;
                    int32_t qb = x_exb;
                    for (int w = 0; w < warp; ++w) {
                        if (qless(sp_md[w], sp_mb[w], qd, qb)) {
                            qd = sp_md[w];
                            qb = sp_mb[w];
                        }
                        x_before += sp_cnt[w];
                        x_ex |= sp_or[w][warp];
                    }
                    const bool anypb = qb != INT_MAX;
                    if (anypb && !(qd >= x_T0 && !qless(qd, qb, x_key, x_kb))) atomicMin(&sp_P, ci0);
                    if ((x_ex >> (ci0 & 31)) & 1u) atomicMin(&sp_S, ci0);  // ci0 >> 5 == warp
                    if (x_mg && (long long)x_before == num_to_merge - sh.merged - 1) atomicMin(&sp_L, ci0 + 1);
                }
                __syncthreads();
                const int x_end = min(sp_P, min(sp_S, sp_L));
                if (lead && ci0 < x_end) {
                    if (x_mg) {
                        sh.m_from[x_before] = x_kb;
                        sh.m_to[x_before] = sh.c_to[ci0];
                        atomicAdd(&sp_nm, 1);
#pragma unroll
                        for (int w = 0; w < kCcWords; ++w) {
                            const uint32_t v = sh.inv[ci0][w];
                            if (v) atomicOr(&sp_stl[w], v);
                        }
                    }
                    if (x_pb) {
                        const int r = sh.a_rank[ci0];
                        atomicOr(&sp_pend[r >> 5], 1u << (r & 31));
                    }
                    atomicAdd(&sp_c[sh.c_src[ci0]], 1);
                }
                __syncthreads();
                if (tid == 0) {
                    const bool hb = sh.has_bound;
                    const long long bnd_dS = sh.b_dS, merged0 = sh.merged;
                    const int32_t bnd_blk = sh.b_blk;
                    uint32_t pend[kCcWords], stl[kCcWords];
#pragma unroll
                    for (int w = 0; w < kCcWords; ++w) {
                        pend[w] = sp_pend[w];
                        stl[w] = sp_stl[w];
                    }
                    auto bit_of = [&](const uint32_t* m, int x) {
                        uint32_t v = 0;
#pragma unroll
                        for (int w = 0; w < kCcWords; ++w) v = (w == (x >> 5)) ? m[w] : v;
                        return (v >> (x & 31)) & 1u;
                    };
                    auto first = [&]() {
                        int r = -1;
#pragma unroll
                        for (int w = kCcWords - 1; w >= 0; --w)
                            if (pend[w]) r = 32 * w + __ffs(pend[w]) - 1;
                        return r;
                    };
                    auto flip = [&](int x) {
#pragma unroll
                        for (int w = 0; w < kCcWords; ++w)
                            if (w == (x >> 5)) pend[w] ^= 1u << (x & 31);
                    };
                    int i = x_end, nm = sp_nm, c0 = sp_c[0], c1 = sp_c[1], c2 = sp_c[2];
                    int pr = first();  // rank of the put-back list's head, or -1
                    // candidate i's fields in registers, the next one's loaded as i advances
                    long long cd = 0, cact = 0;
                    int32_t cb = 0, cto = 0, csrc = 0;
                    auto load_c = [&]() {
                        if (i < ncand) {
                            cd = sh.c_dS[i];
                            cb = sh.c_blk[i];
                            cto = sh.c_to[i];
                            csrc = sh.c_src[i];
                            cact = sh.c_act[i];
                        }
                    };
                    load_c();
                    long long qd = pr >= 0 ? sh.a_d[pr] : 0;
                    int32_t qb = pr >= 0 ? sh.a_b[pr] : 0;
                    // resume where the parallel pass could not decide (nothing left otherwise)
                    const bool resume = x_end == sp_P && x_end < sp_L;
                    while (resume && merged0 + nm < num_to_merge) {
                        const bool hc = i < ncand, hq = pr >= 0;
                        if (!hc && !hq) break;  // queue empty
                        const bool fromq = hq && (!hc || qless(qd, qb, cd, cb));
                        const long long kd = fromq ? qd : cd;
                        const int32_t kb = fromq ? qb : cb;
                        if (hb && qless(bnd_dS, bnd_blk, kd, kb)) break;  // next pop not evaluated
                        if (fromq) {
                            // popped again: unless a merge since touched what it read, its value
                            // is the one it was put back with, the smallest key left, so it merges
                            const int ci = sh.a_c[pr];
                            if (bit_of(stl, ci)) break;
                            flip(pr);
                            pr = first();
                            if (pr >= 0) {
                                qd = sh.a_d[pr];
                                qb = sh.a_b[pr];
                            }
                            sh.m_from[nm] = kb;
                            sh.m_to[nm] = sh.c_to[ci];
#pragma unroll
                            for (int w = 0; w < kCcWords; ++w) stl[w] |= sh.inv[ci][w];
                            ++nm;
                            continue;
                        }
                        if (bit_of(stl, i)) break;  // its value is stale: re-score it next round
                        const int ci = i++;
                        const long long act = cact;
                        const int32_t to = cto;
                        c0 += csrc == 0;
                        c1 += csrc == 1;
                        c2 += csrc == 2;
                        load_c();
                        if (to == kb) continue;  // already in the same block
                        const bool hc2 = i < ncand;
                        if (hc2 || hq || hb) {
                            long long top = hb ? bnd_dS : LLONG_MAX;
                            if (hc2) top = min(top, cd);
                            if (hq) top = min(top, qd);
                            if (act > top) {  // put back with the recomputed delta
                                const int r = sh.a_rank[ci];
                                flip(r);
                                if (pr < 0 || r < pr) {
                                    pr = r;
                                    qd = act;
                                    qb = kb;
                                }
                                continue;
                            }
                        }
                        sh.m_from[nm] = kb;
                        sh.m_to[nm] = to;
#pragma unroll
                        for (int w = 0; w < kCcWords; ++w) stl[w] |= sh.inv[ci][w];
                        ++nm;
                    }
                    // the put-back entries left, in order, for the shared buffer
                    int k = 0;
#pragma unroll
                    for (int w = 0; w < kCcWords; ++w) {
                        uint32_t m = pend[w];
                        while (m) {
                            const int r = 32 * w + __ffs(m) - 1;
                            m &= m - 1;
                            sh.h_d[k] = sh.a_d[r];
                            sh.h_b[k] = sh.a_b[r];
                            ++k;
                        }
                    }
                    sh.qh = 0;
                    sh.nq = k;
                    sh.p += c0;
                    sh.q += c1;
                    sh.cS = c2;
                    sh.nm = nm;
                    sh.merged += nm;
                    sh.rounds += 1;
                }
            } else if (warp == 0) {
                // The replay, uniform over the warp.  Put-back entries wait in a sorted list
                // h[qh, qh + nq): a pop advances qh, a put-back shifts the entries after its
                // place up by one (each lane moves up to 16 of them).
                const bool hb = sh.has_bound;
                const long long bnd_dS = sh.b_dS, merged0 = sh.merged;
                const int32_t bnd_blk = sh.b_blk, ne0 = sh.ne;
                int i = 0, qh = 0, nq = 0, nm = 0, c0 = 0, c1 = 0, c2 = 0;
                auto stale = [&](int ci) { return ((sh.smask[ci >> 5] >> (ci & 31)) & 1u) != 0u; };
                for (int guard = 0; merged0 + nm < num_to_merge && guard < 8 * kCcMaxW; ++guard) {
                    const bool hc = i < ncand, hq = nq > 0;
                    if (!hc && !hq) break;  // queue empty
                    const long long qd = hq ? sh.h_d[qh] : 0;
                    const int32_t qb = hq ? sh.h_b[qh] : 0;
                    const long long cd = hc ? sh.c_dS[i] : 0;
                    const int32_t cb = hc ? sh.c_blk[i] : 0;
                    const bool fromq = hq && (!hc || qless(qd, qb, cd, cb));
                    if (!kNP && !fromq) {
                        // -- a run of candidates popped before the put-back list's head, each
                        // merged or skipped without a put-back and unchanged by the merges
                        // before it, taken 32 at a time (greedy entropy only: the
                        // nonparametric count term changes with every merge)
                        const int c = i + lane;
                        bool valid = c < ncand;
                        long long kd = 0;
                        int32_t kb = 0;
                        if (valid) {
                            kd = sh.c_dS[c];
                            kb = sh.c_blk[c];
                            if (hq && !qless(kd, kb, qd, qb)) valid = false;          // the list pops first
                            if (hb && qless(bnd_dS, bnd_blk, kd, kb)) valid = false;  // not evaluated
                        }
                        int32_t to = 0;
                        bool same = false, ok = false;
                        if (valid) {
                            to = sh.c_to[c];
                            same = to == kb;
                            const bool more = (c + 1 < ncand) || hq || hb;  // queue not empty after it
                            long long top = hb ? bnd_dS : LLONG_MAX;
                            if (c + 1 < ncand) top = min(top, sh.c_dS[c + 1]);
                            if (hq) top = min(top, qd);
                            ok = (same || !more || sh.c_act[c] <= top) && !stale(c);
                        }
                        const unsigned okm = __ballot_sync(SBP_FULL_MASK, valid && ok);
                        int nf = ~okm ? __ffs(~okm) - 1 : 32;
                        // a merge of an earlier lane of the run may change a later one
                        uint32_t win = 0;
                        if (lane < nf && !same) {
                            const int w0 = i >> 5, sft = i & 31;
                            const uint32_t lo = sh.inv[c][w0];
                            const uint32_t hi = w0 + 1 < kCcWords ? sh.inv[c][w0 + 1] : 0u;
                            win = sft ? (lo >> sft) | (hi << (32 - sft)) : lo;
                        }
                        uint32_t incl = win;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const uint32_t y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
                            if (lane >= o) incl |= y;
                        }
                        uint32_t ex = __shfl_up_sync(SBP_FULL_MASK, incl, 1);
                        if (lane == 0) ex = 0u;
                        const unsigned stm = __ballot_sync(SBP_FULL_MASK, lane < nf && ((ex >> lane) & 1u));
                        if (stm) nf = min(nf, __ffs(stm) - 1);
                        // no merges beyond the pass's count: stop after the last one wanted
                        const unsigned mgm = __ballot_sync(SBP_FULL_MASK, lane < nf && !same);
                        const long long need = num_to_merge - merged0 - nm;
                        if (__popc(mgm) >= need) {
                            const bool last = lane < nf && !same && __popc(mgm & lanemask_lt()) == need - 1;
                            nf = min(nf, __ffs(__ballot_sync(SBP_FULL_MASK, last)));
                        }
                        if (nf > 0) {
                            const bool com = lane < nf, cm = com && !same;
                            const unsigned cmm = __ballot_sync(SBP_FULL_MASK, cm);
                            if (cm) {
                                const int pos = nm + __popc(cmm & lanemask_lt());
                                sh.m_from[pos] = kb;
                                sh.m_to[pos] = to;
                            }
#pragma unroll
                            for (int w = 0; w < kCcWords; ++w) {
                                uint32_t v = cm ? sh.inv[c][w] : 0u;
#pragma unroll
                                for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(SBP_FULL_MASK, v, o);
                                if (lane == 0) sh.smask[w] |= v;
                            }
                            const int src = com ? sh.c_src[c] : -1;
                            c0 += __popc(__ballot_sync(SBP_FULL_MASK, src == 0));
                            c1 += __popc(__ballot_sync(SBP_FULL_MASK, src == 1));
                            c2 += __popc(__ballot_sync(SBP_FULL_MASK, src == 2));
                            i += nf;
                            nm += __popc(cmm);
                            __syncwarp();
                            continue;
                        }
                    }
                    // -- one pop under the full rule
                    const long long kd = fromq ? qd : cd;
                    const int32_t kb = fromq ? qb : cb;
                    if (hb && qless(bnd_dS, bnd_blk, kd, kb)) break;  // next pop not evaluated
                    int ci;
                    if (fromq) {
                        // popped again: unless a merge since touched what it read, its value is
                        // the one it was put back with (kNP: up to the count term)
                        ci = sh.h_c[qh];
                        if (stale(ci)) break;
                        ++qh;
                        --nq;
                    } else {
                        if (stale(i)) break;  // its value is stale: re-score it next round
                        if (nq >= kCcQCap) break;  // no room for a put-back: end the round here
                        ci = i++;
                        const int src = sh.c_src[ci];
                        c0 += src == 0;
                        c1 += src == 1;
                        c2 += src == 2;
                        if (sh.c_to[ci] == kb) continue;  // already in the same block
                    }
                    const int32_t to = sh.c_to[ci];
                    long long act = sh.c_act[ci];
                    if (kNP && sh.c_count[ci]) act += __ldg(g.Dm + min(max(ne0 - nm, 0), g.N + 1));
                    const bool hc2 = i < ncand, hq2 = nq > 0;
                    bool put_back = false;
                    if (hc2 || hq2 || hb) {
                        long long top = hb ? bnd_dS : LLONG_MAX;
                        if (hc2) top = min(top, sh.c_dS[i]);
                        if (hq2) top = min(top, sh.h_d[qh]);
                        put_back = act > top;
                    }
                    if (put_back) {
                        // put back with the recomputed delta: its place in the sorted list
                        int before = 0;
                        for (int k = lane; k < nq; k += 32) before += qless(sh.h_d[qh + k], sh.h_b[qh + k], act, kb);
                        const int pos = warp_sum_i(before);
                        if (qh + nq + 1 > kCcQCap) {  // move the list to the front of its array
                            long long vd[kCcQCap / 32];
                            int32_t vb[kCcQCap / 32], vc[kCcQCap / 32];
#pragma unroll
                            for (int t = 0; t < kCcQCap / 32; ++t) {
                                const int k = lane + 32 * t;
                                if (k < nq) {
                                    vd[t] = sh.h_d[qh + k];
                                    vb[t] = sh.h_b[qh + k];
                                    vc[t] = sh.h_c[qh + k];
                                }
                            }
                            __syncwarp();
#pragma unroll
                            for (int t = 0; t < kCcQCap / 32; ++t) {
                                const int k = lane + 32 * t;
                                if (k < nq) {
                                    sh.h_d[k] = vd[t];
                                    sh.h_b[k] = vb[t];
                                    sh.h_c[k] = vc[t];
                                }
                            }
                            __syncwarp();
                            qh = 0;
                        }
                        {
                            long long vd[kCcQCap / 32];
                            int32_t vb[kCcQCap / 32], vc[kCcQCap / 32];
#pragma unroll
                            for (int t = 0; t < kCcQCap / 32; ++t) {
                                const int k = pos + lane + 32 * t;
                                if (k < nq) {
                                    vd[t] = sh.h_d[qh + k];
                                    vb[t] = sh.h_b[qh + k];
                                    vc[t] = sh.h_c[qh + k];
                                }
                            }
                            __syncwarp();
#pragma unroll
                            for (int t = 0; t < kCcQCap / 32; ++t) {
                                const int k = pos + lane + 32 * t;
                                if (k < nq) {
                                    sh.h_d[qh + k + 1] = vd[t];
                                    sh.h_b[qh + k + 1] = vb[t];
                                    sh.h_c[qh + k + 1] = vc[t];
                                }
                            }
                            if (lane == 0) {
                                sh.h_d[qh + pos] = act;
                                sh.h_b[qh + pos] = kb;
                                sh.h_c[qh + pos] = ci;
                            }
                            __syncwarp();
                        }
                        ++nq;
                        continue;
                    }
                    if (lane == 0) {
                        sh.m_from[nm] = kb;
                        sh.m_to[nm] = to;
                    }
                    if (lane < kCcWords) sh.smask[lane] |= sh.inv[ci][lane];
                    ++nm;
                    __syncwarp();
                }
                if (lane == 0) {
                    sh.qh = qh;
                    sh.nq = nq;
                    sh.p += c0;
                    sh.q += c1;
                    sh.cS = c2;
                    sh.nm = nm;
                    sh.merged += nm;
                    sh.ne -= nm;  // every merge lowers the count (blockmodel.cpp:356)
                    sh.rounds += 1;
                }
            }
            __syncthreads();
            // S := S[cS..ns) merged with the round's put-backs
            {
                const int cS = sh.cS, nq = sh.nq, ns = sh.ns, ssel = sh.ssel;
                const long long* q_dS = sh.h_d + sh.qh;
                const int32_t* q_blk = sh.h_b + sh.qh;
                if (cS > 0 || nq > 0) {
                    const int rest = ns - cS;
                    const long long* sd = sh.s_dS[ssel] + cS;
                    const int32_t* sb = sh.s_blk[ssel] + cS;
                    long long* od = sh.s_dS[ssel ^ 1];
                    int32_t* ob = sh.s_blk[ssel ^ 1];
                    for (int i = tid; i < rest; i += kCcThreads) {
                        const int pos = i + count_before(q_dS, q_blk, nq, sd[i], sb[i]);
                        od[pos] = sd[i];
                        ob[pos] = sb[i];
                    }
                    for (int k = tid; k < nq; k += kCcThreads) {
                        const int pos = k + count_before(sd, sb, rest, q_dS[k], q_blk[k]);
                        od[pos] = q_dS[k];
                        ob[pos] = q_blk[k];
                    }
                    __syncthreads();
                    if (tid == 0) {
                        sh.ns = rest + nq;
                        sh.ssel = ssel ^ 1;
                    }
                    __syncthreads();
                }
            }
            // spill S into the global run when it could not take another round's put-backs
            if (sh.ns > kCcQS - kCcQCap - 1) {
                const int ns = sh.ns, ssel = sh.ssel, q = sh.q, nr = sh.nR - sh.q;
                const long long* rdS = (sh.rsel ? r1_dS : r0_dS) + q;
                const int32_t* rb = (sh.rsel ? r1_blk : r0_blk) + q;
                long long* od = sh.rsel ? r0_dS : r1_dS;
                int32_t* ob = sh.rsel ? r0_blk : r1_blk;
                const long long* sd = sh.s_dS[ssel];
                const int32_t* sb = sh.s_blk[ssel];
                for (int i = tid; i < nr; i += kCcThreads) {
                    const int pos = i + count_before(sd, sb, ns, rdS[i], rb[i]);
                    od[pos] = rdS[i];
                    ob[pos] = rb[i];
                }
                for (int k = tid; k < ns; k += kCcThreads) {
                    int lo = 0, hi = nr;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (qless(rdS[mid], rb[mid], sd[k], sb[k])) lo = mid + 1;
                        else hi = mid;
                    }
                    od[k + lo] = sd[k];
                    ob[k + lo] = sb[k];
                }
                __syncthreads();
                if (tid == 0) {
                    sh.nR = nr + ns;
                    sh.q = 0;
                    sh.rsel ^= 1;
                    sh.ns = 0;
                }
                __syncthreads();
            }
        }
        cluster.sync();
        // ---- 5. Blockmodel::merge_block (blockmodel.cpp:337-363) for the round's merges:
        // merge k goes to CTA k % cs; a CTA's merges share its warps (row walk and column
        // walk on separate warps when there are few).  The target's own row and column
        // receive their new keys through a staging slice and one bulk append; the lists of
        // third blocks, which several merges may extend at once, take single keys.  A third
        // block may be another merge's target (a key of this merge's source), so every CTA
        // finishes its single-key appends before any CTA reserves room in a target's list:
        // all CTAs take the same number of passes, with cluster barriers between the phases.
        {
            const int nm = ctl.nm;
            const int mine = nm > rank ? (nm - rank + cs - 1) / cs : 0;
            const int passes = (((nm + cs - 1) / cs) + kCcWarps / 2 - 1) / (kCcWarps / 2);
            int32_t* my_stage = stage_buf + (int64_t)rank * (kCcWarps / 2) * 2 * kCcStage;
            for (int pass = 0; pass < passes; ++pass) {
                const int base = pass * (kCcWarps / 2);
                const int here = max(0, min(kCcWarps / 2, mine - base));
                const int wpm = here == 1 ? 16 : here == 2 ? 8 : here <= 4 ? 4 : 2;
                const int slot = warp / wpm;
                if (tid < kCcWarps) (&sh.st_n[0][0])[tid] = 0;
                __syncthreads();
                if (slot < here) {
                    const int k = rank + cs * (base + slot);
                    const int32_t mf = ctl.m_from[k], mt = ctl.m_to[k];
                    const int half = (warp % wpm) >= wpm / 2;
                    const int nth = 32 * wpm / 2, ht = tid - (slot * wpm + half * wpm / 2) * 32;
                    int32_t* srow = my_stage + (int64_t)(2 * slot) * kCcStage;
                    int32_t* scol = srow + kCcStage;
                    // a new key of the target's row (which 0) or column (which 1)
                    auto stage_key = [&](int which, int32_t key) {
                        const int p = atomicAdd(&sh.st_n[slot][which], 1);
                        if (p < kCcStage) (which ? scol : srow)[p] = key;
                        else list_push1_shared(which ? ch.col_head : ch.row_head, ch, mt, key, flags);
                    };
                    if (half == 0) {
                        list_for_each(bm.row_col, bm.row_off[mf], bm.row_off[mf + 1], ch.row_head[mf], ch, ht, nth,
                                      [&](int32_t c) {
                                          const int32_t m = cells.take(mf, c, flags);
                                          if (m == 0) return;
                                          const int32_t c2 = (c == mf || c == mt) ? mt : c;
                                          if (cells.add(mt, c2, m, flags)) {
                                              stage_key(0, c2);
                                              if (c2 == mt) stage_key(1, mt);
                                              else list_push1_shared(ch.col_head, ch, c2, mt, flags);
                                          }
                                      });
                    } else {
                        list_for_each(bm.col_row, bm.col_off[mf], bm.col_off[mf + 1], ch.col_head[mf], ch, ht, nth,
                                      [&](int32_t x) {
                                          if (x == mf) return;
                                          const int32_t m = cells.take(x, mf, flags);
                                          if (m == 0) return;
                                          const int32_t x2 = x == mt ? mt : x;
                                          if (cells.add(x2, mt, m, flags)) {
                                              stage_key(1, x2);
                                              if (x2 == mt) stage_key(0, mt);
                                              else list_push1_shared(ch.row_head, ch, x2, mt, flags);
                                          }
                                      });
                    }
                }
                cluster.sync();  // every CTA's single-key appends of this pass are done
                if (tid < 2 * here) {
                    const int sl = tid >> 1, which = tid & 1;
                    const int32_t mt = ctl.m_to[rank + cs * (base + sl)];
                    const int n = min(sh.st_n[sl][which], kCcStage);
                    sh.st_slot[sl][which] = n > 0 ? list_reserve(which ? ch.col_head : ch.row_head, ch, mt, n, flags) : -1;
                }
                __syncthreads();
                for (int sl = 0; sl < here; ++sl)
                    for (int which = 0; which < 2; ++which) {
                        const int n = min(sh.st_n[sl][which], kCcStage);
                        const int32_t at = sh.st_slot[sl][which];
                        const int32_t* src = my_stage + (int64_t)(2 * sl + which) * kCcStage;
                        if (at >= 0)
                            for (int i = tid; i < n; i += kCcThreads) ch.pool[at + i] = src[i];
                    }
                if (tid < here) {
                    const int k = rank + cs * (base + tid);
                    const int32_t mf = ctl.m_from[k], mt = ctl.m_to[k];
                    bm.d_out[mt] += bm.d_out[mf];
                    bm.d_in[mt] += bm.d_in[mf];
                    bm.d_out[mf] = 0;
                    bm.d_in[mf] = 0;
                    bm.d_tot[mf] = 0;
                    bm.d_tot[mt] = bm.d_out[mt] + bm.d_in[mt] - cells.get(mt, mt);
                    bm.sizes[mt] += bm.sizes[mf];
                    bm.sizes[mf] = 0;
                    parent[mf] = mt;
                }
                cluster.sync();  // and the reservations before the next pass appends again
            }
            // this round's candidate blocks leave cand_of
            if (j < ncand && lane == 0) cand_of[ctl.c_blk[j]] = -1;
        }
        cluster.sync();
    }
    keys_seen = warp_sum_ll((long long)keys_seen);
    evals = warp_sum_ll((long long)evals);
    if (lane == 0) {
        atomicAdd(&flags->counters[9], keys_seen);
        atomicAdd(&flags->counters[10], evals);
    }
    if (controller && tid == 0) {
        *out_merged = (int32_t)sh.merged;
        atomicAdd(&flags->counters[0], (unsigned long long)sh.rounds);
    }
}

// Largest cluster (16, else 8, else 4) the device holds for this kernel.
template <class K>
int carry_cluster_pick(K kernel) {
    static int cached = -1;
    if (cached >= 0) return cached;
    const int smem = (int)sizeof(CcShared);
    cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    for (int cs = kCcMaxCluster; cs >= 4; cs /= 2) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(kCcThreads);
        cfg.dynamicSmemBytes = smem;
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
void launch_carry_cluster(const DevGraph& g, DevBM& bm, const Cells& cells, int64_t num_to_merge, int cs,
                          int32_t* d_merged, Work& w, cudaStream_t st) {
    auto kernel = k_carry_cluster<Cells, kNP>;
    const int smem = (int)sizeof(CcShared);
    cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kCcThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(
        &cfg, kernel, g, bm, w.chain, cells, (const uint64_t*)w.keys, (const int32_t*)w.vals, bm.B,
        (const int32_t*)w.best, reinterpret_cast<long long*>(w.heap_dS), w.heap_blk,
        reinterpret_cast<long long*>(w.keys_alt), w.vals_alt, w.parent, (long long)num_to_merge, w.cc_head, w.cc_stage,
        d_merged, w.flags_dev);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cluster carry-out launch: ") + cudaGetErrorString(e));
}

__global__ void k_cc_dense_fill(DevBM bm, int32_t* M) {
    const int64_t B = bm.B;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < bm.nnz; j += (int64_t)gridDim.x * blockDim.x)
        M[bm.row_of[j] * B + bm.row_col[j]] = bm.row_cnt[j];
}

}  // namespace

int carry_cluster_size() { return carry_cluster_pick(k_carry_cluster<HashCells, false>); }

size_t carry_cluster_stage_ints(int cs) { return (size_t)cs * (kCcWarps / 2) * 2 * kCcStage; }

void carry_out_cluster(const DevGraph& g, DevBM& bm, int64_t num_to_merge, Work& w, cudaStream_t st, bool np) {
    if (np && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    const int cs = carry_cluster_size();
    if (cs <= 0 || !w.cc_head || !w.cc_stage)
        throw std::logic_error("cluster carry-out buffers missing");
    const int32_t B = bm.B;
    const bool dense = w.cells && (uint64_t)B * (uint64_t)B <= w.cells_elems;
    int32_t* d_merged = w.d_scalar + 1;
    cudaMemsetAsync(w.cc_head, 0xff, sizeof(int32_t) * (size_t)B, st);
    if (dense) {
        lists_init(bm, w, st);
        cudaMemsetAsync(w.cells, 0, sizeof(int32_t) * (size_t)B * (size_t)B, st);
        const int64_t blocks = std::min<int64_t>((bm.nnz + 255) / 256 + 1, (int64_t)device_sms() * 16);
        k_cc_dense_fill<<<(unsigned)blocks, 256, 0, st>>>(bm, w.cells);
        const DenseCells dc{w.cells, (int64_t)B};
        if (np) launch_carry_cluster<DenseCells, true>(g, bm, dc, num_to_merge, cs, d_merged, w, st);
        else launch_carry_cluster<DenseCells, false>(g, bm, dc, num_to_merge, cs, d_merged, w, st);
        count_launches(2);
    } else {
        chain_init(bm, w, (uint64_t)2 * (uint64_t)bm.nnz, st);
        const HashCells hc{w.chain};
        if (np) launch_carry_cluster<HashCells, true>(g, bm, hc, num_to_merge, cs, d_merged, w, st);
        else launch_carry_cluster<HashCells, false>(g, bm, hc, num_to_merge, cs, d_merged, w, st);
        count_launches(1);
    }
}

}  // namespace sbp

// Exact block-merge carry-out: block_merge::carry_out_best_merges_advanced (reference
// src/block_merge.cpp:40-117) on one CTA.
//
// The reference pops merges one at a time from a priority queue ordered by delta,
// recomputes the popped merge's delta against the current blockmodel, puts it back with
// the recomputed delta when that is larger than the delta now on top of the queue, and
// merges otherwise.  Between two merges the blockmodel does not change, so the deltas of
// the next pops do not depend on one another.  Each round here therefore
//   1. selects the W smallest live queue entries (and the (W+1)-th as a bound),
//   2. recomputes their deltas at once, one team of warps per entry,
//   3. replays the reference's pop / put-back / merge rule over those values on one
//      warp, up to the first entry it holds no value for,
//   4. applies the merges of the round together, a team of warps each (up to 8 at once).
// A merge r -> s changes only rows / columns r and s and the degrees of r and s, so an
// evaluation stays exact after it unless it read one of them: each evaluation records
// the blocks it read (its two blocks, every key of the moving row and column) in a
// 2048-bit filter, and the replay continues past a merge only through entries whose
// filter holds neither block (a false positive merely ends the round early).  The same
// property lets the round's merges run concurrently: they move disjoint rows and columns
// into distinct targets, so they share only the key lists of third blocks, which take
// their keys through list_push1_shared; each merge stages the new keys of its target's row
// and column in its own slice of the staging buffers, sized from the keys its evaluation
// walked.
// Merges, their order and every put-back delta equal those of the one-at-a-time loop;
// ties of equal delta pop in ascending block order.
//
// Deltas are handled as exact int64 multiples of 2^-24 (the reference's doubles compare
// the same way), which keeps the sequential queue logic off the slow FP64 pipe.
//
// Nonparametric entropy (kNP): every merge lowers the number of non-empty blocks by one
// (blockmodel.cpp:356), which changes the partition and edge-count terms of every later
// merge by the same amount.  An evaluation therefore leaves that term out and the replay
// adds it for the count at the moment of the pop, so evaluations stay exact across the
// round's merges; a put-back entry popped again is re-scored the same way.
// Queue: the proposals sorted by (delta, block) (P, read through a cursor), put-back
// entries in a sorted shared-memory buffer (S) that spills into a sorted global run (R)
// through a parallel merge.  Each block is in the queue at most once.
//
// Cell values: a dense B x B int32 matrix when it fits the dense budget (no hashing; a
// cell of two live blocks is non-zero exactly when its key is in the row / column
// lists, because the only cells a merge empties are those of the block that dies), else
// the chain hash.  Keys always come from the chain's row / column lists.
#include <algorithm>
#include <cfloat>
#include <climits>

#include <stdexcept>

#include "carry.cuh"

namespace sbp {

namespace {

constexpr int kCarryThreads = 512;
constexpr int kCarryWarps = kCarryThreads / 32;
constexpr int kQS = 1024;   // shared put-back buffer
constexpr int kMaxW = 16;   // entries evaluated per round (kCarryWarps / warps per team)
constexpr int kBloomWords = 64;  // 2048-bit filter of the blocks an evaluation read

struct CarryShared {
    long long s_dS[2][kQS];
    int32_t s_blk[2][kQS];
    long long h_dS[3][32];
    int32_t h_blk[3][32];
    long long c_dS[kMaxW];
    int32_t c_blk[kMaxW];
    int32_t c_src[kMaxW];
    int32_t c_to[kMaxW];
    long long part[kCarryWarps];
    long long q_dS[kMaxW];
    int32_t q_blk[kMaxW];
    int32_t q_to[kMaxW];
    int32_t q_cand[kMaxW];
    uint32_t bloom[kMaxW][kBloomWords];
    int32_t m_from[kMaxW], m_to[kMaxW], m_keys[kMaxW];
    int32_t m_off[kMaxW], m_nrt[kMaxW], m_nct[kMaxW], m_slot_r[kMaxW], m_slot_c[kMaxW];
    int32_t c_keys[kMaxW];
    uint32_t conf[kMaxW];    // bit i of conf[j]: a merge of candidate i would change j's value
    long long c_act[kMaxW];  // recomputed delta of candidate i
    int32_t c_count[kMaxW];  // kNP: the candidate's delta takes the non-empty-count term
    int32_t ne;              // kNP: current number of non-empty blocks
    int32_t nm, np;
    long long b_dS;
    int32_t b_blk;
    int32_t has_bound, ncand, nq, cS;
    int32_t p, q, nR, rsel, ns, ssel;
    int32_t nrt, nct, slot_r, slot_c;
    long long merged, rounds;
};

// W = kCarryWarps / team_warps entries per round; team_warps in {1, 2, 4, 8}.
template <class Cells, bool kNP>
__global__ void __launch_bounds__(kCarryThreads, 1) k_carry_out(
    DevGraph g, DevBM bm, DevChain ch, Cells cells, const uint64_t* __restrict__ pkeys,
    const int32_t* __restrict__ pblk, int32_t nP, const int32_t* __restrict__ best, long long* r0_dS, int32_t* r0_blk,
    long long* r1_dS, int32_t* r1_blk, int32_t* parent, long long num_to_merge, int team_warps, int32_t* stage_row,
    int32_t* stage_col, int stage_cap, int32_t* out_merged, DevFlags* flags) {
    __shared__ CarryShared sh;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int W = min(kMaxW, kCarryWarps / team_warps);
    if (tid == 0) {
        sh.p = 0;
        sh.q = 0;
        sh.nR = 0;
        sh.rsel = 0;
        sh.ns = 0;
        sh.ssel = 0;
        sh.merged = 0;
        sh.rounds = 0;
        sh.ne = kNP ? *bm.nonempty : 0;
    }
    const long long max_rounds = 64ll * (nP + 1) + 4096;
    unsigned long long keys_seen = 0, evals = 0;  // this thread's share of the work counters
    __syncthreads();
    while (true) {
        if (sh.merged >= num_to_merge) break;
        if (sh.rounds >= max_rounds) {
            if (tid == 0) atomicOr(&flags->err, ERR_STATE);
            break;
        }
        for (int i = tid; i < kMaxW * kBloomWords; i += kCarryThreads) (&sh.bloom[0][0])[i] = 0u;
        if (tid < kMaxW) {
            sh.c_keys[tid] = 0;
            sh.conf[tid] = 0u;
        }
        // ---- 1. the W smallest live entries and the bound (warp 0)
        if (warp == 0) {
            const int p = sh.p, q = sh.q, nR = sh.nR, ns = sh.ns, ssel = sh.ssel;
            const long long* rd = sh.rsel ? r1_dS : r0_dS;
            const int32_t* rb = sh.rsel ? r1_blk : r0_blk;
            const int n0 = max(0, min(W + 1, nP - p)), n1 = max(0, min(W + 1, nR - q)), n2 = min(W + 1, ns);
            if (lane < n0) {
                sh.h_dS[0][lane] = key_to_fixed(pkeys[p + lane]);
                sh.h_blk[0][lane] = pblk[p + lane];
            }
            if (lane < n1) {
                sh.h_dS[1][lane] = rd[q + lane];
                sh.h_blk[1][lane] = rb[q + lane];
            }
            if (lane < n2) {
                sh.h_dS[2][lane] = sh.s_dS[ssel][lane];
                sh.h_blk[2][lane] = sh.s_blk[ssel][lane];
            }
            __syncwarp();
            const int n[3] = {n0, n1, n2};
#pragma unroll
            for (int src = 0; src < 3; ++src) {
                if (lane < n[src]) {
                    const long long d = sh.h_dS[src][lane];
                    const int32_t b = sh.h_blk[src][lane];
                    int rank = lane;
#pragma unroll
                    for (int o = 0; o < 3; ++o)
                        if (o != src) rank += count_before(sh.h_dS[o], sh.h_blk[o], n[o], d, b);
                    if (rank < W) {
                        sh.c_dS[rank] = d;
                        sh.c_blk[rank] = b;
                        sh.c_src[rank] = src;
                    } else if (rank == W) {
                        sh.b_dS = d;
                        sh.b_blk = b;
                    }
                }
            }
            if (lane == 0) {
                const int tot = n0 + n1 + n2;
                sh.ncand = min(W, tot);
                sh.has_bound = tot > W;
            }
        }
        __syncthreads();
        const int ncand = sh.ncand;
        if (ncand == 0) break;
        // ---- 2. recompute the deltas, one team per entry
        {
            const int team = warp / team_warps;
            if (team < ncand) {
                const int32_t from = sh.c_blk[team];
                int32_t to = 0;
                if (lane == 0) {
                    const int32_t b = best[from];
                    to = (b < 0 || b >= bm.B) ? from : uf_find(parent, b);
                }
                to = __shfl_sync(SBP_FULL_MASK, to, 0);
                long long part = 0;
                // nonparametric: zero when either block is empty (entropy.cpp:1203-1204)
                const bool counted = !kNP || (to != from && bm.sizes[from] != 0 && bm.sizes[to] != 0);
                if (lane == 0 && warp % team_warps == 0) sh.c_count[team] = kNP && counted;
                if (to != from && counted) {
                    const int nt = 32 * team_warps, t = tid - team * nt;
                    const unsigned long long before = keys_seen;
                    uint32_t* bloom = sh.bloom[team];
                    part = merge_delta_part<Cells, kNP>(g, bm, ch, cells, from, to, t, nt, (warp % team_warps) == 0,
                                                        [&](int32_t x) { bloom_add(bloom, x); }, keys_seen);
                    const int kc = warp_sum_i((int)(keys_seen - before));
                    if (lane == 0) atomicAdd(&sh.c_keys[team], kc);
                    if (lane == 0 && warp % team_warps == 0) ++evals;
                }
                if (lane == 0) {
                    sh.part[warp] = part;
                    if (warp % team_warps == 0) sh.c_to[team] = to;
                }
            }
        }
        __syncthreads();
        // ---- which candidate's merge would change which evaluation, all pairs at once
        if (tid < ncand * ncand) {
            const int i = tid / ncand, j = tid % ncand;
            if (i != j) {
                const int32_t a = sh.c_blk[i], b = sh.c_to[i];
                if (a == sh.c_blk[j] || b == sh.c_blk[j] || a == sh.c_to[j] || b == sh.c_to[j] ||
                    bloom_has(sh.bloom[j], a) || bloom_has(sh.bloom[j], b))
                    atomicOr(&sh.conf[j], 1u << i);
            }
        }
        if (tid < ncand) {
            long long aq = 0;
            for (int k = 0; k < team_warps; ++k) aq += sh.part[tid * team_warps + k];
            sh.c_act[tid] = aq;
        }
        __syncthreads();
        // ---- 3. replay the queue rule (block_merge.cpp:54-95) on warp 0.  Lane l holds
        // candidate l and entry l of the round's put-back list (sorted by delta, block) in
        // registers: a pop shifts the list down one lane, a put-back finds its place with a
        // ballot (the list holds each block at most once, so no two keys are equal) and
        // shifts the entries above it up one lane.
        if (warp == 0) {
            const bool lc = lane < ncand;
            const long long cd = lc ? sh.c_dS[lane] : 0, cact = lc ? sh.c_act[lane] : 0;
            const int32_t cb = lc ? sh.c_blk[lane] : 0, cto = lc ? sh.c_to[lane] : 0;
            const int32_t csrc = lc ? sh.c_src[lane] : 0, ckeys = lc ? sh.c_keys[lane] : 0;
            const int32_t ccount = lc ? sh.c_count[lane] : 0;
            const uint32_t cconf = lc ? sh.conf[lane] : 0u;
            long long qd = 0;
            int32_t qb = 0, qt = 0, qc = 0;
            int i = 0, nq = 0, nm = 0, cons0 = 0, cons1 = 0, cons2 = 0;
            uint32_t merged_mask = 0u;  // candidates merged in this round
            const bool hb = sh.has_bound;
            const long long bnd_dS = sh.b_dS, merged0 = sh.merged;
            const int32_t bnd_blk = sh.b_blk, ne0 = sh.ne;
            // each candidate is taken once and put back at most once
            for (int it = 0; it <= 2 * kMaxW + 1 && merged0 + nm < num_to_merge; ++it) {
                const long long hc_d = __shfl_sync(SBP_FULL_MASK, cd, i & 31);
                const int32_t hc_b = __shfl_sync(SBP_FULL_MASK, cb, i & 31);
                const long long hq_d = __shfl_sync(SBP_FULL_MASK, qd, 0);
                const int32_t hq_b = __shfl_sync(SBP_FULL_MASK, qb, 0);
                int pick = i < ncand ? 0 : -1;
                long long bd = hc_d;
                int32_t bb = hc_b;
                if (nq > 0 && (pick < 0 || qless(hq_d, hq_b, bd, bb))) {
                    pick = 1;
                    bd = hq_d;
                    bb = hq_b;
                }
                if (pick < 0) break;                                  // queue empty
                if (hb && qless(bnd_dS, bnd_blk, bd, bb)) break;      // next pop not evaluated
                int ci;
                int32_t from, to;
                if (pick == 1) {
                    // popped again: if no merge since touched what it read, its recomputed
                    // delta is the one it was put back with (kNP: up to the count term)
                    ci = __shfl_sync(SBP_FULL_MASK, qc, 0);
                    if (__shfl_sync(SBP_FULL_MASK, cconf, ci) & merged_mask) break;
                    from = hq_b;
                    to = __shfl_sync(SBP_FULL_MASK, qt, 0);
                    qd = __shfl_down_sync(SBP_FULL_MASK, qd, 1);
                    qb = __shfl_down_sync(SBP_FULL_MASK, qb, 1);
                    qt = __shfl_down_sync(SBP_FULL_MASK, qt, 1);
                    qc = __shfl_down_sync(SBP_FULL_MASK, qc, 1);
                    --nq;
                } else {
                    // its value is stale: re-evaluate it next round
                    if (__shfl_sync(SBP_FULL_MASK, cconf, i) & merged_mask) break;
                    from = hc_b;
                    to = __shfl_sync(SBP_FULL_MASK, cto, i);
                    const int32_t src = __shfl_sync(SBP_FULL_MASK, csrc, i);
                    cons0 += src == 0;
                    cons1 += src == 1;
                    cons2 += src == 2;
                    ci = i++;
                    if (to == from) continue;  // already in the same block
                }
                long long act = __shfl_sync(SBP_FULL_MASK, cact, ci);
                if (kNP && __shfl_sync(SBP_FULL_MASK, ccount, ci)) {
                    const int32_t b = min(max(ne0 - nm, 0), g.N + 1);
                    act += __ldg(g.Dm + b);
                }
                const int32_t keys_ci = __shfl_sync(SBP_FULL_MASK, ckeys, ci);
                const long long nc_d = __shfl_sync(SBP_FULL_MASK, cd, i & 31);
                const long long nq_d = __shfl_sync(SBP_FULL_MASK, qd, 0);
                if (i < ncand || nq > 0 || hb) {
                    long long top = hb ? bnd_dS : LLONG_MAX;
                    if (i < ncand) top = min(top, nc_d);
                    if (nq > 0) top = min(top, nq_d);
                    if (act > top) {  // put back with the recomputed delta
                        const int k = __popc(__ballot_sync(SBP_FULL_MASK, lane < nq && qless(qd, qb, act, from)));
                        const long long ud = __shfl_up_sync(SBP_FULL_MASK, qd, 1);
                        const int32_t ub = __shfl_up_sync(SBP_FULL_MASK, qb, 1);
                        const int32_t ut = __shfl_up_sync(SBP_FULL_MASK, qt, 1);
                        const int32_t uc = __shfl_up_sync(SBP_FULL_MASK, qc, 1);
                        if (lane > k) {
                            qd = ud;
                            qb = ub;
                            qt = ut;
                            qc = uc;
                        } else if (lane == k) {
                            qd = act;
                            qb = from;
                            qt = to;
                            qc = ci;
                        }
                        ++nq;
                        continue;
                    }
                }
                if (lane == 0) {
                    sh.m_from[nm] = from;
                    sh.m_to[nm] = to;
                    sh.m_keys[nm] = keys_ci;
                }
                merged_mask |= 1u << ci;
                ++nm;
            }
            if (lane < nq) {
                sh.q_dS[lane] = qd;
                sh.q_blk[lane] = qb;
            }
            if (lane == 0) {
                sh.p += cons0;
                sh.q += cons1;
                sh.cS = cons2;
                sh.nq = nq;
                sh.nm = nm;
                sh.ne -= nm;  // every merge lowers the count (blockmodel.cpp:356)
                sh.rounds += 1;
            }
        }
        __syncthreads();
        // ---- 4. S := S[cS..ns) merged with the put-back entries
        {
            const int cS = sh.cS, nq = sh.nq, ns = sh.ns, ssel = sh.ssel;
            if (cS > 0 || nq > 0) {
                const int rest = ns - cS;
                const long long* sd = sh.s_dS[ssel] + cS;
                const int32_t* sb = sh.s_blk[ssel] + cS;
                long long* od = sh.s_dS[ssel ^ 1];
                int32_t* ob = sh.s_blk[ssel ^ 1];
                for (int i = tid; i < rest; i += kCarryThreads) {
                    int pos = i;
                    for (int k = 0; k < nq; ++k) pos += qless(sh.q_dS[k], sh.q_blk[k], sd[i], sb[i]);
                    od[pos] = sd[i];
                    ob[pos] = sb[i];
                }
                for (int j = tid; j < nq; j += kCarryThreads) {
                    const int pos = j + count_before(sd, sb, rest, sh.q_dS[j], sh.q_blk[j]);
                    od[pos] = sh.q_dS[j];
                    ob[pos] = sh.q_blk[j];
                }
                __syncthreads();
                if (tid == 0) {
                    sh.ns = rest + nq;
                    sh.ssel = ssel ^ 1;
                }
                __syncthreads();
            }
        }
        // ---- spill S into R when it could not take another round's put-backs
        if (sh.ns > kQS - kMaxW - 1) {
            const int ns = sh.ns, ssel = sh.ssel, q = sh.q, nr = sh.nR - sh.q;
            const long long* rd = (sh.rsel ? r1_dS : r0_dS) + q;
            const int32_t* rb = (sh.rsel ? r1_blk : r0_blk) + q;
            long long* od = sh.rsel ? r0_dS : r1_dS;
            int32_t* ob = sh.rsel ? r0_blk : r1_blk;
            const long long* sd = sh.s_dS[ssel];
            const int32_t* sb = sh.s_blk[ssel];
            for (int i = tid; i < nr; i += kCarryThreads) {
                const long long d = rd[i];
                const int32_t b = rb[i];
                const int pos = i + count_before(sd, sb, ns, d, b);
                od[pos] = d;
                ob[pos] = b;
            }
            for (int j = tid; j < ns; j += kCarryThreads) {
                int lo = 0, hi = nr;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (qless(rd[mid], rb[mid], sd[j], sb[j])) lo = mid + 1;
                    else hi = mid;
                }
                od[j + lo] = sd[j];
                ob[j + lo] = sb[j];
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
        // ---- 5. Blockmodel::merge_block (src/blockmodel/blockmodel.cpp:337-363) for the
        // round's merges, up to 8 at once: merge j of a pass gets wpm warps, the first half
        // moving row mf, the second half column mf.
        const int nm = sh.nm;
        for (int j0 = 0; j0 < nm; j0 += sh.np) {
            __syncthreads();  // every thread has read sh.np of the previous pass
            if (tid == 0) {
                // as many merges (up to 8) as the staging buffers hold
                int off = 0, np = 0;
                while (np < 8 && j0 + np < nm && (np == 0 || off + sh.m_keys[j0 + np] + 2 <= stage_cap)) {
                    sh.m_off[np] = off;
                    off += sh.m_keys[j0 + np] + 2;
                    sh.m_nrt[np] = 0;
                    sh.m_nct[np] = 0;
                    ++np;
                }
                sh.np = np;
            }
            __syncthreads();
            const int np = sh.np;
            const int wpm = np <= 1 ? 16 : np <= 2 ? 8 : np <= 4 ? 4 : 2;
            const int j = warp / wpm;
            if (j < np) {
                const int32_t mf = sh.m_from[j0 + j], mt = sh.m_to[j0 + j];
                const int half = (warp % wpm) >= wpm / 2;
                const int nth = 32 * wpm / 2, ht = tid - (j * wpm + half * wpm / 2) * 32;
                const int slice = sh.m_keys[j0 + j] + 2;
                int32_t* srow = stage_row + sh.m_off[j];
                int32_t* scol = stage_col + sh.m_off[j];
                const bool solo = np == 1;
                if (half == 0) {
                    list_for_each(bm.row_col, bm.row_off[mf], bm.row_off[mf + 1], ch.row_head[mf], ch, ht, nth,
                                  [&](int32_t c) {
                                      const int32_t m = cells.take(mf, c, flags);
                                      if (m == 0) return;
                                      const int32_t c2 = (c == mf || c == mt) ? mt : c;
                                      if (cells.add(mt, c2, m, flags)) {
                                          stage(srow, &sh.m_nrt[j], slice, c2, flags);
                                          if (c2 == mt) stage(scol, &sh.m_nct[j], slice, mt, flags);
                                          else if (solo) list_push1(ch.col_head, ch, c2, mt, flags);
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
                                          stage(scol, &sh.m_nct[j], slice, x2, flags);
                                          if (x2 == mt) stage(srow, &sh.m_nrt[j], slice, mt, flags);
                                          else if (solo) list_push1(ch.row_head, ch, x2, mt, flags);
                                          else list_push1_shared(ch.row_head, ch, x2, mt, flags);
                                      }
                                  });
                }
            }
            __syncthreads();
            if (tid < np) {
                const int32_t mt = sh.m_to[j0 + tid];
                const int nr = min(sh.m_nrt[tid], sh.m_keys[j0 + tid] + 2);
                sh.m_slot_r[tid] = nr > 0 ? list_reserve(ch.row_head, ch, mt, nr, flags) : -1;
            } else if (tid >= 64 && tid < 64 + np) {
                const int q = tid - 64;
                const int32_t mt = sh.m_to[j0 + q];
                const int nc = min(sh.m_nct[q], sh.m_keys[j0 + q] + 2);
                sh.m_slot_c[q] = nc > 0 ? list_reserve(ch.col_head, ch, mt, nc, flags) : -1;
            }
            __syncthreads();
            for (int q = 0; q < np; ++q) {
                const int slice = sh.m_keys[j0 + q] + 2;
                const int nr = min(sh.m_nrt[q], slice), nc = min(sh.m_nct[q], slice);
                const int32_t pr = sh.m_slot_r[q], pc = sh.m_slot_c[q];
                const int32_t* srow = stage_row + sh.m_off[q];
                const int32_t* scol = stage_col + sh.m_off[q];
                if (pr >= 0)
                    for (int i = tid; i < nr; i += kCarryThreads) ch.pool[pr + i] = srow[i];
                if (pc >= 0)
                    for (int i = tid; i < nc; i += kCarryThreads) ch.pool[pc + i] = scol[i];
            }
            if (tid < np) {
                const int32_t mf = sh.m_from[j0 + tid], mt = sh.m_to[j0 + tid];
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
            __syncthreads();
        }
        if (tid == 0) sh.merged += nm;
        __syncthreads();
    }
    keys_seen = warp_sum_ll((long long)keys_seen);
    evals = warp_sum_ll((long long)evals);
    if (lane == 0) {
        atomicAdd(&flags->counters[9], keys_seen);
        atomicAdd(&flags->counters[10], evals);
    }
    if (tid == 0) {
        *out_merged = (int32_t)sh.merged;
        atomicAdd(&flags->counters[0], (unsigned long long)sh.rounds);
    }
}

__global__ void k_dense_cells_fill(DevBM bm, int32_t* M) {
    const int64_t B = bm.B;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < bm.nnz; j += (int64_t)gridDim.x * blockDim.x)
        M[bm.row_of[j] * B + bm.row_col[j]] = bm.row_cnt[j];
}

}  // namespace

template <class Cells>
void launch_carry(bool np, const DevGraph& g, DevBM& bm, const Cells& cells, int64_t num_to_merge, int team_warps,
                  int32_t* d_merged, Work& w, cudaStream_t st) {
    auto k = np ? k_carry_out<Cells, true> : k_carry_out<Cells, false>;
    k<<<1, kCarryThreads, 0, st>>>(g, bm, w.chain, cells, w.keys, w.vals, bm.B, w.best,
                                   reinterpret_cast<long long*>(w.heap_dS), w.heap_blk,
                                   reinterpret_cast<long long*>(w.keys_alt), w.vals_alt, w.parent, num_to_merge,
                                   team_warps, w.list_small, w.list_big, 2 * g.N, d_merged, w.flags_dev);
}

void carry_out_exact(const DevGraph& g, DevBM& bm, int64_t num_to_merge, Work& w, cudaStream_t st, bool np) {
    if (np && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    const int32_t B = bm.B;
    const bool dense = w.cells && (uint64_t)B * (uint64_t)B <= w.cells_elems;
    // team size from the mean number of row + column keys per block
    const double keys = 2.0 * (double)bm.nnz / (double)(B > 0 ? B : 1);
    const int team_warps = keys <= 512 ? 1 : keys <= 1024 ? 2 : keys <= 2048 ? 4 : 8;
    int32_t* d_merged = w.d_scalar + 1;
    if (dense) {
        lists_init(bm, w, st);
        cudaMemsetAsync(w.cells, 0, sizeof(int32_t) * (size_t)B * (size_t)B, st);
        const int64_t blocks = std::min<int64_t>((bm.nnz + 255) / 256 + 1, (int64_t)device_sms() * 16);
        k_dense_cells_fill<<<(unsigned)blocks, 256, 0, st>>>(bm, w.cells);
        launch_carry(np, g, bm, DenseCells{w.cells, (int64_t)B}, num_to_merge, team_warps, d_merged, w, st);
        count_launches(2);
    } else {
        chain_init(bm, w, (uint64_t)2 * (uint64_t)bm.nnz, st);
        launch_carry(np, g, bm, HashCells{w.chain}, num_to_merge, team_warps, d_merged, w, st);
        count_launches(1);
    }
}

}  // namespace sbp

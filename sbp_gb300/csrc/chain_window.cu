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

#include "delta.cuh"
#include "kernels.cuh"

namespace sbp {

namespace {

constexpr int kWinMaxWarps = 16;
constexpr int kSmemHashL2 = 9;     // neighbour hashes up to 512 slots live in shared memory
constexpr int kGlobalHashL2 = 13;  // larger ones (degree > 256) in a per-warp global region
constexpr int kLqCache = 2048;     // log-table entries copied into shared memory

enum : int32_t { ST_SKIP = 0, ST_NOMOVE = 1, ST_REJECT = 2, ST_ACCEPT = 3 };

struct SharedCells {
    const int32_t* M;
    int32_t ld;
    __device__ __forceinline__ int32_t row_get(int32_t r, int32_t c) const { return M[r * ld + c]; }
    __device__ __forceinline__ int32_t col_get(int32_t c, int32_t r) const { return M[r * ld + c]; }
};

// Dense M and its transpose in global memory, each with the sums of its rows' 128-entry
// tiles (TS for M, TST for the transpose) so that a multinomial draw over a row reads the
// row's tile sums and one tile instead of the whole row.
struct GlobalCells {
    int32_t* M;
    int32_t* MT;
    int32_t* TS;
    int32_t* TST;
    int64_t ld;
    int32_t nt;  // tiles per row
    __device__ __forceinline__ int32_t row_get(int32_t r, int32_t c) const { return __ldcg(M + r * ld + c); }
    __device__ __forceinline__ int32_t col_get(int32_t c, int32_t r) const { return __ldcg(MT + c * ld + r); }
    // M[r][c] += d, with the transpose and both tile sums
    __device__ __forceinline__ void add(int32_t r, int32_t c, int32_t d) const {
        atomicAdd(M + r * ld + c, d);
        atomicAdd(TS + (int64_t)r * nt + (c >> 7), d);
        atomicAdd(MT + c * ld + r, d);
        atomicAdd(TST + (int64_t)c * nt + (r >> 7), d);
    }
};

struct WinResult {
    long long dS;
    int32_t v, r, s, nb, status, k, kout, kin, L, l2;  // l2: log2 of this vertex's hash size
    int32_t dB;  // kNP: change of the number of non-empty blocks if the move is applied
    int32_t ni;  // slots of the hash taken by the neighbour blocks
};

// log2 of the neighbour-hash size for a vertex of degree k (at least twice k slots).
__device__ __forceinline__ int hash_log2(int32_t k, int log2max) {
    const int32_t need = 2 * (k > 16 ? k : 16);
    const int l = 32 - __clz(need - 1);
    return l < log2max ? l : log2max;
}

// Entry at cumulative unit t in ascending index order over x(i), i < B, one warp.
// get(i) returns the weight of index i.  Returns -1 when t is out of range.
template <typename Get>
__device__ __forceinline__ int32_t warp_select(int32_t B, long long t, Get get) {
    const int lane = threadIdx.x & 31;
    for (int32_t base = 0; base < B; base += 32) {
        const int32_t i = base + lane;
        const long long x = i < B ? (long long)get(i) : 0ll;
        long long incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
            if (lane >= o) incl += y;
        }
        const long long tot = __shfl_sync(SBP_FULL_MASK, incl, 31);
        if (t < tot) {
            const unsigned hit = __ballot_sync(SBP_FULL_MASK, incl > t);
            return base + __ffs(hit) - 1;
        }
        t -= tot;
    }
    return -1;
}

// The same over a 16-byte aligned global row (ld a multiple of 4): 128 entries per step.
__device__ __forceinline__ int32_t warp_select_row4(const int32_t* __restrict__ row, int32_t B, long long t,
                                                    int32_t skip) {
    const int lane = threadIdx.x & 31;
    for (int32_t base = 0; base < B; base += 128) {
        const int32_t i = base + 4 * lane;
        int4 q = make_int4(0, 0, 0, 0);
        if (i < B) q = __ldcg(reinterpret_cast<const int4*>(row + i));
        int32_t x[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (i + j >= B || i + j == skip) x[j] = 0;
        const long long s4 = (long long)x[0] + x[1] + x[2] + x[3];
        long long incl = s4;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
            if (lane >= o) incl += y;
        }
        const long long tot = __shfl_sync(SBP_FULL_MASK, incl, 31);
        if (t < tot) {
            const unsigned hit = __ballot_sync(SBP_FULL_MASK, incl > t);
            const int src = __ffs(hit) - 1;
            int32_t pick = -1;
            if (lane == src) {
                long long u = t - (incl - s4);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (pick < 0 && u < x[j]) pick = i + j;
                    u -= x[j];
                }
            }
            return __shfl_sync(SBP_FULL_MASK, pick, src);
        }
        t -= tot;
    }
    return -1;
}

__device__ __forceinline__ bool hash_has(const int32_t* hk, int log2cap, int32_t b) {
    const uint32_t mask = (1u << log2cap) - 1u;
    uint32_t s = hslot(b, log2cap);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int32_t k = hk[s];
        if (k == b) return true;
        if (k == -1) return false;
        s = (s + 1) & mask;
    }
    return false;
}

__device__ __forceinline__ int32_t hash_get(const int32_t* hk, const int32_t* cnt, int log2cap, int32_t b) {
    const uint32_t mask = (1u << log2cap) - 1u;
    uint32_t s = hslot(b, log2cap);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int32_t k = hk[s];
        if (k == b) return cnt[s];
        if (k == -1) return 0;
        s = (s + 1) & mask;
    }
    return 0;
}

// Entry at cumulative unit t of a global row through its tile sums: lane l takes tiles
// [8l, 8l + 8) of each group of 256 tiles (one load each), a warp scan over the lanes'
// totals finds the tile, then one pass over that tile (16-byte loads) finds the entry.
// Entry `skip` (weight skip_w) is left out.  pre, when given, holds this lane's tile sums
// of the first group, loaded earlier.
__device__ __forceinline__ int32_t warp_select_tiles(const int32_t* __restrict__ row, const int32_t* __restrict__ ts,
                                                     int32_t B, int32_t nt, long long t, int32_t skip,
                                                     int32_t skip_w, const int32_t* pre = nullptr) {
    const int lane = threadIdx.x & 31;
    const int32_t skip_tile = skip >= 0 ? skip >> 7 : -1;
    for (int32_t tb = 0; tb < nt; tb += 256) {
        int32_t x[8];
        long long mine = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int32_t tile = tb + 8 * lane + j;
            x[j] = tile < nt ? (pre && tb == 0 ? pre[j] : __ldcg(ts + tile)) - (tile == skip_tile ? skip_w : 0) : 0;
            mine += x[j];
        }
        long long incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
            if (lane >= o) incl += y;
        }
        const long long tot = __shfl_sync(SBP_FULL_MASK, incl, 31);
        if (t < tot) {
            const int src = __ffs(__ballot_sync(SBP_FULL_MASK, incl > t)) - 1;
            int32_t tile = -1;
            long long before = 0;
            if (lane == src) {
                long long u = t - (incl - mine);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (tile < 0 && u < x[j]) tile = tb + 8 * lane + j;
                    else if (tile < 0) u -= x[j];
                }
                before = t - u;
            }
            tile = __shfl_sync(SBP_FULL_MASK, tile, src);
            before = __shfl_sync(SBP_FULL_MASK, before, src);
            if (tile < 0) return -1;
            const int32_t base = tile << 7;
            const int32_t r = warp_select_row4(row + base, min(128, B - base), t - before, skip - base);
            return r < 0 ? -1 : base + r;
        }
        t -= tot;
    }
    return -1;
}

// Adds one to the count of key b, taking a slot for b when it is absent, probing from slot
// s.  Returns the slot when this call took it, else -1.
__device__ __forceinline__ int32_t hinsert_fresh(int32_t* keys, int32_t* cnt, int log2cap, int32_t b, uint32_t s) {
    const uint32_t mask = (1u << log2cap) - 1u;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int32_t k = ((volatile int32_t*)keys)[s];
        if (k == -1) {
            const int32_t prev = atomicCAS(keys + s, -1, b);
            if (prev == -1 || prev == b) {
                atomicAdd(cnt + s, 1);
                return prev == -1 ? (int32_t)s : -1;
            }
        } else if (k == b) {
            atomicAdd(cnt + s, 1);
            return -1;
        }
        s = (s + 1) & mask;
    }
    return -1;
}

// Neighbour-block counts of v into the warp's hash (edge_weights + the block lookups of
// blockmodel_delta): out-neighbours except v itself into hO, in-neighbours (self-loops
// already excluded) into hI, the slots taken listed in items[] (their number in n, which
// the caller zeroes).  Neighbour ids, then their blocks, are loaded 8 per lane before any
// insert; each lane keeps the slots it took and one warp scan places them in the list.
// on_nb(nb) is called as soon as the block nb of neighbour number `pick` (the proposal's
// sampled neighbour) is known.  The hash must be clean (keys -1, counts 0).  Returns nb,
// or -1 when pick is out of range.
template <class OnNb>
__device__ __forceinline__ int32_t warp_gather(const DevGraph& g, const int32_t* asg, int32_t v, int32_t r,
                                               int32_t o0, int32_t kout, int32_t i0, int32_t k, int32_t pick,
                                               int32_t* hk, int32_t* hO, int32_t* hI, int log2cap, int32_t* items,
                                               int32_t& n, OnNb on_nb) {
    const int lane = threadIdx.x & 31;
    int32_t nb = -1;
    for (int32_t base = 0; base < k; base += 256) {
        int32_t u[8], b[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int32_t idx = base + lane + 32 * j;
            u[j] = idx < k ? (idx < kout ? __ldg(g.out_nbr + o0 + idx) : __ldg(g.inns_nbr + i0 + idx - kout)) : -1;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int32_t idx = base + lane + 32 * j;
            b[j] = (u[j] >= 0 && !(idx < kout && u[j] == v)) ? __ldcg(asg + u[j]) : -1;
        }
        if (pick >= base && pick < base + 256) {  // the sampled neighbour's block (its own block for a self-loop)
            const int q = (pick - base) >> 5, owner = (pick - base) & 31;
            int32_t bq = b[0], uq = u[0];
#pragma unroll
            for (int j = 1; j < 8; ++j)
                if (j == q) {
                    bq = b[j];
                    uq = u[j];
                }
            nb = __shfl_sync(SBP_FULL_MASK, uq == v ? r : bq, owner);
            on_nb(nb);  // loads that need only nb start before the inserts
        }
        // The eight inserts of a lane in three batches: the home slots' keys, then a take of
        // every empty home slot, then the counts; a key whose home slot holds another key
        // probes on alone.
        uint32_t sl[8];
        int32_t kk[8], fresh[8], nf = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            sl[j] = b[j] >= 0 ? hslot(b[j], log2cap) : 0u;
            kk[j] = b[j] >= 0 ? ((volatile int32_t*)hk)[sl[j]] : 0;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (b[j] >= 0 && kk[j] == -1) {
                const int32_t prev = atomicCAS(hk + sl[j], -1, b[j]);
                kk[j] = prev == -1 ? INT_MIN : prev;  // INT_MIN: taken by this insert
            }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int32_t idx = base + lane + 32 * j;
            int32_t* cnt = idx < kout ? hO : hI;
            fresh[j] = -1;
            if (b[j] < 0) continue;
            if (kk[j] == INT_MIN || kk[j] == b[j]) {
                atomicAdd(cnt + sl[j], 1);
                if (kk[j] == INT_MIN) fresh[j] = (int32_t)sl[j];
            } else {
                fresh[j] = hinsert_fresh(hk, cnt, log2cap, b[j], (sl[j] + 1) & ((1u << log2cap) - 1u));
            }
            nf += fresh[j] >= 0;
        }
        // the slots this lane took, appended after those of the lanes below it
        int32_t off = nf;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(SBP_FULL_MASK, off, o);
            if (lane >= o) off += y;
        }
        const int32_t tot = __shfl_sync(SBP_FULL_MASK, off, 31);
        off += n - nf;
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (fresh[j] >= 0) items[off++] = fresh[j];
        n += tot;
    }
    __syncwarp();
    return nb;
}

// entropy::delta_mdl for moving v from r to s over the gathered neighbour blocks; the same
// terms as vertex_delta_fixed (exact int64, units of 2^-24) over the n occupied hash slots
// listed in items[], every cell of a pass loaded before it is used.  Log-table
// entries are 32-bit and a cell term v * (L[v] - L[d_in] - L[d_out]) is formed without a
// test for v = 0 (the product is 0 then); the logs of the degrees of r and s before and
// after the move are looked up once, and the four cells of rows / columns r and s are
// loaded before the hash is scanned.
// kNP: nonparametric::delta_mdl (src/entropy.cpp:1146-1178) with block sizes `size` and
// `nonempty` non-empty blocks.
template <class Cells, bool kNP>
__device__ long long warp_delta(const DevGraph& g, const int32_t* d_out, const int32_t* d_in, const Cells& M,
                                int32_t r, int32_t s, int32_t kout, int32_t kin, int32_t L, const int32_t* hk,
                                const int32_t* hO, const int32_t* hI, const int32_t* items, int32_t n,
                                const int32_t* lq_cache, const int32_t* size, int32_t nonempty) {
    const int lane = threadIdx.x & 31;
    const int32_t hi = g.E + 1;
    // fastlog table entry: the first kLqCache entries from shared memory
    auto L32 = [&](int32_t x) -> int32_t {
        x = max(0, min(x, hi));
        return x < kLqCache ? lq_cache[x] : __ldg(g.Lq + x);
    };
    const int32_t selfw = L > 0 ? 1 : 0;
    const int32_t dout_r = d_out[r], dout_s = d_out[s], din_r = d_in[r], din_s = d_in[s];
    const int32_t Mrr = M.row_get(r, r), Mrs = M.row_get(r, s), Msr = M.row_get(s, r), Mss = M.row_get(s, s);
    const int32_t dout_r2 = dout_r - kout, dout_s2 = dout_s + kout;
    const int32_t din_r2 = din_r - (kin + selfw), din_s2 = din_s + (kin + selfw);
    int32_t lo_r = 0, lo_s = 0, li_r = 0, li_s = 0, lo_r2 = 0, lo_s2 = 0, li_r2 = 0, li_s2 = 0;
    if (!kNP) {
        lo_r = L32(dout_r);
        lo_r2 = L32(dout_r2);
        lo_s = L32(dout_s);
        lo_s2 = L32(dout_s2);
        li_r = L32(din_r);
        li_r2 = L32(din_r2);
        li_s = L32(din_s);
        li_s2 = L32(din_s2);
    }
    int32_t Or = 0, Ir = 0, Os = 0, Is = 0;
    long long acc = 0;
    int32_t sRo = 0, sSo = 0, sRi = 0, sSi = 0;  // row / column sums of cells <= E
    for (int j0 = 0; j0 < n; j0 += 128) {
        int32_t b[4], O[4], I[4], Mrb[4], Msb[4], Mbr[4], Mbs[4], dib[4], dob[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int jj = j0 + lane + 32 * q;
            const int sl = jj < n ? items[jj] : -1;
            b[q] = sl >= 0 ? hk[sl] : -1;
            O[q] = sl >= 0 ? hO[sl] : 0;
            I[q] = sl >= 0 ? hI[sl] : 0;
            if (b[q] == r || b[q] == s) {  // the cells of r and s are handled after the loop
                if (b[q] == r) {
                    Or += O[q];
                    Ir += I[q];
                } else {
                    Os += O[q];
                    Is += I[q];
                }
                b[q] = -1;
                O[q] = 0;
                I[q] = 0;
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            Mrb[q] = O[q] > 0 ? M.row_get(r, b[q]) : 0;
            Msb[q] = O[q] > 0 ? M.row_get(s, b[q]) : 0;
            Mbr[q] = I[q] > 0 ? M.col_get(r, b[q]) : 0;
            Mbs[q] = I[q] > 0 ? M.col_get(s, b[q]) : 0;
            dib[q] = !kNP && O[q] > 0 ? d_in[b[q]] : 0;
            dob[q] = !kNP && I[q] > 0 ? d_out[b[q]] : 0;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if constexpr (kNP) {
                if (O[q] > 0) acc += np_cell(g, Mrb[q], -O[q]) + np_cell(g, Msb[q], O[q]);
                if (I[q] > 0) acc += np_cell(g, Mbr[q], -I[q]) + np_cell(g, Mbs[q], I[q]);
                continue;
            }
            if (O[q] > 0) {
                const int32_t ld = L32(dib[q]);
                const int32_t a0 = L32(Mrb[q]), a1 = L32(Mrb[q] - O[q]), a2 = L32(Msb[q]), a3 = L32(Msb[q] + O[q]);
                acc += (long long)Mrb[q] * (a0 - ld - lo_r) - (long long)(Mrb[q] - O[q]) * (a1 - ld - lo_r2) +
                       (long long)Msb[q] * (a2 - ld - lo_s) - (long long)(Msb[q] + O[q]) * (a3 - ld - lo_s2);
                sRo += Mrb[q];
                sSo += Msb[q];
            }
            if (I[q] > 0) {
                const int32_t ld = L32(dob[q]);
                const int32_t a0 = L32(Mbr[q]), a1 = L32(Mbr[q] - I[q]), a2 = L32(Mbs[q]), a3 = L32(Mbs[q] + I[q]);
                acc += (long long)Mbr[q] * (a0 - li_r - ld) - (long long)(Mbr[q] - I[q]) * (a1 - li_r2 - ld) +
                       (long long)Mbs[q] * (a2 - li_s - ld) - (long long)(Mbs[q] + I[q]) * (a3 - li_s2 - ld);
                sRi += Mbr[q];
                sSi += Mbs[q];
            }
        }
    }
    Or = warp_sum_i(Or);
    Ir = warp_sum_i(Ir);
    Os = warp_sum_i(Os);
    Is = warp_sum_i(Is);
    acc = warp_sum_ll(acc);
    sRo = warp_sum_i(sRo);
    sSo = warp_sum_i(sSo);
    sRi = warp_sum_i(sRi);
    sSi = warp_sum_i(sSi);
    const int32_t d_rr = -Or - Ir - L, d_rs = Ir - Os, d_sr = Or - Is, d_ss = Os + Is + L;
    long long tot = acc;
    if constexpr (kNP) {
        tot += np_cell_diag(g, Mrr, d_rr) + np_cell(g, Mrs, d_rs) + np_cell(g, Msr, d_sr) + np_cell_diag(g, Mss, d_ss);
        return tot + np_block_terms(g, dout_r, din_r, size[r], dout_s, din_s, size[s], kout, kin, 1, nonempty);
    }
    const int32_t c0 = L32(Mrr), c1 = L32(Mrr + d_rr), c2 = L32(Mrs), c3 = L32(Mrs + d_rs);
    const int32_t c4 = L32(Msr), c5 = L32(Msr + d_sr), c6 = L32(Mss), c7 = L32(Mss + d_ss);
    // ce_fixed(v, d_in, d_out) - ce_fixed(v + d, d_in', d_out') of a changed cell, and
    // ce_delta of an unchanged one (its degrees change only)
    auto changed = [](int32_t v, int32_t d, int32_t lv, int32_t lvd, int32_t li, int32_t lo, int32_t li2,
                      int32_t lo2) { return (long long)v * (lv - li - lo) - (long long)(v + d) * (lvd - li2 - lo2); };
    auto unchanged = [](int32_t v, int32_t li, int32_t lo, int32_t li2, int32_t lo2) {
        return (long long)v * ((li2 - li) + (lo2 - lo));
    };
    if (Or | Ir | L) tot += changed(Mrr, d_rr, c0, c1, li_r, lo_r, li_r2, lo_r2);
    else tot += unchanged(Mrr, li_r, lo_r, li_r2, lo_r2);
    if (Os | Ir) tot += changed(Mrs, d_rs, c2, c3, li_s, lo_r, li_s2, lo_r2);
    if (d_rs == 0) tot += unchanged(Mrs, li_s, lo_r, li_s2, lo_r2);
    if (Or | Is) tot += changed(Msr, d_sr, c4, c5, li_r, lo_s, li_r2, lo_s2);
    if (d_sr == 0) tot += unchanged(Msr, li_r, lo_s, li_r2, lo_s2);
    if (Os | Is | L) tot += changed(Mss, d_ss, c6, c7, li_s, lo_s, li_s2, lo_s2);
    else tot += unchanged(Mss, li_s, lo_s, li_s2, lo_s2);
    tot += ((long long)dout_r - Mrr - Mrs - sRo) * (lo_r2 - lo_r);
    tot += ((long long)dout_s - Msr - Mss - sSo) * (lo_s2 - lo_s);
    tot += ((long long)din_r - Mrr - Msr - sRi) * (li_r2 - li_r);
    tot += ((long long)din_s - Mrs - Mss - sSi) * (li_s2 - li_s);
    return tot;
}

// x in T(candidate)?
__device__ __forceinline__ bool in_touched(const WinResult& c, const int32_t* hk, int32_t x) {
    if (x == c.r) return true;
    if (c.status >= ST_NOMOVE && x == c.nb) return true;
    if (c.status >= ST_REJECT && (x == c.s || hash_has(hk, c.l2, x))) return true;
    return false;
}

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

// The snapshot's cells into the zeroed dense matrices and tile sums.
__global__ void k_window_fill(DevBM bm, GlobalCells gc) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < bm.nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = bm.row_of[j], c = bm.row_col[j], v = bm.row_cnt[j];
        gc.M[r * gc.ld + c] = v;
        gc.MT[c * gc.ld + r] = v;
        atomicAdd(gc.TS + (int64_t)r * gc.nt + (c >> 7), v);
        atomicAdd(gc.TST + (int64_t)c * gc.nt + (r >> 7), v);
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
    cudaMemsetAsync(w.cells, 0, sizeof(int32_t) * mh_window_cells(bm.B), st);
    int64_t blocks = ((int64_t)bm.nnz + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > (int64_t)device_sms() * 16) blocks = (int64_t)device_sms() * 16;
    k_window_fill<<<(unsigned)blocks, 256, 0, st>>>(bm, gc);
    if (p.mode == 1) launch_window<1>(np, g, bm, order, n, p, seed, iter, step, greedy, gc, smem, w, st);
    else launch_window<2>(np, g, bm, order, n, p, seed, iter, step, greedy, gc, smem, w, st);
    count_launches(2);
}

}  // namespace sbp

// Device helpers shared by the windowed Metropolis-Hastings chains (chain_window.cu: one CTA;
// chain_cluster.cu: a thread-block cluster): window entries, per-warp neighbour hashes,
// multinomial draws over dense rows, and the warp-level gather and delta of one proposal.
#pragma once

#include <climits>

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

// Zeroes the dense matrices and tile sums of gc (laid out from gc.M: M, MT, TS, TST) and
// fills them from the snapshot.
inline void window_fill(const DevBM& bm, const GlobalCells& gc, cudaStream_t st) {
    const int64_t B = bm.B;
    cudaMemsetAsync(gc.M, 0, sizeof(int32_t) * (2 * B * gc.ld + 2 * B * (int64_t)gc.nt), st);
    int64_t blocks = ((int64_t)bm.nnz + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > (int64_t)device_sms() * 16) blocks = (int64_t)device_sms() * 16;
    k_window_fill<<<(unsigned)blocks, 256, 0, st>>>(bm, gc);
}

}  // namespace

}  // namespace sbp

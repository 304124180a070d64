// Device helpers of the exact block-merge carry-out (carry.cu: one CTA; carry_cluster.cu:
// a thread-block cluster): cell stores, the merge queue's order, the union-find block map
// and one team's share of a merge delta.
#pragma once

#include <climits>

#include "chain.cuh"
#include "kernels.cuh"
#include "np.cuh"

namespace sbp {

namespace {

// Two bits of the 2048-bit filter per block.
__device__ __forceinline__ void bloom_add(uint32_t* f, int32_t x) {
    const uint32_t h = (uint32_t)x * 0x9E3779B1u;
    const uint32_t a = h >> 21, b = (h >> 10) & 2047u;
    atomicOr(f + (a >> 5), 1u << (a & 31));
    atomicOr(f + (b >> 5), 1u << (b & 31));
}
__device__ __forceinline__ bool bloom_has(const uint32_t* f, int32_t x) {
    const uint32_t h = (uint32_t)x * 0x9E3779B1u;
    const uint32_t a = h >> 21, b = (h >> 10) & 2047u;
    return ((f[a >> 5] >> (a & 31)) & 1u) && ((f[b >> 5] >> (b & 31)) & 1u);
}

struct DenseCells {
    int32_t* M;
    int64_t ld;
    __device__ __forceinline__ int32_t* at(int32_t r, int32_t c) const { return M + (int64_t)r * ld + c; }
    __device__ __forceinline__ int32_t get(int32_t r, int32_t c) const { return __ldcg(at(r, c)); }
    // Reads and clears a cell owned by the calling thread.
    __device__ __forceinline__ int32_t take(int32_t r, int32_t c, DevFlags*) const {
        int32_t* p = at(r, c);
        const int32_t v = __ldcg(p);
        if (v != 0) __stcg(p, 0);
        return v;
    }
    // Adds d > 0; true when the cell was empty (its key is new to the lists).
    __device__ __forceinline__ bool add(int32_t r, int32_t c, int32_t d, DevFlags*) const {
        return atomicAdd(at(r, c), d) == 0;
    }
};

struct HashCells {
    DevChain ch;
    __device__ __forceinline__ int32_t get(int32_t r, int32_t c) const { return chain_get(ch, r, c); }
    __device__ __forceinline__ int32_t take(int32_t r, int32_t c, DevFlags*) const {
        const unsigned long long k = cell_key(r, c);
        uint32_t s = cell_slot(k, ch.mask);
        for (uint32_t probe = 0; probe <= ch.mask; ++probe) {
            const ulonglong2 v = ld_slot(ch.slots + s);
            if (v.x == k) return (int32_t)(uint32_t)v.y == 0 ? 0 : atomicExch(slot_val(ch, (int32_t)s), 0);
            if (v.x == kEmptyKey) return 0;
            s = (s + 1) & ch.mask;
        }
        return 0;
    }
    __device__ __forceinline__ bool add(int32_t r, int32_t c, int32_t d, DevFlags* flags) const {
        return chain_add(ch, r, c, d, flags);
    }
};

__device__ __forceinline__ bool qless(long long a, int32_t ab, long long b, int32_t bb) {
    return a < b || (a == b && ab < bb);
}

// Inverse of the order-preserving key of the proposal sort (k_merge_keys): the delta in
// units of 2^-24.
__device__ __forceinline__ long long key_to_fixed(uint64_t k) { return (long long)(k ^ 0x8000000000000000ull); }

// Number of entries of the sorted list (d[i], b[i]), i < n, ordered before (x, xb).
__device__ __forceinline__ int count_before(const long long* d, const int32_t* b, int n, long long x, int32_t xb) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (qless(d[mid], b[mid], x, xb)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Root of x in the block map (union-find with path halving; concurrent halving only
// ever links a node to one of its ancestors).
__device__ __forceinline__ int32_t uf_find(int32_t* parent, int32_t x) {
    int guard = 0;
    while (guard++ < (1 << 24)) {
        const int32_t p = parent[x];
        if (p == x) return x;
        const int32_t gp = parent[p];
        if (gp != p) parent[x] = gp;
        x = gp;
    }
    return x;
}

// One team's share of entropy::block_merge_delta_mdl (reference src/entropy.cpp:129-182)
// for merging r into s, in units of 2^-24.  Thread t of nt walks its stride of the row
// and column key lists of r; the warp sum of the returned values over the team is the
// delta.  The terms that need no walk are added by the leader warp.  rec(key) is called
// for every third block whose cell the delta reads (a merge of that block would change
// the result).
//
// Row cell (r, c) with count m moves to (s, c): its term, the change of (s, c) and, for
// the cells of row s that do not receive anything, the change of their d_out factor
// collapse into (d_out[s] - M[s][s] - M[s][r] - sum over moved c of M[s][c]) times the
// log-degree difference; columns likewise.
// kNP: nonparametric::block_merge_delta_mdl (src/entropy.cpp:1198-1223) without its
// non-empty-count term; both blocks are non-empty (the caller checks).
template <class Cells, bool kNP, class Rec>
__device__ long long merge_delta_part(const DevGraph& g, const DevBM& bm, const DevChain& ch, const Cells& cells,
                                      int32_t r, int32_t s, int t, int nt, bool leader, Rec rec,
                                      unsigned long long& keys_seen) {
    const int32_t hi = g.E + 1;
    // fastlog table entry, 32-bit (cells and degrees are at most E)
    auto L32 = [&](int32_t x) -> int32_t { return __ldg(g.Lq + max(0, min(x, hi))); };
    const int32_t dout_r = bm.d_out[r], din_r = bm.d_in[r], dout_s = bm.d_out[s], din_s = bm.d_in[s];
    const int32_t dout_s2 = dout_s + dout_r, din_s2 = din_s + din_r;
    const int32_t lo_r = L32(dout_r), li_r = L32(din_r), lo_s = L32(dout_s), li_s = L32(din_s);
    const int32_t lo_s2 = L32(dout_s2), li_s2 = L32(din_s2);
    const long long Lout = lo_s2 - lo_s, Lin = li_s2 - li_s;
    long long acc = 0;
    // is_row: cell (r, key) moving to (s, key), factor d_in[key]; else (key, r) -> (key, s),
    // factor d_out[key].  Both forms load their three values before using any of them; a
    // cell term v * (L[v] - L[deg] - L[own]) needs no test for v = 0 (the product is 0).
    auto term = [&](int32_t key, bool is_row, int32_t m, int32_t o, int32_t deg) {
        if (m == 0 || (!is_row && key == r)) return;
        rec(key);
        if constexpr (kNP) {  // the cell empties; a third block's cell adds into row / column s
            acc += is_row && key == r ? np_cell_diag(g, m, -m) : np_lg(g, m);
            if (is_row ? (key != r && key != s) : (key != s)) acc += np_cell(g, o, m);
            return;
        }
        const bool third = is_row ? (key != r && key != s) : (key != s);
        const int32_t ld = L32(deg), lm = L32(m), lo = L32(third ? o : 0), lom = L32(third ? o + m : 0);
        acc += (long long)m * (lm - ld - (is_row ? lo_r : li_r));
        if (third) {
            const int32_t ls = is_row ? lo_s : li_s, ls2 = is_row ? lo_s2 : li_s2;
            acc += (long long)o * (lo - ld - ls) - (long long)(o + m) * (lom - ld - ls2) -
                   (long long)o * (is_row ? Lout : Lin);
        }
    };
    // The appended chunks of row r and of column r, walked together: each step takes the next
    // chunk of each list, loads the headers of the chunks after them before using its keys,
    // and handles the keys four per thread per pass with all their cells loaded first, so the
    // two list walks overlap their memory latencies.
    auto walk = [&](int32_t rh, int32_t chd) {
        const volatile int32_t* vp = ch.pool;
        int32_t c[2] = {rh, chd}, nxt[2] = {-1, -1}, cnt[2] = {0, 0}, cap[2] = {0, 0};
#pragma unroll
        for (int l = 0; l < 2; ++l)
            if (c[l] >= 0) {
                nxt[l] = vp[c[l]];
                cnt[l] = vp[c[l] + 1];
                cap[l] = vp[c[l] + 2];
            }
        int guard = 0;
        while ((c[0] >= 0 || c[1] >= 0) && guard++ < (1 << 26)) {
            int32_t nxt2[2] = {-1, -1}, cnt2[2] = {0, 0}, cap2[2] = {0, 0};
#pragma unroll
            for (int l = 0; l < 2; ++l)
                if (nxt[l] >= 0) {
                    nxt2[l] = vp[nxt[l]];
                    cnt2[l] = vp[nxt[l] + 1];
                    cap2[l] = vp[nxt[l] + 2];
                }
            const int32_t n0 = c[0] >= 0 ? min(cnt[0], cap[0]) : 0, n1 = c[1] >= 0 ? min(cnt[1], cap[1]) : 0;
            // one index space over the two chunks: [0, n0) row keys, [n0, n0 + n1) column keys
            for (int32_t i0 = t; i0 < n0 + n1; i0 += 4 * nt) {
                int32_t key[4], m[4], o[4], deg[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int32_t i = i0 + q * nt;
                    key[q] = i < n0 ? vp[c[0] + 3 + i] : (i < n0 + n1 ? vp[c[1] + 3 + i - n0] : -1);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const bool is_row = i0 + q * nt < n0;
                    const int32_t k = key[q] < 0 ? r : key[q];
                    m[q] = cells.get(is_row ? r : k, is_row ? k : r);
                    o[q] = cells.get(is_row ? s : k, is_row ? k : s);
                    deg[q] = (is_row ? bm.d_in : bm.d_out)[k];
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (key[q] >= 0) {
                        ++keys_seen;
                        term(key[q], i0 + q * nt < n0, m[q], o[q], deg[q]);
                    }
            }
#pragma unroll
            for (int l = 0; l < 2; ++l) {
                c[l] = nxt[l];
                nxt[l] = nxt2[l];
                cnt[l] = cnt2[l];
                cap[l] = cap2[l];
            }
        }
    };
    // Snapshot segments of row r and column r as one index space, four keys per thread
    // per pass: the keys, then all their cells and degrees, are loaded before any is used.
    const int32_t rlo = bm.row_off[r], rn = bm.row_off[r + 1] - rlo;
    const int32_t clo = bm.col_off[r], cn = bm.col_off[r + 1] - clo;
    const int32_t rhead = ch.row_head[r], chead = ch.col_head[r];
    for (int32_t j0 = t; j0 < rn + cn; j0 += 4 * nt) {
        int32_t key[4], m[4], o[4], deg[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int32_t j = j0 + q * nt;
            key[q] = j < rn ? bm.row_col[rlo + j] : (j < rn + cn ? bm.col_row[clo + j - rn] : -1);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const bool is_row = j0 + q * nt < rn;
            const int32_t k = key[q] < 0 ? r : key[q];
            m[q] = cells.get(is_row ? r : k, is_row ? k : r);
            o[q] = cells.get(is_row ? s : k, is_row ? k : s);
            deg[q] = (is_row ? bm.d_in : bm.d_out)[k];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (key[q] >= 0) {
                ++keys_seen;
                term(key[q], j0 + q * nt < rn, m[q], o[q], deg[q]);
            }
    }
    walk(rhead, chead);
    acc = warp_sum_ll(acc);
    if (leader && kNP) {
        const int32_t Mrr = cells.get(r, r), Mrs = cells.get(r, s), Msr = cells.get(s, r), Mss = cells.get(s, s);
        acc += np_cell_diag(g, Mss, Mrr + Mrs + Msr);
        acc += np_block_terms(g, dout_r, din_r, bm.sizes[r], dout_s, din_s, bm.sizes[s], dout_r, din_r, bm.sizes[r], 0,
                              false);
    } else if (leader) {
        const int32_t Mrr = cells.get(r, r), Mrs = cells.get(r, s), Msr = cells.get(s, r), Mss = cells.get(s, s);
        const int32_t dss = Mrr + Mrs + Msr;
        if (dss > 0)
            acc += (long long)Mss * (L32(Mss) - li_s - lo_s) - (long long)(Mss + dss) * (L32(Mss + dss) - li_s2 - lo_s2);
        else acc += (long long)Mss * ((li_s2 - li_s) + (lo_s2 - lo_s));
        acc += ((long long)dout_s - Msr - Mss) * Lout + ((long long)din_s - Mrs - Mss) * Lin;
    }
    return acc;
}

}  // namespace

}  // namespace sbp

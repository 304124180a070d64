// Proposal samplers and delta-MDL evaluation on the device.
//
// Delta-MDL follows entropy::delta_mdl (reference src/entropy.cpp:298-403) and
// entropy::block_merge_delta_mdl (:129-182) term by term, with two differences of
// method that leave the value unchanged:
//  * every term v * (L[v] - L[din] - L[dout]) is accumulated as an exact int64 in units
//    of 2^-24 (each logf value of an integer is a multiple of 2^-24), so the sum does
//    not depend on the order of summation;
//  * the reference's loops over the unchanged cells of rows r, s and columns r, s only
//    change their block degrees, so their contribution is
//    (sum of the unchanged counts) * (L[new degree] - L[old degree]); the unchanged
//    count is the block degree minus the counts of the cells the move touches.  Only
//    the O(k) touched cells are looked up.
// Key presence (a Delta cell whose net change is zero is visited by both loops of the
// reference) is reproduced exactly: for a vertex move only cells (r,s) and (s,r) can
// be present with a zero change.
#pragma once

#include "common.cuh"
#include "np.cuh"

namespace sbp {

// Matrix accessors.  row_get(r, c) = M[r, c] searching row r; col_get(c, r) = M[r, c]
// searching column c.
struct CsrAcc {
    DevBM bm;
    __device__ __forceinline__ int32_t row_get(int32_t r, int32_t c) const {
        return csr_get(bm.row_off, bm.row_col, bm.row_cnt, r, c);
    }
    __device__ __forceinline__ int32_t col_get(int32_t c, int32_t r) const {
        return csr_get(bm.col_off, bm.col_row, bm.col_cnt, c, r);
    }
};

struct ChainAcc {
    DevChain ch;
    __device__ __forceinline__ int32_t row_get(int32_t r, int32_t c) const { return chain_get(ch, r, c); }
    __device__ __forceinline__ int32_t col_get(int32_t c, int32_t r) const { return chain_get(ch, r, c); }
};

// Thread-group abstraction: one warp (kThreads == 32) or the whole CTA.
template <int kThreads>
struct Group {
    __device__ __forceinline__ static int rank() { return kThreads == 32 ? (int)(threadIdx.x & 31) : (int)threadIdx.x; }
    __device__ __forceinline__ static void sync() {
        if (kThreads == 32) __syncwarp();
        else __syncthreads();
    }
    // Sums N values over the group in one pass; red is [32][8] long longs of shared
    // memory (unused for a warp).  Every thread receives the totals.
    template <int N>
    __device__ __forceinline__ static void sum(long long v[N], long long (*red)[8]) {
#pragma unroll
        for (int j = 0; j < N; ++j) v[j] = warp_sum_ll(v[j]);
        if (kThreads == 32) return;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        __syncthreads();
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) red[w][j] = v[j];
        __syncthreads();
#pragma unroll
        for (int j = 0; j < N; ++j) {
            long long t = 0;
            for (int i = 0; i < kThreads / 32; ++i) t += red[i][j];
            v[j] = t;
        }
        __syncthreads();
    }
};

// ------------------------------------------------------------------ group hash
// Open-addressing table in shared (or global) memory aggregating per-block counts.
__device__ __forceinline__ uint32_t hslot(int32_t b, int log2cap) {
    return ((uint32_t)b * 0x9E3779B1u) >> (32 - log2cap);
}
__device__ __forceinline__ void hinsert(int32_t* keys, int32_t* cnt, int log2cap, int32_t b) {
    const uint32_t mask = (1u << log2cap) - 1u;
    uint32_t s = hslot(b, log2cap);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int32_t k = ((volatile int32_t*)keys)[s];
        if (k == b) {
            atomicAdd(cnt + s, 1);
            return;
        }
        if (k == -1) {
            const int32_t prev = atomicCAS(keys + s, -1, b);
            if (prev == -1 || prev == b) {
                atomicAdd(cnt + s, 1);
                return;
            }
        }
        s = (s + 1) & mask;
    }
}

// ------------------------------------------------------------------ samplers
// common::propose_new_block(..., block_merge=false) (reference src/common.cpp:138-198):
// a uniform neighbour among out-neighbours then in-neighbours without the vertex itself,
// its block nb, then a multinomial over nb's row (ascending column) followed by nb's
// column without the diagonal (ascending row).  Static CSR/CSC only.
__device__ __forceinline__ int32_t sample_vertex_proposal(const DevGraph& g, const DevBM& bm, int32_t v, int32_t r,
                                                          const uint32_t w[4]) {
    const int32_t o0 = __ldg(g.out_off + v), o1 = __ldg(g.out_off + v + 1);
    const int32_t i0 = __ldg(g.inns_off + v), i1 = __ldg(g.inns_off + v + 1);
    const int32_t kout = o1 - o0, k = kout + (i1 - i0);
    if (k == 0) return random_block(r, bm.B, w[1]);
    const int32_t idx = (int32_t)u32_below(w[0], (uint32_t)k);
    const int32_t nbr = idx < kout ? __ldg(g.out_nbr + o0 + idx) : __ldg(g.inns_nbr + i0 + idx - kout);
    const int32_t nb = bm.asg[nbr];
    const long long R = bm.d_out[nb];
    const int32_t dg = bm.diag[nb];
    const long long C = (long long)bm.d_in[nb] - dg;
    const long long t = (long long)u64_below(w[1], w[2], (uint64_t)(R + C));
    if (t < R) return seg_select(bm.row_col, bm.row_cum, bm.row_off[nb], bm.row_off[nb + 1], t, -1, 0, -1, 0);
    const int32_t p = dg > 0 ? csr_find(bm.col_off, bm.col_row, nb, nb) : -1;
    return seg_select(bm.col_row, bm.col_cum, bm.col_off[nb], bm.col_off[nb + 1], t - R, p, dg, -1, 0);
}

// common::propose_new_block(..., block_merge=true) as used by propose_merge_sparse
// (reference src/block_merge.cpp:251-256): neighbour block drawn from row r then column r
// weighted by counts; then nb's neighbour weights without block r.
__device__ __forceinline__ int32_t sample_merge_proposal(const DevBM& bm, int32_t r, const uint32_t w[4]) {
    const long long Rr = bm.d_out[r], Cr = bm.d_in[r];
    if (Rr + Cr == 0) return random_block(r, bm.B, w[0]);
    const long long t = (long long)u64_below(w[0], w[1], (uint64_t)(Rr + Cr));
    const int32_t nb = t < Rr ? seg_select(bm.row_col, bm.row_cum, bm.row_off[r], bm.row_off[r + 1], t, -1, 0, -1, 0)
                              : seg_select(bm.col_row, bm.col_cum, bm.col_off[r], bm.col_off[r + 1], t - Rr, -1, 0,
                                           -1, 0);
    if (nb < 0) return -1;
    const int32_t pr = csr_find(bm.row_off, bm.row_col, nb, r);  // (nb, r) in row nb
    const long long wr = pr >= 0 ? bm.row_cnt[pr] : 0;
    const long long R2 = (long long)bm.d_out[nb] - wr;
    int32_t pa = csr_find(bm.col_off, bm.col_row, nb, nb);        // (nb, nb) in column nb
    long long wa = pa >= 0 ? bm.col_cnt[pa] : 0;
    int32_t pb = -1;
    long long wb = 0;
    if (nb != r) {
        pb = csr_find(bm.col_off, bm.col_row, nb, r);             // (r, nb) in column nb
        wb = pb >= 0 ? bm.col_cnt[pb] : 0;
    }
    const long long C2 = (long long)bm.d_in[nb] - wa - wb;
    if (R2 + C2 == 0) return random_block(r, bm.B, w[2]);
    const long long t2 = (long long)u64_below(w[2], w[3], (uint64_t)(R2 + C2));
    if (t2 < R2) return seg_select(bm.row_col, bm.row_cum, bm.row_off[nb], bm.row_off[nb + 1], t2, pr, wr, -1, 0);
    if (pa > pb && pb >= 0) {
        const int32_t tp = pa;
        pa = pb;
        pb = tp;
        const long long tw = wa;
        wa = wb;
        wb = tw;
    }
    if (pa < 0) {
        pa = pb;
        wa = wb;
        pb = -1;
        wb = 0;
    }
    return seg_select(bm.col_row, bm.col_cum, bm.col_off[nb], bm.col_off[nb + 1], t2 - R2, pa, wa, pb, wb);
}

// ------------------------------------------------------------------ vertex delta-MDL
struct VertexScalars {
    int32_t kout, kin, L, selfw;
};

// Accumulates the touched-cell terms of moving v from r to s and returns the exact
// delta-MDL in units of 2^-24.  hk/hO/hI: group hash of 2^log2cap slots (>= 2k).
// kNP: nonparametric::delta_mdl (reference src/entropy.cpp:1146-1178) instead, which reads
// the block sizes and the number of non-empty blocks as well.
template <int kThreads, typename Acc, bool kNP = false>
__device__ long long vertex_delta_fixed(const DevGraph& g, const int32_t* asg, const int32_t* d_out,
                                        const int32_t* d_in, const Acc& M, int32_t v, int32_t r, int32_t s,
                                        int32_t* hk, int32_t* hO, int32_t* hI, int log2cap, long long (*red)[8],
                                        const int32_t* sizes = nullptr, int32_t nonempty = 0) {
    typedef Group<kThreads> G;
    const int t = G::rank();
    const int cap = 1 << log2cap;
    for (int i = t; i < cap; i += kThreads) {
        hk[i] = -1;
        hO[i] = 0;
        hI[i] = 0;
    }
    G::sync();
    const int32_t o0 = __ldg(g.out_off + v), o1 = __ldg(g.out_off + v + 1);
    const int32_t i0 = __ldg(g.inns_off + v), i1 = __ldg(g.inns_off + v + 1);
    for (int32_t i = o0 + t; i < o1; i += kThreads) {
        const int32_t u = __ldg(g.out_nbr + i);
        if (u != v) hinsert(hk, hO, log2cap, asg[u]);
    }
    for (int32_t i = i0 + t; i < i1; i += kThreads) hinsert(hk, hI, log2cap, asg[__ldg(g.inns_nbr + i)]);
    G::sync();
    const int32_t hi = g.E + 1;
    // fastlog table entry, 32-bit (cells and degrees are at most E); a cell term
    // v * (L[v] - L[d_in] - L[d_out]) is formed without a test for v = 0 (the product is 0)
    auto L32 = [&](int32_t x) -> int32_t { return __ldg(g.Lq + max(0, min(x, hi))); };
    const int32_t kout = o1 - o0, kin = i1 - i0, L = __ldg(g.selfcnt + v), selfw = L > 0 ? 1 : 0;
    const int32_t dout_r = d_out[r], dout_s = d_out[s], din_r = d_in[r], din_s = d_in[s];
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
    long long acc = 0, sRo = 0, sSo = 0, sRi = 0, sSi = 0, spec = 0;
    for (int i = t; i < cap; i += kThreads) {
        const int32_t b = hk[i];
        if (b < 0) continue;
        const int32_t O = hO[i], I = hI[i];
        if (b == r) {
            spec += ((long long)O << 48) | ((long long)I << 32);
            continue;
        }
        if (b == s) {
            spec += ((long long)O << 16) | (long long)I;
            continue;
        }
        if constexpr (kNP) {  // entries_dS: only the cells that change
            if (O > 0) acc += np_cell(g, M.row_get(r, b), -O) + np_cell(g, M.row_get(s, b), O);
            if (I > 0) acc += np_cell(g, M.col_get(r, b), -I) + np_cell(g, M.col_get(s, b), I);
            continue;
        }
        if (O > 0) {
            const int32_t Mrb = M.row_get(r, b), Msb = M.row_get(s, b), ld = L32(d_in[b]);
            const int32_t a0 = L32(Mrb), a1 = L32(Mrb - O), a2 = L32(Msb), a3 = L32(Msb + O);
            acc += (long long)Mrb * (a0 - ld - lo_r) - (long long)(Mrb - O) * (a1 - ld - lo_r2) +
                   (long long)Msb * (a2 - ld - lo_s) - (long long)(Msb + O) * (a3 - ld - lo_s2);
            sRo += Mrb;
            sSo += Msb;
        }
        if (I > 0) {
            const int32_t Mbr = M.col_get(r, b), Mbs = M.col_get(s, b), ld = L32(d_out[b]);
            const int32_t a0 = L32(Mbr), a1 = L32(Mbr - I), a2 = L32(Mbs), a3 = L32(Mbs + I);
            acc += (long long)Mbr * (a0 - li_r - ld) - (long long)(Mbr - I) * (a1 - li_r2 - ld) +
                   (long long)Mbs * (a2 - li_s - ld) - (long long)(Mbs + I) * (a3 - li_s2 - ld);
            sRi += Mbr;
            sSi += Mbs;
        }
    }
    {
        long long v[6] = {acc, sRo, sSo, sRi, sSi, spec};
        G::template sum<6>(v, red);
        acc = v[0];
        sRo = v[1];
        sSo = v[2];
        sRi = v[3];
        sSi = v[4];
        spec = v[5];
    }
    // Each count is < 2^16 in this packing only when k < 65536; the callers guarantee it.
    const int32_t Or = (int32_t)((spec >> 48) & 0xffff), Ir = (int32_t)((spec >> 32) & 0xffff);
    const int32_t Os = (int32_t)((spec >> 16) & 0xffff), Is = (int32_t)(spec & 0xffff);
    const int32_t Mrr = M.row_get(r, r), Mrs = M.row_get(r, s), Msr = M.row_get(s, r), Mss = M.row_get(s, s);
    long long tot = acc;
    if constexpr (kNP) {
        tot += np_cell_diag(g, Mrr, -Or - Ir - L) + np_cell(g, Mrs, Ir - Os) + np_cell(g, Msr, Or - Is) +
               np_cell_diag(g, Mss, Os + Is + L);
        return tot + np_block_terms(g, dout_r, din_r, sizes[r], dout_s, din_s, sizes[s], kout, kin, 1, nonempty);
    }
    const int32_t d_rr = -Or - Ir - L, d_rs = Ir - Os, d_sr = Or - Is, d_ss = Os + Is + L;
    const int32_t c0 = L32(Mrr), c1 = L32(Mrr + d_rr), c2 = L32(Mrs), c3 = L32(Mrs + d_rs);
    const int32_t c4 = L32(Msr), c5 = L32(Msr + d_sr), c6 = L32(Mss), c7 = L32(Mss + d_ss);
    // ce_fixed(v, d_in, d_out) - ce_fixed(v + d, d_in', d_out') of a changed cell, and
    // ce_delta of an unchanged one (its degrees change only)
    auto changed = [](int32_t x, int32_t d, int32_t lv, int32_t lvd, int32_t li, int32_t lo, int32_t li2,
                      int32_t lo2) { return (long long)x * (lv - li - lo) - (long long)(x + d) * (lvd - li2 - lo2); };
    auto unchanged = [](int32_t x, int32_t li, int32_t lo, int32_t li2, int32_t lo2) {
        return (long long)x * ((li2 - li) + (lo2 - lo));
    };
    // (r, r): present iff a neighbour lies in r or a self-loop exists; its change is never zero.
    if (Or | Ir | L) tot += changed(Mrr, d_rr, c0, c1, li_r, lo_r, li_r2, lo_r2);
    else tot += unchanged(Mrr, li_r, lo_r, li_r2, lo_r2);
    // (r, s): may be present with a zero change; then both loops count it.
    if (Os | Ir) tot += changed(Mrs, d_rs, c2, c3, li_s, lo_r, li_s2, lo_r2);
    if (d_rs == 0) tot += unchanged(Mrs, li_s, lo_r, li_s2, lo_r2);
    // (s, r)
    if (Or | Is) tot += changed(Msr, d_sr, c4, c5, li_r, lo_s, li_r2, lo_s2);
    if (d_sr == 0) tot += unchanged(Msr, li_r, lo_s, li_r2, lo_s2);
    // (s, s)
    if (Os | Is | L) tot += changed(Mss, d_ss, c6, c7, li_s, lo_s, li_s2, lo_s2);
    else tot += unchanged(Mss, li_s, lo_s, li_s2, lo_s2);
    // Unchanged cells of rows r, s and columns r, s (entropy.cpp:346-401).
    tot += ((long long)dout_r - Mrr - Mrs - sRo) * (lo_r2 - lo_r);
    tot += ((long long)dout_s - Msr - Mss - sSo) * (lo_s2 - lo_s);
    tot += ((long long)din_r - Mrr - Msr - sRi) * (li_r2 - li_r);
    tot += ((long long)din_s - Mrs - Mss - sSi) * (li_s2 - li_s);
    return tot;
}

// ------------------------------------------------------------------ Hastings correction
// entropy::hastings_correction (reference src/entropy.cpp:497-561) for the non-greedy
// acceptance.  Each term counts * weights / degrees is the same IEEE double as on the
// host; the two sums are accumulated exactly as integers of 2^-64 units (truncated), so
// they do not depend on the order in which the neighbour blocks are visited, and the
// ratio is taken of the sums converted back to double.
__device__ __forceinline__ __int128 to_fix64(double x) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0 || (bits >> 63)) return 0;
    const unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = e - 1075 + 64;
    if (sh >= 0) return (__int128)mant << sh;
    if (sh <= -64) return 0;
    return (__int128)(mant >> (-sh));
}
__device__ __forceinline__ double fix64_to_double(__int128 q) {
    const long long hi = (long long)(q >> 64);
    const unsigned long long lo = (unsigned long long)q;
    return __dadd_rn(__dmul_rn((double)hi, 18446744073709551616.0), (double)lo);
}
__device__ __forceinline__ __int128 warp_sum_i128(__int128 x) {
    unsigned long long lo = (unsigned long long)x;
    long long hi = (long long)(x >> 64);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long lo2 = __shfl_xor_sync(SBP_FULL_MASK, lo, o);
        const long long hi2 = __shfl_xor_sync(SBP_FULL_MASK, hi, o);
        const unsigned long long sum = lo + lo2;
        hi = hi + hi2 + (sum < lo ? 1 : 0);
        lo = sum;
    }
    return ((__int128)hi << 64) | (__int128)lo;
}

// One neighbour block's terms of the forward and backward proposal sums.
struct HastingsTerm {
    __int128 pf, pb;
};

// Sums over the group's neighbour hash (blocks b with out / in neighbour counts O, I of v)
// for moving v from r to s.  M: cells before the move; dtot(b): block total degree before
// the move.  kout counts v's out-edges including self-loops, kin its in-edges without them,
// L its self-loops (they count toward block r).
template <int kThreads, typename Acc, typename DTot>
__device__ double hastings_fixed(const Acc& M, DTot dtot, const int32_t* d_out, const int32_t* d_in, int32_t B,
                                 int32_t r, int32_t s, int32_t kout, int32_t kin, int32_t L, const int32_t* hk,
                                 const int32_t* hO, const int32_t* hI, int log2cap, long long (*red)[8]) {
    typedef Group<kThreads> G;
    const int t = G::rank();
    const int cap = 1 << log2cap;
    const double Bd = (double)B;
    // cells of the move's own rows / columns before and after (blockmodel_delta, finetune.cpp:201-235)
    int32_t Or = 0, Ir = 0, Os = 0, Is = 0, has_r = 0;
    for (int i = t; i < cap; i += kThreads) {
        const int32_t b = hk[i];
        if (b == r) {
            Or = hO[i];
            Ir = hI[i];
            has_r = 1;
        } else if (b == s) {
            Os = hO[i];
            Is = hI[i];
        }
    }
    {
        long long v[5] = {Or, Ir, Os, Is, has_r};
        G::template sum<5>(v, red);
        Or = (int32_t)v[0];
        Ir = (int32_t)v[1];
        Os = (int32_t)v[2];
        Is = (int32_t)v[3];
        has_r = (int32_t)v[4];
    }
    const int32_t Mrr = M.row_get(r, r), Mrs = M.row_get(r, s), Msr = M.row_get(s, r), Mss = M.row_get(s, s);
    const int32_t drr = -Or - Ir - L, drs = Ir - Os, dsr = Or - Is, dss = Os + Is + L;
    auto term = [&](int32_t b, int32_t cntO, int32_t cntI) {
        const int32_t cnt = cntO + cntI + (b == r ? L : 0);
        const double pw = (double)(M.row_get(s, b) + M.col_get(s, b)) + 1.0;
        const double bd = (double)dtot(b) + Bd;
        long long bw, nd;
        if (b == r) {
            bw = 2ll * (Mrr + drr);
            nd = ((long long)d_out[r] - kout) + ((long long)d_in[r] - kin) - (Mrr + drr);
        } else if (b == s) {
            bw = (long long)(Mrs + drs) + (Msr + dsr);
            nd = ((long long)d_out[s] + kout) + ((long long)d_in[s] + kin) - (Mss + dss);
        } else {
            bw = (long long)(M.row_get(r, b) - cntO) + (M.col_get(r, b) - cntI);
            nd = dtot(b);
        }
        HastingsTerm h;
        h.pf = to_fix64(__ddiv_rn(__dmul_rn((double)cnt, pw), bd));
        h.pb = to_fix64(__ddiv_rn(__dmul_rn((double)cnt, (double)bw + 1.0), (double)nd + Bd));
        return h;
    };
    __int128 pf = 0, pb = 0;
    for (int i = t; i < cap; i += kThreads) {
        const int32_t b = hk[i];
        if (b < 0) continue;
        const HastingsTerm h = term(b, hO[i], hI[i]);
        pf += h.pf;
        pb += h.pb;
    }
    if (t == 0 && L > 0 && !has_r) {  // block r reached only through self-loops
        const HastingsTerm h = term(r, 0, 0);
        pf += h.pf;
        pb += h.pb;
    }
    pf = warp_sum_i128(pf);
    pb = warp_sum_i128(pb);
    if (kThreads > 32) {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        __syncthreads();
        if (lane == 0) {
            red[w][0] = (long long)(unsigned long long)pf;
            red[w][1] = (long long)(pf >> 64);
            red[w][2] = (long long)(unsigned long long)pb;
            red[w][3] = (long long)(pb >> 64);
        }
        __syncthreads();
        pf = 0;
        pb = 0;
        for (int i = 0; i < kThreads / 32; ++i) {
            pf += ((__int128)red[i][1] << 64) | (__int128)(unsigned long long)red[i][0];
            pb += ((__int128)red[i][3] << 64) | (__int128)(unsigned long long)red[i][2];
        }
        __syncthreads();
    }
    return __ddiv_rn(fix64_to_double(pb), fix64_to_double(pf));
}

// finetune::accept (reference src/finetune.cpp:22-32): greedy takes dS < 0; otherwise the
// uniform draw u = w3 / 2^32 of the proposal's counter against min(1, e^(-3 dS) H).
__device__ __forceinline__ bool accept_move(long long dS_fixed, double H, bool greedy, uint32_t w3) {
    if (greedy) return dS_fixed < 0;
    const double u = (double)w3 * (1.0 / 4294967296.0);
    double p = exp(-3.0 * fixed_to_double(dS_fixed)) * H;
    p = p >= 1.0 ? 1.0 : p;
    return u <= p;
}

// ------------------------------------------------------------------ merge delta-MDL
// entropy::block_merge_delta_mdl for merging r into s over the static CSR/CSC.
template <int kThreads>
__device__ long long merge_delta_fixed_csr(const DevGraph& g, const DevBM& bm, int32_t r, int32_t s,
                                        long long (*red)[8]) {
    typedef Group<kThreads> G;
    const int t = G::rank();
    const LogTab Lq{g.Lq, g.E + 1};
    const int32_t dout_r = bm.d_out[r], din_r = bm.d_in[r], dout_s = bm.d_out[s], din_s = bm.d_in[s];
    const int32_t dout_s2 = dout_s + dout_r, din_s2 = din_s + din_r;
    long long acc = 0, sRow = 0, sCol = 0;
    const int32_t ro0 = bm.row_off[r], ro1 = bm.row_off[r + 1];
    for (int32_t j = ro0 + t; j < ro1; j += kThreads) {
        const int32_t c = bm.row_col[j], m = bm.row_cnt[j], dinc = bm.d_in[c];
        acc += ce_fixed(Lq, m, dinc, dout_r);
        if (c != r && c != s) {
            const int32_t Msc = csr_get(bm.row_off, bm.row_col, bm.row_cnt, s, c);
            acc += ce_fixed(Lq, Msc, dinc, dout_s) - ce_fixed(Lq, Msc + m, dinc, dout_s2);
            sRow += Msc;
        }
    }
    const int32_t co0 = bm.col_off[r], co1 = bm.col_off[r + 1];
    for (int32_t j = co0 + t; j < co1; j += kThreads) {
        const int32_t x = bm.col_row[j], m = bm.col_cnt[j];
        if (x == r) continue;
        const int32_t doutx = bm.d_out[x];
        acc += ce_fixed(Lq, m, din_r, doutx);
        if (x != s) {
            const int32_t Mxs = csr_get(bm.col_off, bm.col_row, bm.col_cnt, s, x);
            acc += ce_fixed(Lq, Mxs, din_s, doutx) - ce_fixed(Lq, Mxs + m, din_s2, doutx);
            sCol += Mxs;
        }
    }
    {
        long long v[3] = {acc, sRow, sCol};
        G::template sum<3>(v, red);
        acc = v[0];
        sRow = v[1];
        sCol = v[2];
    }
    const int32_t Mrr = csr_get(bm.row_off, bm.row_col, bm.row_cnt, r, r);
    const int32_t Mrs = csr_get(bm.row_off, bm.row_col, bm.row_cnt, r, s);
    const int32_t Msr = csr_get(bm.row_off, bm.row_col, bm.row_cnt, s, r);
    const int32_t Mss = csr_get(bm.row_off, bm.row_col, bm.row_cnt, s, s);
    const int32_t dss = Mrr + Mrs + Msr;
    long long tot = acc;
    if (dss > 0) tot += ce_fixed(Lq, Mss, din_s, dout_s) - ce_fixed(Lq, Mss + dss, din_s2, dout_s2);
    else tot += ce_delta(Lq, Mss, din_s, dout_s, din_s2, dout_s2);
    tot += ((long long)dout_s - Msr - Mss - sRow) * (Lx(Lq, dout_s2) - Lx(Lq, dout_s));
    tot += ((long long)din_s - Mrs - Mss - sCol) * (Lx(Lq, din_s2) - Lx(Lq, din_s));
    return tot;
}

// nonparametric::block_merge_delta_mdl (reference src/entropy.cpp:1198-1223) for merging r
// into s over the static CSR/CSC: every cell of row and column r empties, row / column
// cells of third blocks add into row / column s, and (r,r), (r,s), (s,r) into (s,s).  Zero
// when either block is empty (:1203-1204).
template <int kThreads>
__device__ long long np_merge_delta_csr(const DevGraph& g, const DevBM& bm, int32_t r, int32_t s, int32_t nonempty,
                                        long long (*red)[8]) {
    typedef Group<kThreads> G;
    const int t = G::rank();
    const int32_t size_r = bm.sizes[r], size_s = bm.sizes[s];
    if (r == s || size_r == 0 || size_s == 0) return 0;
    long long acc = 0;
    const int32_t ro0 = bm.row_off[r], ro1 = bm.row_off[r + 1];
    for (int32_t j = ro0 + t; j < ro1; j += kThreads) {
        const int32_t c = bm.row_col[j], m = bm.row_cnt[j];
        acc += c == r ? np_cell_diag(g, m, -m) : np_lg(g, m);  // the cell empties
        if (c != r && c != s) acc += np_cell(g, csr_get(bm.row_off, bm.row_col, bm.row_cnt, s, c), m);
    }
    const int32_t co0 = bm.col_off[r], co1 = bm.col_off[r + 1];
    for (int32_t j = co0 + t; j < co1; j += kThreads) {
        const int32_t x = bm.col_row[j], m = bm.col_cnt[j];
        if (x == r) continue;
        acc += np_lg(g, m);
        if (x != s) acc += np_cell(g, csr_get(bm.col_off, bm.col_row, bm.col_cnt, s, x), m);
    }
    {
        long long v[1] = {acc};
        G::template sum<1>(v, red);
        acc = v[0];
    }
    const int32_t Mrr = csr_get(bm.row_off, bm.row_col, bm.row_cnt, r, r);
    const int32_t Mrs = csr_get(bm.row_off, bm.row_col, bm.row_cnt, r, s);
    const int32_t Msr = csr_get(bm.row_off, bm.row_col, bm.row_cnt, s, r);
    const int32_t Mss = csr_get(bm.row_off, bm.row_col, bm.row_cnt, s, s);
    acc += np_cell_diag(g, Mss, Mrr + Mrs + Msr);
    const int32_t dout_r = bm.d_out[r], din_r = bm.d_in[r];
    return acc + np_block_terms(g, dout_r, din_r, size_r, bm.d_out[s], bm.d_in[s], size_s, dout_r, din_r, size_r,
                                nonempty);
}

}  // namespace sbp

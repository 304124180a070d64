// Nonparametric description length on the device: entropy::nonparametric (reference
// src/entropy.cpp:617-1225, include/entropy.hpp:101-190) for a directed graph without
// degree correction.
//
// Terms, in units of 2^-24 as int64 so that every sum is exact and order-free:
//   * eterm_exact(w) = -lgamma(w + 1): the table LG[x] = round(lgamma(x + 1) * 2^24);
//   * vterm_exact(d_out, d_in, size) = (d_out + d_in) * fastlog(size): the exact fastlog
//     table Lq (logf of an integer is a multiple of 2^-24);
//   * get_delta_partition_dl: -lgamma(size + 1) from LG, plus lbinom(N - 1, B' - 1);
//   * get_delta_edges_dl: lbinom(B'^2 + E - 1, E),
// where B' is the number of non-empty blocks.  The two B'-dependent terms change only when
// a move empties or fills a block; Dm[b] (Dp[b]) holds the rounded change of their sum
// when B' goes from b to b - 1 (b + 1), computed on the host in the reference's double
// arithmetic.  A vertex move's delta is then
//   sum over changed cells (LG[M] - LG[M + change])          (entries_dS, :782-809)
// + the vterm changes of blocks r and s                      (virtual_move_sparse, :822-889)
// + LG[size_r] + LG[size_s] - LG[size_r - w] - LG[size_s + w] (get_delta_partition_dl)
// + Dm / Dp when the move empties r or fills s,
// with w = 1 for a vertex and w = size_r for a block merge (:1198-1223).
#pragma once

#include "common.cuh"

namespace sbp {

// lgamma(x + 1) in units of 2^-24, clamped to the table.
__device__ __forceinline__ long long np_lg(const DevGraph& g, long long x) {
    x = x < 0 ? 0 : (x > g.nlq ? g.nlq : x);
    return __ldg(g.LG + x);
}
// fastlog(x) in units of 2^-24 over the block-size range.
__device__ __forceinline__ long long np_log(const DevGraph& g, long long x) {
    x = x < 0 ? 0 : (x > g.nlq ? g.nlq : x);
    return (long long)__ldg(g.Lq + x);
}
// vterm_exact (include/entropy.hpp:117-133): (d_out + d_in) log w, or d_out log w for an
// undirected graph; degree-corrected: lgamma(d_out + 1) + lgamma(d_in + 1), or the first
// alone when undirected, whatever w.
__device__ __forceinline__ long long np_vterm(const DevGraph& g, long long dout, long long din, long long w) {
    if (g.dc) return np_lg(g, dout) + (g.np_und ? 0 : np_lg(g, din));
    return w == 0 ? 0 : (g.np_und ? dout : dout + din) * np_log(g, w);
}
// One changed cell of entries_dS: eterm(M + d) - eterm(M), off the diagonal.
__device__ __forceinline__ long long np_cell(const DevGraph& g, long long m, long long d) {
    return np_lg(g, m) - np_lg(g, m + d);
}
// The same for a diagonal cell: eterm_exact(r, r, w) carries -w log 2 more when the graph
// is undirected (include/entropy.hpp:102-111).
__device__ __forceinline__ long long np_cell_diag(const DevGraph& g, long long m, long long d) {
    return np_cell(g, m, d) - (g.np_und ? d * g.ln2q : 0);
}
// The block, partition and edge-count terms of moving `w` vertices with kout / kin edges
// from r to s; nonempty = the current number of non-empty blocks.  The terms that depend
// on it are left out when with_count is false (the caller adds them).
__device__ __forceinline__ long long np_block_terms(const DevGraph& g, long long dout_r, long long din_r,
                                                    long long size_r, long long dout_s, long long din_s,
                                                    long long size_s, long long kout, long long kin, long long w,
                                                    int32_t nonempty, bool with_count = true) {
    long long t = np_vterm(g, dout_r - kout, din_r - kin, size_r - w) - np_vterm(g, dout_r, din_r, size_r);
    t += np_vterm(g, dout_s + kout, din_s + kin, size_s + w) - np_vterm(g, dout_s, din_s, size_s);
    t += np_lg(g, size_r) + np_lg(g, size_s) - np_lg(g, size_r - w) - np_lg(g, size_s + w);
    if (with_count) {
        const int dB = (size_r == w ? -1 : 0) + (size_s == 0 ? 1 : 0);
        const int32_t b = nonempty < 0 ? 0 : (nonempty > g.N + 1 ? g.N + 1 : nonempty);
        if (dB < 0) t += __ldg(g.Dm + b);
        else if (dB > 0) t += __ldg(g.Dp + b);
    }
    return t;
}
// Does moving w vertices from a block of size_r into one of size_s change the number of
// non-empty blocks?
__device__ __forceinline__ int np_count_change(long long size_r, long long size_s, long long w) {
    return (size_r == w ? -1 : 0) + (size_s == 0 ? 1 : 0);
}

}  // namespace sbp

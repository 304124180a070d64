/*
 * CPU oracle for the SBP hot path -- TEST INFRASTRUCTURE ONLY (see sbp_oracle.h).
 *
 * A restatement of vtsynergy/SBP's serial semantics with ordered maps (so every
 * iteration is in ascending block order) and the canonical seeded proposal stream.
 * Citations are path:line inside the reference project.
 *
 * Canonical stream (shared with the device implementation, which has its own code):
 *   key   = (seed & 0xffffffff, seed >> 32)
 *   ctr   = (c0, c1, c2, c3); outputs w[0..3] of Philox4x32-10.
 *   Gibbs vertex proposal : ctr = (vertex, iteration, step, DOM_GIBBS)
 *   MH vertex proposal    : ctr = (vertex, iteration, step, DOM_MH)
 *   merge proposal i      : ctr = (block, 0, step, DOM_MERGE | i << 8)
 *   shuffles              : ctr = (position, iteration, step, DOM_SHUFFLE_*)
 *   random sample         : shuffle with ctr = (position, 0, 0, DOM_SAMPLE = 6)
 *   extend, random block  : ctr = (vertex, 0, 0, DOM_EXTEND = 7), block = u32_below(w[0], B)
 *   finetune_assignment   : MH draws with step = 0xffffffff
 *   reattach, random block: ctr = (vertex, 0, 0, DOM_REATTACH = 10), block = u32_below(w[0], B)
 *   snowball samplers     : the k-th draw of a run, ctr = (k, 0, 0, DOM_SNOWBALL = 11),
 *                           random_integer(lo, hi) = lo + u64_below(w[0], w[1], hi - lo + 1)
 *   top-down split size   : ctr = (cluster, proposal, step, DOM_SPLIT_SIZE = 8),
 *                           size = lo + u64_below(w[0], w[1], hi - lo + 1)
 *   top-down split side   : ctr = (vertex, proposal, step, DOM_SPLIT_SIDE = 9),
 *                           side 0 iff w[0] * n < size * 2^32
 *   snowball splits       : the k-th draw of (cluster, proposal, step),
 *                           ctr = (cluster, proposal | k << 8, step, DOM_SPLIT_SNOWBALL = 12)
 *   u32_below(w, n) = (w * n) >> 32;  u64_below(hi, lo, n) = ((hi:lo) * n) >> 64.
 *   Multinomials over a block's neighbour weights enumerate the row part (ascending
 *   column) and then the column part (ascending row), the same concatenation the
 *   reference builds in DictTransposeMatrix::neighbors_weights
 *   (dict_transpose_matrix.cpp:176-188) and in propose_new_block's concatenated
 *   out/in lists (common.cpp:141-142).
 */
#include "sbp_oracle.h"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <queue>
#include <tuple>
#include <set>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum : uint32_t {
    DOM_GIBBS = 1, DOM_MH = 2, DOM_MERGE = 3, DOM_SHUFFLE_HDV = 4, DOM_SHUFFLE_ALL = 5, DOM_SAMPLE = 6,
    DOM_EXTEND = 7, DOM_SPLIT_SIZE = 8, DOM_SPLIT_SIDE = 9, DOM_REATTACH = 10, DOM_SNOWBALL = 11,
    DOM_SPLIT_SNOWBALL = 12,
};

// ---------------------------------------------------------------- Philox4x32-10
inline void philox_round(uint32_t c[4], const uint32_t k[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k[0];
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k[1];
    const uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
}

inline void philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    uint32_t k[2] = {key[0], key[1]};
    for (int r = 0; r < 10; ++r) {
        if (r) { k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u; }
        philox_round(c, k);
    }
    out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
}

inline void draw(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t w[4]) {
    const uint32_t ctr[4] = {c0, c1, c2, c3};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    philox(ctr, key, w);
}

inline uint32_t u32_below(uint32_t w, uint32_t n) { return (uint32_t)(((uint64_t)w * n) >> 32); }
inline uint64_t u64_below(uint32_t hi, uint32_t lo, uint64_t n) {
    const unsigned __int128 x = (unsigned __int128)((((uint64_t)hi) << 32) | lo) * n;
    return (uint64_t)(x >> 64);
}
/* common::propose_random_block (common.cpp:200-209): uniform over [0, B-2], skip current. */
inline int64_t random_block(int64_t current, int64_t B, uint32_t w) {
    int64_t x = (int64_t)u32_below(w, (uint32_t)(B - 1));
    if (x >= current) x++;
    return x;
}

}  // namespace

// ---------------------------------------------------------------- graph
struct ora_graph {
    int64_t N = 0, E = 0;
    // Graph::num_edges (graph.hpp:99), the count every description length uses: the stored
    // directed edges, or half of them for an undirected edge list (graph.cpp:145-147)
    int64_t Em = 0;
    // args.undirected for the nonparametric entropy (entropy.hpp:102-133, entropy.cpp:745):
    // diagonal cells carry -w log 2, a block's vertex term counts its out-degree only, and
    // the edge count is spread over B (B + 1) / 2 block pairs
    bool und = false;
    // args.degreecorrected (entropy.hpp:117-133, entropy.cpp:617-764): the degree-corrected
    // vertex terms and prior, for the description length and vertex-move deltas
    bool dc = false;
    std::vector<std::vector<int32_t>> out, in, inns;  // inns = in-neighbours without self
    std::vector<int32_t> selfcnt;
    std::vector<double> Ld;     // fastlog table: logf((float)x) (fastlog.hpp:21-30)
    std::vector<int64_t> Lq;    // the same values in units of 2^-24 (exact)
    std::vector<int64_t> LG;    // lgamma(x + 1) rounded to units of 2^-24 (nonparametric terms)
};

namespace {

const double kFix = 16777216.0;  // 2^24
const double kInvFix = 1.0 / 16777216.0;

void build_log_tables(ora_graph* g) {
    const int64_t n = std::max(g->E, g->N) + 2;  // edge counts, degrees and block sizes
    g->Ld.resize(n);
    g->Lq.resize(n);
    g->LG.resize(n);
    g->Ld[0] = 0.0;
    g->Lq[0] = 0;
    for (int64_t x = 1; x < n; ++x) {
        const double v = (double)logf((float)x);
        g->Ld[x] = v;
        g->Lq[x] = (int64_t)(v * kFix);
    }
    for (int64_t x = 0; x < n; ++x) g->LG[x] = llrint(lgamma((double)(x + 1)) * kFix);
}

}  // namespace

extern "C" void ora_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox(ctr, key, out);
}

extern "C" ora_graph* ora_graph_create(int64_t N, int64_t E, const int32_t* src, const int32_t* dst) {
    auto* g = new ora_graph();
    g->N = N;
    g->E = E;
    g->Em = E;
    g->out.assign(N, {});
    g->in.assign(N, {});
    g->inns.assign(N, {});
    g->selfcnt.assign(N, 0);
    // Graph::add_edge / utils::insert (graph.cpp:10-18): append in input order.
    for (int64_t e = 0; e < E; ++e) {
        const int32_t u = src[e], v = dst[e];
        g->out[u].push_back(v);
        g->in[v].push_back(u);
        if (u == v) g->selfcnt[u]++;
        else g->inns[v].push_back(u);
    }
    build_log_tables(g);
    return g;
}

extern "C" void ora_graph_destroy(ora_graph* g) { delete g; }

// ---------------------------------------------------------------- blockmodel
struct ora_bm {
    const ora_graph* g = nullptr;
    int64_t B = 0;
    std::vector<int32_t> asg;
    std::vector<int64_t> dout, din, dtot, sizes;
    std::vector<std::map<int32_t, int64_t>> row, col;  // matrix and transpose
    double entropy = DBL_MAX;
    int64_t num_blocks_to_merge = 0;
    int64_t nonempty = 0;  // Blockmodel::_num_nonempty_blocks
    bool empty = false;

    int64_t get(int64_t r, int64_t c) const {
        auto it = row[r].find((int32_t)c);
        return it == row[r].end() ? 0 : it->second;
    }
    /* DictTransposeMatrix::add + add_transpose; erase on zero as sub() and
     * update_edge_counts() do (dict_transpose_matrix.cpp:3-16, 225-235, 430-446). */
    void add(int64_t r, int64_t c, int64_t v) {
        int64_t& a = row[r][(int32_t)c];
        a += v;
        int64_t& b = col[c][(int32_t)r];
        b += v;
        if (a == 0) {
            row[r].erase((int32_t)c);
            col[c].erase((int32_t)r);
        }
    }
};

namespace {

/* Blockmodel::initialize_edge_counts (blockmodel.cpp:193-276). */
void build(ora_bm* bm) {
    const ora_graph* g = bm->g;
    const int64_t B = bm->B;
    bm->dout.assign(B, 0);
    bm->din.assign(B, 0);
    bm->dtot.assign(B, 0);
    bm->sizes.assign(B, 0);
    bm->row.assign(B, {});
    bm->col.assign(B, {});
    for (int64_t v = 0; v < g->N; ++v) {
        const int32_t b = bm->asg[v];
        bm->sizes[b]++;
        for (int32_t u : g->out[v]) {
            bm->row[b][bm->asg[u]] += 1;
            bm->dout[b] += 1;
            bm->dtot[b] += 1;
        }
        for (int32_t w : g->in[v]) {
            const int32_t nb = bm->asg[w];
            bm->col[b][nb] += 1;
            bm->din[b] += 1;
            if (b != nb) bm->dtot[b] += 1;
        }
    }
    bm->nonempty = 0;  // blockmodel.cpp:194, :231
    for (int64_t b = 0; b < B; ++b) bm->nonempty += bm->sizes[b] > 0;
}

/* common::cell_entropy (common.hpp:39-50) in the reference's double arithmetic. */
inline double ce_double(const ora_graph* g, int64_t v, int64_t din, int64_t dout) {
    if (v == 0) return 0.0;
    return (double)v * (g->Ld[v] - (g->Ld[din] + g->Ld[dout]));
}
/* The same term in units of 2^-24: every fastlog value is a multiple of 2^-24. */
inline int64_t ce_fixed(const ora_graph* g, int64_t v, int64_t din, int64_t dout) {
    if (v == 0) return 0;
    return v * (g->Lq[v] - g->Lq[din] - g->Lq[dout]);
}

typedef std::map<std::pair<int32_t, int32_t>, int64_t> DeltaMap;  // key presence matters (H3)

inline int64_t delta_get(const DeltaMap& d, int64_t r, int64_t c) {
    auto it = d.find({(int32_t)r, (int32_t)c});
    return it == d.end() ? 0 : it->second;
}

struct VertexInfo {
    int64_t kout, kin, selfw;
};

inline VertexInfo vinfo(const ora_graph* g, int64_t v) {
    return {(int64_t)g->out[v].size(), (int64_t)g->inns[v].size(), g->selfcnt[v] > 0 ? 1 : 0};
}

/* finetune::blockmodel_delta (finetune.cpp:201-235) with out_edges = all out-neighbours
 * and in_edges = in-neighbours without the vertex itself (finetune.cpp:880-881). */
DeltaMap vertex_delta(const ora_bm* bm, int64_t v, int64_t s) {
    const ora_graph* g = bm->g;
    const int64_t r = bm->asg[v];
    DeltaMap d;
    for (int32_t u : g->out[v]) {
        const int32_t ob = bm->asg[u];
        if (u == v) d[{(int32_t)s, (int32_t)s}] += 1;
        else d[{(int32_t)s, ob}] += 1;
        d[{(int32_t)r, ob}] -= 1;
    }
    for (int32_t w : g->inns[v]) {
        const int32_t ib = bm->asg[w];
        d[{ib, (int32_t)s}] += 1;
        d[{ib, (int32_t)r}] -= 1;
    }
    return d;
}

/* block_merge::blockmodel_delta (block_merge.cpp:14-38). */
DeltaMap merge_delta(const ora_bm* bm, int64_t r, int64_t s) {
    DeltaMap d;
    for (const auto& e : bm->row[r]) {
        const int32_t c = e.first;
        const int64_t v = e.second;
        if (c == r || c == s) d[{(int32_t)s, (int32_t)s}] += v;
        else d[{(int32_t)s, c}] += v;
        d[{(int32_t)r, c}] -= v;
    }
    for (const auto& e : bm->col[r]) {
        const int32_t x = e.first;
        if (x == r) continue;
        const int64_t v = e.second;
        if (x == s) d[{(int32_t)s, (int32_t)s}] += v;
        else d[{x, (int32_t)s}] += v;
        d[{x, (int32_t)r}] -= v;
    }
    return d;
}

/* entropy::delta_mdl(Blockmodel, Delta, proposal) (entropy.cpp:298-403). */
template <typename Acc, typename CE>
Acc delta_mdl_generic(const ora_bm* bm, int64_t v, int64_t s, const DeltaMap& d, CE ce) {
    const ora_graph* g = bm->g;
    const int64_t r = bm->asg[v];
    const VertexInfo vi = vinfo(g, v);
    auto gin = [&](int64_t i) -> int64_t {
        int64_t x = bm->din[i];
        if (i == r) x -= (vi.kin + vi.selfw);
        else if (i == s) x += (vi.kin + vi.selfw);
        return x;
    };
    auto gout = [&](int64_t i) -> int64_t {
        int64_t x = bm->dout[i];
        if (i == r) x -= vi.kout;
        else if (i == s) x += vi.kout;
        return x;
    };
    Acc dS = 0;
    for (const auto& e : d) {
        const int64_t row = e.first.first, col = e.first.second, ch = e.second;
        const int64_t m = bm->get(row, col);
        dS += ce(g, m, bm->din[col], bm->dout[row]);
        dS -= ce(g, m + ch, gin(col), gout(row));
    }
    for (const auto& e : bm->row[r]) {
        const int64_t col = e.first, m = e.second;
        if (delta_get(d, r, col) != 0) continue;
        dS += ce(g, m, bm->din[col], bm->dout[r]);
        dS -= ce(g, m, gin(col), gout(r));
    }
    for (const auto& e : bm->row[s]) {
        const int64_t col = e.first, m = e.second;
        if (delta_get(d, s, col) != 0) continue;
        dS += ce(g, m, bm->din[col], bm->dout[s]);
        dS -= ce(g, m, gin(col), gout(s));
    }
    for (const auto& e : bm->col[r]) {
        const int64_t row = e.first, m = e.second;
        if (delta_get(d, row, r) != 0 || row == r || row == s) continue;
        dS += ce(g, m, bm->din[r], bm->dout[row]);
        dS -= ce(g, m, gin(r), gout(row));
    }
    for (const auto& e : bm->col[s]) {
        const int64_t row = e.first, m = e.second;
        if (delta_get(d, row, s) != 0 || row == r || row == s) continue;
        dS += ce(g, m, bm->din[s], bm->dout[row]);
        dS -= ce(g, m, gin(s), gout(row));
    }
    return dS;
}

/* entropy::block_merge_delta_mdl (entropy.cpp:129-182). */
template <typename Acc, typename CE>
Acc merge_delta_mdl_generic(const ora_bm* bm, int64_t r, int64_t s, const DeltaMap& d, CE ce) {
    const ora_graph* g = bm->g;
    int64_t kout = 0, kin = 0;  // block_merge.cpp:65-69 (std::accumulate of row / column r)
    for (const auto& e : bm->row[r]) kout += e.second;
    for (const auto& e : bm->col[r]) kin += e.second;
    auto gin = [&](int64_t i) -> int64_t {
        int64_t x = bm->din[i];
        if (i == r) x -= kin;
        else if (i == s) x += kin;
        return x;
    };
    auto gout = [&](int64_t i) -> int64_t {
        int64_t x = bm->dout[i];
        if (i == r) x -= kout;
        else if (i == s) x += kout;
        return x;
    };
    Acc dS = 0;
    for (const auto& e : d) {
        const int64_t row = e.first.first, col = e.first.second, ch = e.second;
        const int64_t m = bm->get(row, col);
        dS += ce(g, m, bm->din[col], bm->dout[row]);
        if (row == r || col == r) continue;
        dS -= ce(g, m + ch, gin(col), gout(row));
    }
    for (const auto& e : bm->row[s]) {
        const int64_t col = e.first, m = e.second;
        if (delta_get(d, s, col) != 0) continue;
        dS += ce(g, m, bm->din[col], bm->dout[s]);
        dS -= ce(g, m, gin(col), gout(s));
    }
    for (const auto& e : bm->col[s]) {
        const int64_t row = e.first, m = e.second;
        if (delta_get(d, row, s) != 0 || row == r || row == s) continue;
        dS += ce(g, m, bm->din[s], bm->dout[row]);
        dS -= ce(g, m, gin(s), gout(row));
    }
    return dS;
}

int64_t merge_dS_fixed(const ora_bm* bm, int64_t r, int64_t s) {
    const DeltaMap d = merge_delta(bm, r, s);
    return merge_delta_mdl_generic<int64_t>(bm, r, s, d, ce_fixed);
}

// ---------------------------------------------------------------- nonparametric entropy
/* entropy::nonparametric (entropy.cpp:617-1225, entropy.hpp:101-190) for a directed graph
 * without degree correction (args.undirected = args.degreecorrected = false).
 * fastlgamma(x) = lgamma((double)x) (fastlgamma.hpp:19-27, fastlgamma.cpp:11-20);
 * fastlog(x) = logf(x) (fastlog.hpp:21-30).  Canonical arithmetic, shared with the device:
 * every lgamma(x + 1) term is rounded to units of 2^-24 (LG), the vterm products use the
 * exact fastlog table, and the partition / edge-count terms that depend on the number of
 * non-empty blocks enter as one rounded value per change of that number. */

/* fastlbinom (entropy.hpp:144-148). */
inline double np_lbinom(int64_t N, int64_t k) {
    if (N == 0 || k == 0 || k > N) return 0.0;
    return (lgamma((double)(N + 1)) - lgamma((double)(k + 1))) - lgamma((double)(N - k + 1));
}
/* get_edges_dl (entropy.cpp:745-749): NB = B * B, or B (B + 1) / 2 when undirected. */
inline double np_edges_dl(int64_t b, int64_t E, bool und = false) {
    return np_lbinom((und ? b * (b + 1) / 2 : b * b) + E - 1, E);
}
/* log 2 in units of 2^-24, rounded: the undirected diagonal term w log 2 of eterm_exact
 * (entropy.hpp:102-111) is w times this constant in the canonical arithmetic. */
const int64_t kLn2Fix = llrint(0.69314718055994530942 * 16777216.0);
/* eterm_exact(r, s, M + d) - eterm_exact(r, s, M), canonical. */
inline int64_t np_cell(const ora_graph* g, bool diag, int64_t m, int64_t d) {
    return g->LG[m] - g->LG[m + d] - (g->und && diag ? d * kLn2Fix : 0);
}
/* Change of lbinom(N - 1, B - 1) (get_delta_partition_dl, entropy.cpp:933-940) plus
 * get_delta_edges_dl (:1111-1143) when the non-empty block count goes from b to b + dB. */
inline int64_t np_dl_step(const ora_graph* g, int64_t b, int dB) {
    const double part = np_lbinom(g->N - 1, b + dB - 1) - np_lbinom(g->N - 1, b - 1);
    const double edges = np_edges_dl(b + dB, g->Em, g->und) - np_edges_dl(b, g->Em, g->und);
    return llrint((part + edges) * kFix);
}
/* vterm_exact (entropy.hpp:117-133): (d_out + d_in) log w, or d_out log w when
 * undirected; degree-corrected: lgamma(d_out + 1) + lgamma(d_in + 1), or the first alone
 * when undirected, whatever the block size. */
inline int64_t np_vterm(const ora_graph* g, int64_t dout, int64_t din, int64_t w) {
    if (g->dc) return g->LG[dout] + (g->und ? 0 : g->LG[din]);
    return w == 0 ? 0 : (g->und ? dout : dout + din) * g->Lq[w];
}

// ---------------------------------------------------------------- degree correction
/* The dilogarithm Li2(z) = sum z^k / k^2 (|z| <= 1/2), continued by Euler's reflection
 * Li2(z) = pi^2/6 - log(z) log(1 - z) - Li2(1 - z) above 1/2 and by Landen's identity
 * Li2(z) = -Li2(z / (z - 1)) - log^2(1 - z) / 2 below 0. */
double dc_li2(double z) {
    if (z < 0.0) {
        const double l = log1p(-z);
        return -dc_li2(z / (z - 1.0)) - 0.5 * l * l;
    }
    if (z >= 1.0) return M_PI * M_PI / 6.0;  // Li2(1); the argument here never exceeds 1
    if (z > 0.5) return M_PI * M_PI / 6.0 - log(z) * log1p(-z) - dc_li2(1.0 - z);
    double sum = 0.0, p = z;
    for (int k = 1; k <= 200; ++k) {
        const double t = p / ((double)k * (double)k);
        sum += t;
        if (t <= 1e-18 * sum) break;
        p *= z;
    }
    return sum;
}
/* spence(x) = -integral_1^x log(t) / (t - 1) dt = Li2(1 - x) (spence.hpp:9-22, the
 * Cephes function the reference carries in spence.cpp); here for x = e^-v, with
 * 1 - e^-v formed as -expm1(-v). */
inline double dc_spence_exp(double v) { return dc_li2(-expm1(-v)); }
/* get_v (entropy.cpp:677-686): the fixed point v = u sqrt(spence(e^-v)), to 1e-8. */
double dc_get_v(double u, double epsilon = 1e-8) {
    double v = u, delta = 1.0;
    for (int it = 0; delta > epsilon && it < 100000; ++it) {
        const double nv = u * sqrt(dc_spence_exp(v));
        delta = fabs(nv - v);
        v = nv;
    }
    return v;
}
/* log_q (entropy.cpp:688-707): log of the number of partitions of n into at most k parts,
 * by the small-k form lbinom(n - 1, k - 1) - lgamma(k + 1) when k < n^(1/4) and by the
 * Szekeres asymptotic otherwise. */
double dc_log_q(int64_t n, int64_t k) {
    if (n <= 0 || k < 1) return 0.0;
    if (k > n) k = n;
    if ((double)k < pow((double)n, 0.25)) return np_lbinom(n - 1, k - 1) - lgamma((double)(k + 1));
    const double u = (double)k / sqrt((double)n);
    const double v = dc_get_v(u);
    const double lf = log(v) - log1p(-exp(-v) * (1 + u * u / 2)) / 2 - log(2.0) * 3 / 2. - log(u) - log(M_PI);
    const double gg = 2 * v / u - u * log1p(-exp(-v));
    return lf - log((double)n) + sqrt((double)n) * gg;
}
/* A vertex's degrees as the degree terms read them: the sizes of its neighbour lists,
 * self-loops in both (get_deg_entropy, entropy.cpp:620-624; blockmodel.cpp:234-235). */
inline int64_t dc_kin(const ora_graph* g, int64_t v) { return (int64_t)g->in[v].size(); }
inline int64_t dc_kout(const ora_graph* g, int64_t v) { return (int64_t)g->out[v].size(); }
/* The per-block in- and out-degree histograms, as Blockmodel's constructor builds them
 * (blockmodel.cpp:209-235), for the current assignment. */
struct DcHist {
    std::vector<std::map<int64_t, int64_t>> in, out;
};
DcHist dc_hist(const ora_bm* bm) {
    DcHist h;
    h.in.resize(bm->B);
    h.out.resize(bm->B);
    for (int64_t v = 0; v < bm->g->N; ++v) {
        h.in[bm->asg[v]][dc_kin(bm->g, v)]++;
        h.out[bm->asg[v]][dc_kout(bm->g, v)]++;
    }
    return h;
}
inline int64_t dc_count(const std::map<int64_t, int64_t>& m, int64_t k) {
    const auto it = m.find(k);
    return it == m.end() ? 0 : it->second;
}
inline int64_t dc_fix(double x) { return llrint(x * kFix); }
/* sum over vertices of get_deg_entropy (entropy.cpp:620-624, :644-655), canonical. */
int64_t dc_deg_entropy_fixed(const ora_graph* g) {
    int64_t t = 0;
    for (int64_t v = 0; v < g->N; ++v) t -= g->LG[dc_kin(g, v)] + g->LG[dc_kout(g, v)];
    return t;
}
double dc_deg_entropy_literal(const ora_graph* g) {
    double t = 0.0;
    for (int64_t v = 0; v < g->N; ++v)
        t += -lgamma((double)(dc_kin(g, v) + 1)) - lgamma((double)(dc_kout(g, v) + 1));
    return t;
}
/* get_deg_dl_dist (entropy.cpp:709-743): per block log_q(d_out, size) + log_q(d_in, size),
 * minus lgamma(count + 1) over the in-degree (directed only) and out-degree histograms,
 * plus lgamma(size + 1) twice (once when undirected).  Canonical: every log_q term and
 * lgamma term rounded to 2^-24, then summed exactly. */
int64_t dc_deg_dl_fixed(const ora_bm* bm, const DcHist& h) {
    const ora_graph* g = bm->g;
    int64_t t = 0;
    for (int64_t b = 0; b < bm->B; ++b) {
        t += dc_fix(dc_log_q(bm->dout[b], bm->sizes[b])) + dc_fix(dc_log_q(bm->din[b], bm->sizes[b]));
        int64_t total = 0;
        if (!g->und)
            for (const auto& e : h.in[b]) t -= g->LG[e.second];
        for (const auto& e : h.out[b]) {
            t -= g->LG[e.second];
            total += e.second;
        }
        t += (g->und ? 1 : 2) * g->LG[total];
    }
    return t;
}
double dc_deg_dl_literal(const ora_bm* bm, const DcHist& h) {
    const ora_graph* g = bm->g;
    double S = 0.0;
    for (int64_t b = 0; b < bm->B; ++b) {
        S += dc_log_q(bm->dout[b], bm->sizes[b]);
        S += dc_log_q(bm->din[b], bm->sizes[b]);
        int64_t total = 0;
        if (!g->und)
            for (const auto& e : h.in[b]) S -= lgamma((double)(e.second + 1));
        for (const auto& e : h.out[b]) {
            S -= lgamma((double)(e.second + 1));
            total += e.second;
        }
        S += (g->und ? 1.0 : 2.0) * lgamma((double)(total + 1));
    }
    return S;
}
/* get_delta_deg_dl_dist_change (entropy.cpp:994-1070) for one vertex with degrees
 * (kin, kout) leaving (diff = -1) or joining (+1) block b; `fix` selects the canonical
 * arithmetic (terms rounded to 2^-24, result in those units) or the literal one. */
double dc_change(const ora_bm* bm, const DcHist& h, int64_t b, int64_t kin, int64_t kout, int diff, bool fix) {
    const ora_graph* g = bm->g;
    const int64_t total = bm->sizes[b], ep = bm->dout[b], em = bm->din[b];
    auto lg1 = [&](int64_t x) { return fix ? (double)g->LG[x] : lgamma((double)(x + 1)); };
    auto lq = [&](int64_t n, int64_t k) { return fix ? (double)dc_fix(dc_log_q(n, k)) : dc_log_q(n, k); };
    auto Sk = [&](int delta) {
        double S = 0.0;
        if (!g->und) S -= lg1(dc_count(h.in[b], kin) + delta);
        return S - lg1(dc_count(h.out[b], kout) + delta);
    };
    auto Se = [&](int delta, int64_t din, int64_t dout) { return lq(em + din, total + delta) + lq(ep + dout, total + delta); };
    auto Sr = [&](int delta) { return (g->und ? 1.0 : 2.0) * lg1(total + delta); };
    const double Sb = Sk(0) + Se(0, 0, 0) + Sr(0);
    const double Sa = Sk(diff) + Se(diff, diff * kin, diff * kout) + Sr(diff);
    return Sa - Sb;
}
/* get_delta_deg_dl (entropy.cpp:1072-1109) for moving v from its block to s. */
double dc_vertex_delta(const ora_bm* bm, const DcHist& h, int64_t v, int64_t s, bool fix) {
    const int64_t r = bm->asg[v];
    if (r == s) return 0.0;
    const int64_t kin = dc_kin(bm->g, v), kout = dc_kout(bm->g, v);
    return dc_change(bm, h, r, kin, kout, -1, fix) + dc_change(bm, h, s, kin, kout, +1, fix);
}
/* The block terms of virtual_move_sparse (entropy.cpp:822-889), the lgamma terms of
 * get_delta_partition_dl (:892-1000) and the non-empty-count terms for moving `weight`
 * vertices with kout / kin edges from r to s. */
int64_t np_block_terms(const ora_bm* bm, int64_t r, int64_t s, int64_t kout, int64_t kin, int64_t weight) {
    const ora_graph* g = bm->g;
    const int64_t sr = bm->sizes[r], ss = bm->sizes[s];
    int64_t t = np_vterm(g, bm->dout[r] - kout, bm->din[r] - kin, sr - weight) - np_vterm(g, bm->dout[r], bm->din[r], sr);
    t += np_vterm(g, bm->dout[s] + kout, bm->din[s] + kin, ss + weight) - np_vterm(g, bm->dout[s], bm->din[s], ss);
    t += g->LG[sr] + g->LG[ss] - g->LG[sr - weight] - g->LG[ss + weight];
    const int dB = (sr == weight ? -1 : 0) + (ss == 0 ? 1 : 0);
    if (dB != 0) t += np_dl_step(g, bm->nonempty, dB);
    return t;
}
/* entries_dS (entropy.cpp:782-809): eterm_exact(M + change) - eterm_exact(M) per entry. */
inline int64_t np_entries(const ora_bm* bm, const DeltaMap& d) {
    int64_t t = 0;
    for (const auto& e : d) {
        const int64_t m = bm->get(e.first.first, e.first.second);
        t += np_cell(bm->g, e.first.first == e.first.second, m, e.second);
    }
    return t;
}
/* nonparametric::delta_mdl (entropy.cpp:1146-1178), units of 2^-24. */
int64_t np_vertex_dS(const ora_bm* bm, int64_t v, int64_t s, const DeltaMap& d) {
    const int64_t r = bm->asg[v];
    if (r == s) return 0;
    const VertexInfo vi = vinfo(bm->g, v);
    int64_t t = np_entries(bm, d) + np_block_terms(bm, r, s, vi.kout, vi.kin, 1);
    if (bm->g->dc) t += (int64_t)dc_vertex_delta(bm, dc_hist(bm), v, s, true);
    return t;
}
/* nonparametric::block_merge_delta_mdl (entropy.cpp:1198-1223), units of 2^-24. */
int64_t np_merge_dS(const ora_bm* bm, int64_t r, int64_t s, const DeltaMap& d) {
    if (r == s || bm->sizes[r] == 0 || bm->sizes[s] == 0) return 0;
    int64_t kout = 0, kin = 0;
    for (const auto& e : bm->row[r]) kout += e.second;
    for (const auto& e : bm->col[r]) kin += e.second;
    return np_entries(bm, d) + np_block_terms(bm, r, s, kout, kin, bm->sizes[r]);
}
/* The reference's double arithmetic of the same two deltas (for the known-answer checks). */
double np_dS_literal(const ora_bm* bm, int64_t r, int64_t s, const DeltaMap& d, int64_t kout, int64_t kin,
                     int64_t weight) {
    const ora_graph* g = bm->g;
    auto lg = [](int64_t x) { return lgamma((double)x); };
    auto vt = [&](int64_t o, int64_t i, int64_t w) {
        if (g->dc) return lgamma((double)(o + 1)) + (g->und ? 0.0 : lgamma((double)(i + 1)));
        return w == 0 ? 0.0 : (double)(g->und ? o : o + i) * g->Ld[w];
    };
    const double log_2 = log(2.0);
    auto et = [&](bool diag, int64_t w) { return -lg(w + 1) - (g->und && diag ? (double)w * log_2 : 0.0); };
    double dS = 0.0;
    for (const auto& e : d) {
        const int64_t m = bm->get(e.first.first, e.first.second);
        const bool diag = e.first.first == e.first.second;
        dS += et(diag, m + e.second) - et(diag, m);
    }
    const int64_t sr = bm->sizes[r], ss = bm->sizes[s];
    dS += vt(bm->dout[r] - kout, bm->din[r] - kin, sr - weight);
    dS -= vt(bm->dout[r], bm->din[r], sr);
    dS += vt(bm->dout[s] + kout, bm->din[s] + kin, ss + weight);
    dS -= vt(bm->dout[s], bm->din[s], ss);
    double Sb = -lg(sr + 1) - lg(ss + 1), Sa = -lg(sr - weight + 1) - lg(ss + weight + 1);
    const int dB = (sr == weight ? -1 : 0) + (ss == 0 ? 1 : 0);
    double edges = 0.0;
    if (dB != 0) {
        Sb += np_lbinom(g->N - 1, bm->nonempty - 1);
        Sa += np_lbinom(g->N - 1, bm->nonempty + dB - 1);
        edges = np_edges_dl(bm->nonempty + dB, g->Em, g->und) - np_edges_dl(bm->nonempty, g->Em, g->und);
    }
    return dS + ((Sa - Sb) + 0.0 + edges);
}
/* nonparametric::mdl (entropy.cpp:751-779), canonical: exact sum of the table terms, then
 * the two terms of the non-empty block count. */
double np_mdl_canonical(const ora_bm* bm) {
    const ora_graph* g = bm->g;
    int64_t fixed = 0;
    for (int64_t r = 0; r < bm->B; ++r)
        for (const auto& e : bm->row[r]) fixed -= np_cell(g, e.first == r, e.second, -e.second);  // + eterm
    for (int64_t b = 0; b < bm->B; ++b) fixed += np_vterm(g, bm->dout[b], bm->din[b], bm->sizes[b]) - g->LG[bm->sizes[b]];
    fixed += g->LG[g->N] + g->Lq[g->N];
    if (g->dc) fixed += dc_deg_entropy_fixed(g) + dc_deg_dl_fixed(bm, dc_hist(bm));
    return (double)fixed * kInvFix +
           (np_lbinom(g->N - 1, bm->nonempty - 1) + np_edges_dl(bm->nonempty, g->Em, g->und));
}
/* The four parts in the reference's arithmetic. */
void np_terms_literal(const ora_bm* bm, double out[4]) {
    const ora_graph* g = bm->g;
    double S = 0.0;
    const double log_2 = log(2.0);
    for (int64_t r = 0; r < bm->B; ++r)
        for (const auto& e : bm->row[r])
            S += -lgamma((double)(e.second + 1)) - (g->und && e.first == r ? (double)e.second * log_2 : 0.0);
    for (int64_t b = 0; b < bm->B; ++b) {
        if (g->dc)
            S += lgamma((double)(bm->dout[b] + 1)) + (g->und ? 0.0 : lgamma((double)(bm->din[b] + 1)));
        else if (bm->sizes[b] != 0)
            S += (double)(g->und ? bm->dout[b] : bm->dout[b] + bm->din[b]) * g->Ld[bm->sizes[b]];
    }
    if (g->dc) S += dc_deg_entropy_literal(g);
    double P = 0.0;
    P += np_lbinom(g->N - 1, bm->nonempty - 1);
    P += lgamma((double)(g->N + 1));
    for (int64_t b = 0; b < bm->B; ++b) P -= lgamma((double)(bm->sizes[b] + 1));
    P += g->Ld[g->N];
    out[0] = S;
    out[1] = P;
    out[2] = g->dc ? dc_deg_dl_literal(bm, dc_hist(bm)) : 0.0;
    out[3] = np_edges_dl(bm->nonempty, g->Em, g->und);
}

/* A non-negative double as an integer count of 2^-64 units (truncated): every term of the
 * Hastings sums goes through this, so the sums are exact integers and do not depend on the
 * order in which the neighbour blocks are visited (the device sums them in parallel). */
inline __int128 to_fix64(double x) {
    uint64_t bits;
    std::memcpy(&bits, &x, 8);
    const int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0 || (bits >> 63)) return 0;
    const uint64_t mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = e - 1075 + 64;
    if (sh >= 0) return (__int128)mant << sh;
    if (sh <= -64) return 0;
    return (__int128)(mant >> (-sh));
}
inline double fix64_to_double(__int128 q) {
    const int64_t hi = (int64_t)(q >> 64);
    const uint64_t lo = (uint64_t)q;
    return (double)hi * 18446744073709551616.0 + (double)lo;
}

/* entropy::hastings_correction(vertex, ...) (entropy.cpp:497-561).  The reference sums
 * counts * weights / degrees over the distinct neighbour blocks in hash-map order; here each
 * term is the same double, accumulated exactly in 2^-64 units, and the ratio is taken of
 * the two sums converted back to double. */
double hastings(const ora_bm* bm, int64_t v, int64_t s, const DeltaMap& d, int64_t num_neighbor_edges,
                const ora_config* cfg) {
    if (num_neighbor_edges == 0 || cfg->greedy || cfg->nonparametric) return 1.0;  // entropy.cpp:499
    const ora_graph* g = bm->g;
    const int64_t r = bm->asg[v];
    const VertexInfo vi = vinfo(g, v);
    std::map<int32_t, int64_t> counts;
    for (int32_t u : g->out[v]) counts[bm->asg[u]] += 1;
    for (int32_t w : g->inns[v]) counts[bm->asg[w]] += 1;
    __int128 pf = 0, pb = 0;
    const double B = (double)bm->B;
    for (const auto& e : counts) {
        const int64_t b = e.first;
        const double cnt = (double)e.second;
        const double pw = (double)(bm->get(s, b) + bm->get(b, s)) + 1.0;
        const double bd = (double)bm->dtot[b] + B;
        const double bw = (double)(bm->get(r, b) + delta_get(d, r, b) + bm->get(b, r) + delta_get(d, b, r)) + 1.0;
        int64_t nd = bm->dtot[b];
        if (b == r) {
            const int64_t self = bm->get(r, r) + delta_get(d, r, r);
            nd = (bm->dout[r] - vi.kout) + (bm->din[r] - vi.kin) - self;
        } else if (b == s) {
            const int64_t self = bm->get(s, s) + delta_get(d, s, s);
            nd = (bm->dout[s] + vi.kout) + (bm->din[s] + vi.kin) - self;
        }
        pf += to_fix64(cnt * pw / bd);
        pb += to_fix64(cnt * bw / ((double)nd + B));
    }
    return fix64_to_double(pb) / fix64_to_double(pf);
}

/* finetune::accept (finetune.cpp:22-32). */
inline bool accept(double dS, double H, const ora_config* cfg, uint32_t w) {
    if (cfg->greedy && !cfg->nonparametric) return dS < 0.0;  // --nonparametric sets greedy off
    const double u = (double)w * (1.0 / 4294967296.0);
    double p = exp(-3.0 * dS) * H;
    p = p >= 1.0 ? 1.0 : p;
    return u <= p;
}

/* Walk `m` in ascending key order and return the key at cumulative position t,
 * skipping keys skip1 / skip2. */
inline int64_t walk(const std::map<int32_t, int64_t>& m, uint64_t t, int64_t skip1, int64_t skip2) {
    uint64_t acc = 0;
    for (const auto& e : m) {
        if (e.first == skip1 || e.first == skip2) continue;
        acc += (uint64_t)e.second;
        if (t < acc) return e.first;
    }
    return -1;
}

inline uint64_t sum_excl(const std::map<int32_t, int64_t>& m, int64_t skip1, int64_t skip2) {
    uint64_t acc = 0;
    for (const auto& e : m)
        if (e.first != skip1 && e.first != skip2) acc += (uint64_t)e.second;
    return acc;
}

/* common::propose_new_block(..., block_merge=false) (common.cpp:138-198) under the
 * canonical stream. */
int64_t propose_vertex(const ora_bm* bm, int64_t v, const uint32_t w[4]) {
    const ora_graph* g = bm->g;
    const int64_t r = bm->asg[v];
    const int64_t kout = (int64_t)g->out[v].size(), kin = (int64_t)g->inns[v].size();
    const int64_t k = kout + kin;
    if (k == 0) return random_block(r, bm->B, w[1]);
    const int64_t idx = u32_below(w[0], (uint32_t)k);
    const int32_t nbr = idx < kout ? g->out[v][idx] : g->inns[v][idx - kout];
    const int64_t nb = bm->asg[nbr];
    const uint64_t R = sum_excl(bm->row[nb], -1, -1);
    const uint64_t C = sum_excl(bm->col[nb], nb, -1);
    const uint64_t t = u64_below(w[1], w[2], R + C);
    if (t < R) return walk(bm->row[nb], t, -1, -1);
    return walk(bm->col[nb], t - R, nb, -1);
}

/* common::propose_new_block(..., block_merge=true) as called by
 * block_merge::propose_merge_sparse (block_merge.cpp:251-256). */
int64_t propose_merge(const ora_bm* bm, int64_t r, const uint32_t w[4]) {
    const uint64_t Rr = sum_excl(bm->row[r], -1, -1);
    const uint64_t Cr = sum_excl(bm->col[r], -1, -1);
    if (Rr + Cr == 0) return random_block(r, bm->B, w[0]);
    const uint64_t t = u64_below(w[0], w[1], Rr + Cr);
    const int64_t nb = t < Rr ? walk(bm->row[r], t, -1, -1) : walk(bm->col[r], t - Rr, -1, -1);
    const uint64_t R2 = sum_excl(bm->row[nb], r, -1);
    const uint64_t C2 = sum_excl(bm->col[nb], nb, r);
    if (R2 + C2 == 0) return random_block(r, bm->B, w[2]);
    const uint64_t t2 = u64_below(w[2], w[3], R2 + C2);
    if (t2 < R2) return walk(bm->row[nb], t2, r, -1);
    return walk(bm->col[nb], t2 - R2, nb, r);
}

/* Blockmodel::move_vertex(const VertexMove_v3&) (blockmodel.cpp:437-494). */
bool apply_v3(ora_bm* bm, int64_t v, int64_t s) {
    const ora_graph* g = bm->g;
    const int64_t r = bm->asg[v];
    if (bm->sizes[r] == 1) return false;
    for (int32_t u : g->out[v]) {
        const int64_t ob = bm->asg[u];
        bm->add(r, ob, -1);
        bm->dout[r]--;
        bm->dout[s]++;
        if (u == v) {
            bm->add(s, s, 1);
            bm->din[r]--;
            bm->din[s]++;
        } else {
            bm->add(s, ob, 1);
        }
    }
    for (int32_t w : g->inns[v]) {
        const int64_t ib = bm->asg[w];
        bm->add(ib, r, -1);
        bm->din[r]--;
        bm->add(ib, s, 1);
        bm->din[s]++;
    }
    bm->dtot[r] = bm->din[r] + bm->dout[r] - bm->get(r, r);
    bm->dtot[s] = bm->din[s] + bm->dout[s] - bm->get(s, s);
    bm->asg[v] = (int32_t)s;
    bm->sizes[r]--;
    bm->sizes[s]++;
    // the count of non-empty blocks as a recount gives it (a move that would empty its
    // block is rejected above, so only a move into an empty block changes it)
    if (bm->sizes[s] == 1) bm->nonempty++;
    return true;
}

/* Blockmodel::move_vertex(Vertex, Delta, proposal) (blockmodel.cpp:408-435). */
void apply_delta_move(ora_bm* bm, int64_t v, int64_t s, const DeltaMap& d) {
    const VertexInfo vi = vinfo(bm->g, v);
    const int64_t r = bm->asg[v];
    bm->asg[v] = (int32_t)s;
    for (const auto& e : d) {
        if (e.second == 0) {
            // update_edge_counts inserts then erases a zero cell: no net change.
            continue;
        }
        bm->add(e.first.first, e.first.second, e.second);
    }
    bm->dout[r] -= vi.kout;
    bm->dout[s] += vi.kout;
    bm->din[r] -= (vi.kin + vi.selfw);
    bm->din[s] += (vi.kin + vi.selfw);
    bm->dtot[r] = bm->dout[r] + bm->din[r] - bm->get(r, r);
    bm->dtot[s] = bm->dout[s] + bm->din[s] - bm->get(s, s);
    bm->sizes[r]--;
    bm->sizes[s]++;
    if (bm->sizes[r] == 0) bm->nonempty--;  // blockmodel.cpp:429-430
    if (bm->sizes[s] == 1) bm->nonempty++;
}

/* Canonical MDL log term: round-to-float(log(x)) in units of 2^-24 (see sbp_oracle.h). */
inline int64_t canon_log_q(double ratio) {
    const float xf = (float)ratio;
    const float lf = (float)log((double)xf);
    return (int64_t)((double)lf * kFix);
}

void mdl_both(const ora_bm* bm, double* literal, double* canonical) {
    const ora_graph* g = bm->g;
    double lp = 0.0;
    __int128 lpq = 0;
    for (int64_t r = 0; r < bm->B; ++r) {
        for (const auto& e : bm->row[r]) {
            const double v = (double)e.second;
            const double ratio = v / ((double)bm->dout[r] * (double)bm->din[e.first]);
            lp += v * (double)logf(ratio);  // utils::nat_log (utils.hpp:228-238)
            lpq += (__int128)e.second * canon_log_q(ratio);
        }
    }
    const double E = (double)g->Em;
    const double x = pow((double)bm->B, 2) / E;
    const double h = ((1 + x) * log(1 + x)) - (x * log(x));
    const double model = (E * h) + ((double)g->N * log((double)bm->B));
    if (literal) *literal = model - lp;
    if (canonical) *canonical = model - (double)(int64_t)lpq * kInvFix;
}

double mdl_canonical(const ora_bm* bm) {
    double c;
    mdl_both(bm, nullptr, &c);
    return c;
}

/* entropy::mdl (entropy.cpp:597-604): the nonparametric form under --nonparametric. */
double mdl_for(const ora_bm* bm, const ora_config* cfg) {
    return cfg->nonparametric ? np_mdl_canonical(bm) : mdl_canonical(bm);
}

/* finetune::early_stop (finetune.cpp:265-283). */
bool early_stop(int64_t iteration, bool golden_ratio_not_reached, double initial_entropy,
                const std::vector<double>& d) {
    const size_t last = d.size() - 1;
    if (d[last] == 0.0) return true;
    if (iteration < 3) return false;
    double average = d[last] + d[last - 1] + d[last - 2];
    average /= -3.0;
    const double threshold = golden_ratio_not_reached ? 5e-4 * initial_entropy : 1e-4 * initial_entropy;
    return average < threshold;
}

/* Graph::sort_vertices (graph.cpp:235-268): stable sort by degree descending; the first
 * (mh_percent * N) become high-degree vertices.  mh_percent is a float in the reference. */
void sort_vertices(const ora_graph* g, float mh_percent, std::vector<int32_t>& hdv, std::vector<int32_t>& ldv) {
    std::vector<int64_t> deg(g->N);
    for (int64_t v = 0; v < g->N; ++v)
        deg[v] = (int64_t)g->out[v].size() + (int64_t)g->in[v].size() - (g->selfcnt[v] > 0 ? 1 : 0);
    std::vector<int32_t> idx(g->N);
    for (int64_t v = 0; v < g->N; ++v) idx[v] = (int32_t)v;
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return deg[a] > deg[b]; });
    const float limit = mh_percent * (float)g->N;
    hdv.clear();
    ldv.clear();
    for (int64_t i = 0; i < g->N; ++i) {
        if ((float)i < limit) hdv.push_back(idx[i]);
        else ldv.push_back(idx[i]);
    }
}

/* Canonical shuffle: order the base list by (philox word, position). */
void shuffle(std::vector<int32_t>& out, const std::vector<int32_t>& base, uint64_t seed, uint32_t iteration,
             uint32_t step, uint32_t dom) {
    std::vector<std::pair<uint64_t, int32_t>> keys(base.size());
    for (size_t i = 0; i < base.size(); ++i) {
        uint32_t w[4];
        draw(seed, (uint32_t)i, iteration, step, dom, w);
        keys[i] = {((uint64_t)w[0] << 32) | (uint64_t)i, base[i]};
    }
    std::sort(keys.begin(), keys.end());
    out.resize(base.size());
    for (size_t i = 0; i < base.size(); ++i) out[i] = keys[i].second;
}

struct Proposal {
    int32_t s;
    double dS;
    bool did_move;
};

/* finetune::propose_gibbs_move_v3 + eval_vertex_move_v3 (finetune.cpp:871-901, 447-462). */
Proposal gibbs_proposal(const ora_bm* bm, int64_t v, uint64_t seed, uint32_t iteration, uint32_t step,
                        const ora_config* cfg) {
    uint32_t w[4];
    draw(seed, (uint32_t)v, iteration, step, DOM_GIBBS, w);
    const int64_t r = bm->asg[v];
    const int64_t s = propose_vertex(bm, v, w);
    if (s == r) return {-1, 0.0, false};
    const DeltaMap d = vertex_delta(bm, v, s);
    const double dS = (double)(cfg->nonparametric ? np_vertex_dS(bm, v, s, d)
                                                  : delta_mdl_generic<int64_t>(bm, v, s, d, ce_fixed)) * kInvFix;
    const VertexInfo vi = vinfo(bm->g, v);
    const double H = hastings(bm, v, s, d, vi.kout + vi.kin, cfg);
    if (accept(dS, H, cfg, w[3])) return {(int32_t)s, dS, true};
    return {-1, dS, false};
}

/* finetune::propose_move + move_vertex (finetune.cpp:842-869, 822-840). */
bool mh_step(ora_bm* bm, int64_t v, uint64_t seed, uint32_t iteration, uint32_t step, const ora_config* cfg,
             double* dS_out) {
    const int64_t r = bm->asg[v];
    if (bm->sizes[r] == 1) return false;
    uint32_t w[4];
    draw(seed, (uint32_t)v, iteration, step, DOM_MH, w);
    const int64_t s = propose_vertex(bm, v, w);
    if (s == r) return false;
    const DeltaMap d = vertex_delta(bm, v, s);
    const double dS = (double)(cfg->nonparametric ? np_vertex_dS(bm, v, s, d)
                                                  : delta_mdl_generic<int64_t>(bm, v, s, d, ce_fixed)) * kInvFix;
    const VertexInfo vi = vinfo(bm->g, v);
    const double H = hastings(bm, v, s, d, vi.kout + vi.kin, cfg);
    if (!accept(dS, H, cfg, w[3])) return false;
    apply_delta_move(bm, v, s, d);
    if (dS_out) *dS_out = dS;
    return true;
}

void add_stats(ora_stats* st, const ora_graph* g, int64_t v) {
    if (!st) return;
    st->proposals++;
    st->edges_swept += (int64_t)g->out[v].size() + (int64_t)g->inns[v].size();
}

/* One batch: parallel proposals against one snapshot, then the serial apply loop in
 * vertex-id order (finetune.cpp:63-86 / 604-623). */
int64_t gibbs_batch(ora_bm* bm, const int32_t* vertices, int64_t n, uint64_t seed, uint32_t iteration,
                    uint32_t step, const ora_config* cfg, int32_t* out_moves, double* out_dS, ora_stats* st) {
    const int64_t N = bm->g->N;
    std::vector<int32_t> moves(N, -1);
    std::vector<double> dSs(n, 0.0);
    std::vector<int32_t> props(n, -1);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        const Proposal p = gibbs_proposal(bm, vertices[i], seed, iteration, step, cfg);
        props[i] = p.did_move ? p.s : -1;
        dSs[i] = p.dS;
    }
    for (int64_t i = 0; i < n; ++i) {
        moves[vertices[i]] = props[i];
        if (out_moves) out_moves[i] = props[i];
        if (out_dS) out_dS[i] = dSs[i];
        add_stats(st, bm->g, vertices[i]);
    }
    int64_t applied = 0;
    for (int64_t v = 0; v < N; ++v) {
        if (moves[v] < 0) continue;
        if (apply_v3(bm, v, moves[v])) applied++;
    }
    if (st) st->moves += applied;
    return applied;
}

/* finetune::asynchronous_gibbs (finetune.cpp:34-107). */
void async_gibbs(ora_bm* bm, const ora_config* cfg, uint64_t seed, uint32_t step, bool golden, ora_stats* st) {
    const ora_graph* g = bm->g;
    if (bm->B == 1) return;
    std::vector<double> deltas;
    const double initial = mdl_for(bm, cfg);
    bm->entropy = initial;
    double last = initial;
    std::vector<int32_t> base(g->N), order;
    for (int64_t v = 0; v < g->N; ++v) base[v] = (int32_t)v;
    for (int it = 0; it < cfg->max_iterations; ++it) {
        const bool shuffled = !cfg->ordered && cfg->batches > 1;
        if (shuffled) shuffle(order, base, seed, (uint32_t)it, step, DOM_SHUFFLE_ALL);
        const std::vector<int32_t>& vs = shuffled ? order : base;
        const double nb = (double)cfg->batches;
        const int64_t batch_size = (int64_t)ceil((double)g->N / nb);
        for (int64_t batch = 0; batch_size > 0 && batch < g->N / batch_size; ++batch) {
            const int64_t start = batch * batch_size;
            const int64_t end = std::min(g->N, (batch + 1) * batch_size);
            gibbs_batch(bm, vs.data() + start, end - start, seed, (uint32_t)it, step, cfg, nullptr, nullptr, st);
        }
        const double e = mdl_for(bm, cfg);
        deltas.push_back(e - last);
        last = e;
        if (st) st->mcmc_iterations++;
        if (early_stop(it, golden, initial, deltas)) break;
    }
    bm->entropy = mdl_for(bm, cfg);
}

/* finetune::hybrid_mcmc (finetune.cpp:563-646). */
void hybrid_mcmc(ora_bm* bm, const ora_config* cfg, uint64_t seed, uint32_t step, bool golden, ora_stats* st) {
    const ora_graph* g = bm->g;
    if (bm->B == 1) return;
    std::vector<double> deltas;
    const double initial = mdl_for(bm, cfg);
    bm->entropy = initial;
    double last = initial;
    std::vector<int32_t> hdv0, ldv0, hdv, ldv;
    sort_vertices(g, cfg->mh_percent, hdv0, ldv0);
    const int64_t nlow = (int64_t)ldv0.size();
    const int64_t batch_size = (int64_t)ceil((double)nlow / (double)cfg->batches);
    for (int it = 0; it < cfg->max_iterations; ++it) {
        if (!cfg->ordered) {
            shuffle(hdv, hdv0, seed, (uint32_t)it, step, DOM_SHUFFLE_HDV);
            if (cfg->batches > 1) shuffle(ldv, ldv0, seed, (uint32_t)it, step, DOM_SHUFFLE_ALL);
            else ldv = ldv0;
        } else {
            hdv = hdv0;
            ldv = ldv0;
        }
        for (int32_t v : hdv) {
            add_stats(st, g, v);
            if (mh_step(bm, v, seed, (uint32_t)it, step, cfg, nullptr) && st) st->moves++;
        }
        for (int64_t batch = 0; batch_size > 0 && batch < nlow / batch_size; ++batch) {
            const int64_t start = batch * batch_size;
            const int64_t end = std::min(nlow, (batch + 1) * batch_size);
            gibbs_batch(bm, ldv.data() + start, end - start, seed, (uint32_t)it, step, cfg, nullptr, nullptr, st);
        }
        const double e = mdl_for(bm, cfg);
        deltas.push_back(e - last);
        last = e;
        if (st) st->mcmc_iterations++;
        if (early_stop(it, golden, initial, deltas)) break;
    }
    bm->entropy = mdl_for(bm, cfg);
}

/* finetune::metropolis_hastings (finetune.cpp:773-820). */
void metropolis_hastings(ora_bm* bm, const ora_config* cfg, uint64_t seed, uint32_t step, bool golden,
                         ora_stats* st) {
    const ora_graph* g = bm->g;
    if (bm->B == 1) return;
    std::vector<double> deltas;
    bm->entropy = mdl_for(bm, cfg);
    std::vector<int32_t> base(g->N), order;
    for (int64_t v = 0; v < g->N; ++v) base[v] = (int32_t)v;
    for (int it = 0; it < cfg->max_iterations; ++it) {
        if (!cfg->ordered) shuffle(order, base, seed, (uint32_t)it, step, DOM_SHUFFLE_ALL);
        const std::vector<int32_t>& vs = cfg->ordered ? base : order;
        double dsum = 0.0;
        for (int32_t v : vs) {
            double dS = 0.0;
            add_stats(st, g, v);
            if (mh_step(bm, v, seed, (uint32_t)it, step, cfg, &dS)) {
                dsum += dS;
                if (st) st->moves++;
            }
        }
        deltas.push_back(dsum);
        if (st) st->mcmc_iterations++;
        if (early_stop(it, golden, bm->entropy, deltas)) break;
    }
    bm->entropy = mdl_for(bm, cfg);
}

/* Blockmodel::build_mapping (blockmodel.cpp:34-46) + relabel. */
void relabel(ora_bm* bm) {
    std::map<int32_t, int32_t> mapping;
    for (int32_t b : bm->asg) mapping[b] = 0;
    int32_t c = 0;
    for (auto& e : mapping) e.second = c++;
    for (auto& b : bm->asg) b = mapping[b];
}

/* Blockmodel::merge_block (blockmodel.cpp:337-363) without the O(N) assignment loop,
 * which the caller replaces by union-find (the resulting labels are identical). */
void merge_block(ora_bm* bm, int64_t from, int64_t to, const DeltaMap& d) {
    int64_t kout = 0, kin = 0;
    for (const auto& e : bm->row[from]) kout += e.second;
    for (const auto& e : bm->col[from]) kin += e.second;
    const int64_t self = bm->get(to, to) + delta_get(d, to, to);
    for (const auto& e : d)
        if (e.second != 0) bm->add(e.first.first, e.first.second, e.second);
    bm->dout[from] = 0;
    bm->dout[to] += kout;
    bm->din[from] = 0;
    bm->din[to] += kin;
    bm->dtot[from] = 0;
    bm->dtot[to] = bm->dout[to] + bm->din[to] - self;
    bm->sizes[to] += bm->sizes[from];
    bm->sizes[from] = 0;
    bm->nonempty--;  // blockmodel.cpp:356, also when `from` was empty
}

int64_t uf_find(std::vector<int64_t>& parent, int64_t x) {
    int64_t root = x;
    while (parent[root] != root) root = parent[root];
    while (parent[x] != root) {
        const int64_t nx = parent[x];
        parent[x] = root;
        x = nx;
    }
    return root;
}

/* block_merge::carry_out_best_merges_advanced (block_merge.cpp:40-117).  The queue is
 * ordered by (delta entropy, block); the reference's std::priority_queue leaves ties in
 * an implementation-defined order. */
int carry_out_advanced(ora_bm* bm, const std::vector<double>& dS, const std::vector<int64_t>& best,
                       int64_t num_to_merge, bool nonparametric, ora_stats* st) {
    std::set<std::pair<double, int64_t>> queue;
    std::vector<int64_t> prop(best);
    for (int64_t i = 0; i < (int64_t)dS.size(); ++i) queue.insert({dS[i], i});
    std::vector<int64_t> parent(bm->B);
    for (int64_t i = 0; i < bm->B; ++i) parent[i] = i;
    int64_t merged = 0;
    while (merged < num_to_merge && !queue.empty()) {
        const auto top = *queue.begin();
        queue.erase(queue.begin());
        const int64_t from = top.second;
        const int64_t to = uf_find(parent, prop[from]);
        if (from == to) continue;
        const DeltaMap d = merge_delta(bm, from, to);
        const double actual = (double)(nonparametric ? np_merge_dS(bm, from, to, d)
                                                     : merge_delta_mdl_generic<int64_t>(bm, from, to, d, ce_fixed)) *
                              kInvFix;
        if (!queue.empty() && actual > queue.begin()->first) {
            queue.insert({actual, from});
            continue;
        }
        merge_block(bm, from, to, d);
        parent[from] = to;
        merged++;
    }
    for (auto& b : bm->asg) b = (int32_t)uf_find(parent, b);
    relabel(bm);
    if (st) st->merges += merged;
    return 0;
}

/* Blockmodel::carry_out_best_merges (blockmodel.cpp:55-122), used with --approximate. */
int carry_out_approximate(ora_bm* bm, const std::vector<double>& dS, const std::vector<int64_t>& best,
                          int64_t num_to_merge, ora_stats* st) {
    const int64_t B = bm->B;
    std::vector<int64_t> order(B);
    for (int64_t i = 0; i < B; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return dS[a] < dS[b]; });
    std::vector<int64_t> block_map(B);
    for (int64_t i = 0; i < B; ++i) block_map[i] = i;
    auto translate = [&](int64_t b) {
        do { b = block_map[b]; } while (block_map[b] != b);
        return b;
    };
    int64_t merged = 0, counter = 0;
    while (merged < num_to_merge && counter < B) {
        const int64_t from = order[counter];
        const int64_t to = translate(best[from]);
        counter++;
        if (to != from) {
            block_map[from] = to;
            merged++;
        }
    }
    for (auto& b : bm->asg) b = (int32_t)translate(b);
    relabel(bm);
    if (st) st->merges += merged;
    return 0;
}

/* block_merge::merge_blocks (block_merge.cpp:178-228). */
int merge_blocks(ora_bm* bm, const ora_config* cfg, uint64_t seed, uint32_t step, int64_t num_to_merge,
                 ora_stats* st) {
    const int64_t B = bm->B;
    std::vector<int64_t> best(B, -1);
    std::vector<double> best_dS(B, DBL_MAX);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t r = 0; r < B; ++r) {
        std::set<int64_t> past;
        for (int i = 0; i < 10; ++i) {  // NUM_AGG_PROPOSALS_PER_BLOCK (block_merge.hpp:23)
            uint32_t w[4];
            draw(seed, (uint32_t)r, 0, step, DOM_MERGE | ((uint32_t)i << 8), w);
            const int64_t s = propose_merge(bm, r, w);
            double dS = DBL_MAX;
            if (!past.count(s)) {
                dS = (double)(cfg->nonparametric ? np_merge_dS(bm, r, s, merge_delta(bm, r, s))
                                                 : merge_dS_fixed(bm, r, s)) * kInvFix;
                past.insert(s);
            }
            if (dS < best_dS[r]) {
                best_dS[r] = dS;
                best[r] = s;
            }
        }
    }
    if (st) st->merge_proposals += 10 * B;
    int rc = cfg->approximate ? carry_out_approximate(bm, best_dS, best, num_to_merge, st)
                              : carry_out_advanced(bm, best_dS, best, num_to_merge, cfg->nonparametric != 0, st);
    if (rc) return rc;
    // blockmodel.num_blocks(num_blocks - num_blocks_to_merge) (block_merge.cpp:115): blocks
    // that were empty before the pass become empty trailing blocks
    bm->B = B - num_to_merge;
    int32_t mx = -1;
    for (int32_t b : bm->asg) mx = std::max(mx, b);
    if (mx + 1 > bm->B) return -2;  // fewer merges than requested: inconsistent labels
    build(bm);
    return 0;
}

int mcmc(ora_bm* bm, const ora_config* cfg, uint64_t seed, int32_t step, bool golden, ora_stats* st) {
    if (cfg->algorithm == 0 && step < cfg->asynciterations)
        async_gibbs(bm, cfg, seed, (uint32_t)step, golden, st);
    else if (cfg->algorithm == 1)
        hybrid_mcmc(bm, cfg, seed, (uint32_t)step, golden, st);
    else
        metropolis_hastings(bm, cfg, seed, (uint32_t)step, golden, st);
    return 0;
}

// ---------------------------------------------------------------- golden-section triplet
/* BlockmodelTriplet (blockmodel_triplet.cpp:4-105), keeping assignments only: a slot is
 * rebuilt from its assignment when resumed, which gives the same blockmodel state. */
struct Slot {
    bool empty = true;
    int64_t B = 0;
    double entropy = DBL_MAX;
    std::vector<int32_t> asg;
};

struct Triplet {
    Slot s[3];
    bool optimal = false;
    bool golden_ratio_not_reached() const { return s[2].empty; }
    void update(const ora_bm* bm) { update(bm->B, bm->entropy, bm->asg); }
    void update(int64_t B, double entropy, const std::vector<int32_t>& asg) {
        int idx;
        if (s[1].empty) {
            idx = 1;
        } else if (entropy <= s[1].entropy) {
            const int old = (s[1].B > B) ? 0 : 2;
            s[old] = s[1];
            idx = 1;
        } else {
            idx = (s[1].B > B) ? 2 : 0;
        }
        s[idx].empty = false;
        s[idx].B = B;
        s[idx].entropy = entropy;
        s[idx].asg = asg;
    }
    /* BlockmodelTriplet::get_next_blockmodel (blockmodel_triplet.cpp:4-37) after update. */
    const Slot* next(int64_t* next_merge) {
        if (golden_ratio_not_reached()) {
            *next_merge = (int64_t)((double)s[1].B * 0.5);
            if (*next_merge == 0) optimal = true;
            return &s[1];
        }
        if (is_done()) {
            *next_merge = 0;
            return &s[1];
        }
        int index = 1;
        if (s[0].empty && s[1].B > s[2].B) index = 1;
        else if ((s[0].B - s[1].B) >= (s[1].B - s[2].B)) index = 0;
        else index = 1;
        int64_t next_try = s[index + 1].B;
        next_try += (int64_t)((double)(s[index].B - s[index + 1].B) * 0.618);
        *next_merge = s[index].B - next_try;
        return &s[index];
    }
    bool is_done() {
        if ((!s[0].empty && s[0].B - s[2].B == 2) || (s[0].empty && s[1].B - s[2].B == 1)) optimal = true;
        return optimal;
    }
};

}  // namespace

// ---------------------------------------------------------------- C API
extern "C" ora_bm* ora_bm_create(const ora_graph* g, int64_t B, const int32_t* asg) {
    auto* bm = new ora_bm();
    bm->g = g;
    bm->B = B;
    bm->asg.assign(asg, asg + g->N);
    bm->num_blocks_to_merge = (int64_t)((double)B * 0.5);
    build(bm);
    return bm;
}
extern "C" ora_bm* ora_bm_copy(const ora_bm* bm) { return new ora_bm(*bm); }
extern "C" void ora_bm_destroy(ora_bm* bm) { delete bm; }
extern "C" int64_t ora_bm_num_blocks(const ora_bm* bm) { return bm->B; }
extern "C" int64_t ora_bm_nnz(const ora_bm* bm) {
    int64_t n = 0;
    for (const auto& r : bm->row) n += (int64_t)r.size();
    return n;
}
extern "C" void ora_bm_read(const ora_bm* bm, int32_t* asg, int64_t* dout, int64_t* din, int64_t* dtot,
                            int64_t* sizes, int32_t* rows, int32_t* cols, int64_t* counts) {
    if (asg) std::copy(bm->asg.begin(), bm->asg.end(), asg);
    if (dout) std::copy(bm->dout.begin(), bm->dout.end(), dout);
    if (din) std::copy(bm->din.begin(), bm->din.end(), din);
    if (dtot) std::copy(bm->dtot.begin(), bm->dtot.end(), dtot);
    if (sizes) std::copy(bm->sizes.begin(), bm->sizes.end(), sizes);
    if (rows || cols || counts) {
        int64_t i = 0;
        for (int64_t r = 0; r < bm->B; ++r)
            for (const auto& e : bm->row[r]) {
                if (rows) rows[i] = (int32_t)r;
                if (cols) cols[i] = e.first;
                if (counts) counts[i] = e.second;
                ++i;
            }
    }
}
extern "C" int64_t ora_bm_get(const ora_bm* bm, int64_t r, int64_t c) { return bm->get(r, c); }

extern "C" void ora_mdl(const ora_bm* bm, double* literal, double* canonical) { mdl_both(bm, literal, canonical); }

extern "C" void ora_delta_mdl(const ora_bm* bm, int64_t v, int64_t s, double* literal, int64_t* fixed) {
    const DeltaMap d = vertex_delta(bm, v, s);
    if (literal) *literal = delta_mdl_generic<double>(bm, v, s, d, ce_double);
    if (fixed) *fixed = delta_mdl_generic<int64_t>(bm, v, s, d, ce_fixed);
}

extern "C" void ora_merge_delta_mdl(const ora_bm* bm, int64_t r, int64_t s, double* literal, int64_t* fixed) {
    const DeltaMap d = merge_delta(bm, r, s);
    if (literal) *literal = merge_delta_mdl_generic<double>(bm, r, s, d, ce_double);
    if (fixed) *fixed = merge_delta_mdl_generic<int64_t>(bm, r, s, d, ce_fixed);
}

static int64_t dump_delta(const DeltaMap& d, int32_t* rows, int32_t* cols, int64_t* vals, int64_t cap) {
    int64_t i = 0;
    for (const auto& e : d) {
        if (i < cap) {
            rows[i] = e.first.first;
            cols[i] = e.first.second;
            vals[i] = e.second;
        }
        ++i;
    }
    return i;
}

extern "C" int64_t ora_vertex_delta(const ora_bm* bm, int64_t v, int64_t s, int32_t* rows, int32_t* cols,
                                    int64_t* vals, int64_t cap) {
    return dump_delta(vertex_delta(bm, v, s), rows, cols, vals, cap);
}

extern "C" int64_t ora_merge_delta(const ora_bm* bm, int64_t r, int64_t s, int32_t* rows, int32_t* cols,
                                   int64_t* vals, int64_t cap) {
    return dump_delta(merge_delta(bm, r, s), rows, cols, vals, cap);
}

extern "C" int64_t ora_propose_vertex(const ora_bm* bm, int64_t v, uint64_t seed, uint32_t c1, uint32_t c2,
                                      uint32_t c3) {
    uint32_t w[4];
    draw(seed, (uint32_t)v, c1, c2, c3, w);
    return propose_vertex(bm, v, w);
}

extern "C" int64_t ora_propose_merge(const ora_bm* bm, int64_t r, uint64_t seed, uint32_t step, int32_t i) {
    uint32_t w[4];
    draw(seed, (uint32_t)r, 0, step, DOM_MERGE | ((uint32_t)i << 8), w);
    return propose_merge(bm, r, w);
}

/* The proposal loop of block_merge::merge_blocks (block_merge.cpp:188-217) over the blocks
 * blocks[0..n) only: 10 draws per block, repeats skipped, the best proposal and its delta
 * per listed block.  OpenMP over blocks as the reference.  Returns the draws made. */
extern "C" int64_t ora_merge_proposals(const ora_bm* bm, const int32_t* blocks, int64_t n, uint64_t seed,
                                       uint32_t step, int32_t nonparametric, int32_t* best_out,
                                       double* dS_out) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t k = 0; k < n; ++k) {
        const int64_t r = blocks[k];
        std::set<int64_t> past;
        int64_t best = -1;
        double best_dS = DBL_MAX;
        for (int i = 0; i < 10; ++i) {
            uint32_t w[4];
            draw(seed, (uint32_t)r, 0, step, DOM_MERGE | ((uint32_t)i << 8), w);
            const int64_t s = propose_merge(bm, r, w);
            double dS = DBL_MAX;
            if (!past.count(s)) {
                dS = (double)(nonparametric ? np_merge_dS(bm, r, s, merge_delta(bm, r, s)) : merge_dS_fixed(bm, r, s)) *
                     kInvFix;
                past.insert(s);
            }
            if (dS < best_dS) {
                best_dS = dS;
                best = s;
            }
        }
        best_out[k] = (int32_t)best;
        dS_out[k] = best_dS;
    }
    return 10 * n;
}

/* A bounded sample of one golden-section step (sbp.cpp:27-35), for timing: the merge pass's
 * proposal loop over blocks[0..n) (block_merge.cpp:188-217), the carry-out
 * (block_merge.cpp:40-117) of their queue until n / 2 merges, and `sweeps` hybrid-MCMC
 * sweeps (finetune.cpp:563-646) over the vertices of the blocks that received a merge:
 * those flagged in hub[] as the sequential chain, the rest as one asynchronous-Gibbs batch.
 * Mutates bm (its blocks keep their ids; merged-away blocks stay empty).  counts[0..2] =
 * proposals drawn, merges, vertex proposals. */
extern "C" void ora_step_sample(ora_bm* bm, const int32_t* blocks, int64_t n, const uint8_t* hub, uint64_t seed,
                                uint32_t step, const ora_config* cfg, int32_t sweeps, int64_t* counts) {
    std::vector<int32_t> best(n);
    std::vector<double> dS(n);
    counts[0] = ora_merge_proposals(bm, blocks, n, seed, step, cfg->nonparametric, best.data(), dS.data());
    std::set<std::pair<double, int64_t>> queue;
    std::vector<int64_t> parent(bm->B), prop(bm->B, -1);
    for (int64_t i = 0; i < bm->B; ++i) parent[i] = i;
    for (int64_t k = 0; k < n; ++k) {
        if (best[k] < 0) continue;
        queue.insert({dS[k], (int64_t)blocks[k]});
        prop[blocks[k]] = best[k];
    }
    std::vector<uint8_t> target(bm->B, 0);
    int64_t merged = 0;
    while (merged < n / 2 && !queue.empty()) {
        const auto top = *queue.begin();
        queue.erase(queue.begin());
        const int64_t from = top.second;
        const int64_t to = uf_find(parent, prop[from]);
        if (from == to) continue;
        const DeltaMap d = merge_delta(bm, from, to);
        const double actual = (double)(cfg->nonparametric ? np_merge_dS(bm, from, to, d)
                                                          : merge_delta_mdl_generic<int64_t>(bm, from, to, d, ce_fixed)) *
                              kInvFix;
        if (!queue.empty() && actual > queue.begin()->first) {
            queue.insert({actual, from});
            continue;
        }
        merge_block(bm, from, to, d);
        parent[from] = to;
        target[to] = 1;
        merged++;
    }
    for (auto& b : bm->asg) b = (int32_t)uf_find(parent, b);
    counts[1] = merged;
    std::vector<int32_t> chain, rest;
    for (int64_t v = 0; v < bm->g->N; ++v)
        if (target[bm->asg[v]]) (hub[v] ? chain : rest).push_back((int32_t)v);
    for (int32_t it = 0; it < sweeps; ++it) {
        for (int32_t v : chain) mh_step(bm, v, seed, (uint32_t)it, step, cfg, nullptr);
        gibbs_batch(bm, rest.data(), (int64_t)rest.size(), seed, (uint32_t)it, step, cfg, nullptr, nullptr, nullptr);
    }
    counts[2] = (int64_t)sweeps * (int64_t)(chain.size() + rest.size());
}

extern "C" int64_t ora_gibbs_batch(ora_bm* bm, const int32_t* vertices, int64_t n, uint64_t seed,
                                   uint32_t iteration, uint32_t step, const ora_config* cfg, int32_t* out_moves,
                                   double* out_dS) {
    return gibbs_batch(bm, vertices, n, seed, iteration, step, cfg, out_moves, out_dS, nullptr);
}

extern "C" int64_t ora_apply_moves(ora_bm* bm, const int32_t* moves) {
    int64_t applied = 0;
    for (int64_t v = 0; v < bm->g->N; ++v)
        if (moves[v] >= 0 && apply_v3(bm, v, moves[v])) applied++;
    return applied;
}

extern "C" int64_t ora_mh_chain(ora_bm* bm, const int32_t* order, int64_t n, uint64_t seed, uint32_t iteration,
                                uint32_t step, const ora_config* cfg) {
    int64_t applied = 0;
    for (int64_t i = 0; i < n; ++i)
        if (mh_step(bm, order[i], seed, iteration, step, cfg, nullptr)) applied++;
    return applied;
}

extern "C" int ora_mcmc(ora_bm* bm, const ora_config* cfg, uint64_t seed, int32_t step,
                        int32_t golden_ratio_not_reached, ora_stats* st) {
    return mcmc(bm, cfg, seed, step, golden_ratio_not_reached != 0, st);
}

extern "C" int ora_merge_blocks(ora_bm* bm, const ora_config* cfg, uint64_t seed, int32_t step,
                                int64_t num_to_merge, ora_stats* st) {
    return merge_blocks(bm, cfg, seed, (uint32_t)step, num_to_merge, st);
}

// ---------------------------------------------------------------- sampling
namespace {

/* Graph::degrees (graph.cpp:24-31): out + in - (has a self-loop). */
std::vector<int64_t> graph_degrees(const ora_graph* g) {
    std::vector<int64_t> d(g->N);
    for (int64_t v = 0; v < g->N; ++v)
        d[v] = (int64_t)g->out[v].size() + (int64_t)g->in[v].size() - (g->selfcnt[v] > 0 ? 1 : 0);
    return d;
}

/* long(args.samplesize * double(N)) */
inline int64_t sample_target(const ora_graph* g, double samplesize) { return (int64_t)(samplesize * (double)g->N); }

/* sample::max_degree (sample.cpp:255-270): stable argsort by degree, descending. */
int64_t sample_max_degree(const ora_graph* g, double samplesize, std::vector<int32_t>& mapping) {
    const std::vector<int64_t> d = graph_degrees(g);
    std::vector<int32_t> idx(g->N);
    for (int64_t v = 0; v < g->N; ++v) idx[v] = (int32_t)v;
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return d[a] > d[b]; });
    const int64_t n = std::min(sample_target(g, samplesize), g->N);
    for (int64_t i = 0; i < n; ++i) mapping[idx[i]] = (int32_t)i;
    return n;
}

/* sample::random (sample.cpp:272-284) with the canonical shuffle. */
int64_t sample_random(const ora_graph* g, double samplesize, uint64_t seed, std::vector<int32_t>& mapping) {
    std::vector<int32_t> base(g->N), order;
    for (int64_t v = 0; v < g->N; ++v) base[v] = (int32_t)v;
    shuffle(order, base, seed, 0, 0, DOM_SAMPLE);
    const int64_t n = std::min(sample_target(g, samplesize), g->N);
    for (int64_t i = 0; i < n; ++i) mapping[order[i]] = (int32_t)i;
    return n;
}

/* sample::degree_product (sample.cpp:28-49) over Graph::sorted_edge_list (graph.cpp:302-315):
 * edges in source order, stable-sorted by degree product, descending. */
int64_t sample_degree_product(const ora_graph* g, double samplesize, std::vector<int32_t>& mapping) {
    const std::vector<int64_t> d = graph_degrees(g);
    std::vector<std::pair<std::pair<int32_t, int32_t>, int64_t>> edges;
    for (int64_t u = 0; u < g->N; ++u)
        for (int32_t v : g->out[u]) edges.push_back({{(int32_t)u, v}, d[u] * d[v]});
    std::stable_sort(edges.begin(), edges.end(), [](const auto& a, const auto& b) { return a.second > b.second; });
    const int64_t target = sample_target(g, samplesize);
    int64_t n = 0;
    for (const auto& e : edges) {
        if (mapping[e.first.first] == -1) mapping[e.first.first] = (int32_t)n++;
        if (mapping[e.first.second] == -1) mapping[e.first.second] = (int32_t)n++;
        if (n >= target) break;
    }
    return n;
}

/* sample::detach (sample.cpp:12-26): vertices of degree above 1. */
int64_t sample_detach(const ora_graph* g, std::vector<int32_t>& mapping) {
    const std::vector<int64_t> d = graph_degrees(g);
    int64_t n = 0;
    for (int64_t v = 0; v < g->N; ++v)
        if (d[v] > 1) mapping[v] = (int32_t)n++;
    return n;
}

/* sample::from_vertices (sample.cpp:240-253): edges between sampled vertices, by source
 * vertex in ascending original id, each source's out-neighbours in order. */
ora_graph* from_vertices(const ora_graph* g, const std::vector<int32_t>& mapping, int64_t n) {
    std::vector<int32_t> src, dst;
    for (int64_t u = 0; u < g->N; ++u) {
        if (mapping[u] < 0) continue;
        for (int32_t v : g->out[u])
            if (mapping[v] >= 0) {
                src.push_back(mapping[u]);
                dst.push_back(mapping[v]);
            }
    }
    ora_graph* sub = ora_graph_create(n, (int64_t)src.size(), src.data(), dst.data());
    sub->und = g->und;  // args.undirected is global in the reference
    return sub;
}

/* sample::extend (sample.cpp:159-199): sampled vertices keep their block; the others, in
 * vertex order, take the block most of their already-assigned neighbours are in (ties to
 * the smallest block: the reference iterates a hash map), or a random block. */
void extend(const ora_graph* g, const std::vector<int32_t>& sample_asg, int64_t B, const std::vector<int32_t>& mapping,
            uint64_t seed, std::vector<int32_t>& asg) {
    asg.assign(g->N, -1);
    for (int64_t v = 0; v < g->N; ++v)
        if (mapping[v] >= 0) asg[v] = sample_asg[mapping[v]];
    for (int64_t v = 0; v < g->N; ++v) {
        if (asg[v] != -1) continue;
        std::map<int32_t, int64_t> counts;
        for (int32_t u : g->out[v])
            if (asg[u] != -1) counts[asg[u]]++;
        for (int32_t u : g->in[v])
            if (asg[u] != -1 && u != v) counts[asg[u]]++;
        if (counts.empty()) {
            uint32_t w[4];
            draw(seed, (uint32_t)v, 0, 0, DOM_EXTEND, w);
            asg[v] = (int32_t)u32_below(w[0], (uint32_t)B);
            continue;
        }
        int64_t best = 0;
        int32_t block = -1;
        for (const auto& e : counts)
            if (e.second > best) {
                best = e.second;
                block = e.first;
            }
        asg[v] = block;
    }
}

/* finetune::early_stop(iteration, initial_entropy, deltas) (finetune.cpp:285-294). */
bool early_stop3(int64_t iteration, double initial_entropy, const std::vector<double>& d) {
    if (iteration < 3) return false;
    const size_t last = d.size() - 1;
    double average = d[last] + d[last - 1] + d[last - 2];
    average /= -3.0;
    return average < 1e-4 * initial_entropy;
}

constexpr uint32_t kFinetuneStep = 0xffffffffu;

/* finetune::finetune_assignment (finetune.cpp:903-932): sequential MH over every vertex in
 * id order until the three-iteration average improvement falls below 1e-4 of the entropy. */
void finetune_assignment(ora_bm* bm, const ora_config* cfg, uint64_t seed, ora_stats* st) {
    const ora_graph* g = bm->g;
    bm->entropy = mdl_for(bm, cfg);
    if (bm->B < 2) return;  // one block: no move can be proposed (as the sweeps, finetune.cpp:567)
    std::vector<double> deltas;
    for (int it = 0; it < cfg->max_iterations; ++it) {
        double dsum = 0.0;
        for (int64_t v = 0; v < g->N; ++v) {
            double dS = 0.0;
            add_stats(st, g, v);
            if (mh_step(bm, v, seed, (uint32_t)it, kFinetuneStep, cfg, &dS)) {
                dsum += dS;
                if (st) st->moves++;
            }
        }
        deltas.push_back(dsum);
        if (st) st->mcmc_iterations++;
        if (early_stop3(it, bm->entropy, deltas)) break;
    }
    bm->entropy = mdl_for(bm, cfg);
}

int64_t sample_expansion_snowball(const ora_graph* g, double samplesize, uint64_t seed, std::vector<int32_t>& mapping);
int64_t sample_degree_product_snowball(const ora_graph* g, double samplesize, uint64_t seed,
                                       std::vector<int32_t>& mapping);

int64_t sample_any(const ora_graph* g, int32_t alg, double samplesize, uint64_t seed, std::vector<int32_t>& mapping) {
    mapping.assign(g->N, -1);
    switch (alg) {
        case 0: return sample_max_degree(g, samplesize, mapping);
        case 1: return sample_random(g, samplesize, seed, mapping);
        case 2: return sample_degree_product(g, samplesize, mapping);
        case 3: return sample_detach(g, mapping);
        case 4: return sample_expansion_snowball(g, samplesize, seed, mapping);
        case 5: return sample_degree_product_snowball(g, samplesize, seed, mapping);
        default: return -1;
    }
}

}  // namespace

namespace {

/* sample::reattach (sample.cpp:365-405) for the detached vertices (degree 0 or 1): a vertex
 * whose one neighbour is assigned takes its block; otherwise the vertex (and its unassigned
 * neighbour) take the vertex's random block. */
void reattach(const ora_graph* g, const std::vector<int32_t>& sample_asg, int64_t B,
              const std::vector<int32_t>& mapping, uint64_t seed, std::vector<int32_t>& asg) {
    asg.assign(g->N, -1);
    for (int64_t v = 0; v < g->N; ++v)
        if (mapping[v] >= 0) asg[v] = sample_asg[mapping[v]];
    for (int64_t v = 0; v < g->N; ++v) {
        if (asg[v] != -1) continue;
        uint32_t w[4];
        draw(seed, (uint32_t)v, 0, 0, DOM_REATTACH, w);
        const int32_t random_block_v = (int32_t)u32_below(w[0], (uint32_t)B);
        for (int32_t u : g->out[v]) {
            if (asg[u] == -1) {
                asg[v] = random_block_v;
                asg[u] = random_block_v;
                break;
            }
            asg[v] = asg[u];
        }
        for (int32_t u : g->in[v]) {
            if (asg[u] == -1) {
                asg[v] = random_block_v;
                asg[u] = random_block_v;
                break;
            }
            asg[v] = asg[u];
        }
        if (asg[v] < 0) asg[v] = random_block_v;
    }
}

/* The k-th draw of a snowball run: common::random_integer(lo, hi). */
struct SeqRng {
    uint64_t seed;
    uint32_t k = 0;
    int64_t operator()(int64_t lo, int64_t hi) {
        uint32_t w[4];
        draw(seed, k++, 0, 0, DOM_SNOWBALL, w);
        return lo + (int64_t)u64_below(w[0], w[1], (uint64_t)(hi - lo + 1));
    }
};

/* sample::expansion_snowball (sample.cpp:125-157, es_add_vertex :103-117,
 * es_update_contribution :119-130): grow the sample by the neighbour that adds the most
 * new neighbours. */
int64_t sample_expansion_snowball(const ora_graph* g, double samplesize, uint64_t seed, std::vector<int32_t>& mapping) {
    const int64_t N = g->N, target = sample_target(g, samplesize);
    SeqRng rng{seed};
    std::vector<int64_t> contribution(N, 0);
    std::vector<char> flag(N, 0);
    std::set<int64_t> neighbors;
    int64_t contribution_sum = 0, n = 0;
    auto update = [&](int64_t vertex) {
        for (int32_t nb : g->out[vertex]) {
            if (flag[nb] || mapping[nb] >= 0) continue;
            contribution[vertex]++;
            contribution_sum++;
        }
        for (int32_t nb : g->in[vertex])
            if (contribution[nb] > 0) {
                contribution[nb]--;
                contribution_sum--;
            }
    };
    auto add = [&](int64_t vertex) {
        mapping[vertex] = (int32_t)n++;
        for (int32_t nb : g->out[vertex]) {
            if (flag[nb] || mapping[nb] >= 0) continue;
            neighbors.insert(nb);
            flag[nb] = 1;
            if (contribution[nb] > 0) continue;
            update(nb);
        }
        neighbors.erase(vertex);
        flag[vertex] = 0;
    };
    add(rng(0, N - 1));
    while (n < target) {
        if (neighbors.empty()) {
            int64_t v;
            do v = rng(0, N - 1);
            while (mapping[v] >= 0);
            add(v);
            continue;
        } else if (contribution_sum == 0) {
            auto it = neighbors.begin();
            std::advance(it, rng(0, (int64_t)neighbors.size() - 1));
            add(*it);
            continue;
        }
        int64_t best = 0;
        for (int64_t v = 1; v < N; ++v)
            if (contribution[v] > contribution[best]) best = v;
        add(best);
    }
    return n;
}

/* sample::degree_product_snowball (sample.cpp:51-101): grow the sample along the frontier
 * edge of the largest degree product (ties: the earliest pushed edge). */
int64_t sample_degree_product_snowball(const ora_graph* g, double samplesize, uint64_t seed,
                                       std::vector<int32_t>& mapping) {
    const int64_t N = g->N;
    const std::vector<int64_t> d = graph_degrees(g);
    SeqRng rng{seed};
    // (degree product, -push sequence, source, destination): the largest product first, then
    // the earliest push
    std::priority_queue<std::tuple<int64_t, int64_t, int32_t, int32_t>> frontier;
    int64_t pushes = 0, n = 0;
    auto add = [&](int64_t vertex) {
        mapping[vertex] = (int32_t)n++;
        for (int32_t nb : g->out[vertex]) {
            if (mapping[nb] != -1) continue;
            frontier.push({d[vertex] * d[nb], -(pushes++), (int32_t)vertex, nb});
        }
        for (int32_t nb : g->in[vertex]) {
            if (mapping[nb] != -1) continue;
            frontier.push({d[nb] * d[vertex], -(pushes++), nb, (int32_t)vertex});
        }
    };
    add(rng(0, N - 1));
    const int64_t target = (int64_t)((double)N * samplesize);
    while (n < target) {
        if (frontier.empty()) {
            int64_t v;
            do v = rng(0, N - 1);
            while (mapping[v] >= 0);
            add(v);
            if (frontier.empty()) continue;  // the vertex had no unsampled neighbour
        }
        const auto next = frontier.top();
        frontier.pop();
        const int32_t src = std::get<2>(next), dst = std::get<3>(next);
        if (mapping[src] == -1) add(src);
        if (mapping[dst] == -1) add(dst);
    }
    return n;
}

}  // namespace

extern "C" void ora_reattach(const ora_graph* g, const int32_t* sample_asg, int64_t sample_n, int64_t B,
                             const int32_t* mapping, uint64_t seed, int32_t* out) {
    std::vector<int32_t> a;
    reattach(g, std::vector<int32_t>(sample_asg, sample_asg + sample_n), B,
             std::vector<int32_t>(mapping, mapping + g->N), seed, a);
    std::copy(a.begin(), a.end(), out);
}

extern "C" int64_t ora_sample(const ora_graph* g, int32_t alg, double samplesize, uint64_t seed, int32_t* mapping) {
    std::vector<int32_t> m;
    const int64_t n = sample_any(g, alg, samplesize, seed, m);
    if (mapping) std::copy(m.begin(), m.end(), mapping);
    return n;
}

extern "C" ora_graph* ora_subgraph(const ora_graph* g, const int32_t* mapping, int64_t n) {
    return from_vertices(g, std::vector<int32_t>(mapping, mapping + g->N), n);
}

extern "C" void ora_graph_edges(const ora_graph* g, int32_t* src, int32_t* dst) {
    int64_t i = 0;
    for (int64_t u = 0; u < g->N; ++u)
        for (int32_t v : g->out[u]) {
            src[i] = (int32_t)u;
            dst[i] = v;
            ++i;
        }
}

extern "C" int64_t ora_graph_num_edges(const ora_graph* g) { return g->E; }
extern "C" int64_t ora_graph_model_edges(const ora_graph* g) { return g->Em; }
extern "C" void ora_graph_set_model_edges(ora_graph* g, int64_t num_edges) { g->Em = num_edges; }
extern "C" void ora_graph_set_undirected(ora_graph* g, int32_t undirected) { g->und = undirected != 0; }

extern "C" void ora_graph_set_degree_corrected(ora_graph* g, int32_t on) { g->dc = on != 0; }

extern "C" double ora_log_q(int64_t n, int64_t k) { return dc_log_q(n, k); }

extern "C" double ora_spence(double x) { return x == 1.0 ? 0.0 : dc_li2(1.0 - x); }

extern "C" void ora_extend(const ora_graph* g, const int32_t* sample_asg, int64_t sample_n, int64_t B,
                           const int32_t* mapping, uint64_t seed, int32_t* out) {
    std::vector<int32_t> a;
    extend(g, std::vector<int32_t>(sample_asg, sample_asg + sample_n), B, std::vector<int32_t>(mapping, mapping + g->N),
           seed, a);
    std::copy(a.begin(), a.end(), out);
}

extern "C" int ora_finetune_assignment(ora_bm* bm, const ora_config* cfg, uint64_t seed, ora_stats* st) {
    finetune_assignment(bm, cfg, seed, st);
    return 0;
}

/* sbp::stochastic_block_partition (sbp.cpp:16-72) with BlockmodelTriplet::get_next_blockmodel
 * (blockmodel_triplet.cpp:4-37). */
extern "C" int64_t ora_sbp(const ora_graph* g, const ora_config* cfg, uint64_t seed, int32_t* out_asg,
                           double* out_mdl, ora_stats* st) {
    std::vector<int32_t> ident(g->N);
    for (int64_t v = 0; v < g->N; ++v) ident[v] = (int32_t)v;
    ora_bm* bm = ora_bm_create(g, g->N, ident.data());
    bm->entropy = DBL_MAX;
    Triplet t;
    int32_t step = 0;
    while (!t.optimal) {
        int rc = merge_blocks(bm, cfg, seed, (uint32_t)step, bm->num_blocks_to_merge, st);
        if (rc) {
            delete bm;
            return -1;
        }
        mcmc(bm, cfg, seed, step, t.golden_ratio_not_reached(), st);
        ++step;
        if (st) st->outer_steps++;
        // get_next_blockmodel
        t.update(bm);
        int64_t next_B, next_merge;
        const Slot* src;
        if (t.golden_ratio_not_reached()) {
            src = &t.s[1];
            next_B = src->B;
            next_merge = (int64_t)((double)next_B * 0.5);
            if (next_merge == 0) t.optimal = true;
        } else if (t.is_done()) {
            src = &t.s[1];
            next_merge = 0;
        } else {
            int index = 1;
            if (t.s[0].empty && t.s[1].B > t.s[2].B) index = 1;
            else if ((t.s[0].B - t.s[1].B) >= (t.s[1].B - t.s[2].B)) index = 0;
            else index = 1;
            int64_t next_try = t.s[index + 1].B;
            next_try += (int64_t)((double)(t.s[index].B - t.s[index + 1].B) * 0.618);
            src = &t.s[index];
            next_merge = src->B - next_try;
        }
        delete bm;
        bm = ora_bm_create(g, src->B, src->asg.data());
        bm->entropy = src->entropy;
        bm->num_blocks_to_merge = next_merge;
    }
    const int64_t B = bm->B;
    if (out_asg) std::copy(bm->asg.begin(), bm->asg.end(), out_asg);
    if (out_mdl) *out_mdl = bm->entropy;
    delete bm;
    return B;
}

extern "C" void ora_np_mdl(const ora_bm* bm, double* literal, double* canonical) {
    if (literal) {
        double t[4];
        np_terms_literal(bm, t);
        *literal = t[0] + (((0.0 + t[1]) + t[2]) + t[3]) * 1.0;  // S + S_dl * BETA_DL (entropy.cpp:751-779)
    }
    if (canonical) *canonical = np_mdl_canonical(bm);
}

extern "C" void ora_np_terms(const ora_bm* bm, double out[4]) { np_terms_literal(bm, out); }

extern "C" void ora_np_delta_mdl(const ora_bm* bm, int64_t v, int64_t s, double* literal, int64_t* fixed) {
    const DeltaMap d = vertex_delta(bm, v, s);
    const VertexInfo vi = vinfo(bm->g, v);
    const int64_t r = bm->asg[v];
    if (literal)
        *literal = r == s ? 0.0
                          : np_dS_literal(bm, r, s, d, vi.kout, vi.kin, 1) +
                                (bm->g->dc ? dc_vertex_delta(bm, dc_hist(bm), v, s, false) : 0.0);
    if (fixed) *fixed = np_vertex_dS(bm, v, s, d);
}

extern "C" void ora_np_merge_delta_mdl(const ora_bm* bm, int64_t r, int64_t s, double* literal, int64_t* fixed) {
    const DeltaMap d = merge_delta(bm, r, s);
    if (literal) {
        int64_t kout = 0, kin = 0;
        for (const auto& e : bm->row[r]) kout += e.second;
        for (const auto& e : bm->col[r]) kin += e.second;
        *literal = (r == s || bm->sizes[r] == 0 || bm->sizes[s] == 0) ? 0.0
                                                                       : np_dS_literal(bm, r, s, d, kout, kin, bm->sizes[r]);
    }
    if (fixed) *fixed = np_merge_dS(bm, r, s, d);
}

extern "C" int64_t ora_bm_nonempty(const ora_bm* bm) { return bm->nonempty; }

/* The sampled partition of main.cpp:98-140: sample, partition the sample, extend the
 * sample's blocks to the full graph, then finetune_assignment on the full graph. */
extern "C" int64_t ora_sbp_sampled(const ora_graph* g, const ora_config* cfg, uint64_t seed, int32_t alg,
                                   double samplesize, int32_t* out_asg, double* out_mdl, ora_stats* st) {
    std::vector<int32_t> mapping;
    const int64_t n = sample_any(g, alg, samplesize, seed, mapping);
    if (n <= 0) return -1;
    ora_graph* sg = from_vertices(g, mapping, n);
    std::vector<int32_t> sasg(n);
    double smdl = 0.0;
    const int64_t B = ora_sbp(sg, cfg, seed, sasg.data(), &smdl, st);
    ora_graph_destroy(sg);
    if (B <= 0) return -1;
    std::vector<int32_t> asg;
    extend(g, sasg, B, mapping, seed, asg);
    ora_bm* bm = ora_bm_create(g, B, asg.data());
    finetune_assignment(bm, cfg, seed, st);
    if (out_asg) std::copy(bm->asg.begin(), bm->asg.end(), out_asg);
    if (out_mdl) *out_mdl = bm->entropy;
    delete bm;
    return B;
}

// ---------------------------------------------------------------- top-down (divisive) SBP
namespace {

/* The random split of a cluster of n vertices (propose_random_split, top_down_sbp.cpp:
 * 248-260): the size of side 0 uniform in [long(0.2 n), long(0.8 n)], then each vertex on
 * side 0 with probability size / n. */
inline int64_t split_size(uint64_t seed, int64_t cluster, int32_t i, uint32_t step, int64_t n) {
    const int64_t lo = (int64_t)((double)n * 0.2), hi = (int64_t)((double)n * 0.8);
    uint32_t w[4];
    draw(seed, (uint32_t)cluster, (uint32_t)i, step, DOM_SPLIT_SIZE, w);
    return lo + (int64_t)u64_below(w[0], w[1], (uint64_t)(hi - lo + 1));
}
inline int split_side(uint64_t seed, int64_t v, int32_t i, uint32_t step, int64_t size, int64_t n) {
    uint32_t w[4];
    draw(seed, (uint32_t)v, (uint32_t)i, step, DOM_SPLIT_SIDE, w);
    return (uint64_t)w[0] * (uint64_t)n < ((uint64_t)size << 32) ? 0 : 1;
}

/* nonparametric::mdl (entropy.cpp:751-779) of a two-block model of a subgraph with n
 * vertices and E edges: sizes[2], cells M[2][2] (row-major).  The canonical form. */
double np_mdl_two_blocks(const ora_graph* g, int64_t n, int64_t E, const int64_t sizes[2], const int64_t M[4]) {
    int64_t fixed = 0;
    for (int k = 0; k < 4; ++k) fixed -= np_cell(g, k == 0 || k == 3, M[k], -M[k]);  // + eterm
    for (int b = 0; b < 2; ++b) {
        const int64_t dout = M[2 * b] + M[2 * b + 1], din = M[b] + M[2 + b];
        fixed += np_vterm(g, dout, din, sizes[b]) - g->LG[sizes[b]];
    }
    fixed += g->LG[n] + g->Lq[n];
    const int64_t ne = (sizes[0] > 0) + (sizes[1] > 0);
    return (double)fixed * kInvFix + (np_lbinom(n - 1, ne - 1) + np_edges_dl(ne, E, g->und));
}

/* entropy::null_mdl_v1 (entropy.cpp:571-585) of a subgraph: the one-block nonparametric
 * MDL under --nonparametric, else the parametric formula. */
double split_null_mdl(const ora_graph* g, int64_t n, int64_t E, bool nonparametric) {
    if (nonparametric) {
        const int64_t sizes[2] = {n, 0}, M[4] = {E, 0, 0, 0};
        return np_mdl_two_blocks(g, n, E, sizes, M);
    }
    const double e = (double)E;
    const double log_posterior_p = e * log(1.0 / e);
    const double x = 1.0 / e;
    const double h = ((1 + x) * log(1 + x)) - (x * log(x));
    return (e * h) - log_posterior_p;
}

/* A cluster's subgraph (extract_subgraph, top_down_sbp.cpp:100-130): local ids in vertex
 * order, the edges between its vertices; neighbors(v) = out-neighbours then in-neighbours
 * (Graph::neighbors, graph.cpp:174-183). */
struct ClusterGraph {
    int64_t n = 0;
    std::vector<std::vector<int32_t>> nbrs;
    std::vector<int64_t> deg;  // Graph::degrees: out + in - (has a self-loop)
};

ClusterGraph cluster_graph(const ora_graph* g, const std::vector<int32_t>& members, const std::vector<int32_t>& local) {
    ClusterGraph cg;
    cg.n = (int64_t)members.size();
    std::vector<std::vector<int32_t>> out(cg.n), in(cg.n);
    std::vector<char> self(cg.n, 0);
    for (int32_t u : members)
        for (int32_t v : g->out[u])
            if (local[v] >= 0) {
                out[local[u]].push_back(local[v]);
                in[local[v]].push_back(local[u]);
                if (u == v) self[local[u]] = 1;
            }
    cg.nbrs.resize(cg.n);
    cg.deg.resize(cg.n);
    for (int64_t x = 0; x < cg.n; ++x) {
        cg.nbrs[x] = out[x];
        cg.nbrs[x].insert(cg.nbrs[x].end(), in[x].begin(), in[x].end());
        cg.deg[x] = (int64_t)out[x].size() + (int64_t)in[x].size() - self[x];
    }
    return cg;
}

/* common::random_integer for the k-th draw of one split proposal. */
struct SplitRng {
    uint64_t seed;
    uint32_t cluster, proposal, step, k = 0;
    uint32_t word() {
        uint32_t w[4];
        draw(seed, cluster, proposal | (k++ << 8), step, DOM_SPLIT_SNOWBALL, w);
        return w[0];
    }
    int64_t operator()(int64_t lo, int64_t hi) {
        uint32_t w[4];
        draw(seed, cluster, proposal | (k++ << 8), step, DOM_SPLIT_SNOWBALL, w);
        return lo + (int64_t)u64_below(w[0], w[1], (uint64_t)(hi - lo + 1));
    }
};

/* split_init (top_down_sbp.cpp:532-583): two start vertices.  The reference's nth_element
 * leaves ties in an unspecified order; here the degree ranking is a stable descending sort.
 * degree-weighted draws from the top max(n / 10, 2) (the reference's n / 10 = 1 never ends). */
std::pair<int64_t, int64_t> split_init(const ClusterGraph& cg, int32_t kind, SplitRng& rng) {
    const int64_t n = cg.n;
    if (kind == 0 || n < 10) {
        const int64_t a = rng(0, n - 1);
        int64_t b = rng(0, n - 1);
        while (b == a) b = rng(0, n - 1);
        return {a, b};
    }
    std::vector<int64_t> idx(n);
    for (int64_t x = 0; x < n; ++x) idx[x] = x;
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return cg.deg[a] > cg.deg[b]; });
    if (kind == 2) return {idx[0], idx[1]};
    const int64_t m = std::max<int64_t>(n / 10, 2);
    const int64_t a = rng(0, m - 1);
    int64_t b = rng(0, m - 1);
    while (b == a) b = rng(0, m - 1);
    return {idx[a], idx[b]};
}

/* propose_snowball_split (top_down_sbp.cpp:313-363): two snowballs; each step picks a side
 * with the split-size odds and takes the smallest vertex of its frontier (or the smallest
 * unsampled vertex). */
std::vector<int8_t> snowball_split(const ClusterGraph& cg, int32_t init, SplitRng& rng) {
    const int64_t n = cg.n;
    std::vector<int8_t> side(n, -1);
    std::set<int64_t> unsampled;
    for (int64_t x = 0; x < n; ++x) unsampled.insert(x);
    std::set<int64_t> frontier[2];
    const auto st = split_init(cg, init, rng);
    const int64_t start[2] = {st.first, st.second};
    for (int id = 0; id < 2; ++id) {
        side[start[id]] = (int8_t)id;
        unsampled.erase(start[id]);
    }
    for (int id = 0; id < 2; ++id)
        for (int32_t y : cg.nbrs[start[id]])
            if (side[y] == -1) frontier[id].insert(y);
    const int64_t size = rng((int64_t)((double)n * 0.2), (int64_t)((double)n * 0.8));
    while (!unsampled.empty()) {
        const int id = (uint64_t)rng.word() * (uint64_t)n < ((uint64_t)size << 32) ? 0 : 1;
        const int64_t sel = frontier[id].empty() ? *unsampled.begin() : *frontier[id].begin();
        side[sel] = (int8_t)id;
        unsampled.erase(sel);
        frontier[0].erase(sel);
        frontier[1].erase(sel);
        for (int32_t y : cg.nbrs[sel])
            if (side[y] == -1) frontier[id].insert(y);
    }
    return side;
}

/* propose_single_snowball_split (top_down_sbp.cpp:382-426): one snowball grown level by level
 * until it holds the target number of vertices.  As in the reference, the membership test
 * `sampled[vertex]` of a map counts every vertex it looks at. */
std::vector<int8_t> single_snowball_split(const ClusterGraph& cg, int32_t init, SplitRng& rng) {
    const int64_t n = cg.n;
    std::vector<int8_t> side(n, 0);
    std::map<int64_t, bool> sampled, frontier, next_frontier;
    const int64_t start = split_init(cg, init, rng).first;
    side[start] = 1;
    sampled[start] = true;
    for (int32_t y : cg.nbrs[start])
        if (side[y] != 1) frontier[y] = true;
    const uint64_t target = (uint64_t)rng((int64_t)((double)n * 0.2), (int64_t)((double)n * 0.8));
    while (sampled.size() < target) {
        if (frontier.empty() && next_frontier.empty()) break;
        for (const auto& e : frontier) {
            const int64_t x = e.first;
            if (!sampled[x]) {
                side[x] = 1;
                sampled[x] = true;
                for (int32_t y : cg.nbrs[x])
                    if (side[y] != 1) next_frontier[y] = true;
            }
            if (sampled.size() >= target) break;
        }
        frontier = std::move(next_frontier);
        next_frontier.clear();
    }
    return side;
}

/* propose_connectivity_snowball_split (top_down_sbp.cpp:262-311): two seeds, then level by
 * level every frontier vertex joins the side most of its assigned neighbours are on. */
std::vector<int8_t> connectivity_snowball_split(const ClusterGraph& cg, int32_t init, SplitRng& rng) {
    const int64_t n = cg.n;
    std::vector<int8_t> side(n, -1);
    std::set<int64_t> unsampled;
    for (int64_t x = 0; x < n; ++x) unsampled.insert(x);
    std::map<int64_t, bool> frontier, next_frontier;
    const auto st = split_init(cg, init, rng);
    const int64_t start[2] = {st.first, st.second};
    for (int id = 0; id < 2; ++id) {
        side[start[id]] = (int8_t)id;
        unsampled.erase(start[id]);
    }
    for (int id = 0; id < 2; ++id)
        for (int32_t y : cg.nbrs[start[id]])
            if (side[y] == -1) frontier[y] = true;
    auto sample_vertex = [&](int64_t x) {
        int e0 = 0, e1 = 0;
        for (int32_t y : cg.nbrs[x]) {
            if (side[y] == 0) e0++;
            if (side[y] == 1) e1++;
            if (side[y] != -1) continue;
            next_frontier[y] = true;
        }
        side[x] = e1 > e0 ? 1 : 0;
        unsampled.erase(x);
        frontier[x] = false;
    };
    while (!unsampled.empty()) {
        if (frontier.empty()) {
            sample_vertex(*unsampled.begin());
            continue;
        }
        for (const auto& e : frontier) sample_vertex(e.first);
        frontier = std::move(next_frontier);
        next_frontier.clear();
    }
    return side;
}

/* The sides of proposal i of cluster c (local ids): propose_random_split or a snowball. */
std::vector<int8_t> split_sides(const ora_graph* g, const ora_config* cfg, const std::vector<int32_t>& members,
                                const ClusterGraph* cg, uint64_t seed, int64_t c, int32_t i, uint32_t step) {
    const int64_t n = (int64_t)members.size();
    std::vector<int8_t> side(n, 0);
    if (n < 2) return side;
    if (cfg->split == 0) {
        const int64_t size = split_size(seed, c, i, step, n);
        for (int64_t x = 0; x < n; ++x) side[x] = (int8_t)split_side(seed, members[x], i, step, size, n);
        return side;
    }
    SplitRng rng{seed, (uint32_t)c, (uint32_t)i, step};
    if (cfg->split == 1) return snowball_split(*cg, cfg->splitinit, rng);
    if (cfg->split == 2) return single_snowball_split(*cg, cfg->splitinit, rng);
    return connectivity_snowball_split(*cg, cfg->splitinit, rng);
}

/* divisive::split_communities (top_down_sbp.cpp:472-530) and apply_best_splits (:30-65). */
void split_communities(ora_bm* bm, const ora_config* cfg, uint64_t seed, uint32_t step, int64_t target) {
    const ora_graph* g = bm->g;
    const int64_t B = bm->B, N = g->N;
    std::vector<std::vector<int32_t>> members(B);
    for (int64_t v = 0; v < N; ++v) members[bm->asg[v]].push_back((int32_t)v);
    std::vector<double> best(B, DBL_MAX);
    std::vector<int32_t> best_i(B, -1);
    std::vector<int64_t> split_n(B, INT64_MAX);  // Split::num_vertices; unset splits are skipped
    std::vector<int32_t> local(N, -1);
    for (int64_t c = 0; c < B; ++c) {
        const int64_t n = (int64_t)members[c].size();
        if ((double)n < 0.001 * (double)N) continue;  // do not split small clusters
        for (int64_t x = 0; x < n; ++x) local[members[c][x]] = (int32_t)x;
        int64_t E = 0;
        for (int32_t u : members[c])
            for (int32_t v : g->out[u]) E += bm->asg[v] == c;
        const double old_entropy = split_null_mdl(g, n, E, cfg->nonparametric != 0);
        ClusterGraph cg;
        if (cfg->split != 0 && n >= 2) cg = cluster_graph(g, members[c], local);
        for (int32_t i = 0; i < 10; ++i) {  // NUM_AGG_PROPOSALS_PER_BLOCK
            const std::vector<int8_t> sd = split_sides(g, cfg, members[c], &cg, seed, c, i, step);
            int64_t sizes[2] = {0, 0}, M[4] = {0, 0, 0, 0};
            for (int32_t u : members[c]) {
                sizes[sd[local[u]]]++;
                for (int32_t v : g->out[u])
                    if (bm->asg[v] == c) M[2 * sd[local[u]] + sd[local[v]]]++;
            }
            const double delta = np_mdl_two_blocks(g, n, E, sizes, M) - old_entropy;
            if (delta < best[c]) {
                best[c] = delta;
                best_i[c] = i;
                split_n[c] = n;
            }
        }
        for (int32_t u : members[c]) local[u] = -1;
    }
    // apply_best_splits: ascending delta (utils::argsort is a stable descending sort, walked
    // from its end)
    std::vector<int64_t> order(B);
    for (int64_t c = 0; c < B; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return best[a] > best[b]; });
    int64_t num_blocks = B;
    for (int64_t k = B - 1; k >= 0; --k) {
        const int64_t c = order[k];
        if (split_n[c] > N) continue;
        const int32_t i = best_i[c];
        for (int64_t x = 0; x < (int64_t)members[c].size(); ++x) local[members[c][x]] = (int32_t)x;
        ClusterGraph cg;
        if (cfg->split != 0 && members[c].size() >= 2) cg = cluster_graph(g, members[c], local);
        const std::vector<int8_t> sd = split_sides(g, cfg, members[c], &cg, seed, c, i, step);
        for (int32_t u : members[c]) local[u] = -1;
        for (int64_t x = 0; x < (int64_t)members[c].size(); ++x)
            if (sd[x] == 1) bm->asg[members[c][x]] = (int32_t)num_blocks;
        num_blocks++;
        if (num_blocks >= target) break;
    }
    bm->B = num_blocks;
    build(bm);
}

/* TopDownBlockmodelTriplet (blockmodel_triplet.cpp:107-193). */
struct TDTriplet {
    Slot s[3];
    bool optimal = false;
    bool golden_ratio_not_reached() const { return s[2].empty; }
    void update(const ora_bm* bm) {
        int idx;
        if (s[1].empty) {
            idx = 1;
        } else if (bm->entropy <= s[1].entropy && std::labs(bm->B - s[1].B) > 0.1 * (double)s[1].B) {
            const int old = s[1].B < bm->B ? 0 : 2;
            s[old] = s[1];
            idx = 1;
        } else {
            idx = s[1].B < bm->B ? 2 : 0;
        }
        s[idx].empty = false;
        s[idx].B = bm->B;
        s[idx].entropy = bm->entropy;
        s[idx].asg = bm->asg;
    }
    bool is_done() {
        if ((!s[0].empty && s[2].B - s[0].B <= 2) || (s[0].empty && s[2].B - s[1].B <= 1)) optimal = true;
        return optimal;
    }
};

}  // namespace

/* divisive::run (top_down_sbp.cpp:435-470) without --mix: from one block, split toward
 * ceil(1.5 B) blocks until the golden-section bracket closes, finetuning after each split. */
extern "C" int64_t ora_top_down(const ora_graph* g, const ora_config* cfg, uint64_t seed, int32_t mix,
                                int32_t* out_asg, double* out_mdl, ora_stats* st) {
    std::vector<int32_t> zeros(g->N, 0);
    ora_bm* bm = ora_bm_create(g, 1, zeros.data());
    bm->entropy = DBL_MAX;
    TDTriplet t;
    uint32_t step = 0;
    auto next = [&](ora_bm* cur, int64_t* target) -> const Slot* {
        t.update(cur);
        if (t.golden_ratio_not_reached()) {
            *target = (int64_t)ceil((double)t.s[1].B * 1.5);
            if (*target == 0 || *target >= g->N) t.optimal = true;
            return &t.s[1];
        }
        if (t.is_done()) return &t.s[1];
        int index;
        if (t.s[0].empty && t.s[1].B < t.s[2].B) index = 1;
        else if ((t.s[1].B - t.s[0].B) <= (t.s[2].B - t.s[1].B)) index = 1;
        else index = 0;
        *target = t.s[index + 1].B + (int64_t)((double)(t.s[index].B - t.s[index + 1].B) * 0.618);
        return &t.s[index];
    };
    int64_t target = 0;
    const Slot* src = next(bm, &target);
    // end_condition_not_reached (top_down_sbp.cpp:428-433): with --mix, until the bracket forms
    while (mix ? t.golden_ratio_not_reached() : !t.optimal) {
        delete bm;
        bm = ora_bm_create(g, src->B, src->asg.data());
        bm->entropy = src->entropy;
        split_communities(bm, cfg, seed, step, target);
        mcmc(bm, cfg, seed, (int32_t)step, t.golden_ratio_not_reached(), st);
        ++step;
        if (st) st->outer_steps++;
        src = next(bm, &target);
    }
    Slot result = *src;
    if (mix) {
        /* continue_agglomerative (top_down_sbp.cpp:67-98): an agglomerative triplet fed the three
         * top-down blockmodels in slot order, then merges and finetuning until it is done; the
         * finetuning keeps the top-down triplet's (reached) golden-ratio state. */
        Triplet gr;
        const Slot* gs = nullptr;
        int64_t next_merge = 0;
        for (int k = 0; k < 3; ++k) {
            gr.update(t.s[k].B, t.s[k].entropy, t.s[k].asg);
            gs = gr.next(&next_merge);
        }
        while (!gr.optimal) {
            delete bm;
            bm = ora_bm_create(g, gs->B, gs->asg.data());
            bm->entropy = gs->entropy;
            merge_blocks(bm, cfg, seed, step, next_merge, st);
            mcmc(bm, cfg, seed, (int32_t)step, t.golden_ratio_not_reached(), st);
            ++step;
            if (st) st->outer_steps++;
            gr.update(bm);
            gs = gr.next(&next_merge);
        }
        result = *gs;
    }
    src = &result;
    const int64_t B = src->B;
    if (out_asg) std::copy(src->asg.begin(), src->asg.end(), out_asg);
    if (out_mdl) *out_mdl = src->entropy;
    delete bm;
    return B;
}

extern "C" int ora_split_communities(ora_bm* bm, const ora_config* cfg, uint64_t seed, uint32_t step,
                                     int64_t target) {
    split_communities(bm, cfg, seed, step, target);
    return 0;
}

extern "C" double ora_null_mdl_v1(double E) {
    const double log_posterior_p = E * log(1.0 / E);
    const double x = 1.0 / E;
    const double h = ((1 + x) * log(1 + x)) - (x * log(x));
    return (E * h) - log_posterior_p;
}

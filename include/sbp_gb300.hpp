/*
 * sbp_gb300.hpp -- C++ host interface over the sbpgpu C ABI (sbpgpu.h), mirroring the
 * hot-path API of vtsynergy/SBP so that callers of the reference can switch:
 *
 *   Args / args                 include/args.hpp:14-213, src/globals.cpp:5
 *   Graph                       include/graph.hpp:29-127
 *   Blockmodel                  include/blockmodel/blockmodel.hpp:46-219
 *   entropy::mdl, delta_mdl, block_merge_delta_mdl, null_mdl_v1, normalize_mdl_v1
 *                               include/entropy.hpp:33-81
 *   finetune::mcmc, asynchronous_gibbs, hybrid_mcmc, metropolis_hastings, accept,
 *   early_stop, edge_weights, blockmodel_delta, propose_move, move_vertex,
 *   propose_gibbs_move_v3 (and the batched propose_gibbs_moves)
 *                               include/finetune.hpp:36-157
 *   EdgeWeights, VertexMove     include/typedefs.hpp:16-38, 124-129
 *   utils::ProposalAndEdgeCounts
 *                               include/utils.hpp:24-30
 *   Delta                       include/blockmodel/sparse/delta.hpp:22-148
 *   BlockMatrix (blockmatrix()) include/blockmodel/sparse/csparse_matrix.hpp:45-112
 *   BlockmodelTriplet           include/blockmodel/blockmodel_triplet.hpp:12-42
 *   sbp::done_blockmodeling     src/sbp.cpp:74-86
 *   block_merge::merge_blocks, merge_proposals (propose_merge_sparse for every block)
 *                               include/block_merge.hpp:32-56
 *   sbp::stochastic_block_partition
 *                               include/sbp.hpp:18
 *
 * Header-only; link with libsbpgpu.so.  All state of a Graph and a Blockmodel lives on
 * the GPU; host vectors returned by the accessors are copies read back on demand and
 * refreshed after every operation that changes the blockmodel.
 *
 * Differences from the reference, by design:
 *   - randomness comes from the seeded Philox stream (Args::seed), so runs repeat;
 *   - finetune::mcmc takes the golden-ratio flag or a BlockmodelTriplet;
 *     block_merge::merge_blocks, propose_move and move_vertex take optional
 *     iteration/step numbers that key their proposal stream;
 *   - blockmatrix() returns a read-only host snapshot, not the live device matrix;
 *   - delta_mdl / block_merge_delta_mdl take (block or vertex, proposal) instead of a
 *     Delta; batched forms score many moves per call.
 * Errors: invalid arguments throw std::invalid_argument (as the reference); device
 * errors and unsupported configurations throw sbp_gb300::Error.
 */
#ifndef SBP_GB300_HPP
#define SBP_GB300_HPP

#include <climits>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <set>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "sbpgpu.h"

namespace sbp_gb300 {

class Error : public std::runtime_error {
  public:
    Error(sbpgpu_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    sbpgpu_status status;
};

inline void check(sbpgpu_status s, const sbpgpu_ctx* ctx) {
    if (s == SBPGPU_OK) return;
    const std::string m = ctx ? sbpgpu_last_error(ctx) : "sbpgpu call failed";
    if (s == SBPGPU_EINVAL) throw std::invalid_argument(m);
    throw Error(s, m);
}

/// One CUDA device and stream.  Context::global() is the process-wide default on device 0.
class Context {
  public:
    explicit Context(int device = 0) { check(sbpgpu_ctx_create(device, &h_), nullptr); }
    ~Context() {
        if (h_) sbpgpu_ctx_destroy(h_);  // device memory is released after its last graph
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    sbpgpu_ctx* get() const { return h_; }
    static Context& global() {
        static Context c(0);
        return c;
    }

  private:
    sbpgpu_ctx* h_ = nullptr;
};

/// The hot-path subset of the reference's Args.
struct Args {
    std::string algorithm = "hybrid_mcmc";  // async_gibbs | hybrid_mcmc | metropolis_hastings
    int batches = 1;
    float mh_percent = 0.075f;
    bool greedy = true;
    bool ordered = false;
    bool approximate = false;
    int asynciterations = INT_MAX;
    bool nonparametric = false;       // entropy::nonparametric
    bool degreecorrected = false;     // args.degreecorrected (include/args.hpp:24): the degree-
                                      // corrected nonparametric description length; graphs built
                                      // while it is set take it (evaluation and single moves only)
    bool undirected = false;          // args.undirected (include/args.hpp:55): the nonparametric
                                      // entropy's undirected form; graphs built while it is set
                                      // take it, and stochastic_block_partition applies it
    int threads = 1;                  // accepted for compatibility; the device uses every SM
    uint64_t seed = 0;                // seeds the proposal stream
    int max_iterations = 100;         // MAX_NUM_ITERATIONS (include/finetune.hpp:34)
    double samplesize = 1.0;          // --samplesize: below 1, partition a sample (src/main.cpp:98-140)
    std::string samplingalg = "random";  // random | max_degree | degree_product | *_snowball
    bool detach = false;              // --detach: set degree-0/1 vertices aside, reattach them
    bool mix = false;                 // --mix: top-down, then agglomerative (top_down_sbp.cpp:67-98)
    std::string split = "random";     // --split: random | snowball | single-snowball | connectivity-snowball
    std::string splitinit = "random";  // --splitinit: random | degree-weighted | high-degree
};

/// The global arguments, as the reference's `args`.
inline Args args;

inline sbpgpu_config to_config(const Args& a) {
    sbpgpu_config c;
    sbpgpu_default_config(&c);
    if (a.algorithm == "async_gibbs") c.algorithm = 0;
    else if (a.algorithm == "hybrid_mcmc") c.algorithm = 1;
    else if (a.algorithm == "metropolis_hastings") c.algorithm = 2;
    else throw std::invalid_argument("unknown algorithm: " + a.algorithm);
    if (a.batches < 1) throw std::invalid_argument("batches must be >= 1");
    c.batches = a.batches;
    c.mh_percent = a.mh_percent;
    c.greedy = a.greedy && !a.nonparametric ? 1 : 0;  // --nonparametric sets greedy off (args.hpp:204-207)
    c.nonparametric = a.nonparametric ? 1 : 0;
    if (a.split == "random") c.split = 0;
    else if (a.split == "snowball") c.split = 1;
    else if (a.split == "single-snowball") c.split = 2;
    else if (a.split == "connectivity-snowball") c.split = 3;
    else throw std::invalid_argument("Invalid split type provided.");
    if (a.splitinit == "random") c.splitinit = 0;
    else if (a.splitinit == "degree-weighted") c.splitinit = 1;
    else if (a.splitinit == "high-degree") c.splitinit = 2;
    else throw std::logic_error("This init split type has not been implemented yet.");
    c.ordered = a.ordered ? 1 : 0;
    c.approximate = a.approximate ? 1 : 0;
    c.asynciterations = a.asynciterations;
    c.max_iterations = a.max_iterations;
    return c;
}

using NeighborList = std::vector<std::vector<long>>;

/// A directed graph resident on the device.  Edges keep their insertion order
/// (Graph::add_edge, src/graph.cpp:10-18); self-loops and duplicates are kept.
class Graph {
  public:
    Graph(long num_vertices, const std::vector<std::pair<long, long>>& edges, Context& ctx = Context::global())
        : ctx_(&ctx), n_(num_vertices), out_(num_vertices), in_(num_vertices) {
        std::vector<int32_t> src, dst;
        src.reserve(edges.size());
        dst.reserve(edges.size());
        for (const auto& e : edges) {
            if (e.first < 0 || e.first >= num_vertices || e.second < 0 || e.second >= num_vertices)
                throw std::invalid_argument("edge endpoint out of range");
            src.push_back((int32_t)e.first);
            dst.push_back((int32_t)e.second);
            out_[e.first].push_back(e.second);
            in_[e.second].push_back(e.first);
        }
        upload(src, dst);
    }
    /// From neighbour lists (Graph(out, in, N, E)): the edges are taken from the
    /// out-neighbour lists in vertex order; num_edges is kept as Graph::num_edges, the count
    /// the description lengths use (half the stored edges for an undirected edge list,
    /// src/graph.cpp:145-147).
    Graph(const NeighborList& out_neighbors, const NeighborList& in_neighbors, long num_vertices, long num_edges,
          Context& ctx = Context::global())
        : ctx_(&ctx), n_(num_vertices), out_(out_neighbors), in_(in_neighbors) {
        std::vector<int32_t> src, dst;
        src.reserve(num_edges);
        dst.reserve(num_edges);
        for (long v = 0; v < (long)out_neighbors.size(); ++v)
            for (long u : out_neighbors[v]) {
                src.push_back((int32_t)v);
                dst.push_back((int32_t)u);
            }
        upload(src, dst);
        if (num_edges != e_) {
            check(sbpgpu_graph_set_model_edges(h_, num_edges), ctx_->get());
            e_ = num_edges;
        }
    }
    Graph(const Graph&) = delete;
    Graph& operator=(const Graph&) = delete;
    ~Graph() {
        if (h_) sbpgpu_graph_destroy(h_);
    }
    long num_vertices() const { return n_; }
    long num_edges() const { return e_; }
    const NeighborList& out_neighbors() const { return out_; }
    const NeighborList& in_neighbors() const { return in_; }
    const std::vector<long>& out_neighbors(long v) const { return out_[v]; }
    const std::vector<long>& in_neighbors(long v) const { return in_[v]; }
    /// The true assignment, -1 where unknown (Graph::assignment, include/graph.hpp:74-78).
    const std::vector<long>& assignment() const { return assignment_; }
    void assignment(const std::vector<long>& a) { assignment_ = a; }
    long assignment(long v) const { return assignment_[v]; }
    void assign(long v, long block) { assignment_[v] = block; }
    sbpgpu_graph* handle() const { return h_; }
    Context& context() const { return *ctx_; }

  private:
    void upload(const std::vector<int32_t>& src, const std::vector<int32_t>& dst) {
        e_ = (long)src.size();
        assignment_.assign(n_, -1);
        check(sbpgpu_graph_create(ctx_->get(), n_, e_, src.data(), dst.data(), &h_), ctx_->get());
        if (args.undirected) check(sbpgpu_graph_set_undirected(h_, 1), ctx_->get());
        if (args.degreecorrected) check(sbpgpu_graph_set_degree_corrected(h_, 1), ctx_->get());
    }
    Context* ctx_;
    long n_ = 0, e_ = 0;
    NeighborList out_, in_;
    std::vector<long> assignment_;
    sbpgpu_graph* h_ = nullptr;
};

/// EdgeWeights (include/typedefs.hpp:16-38): the far endpoint of each edge (or the block of
/// each cell) and its weight.
struct EdgeWeights {
    std::vector<long> indices;
    std::vector<long> values;
};

/// A read-only host snapshot of the block-edge-count matrix with the reference's
/// ISparseMatrix query interface (include/blockmodel/sparse/csparse_matrix.hpp:45-112).
/// Rows and columns iterate in ascending block order, the canonical order of this
/// implementation.  Taken by Blockmodel::blockmatrix(); it does not follow later changes.
class BlockMatrix {
  public:
    using SparseVector = std::map<long, long>;
    BlockMatrix(long num_blocks, const std::vector<std::tuple<long, long, long>>& cells)
        : rows_(num_blocks), cols_(num_blocks) {
        for (const auto& c : cells) {
            rows_[std::get<0>(c)][std::get<1>(c)] = std::get<2>(c);
            cols_[std::get<1>(c)][std::get<0>(c)] = std::get<2>(c);
            edges_ += std::get<2>(c);
        }
    }
    long get(long row, long col) const {
        check_index(row);
        check_index(col);
        const auto it = rows_[row].find(col);
        return it == rows_[row].end() ? 0 : it->second;
    }
    std::vector<long> getrow(long row) const {
        check_index(row);
        std::vector<long> v(rows_.size(), 0);
        for (const auto& e : rows_[row]) v[e.first] = e.second;
        return v;
    }
    std::vector<long> getcol(long col) const {
        check_index(col);
        std::vector<long> v(cols_.size(), 0);
        for (const auto& e : cols_[col]) v[e.first] = e.second;
        return v;
    }
    const SparseVector& getrow_sparse(long row) const {
        check_index(row);
        return rows_[row];
    }
    const SparseVector& getcol_sparse(long col) const {
        check_index(col);
        return cols_[col];
    }
    /// Blocks with edges out of / into `block`, with the edge counts.
    EdgeWeights outgoing_edges(long block) const { return weights(getrow_sparse(block)); }
    EdgeWeights incoming_edges(long block) const { return weights(getcol_sparse(block)); }
    /// Row and column of `block` summed per neighbouring block (neighbors_weights).
    SparseVector neighbors_weights(long block) const {
        SparseVector w = getrow_sparse(block);
        for (const auto& e : getcol_sparse(block)) w[e.first] += e.second;
        return w;
    }
    std::set<long> neighbors(long block) const {
        std::set<long> n;
        for (const auto& e : neighbors_weights(block)) n.insert(e.first);
        return n;
    }
    long distinct_edges(long block) const { return (long)neighbors_weights(block).size(); }
    std::vector<std::tuple<long, long, long>> entries() const {
        std::vector<std::tuple<long, long, long>> out;
        for (long r = 0; r < (long)rows_.size(); ++r)
            for (const auto& e : rows_[r]) out.emplace_back(r, e.first, e.second);
        return out;
    }
    long edges() const { return edges_; }
    long trace() const {
        long t = 0;
        for (long b = 0; b < (long)rows_.size(); ++b) t += get(b, b);
        return t;
    }
    /// Row sums (axis 0) or column sums (axis 1).
    std::vector<long> sum(long axis = 0) const {
        std::vector<long> out(rows_.size(), 0);
        const auto& lines = axis == 0 ? rows_ : cols_;
        for (long b = 0; b < (long)lines.size(); ++b)
            for (const auto& e : lines[b]) out[b] += e.second;
        return out;
    }

  private:
    void check_index(long b) const {
        if (b < 0 || b >= (long)rows_.size()) throw std::out_of_range("block index out of range");
    }
    static EdgeWeights weights(const SparseVector& v) {
        EdgeWeights w;
        for (const auto& e : v) {
            w.indices.push_back(e.first);
            w.values.push_back(e.second);
        }
        return w;
    }
    std::vector<SparseVector> rows_, cols_;
    long edges_ = 0;
};

/// The blockmodel: assignment, block degrees and sizes, and the block-edge-count matrix,
/// all on the device (Blockmodel::initialize_edge_counts, src/blockmodel/blockmodel.cpp:193-276).
class Blockmodel {
  public:
    Blockmodel(long num_blocks, const Graph& graph, double block_reduction_rate,
               const std::vector<long>& block_assignment)
        : graph_(&graph), rate_(block_reduction_rate) {
        if ((long)block_assignment.size() != graph.num_vertices())
            throw std::invalid_argument("assignment must have one block per vertex");
        std::vector<int32_t> a(block_assignment.begin(), block_assignment.end());
        sbpgpu_bm* h = nullptr;
        check(sbpgpu_bm_create(graph.handle(), num_blocks, a.data(), &h), ctx());
        h_.reset(h);
        num_blocks_to_merge_ = (long)(num_blocks * rate_);
    }
    /// Every vertex in its own block is the reference's starting point (src/sbp.cpp:23);
    /// here num_blocks must equal the number of vertices.
    Blockmodel(long num_blocks, const Graph& graph, double block_reduction_rate)
        : Blockmodel(num_blocks, graph, block_reduction_rate, range(graph.num_vertices())) {}
    /// An empty Blockmodel (Blockmodel(), include/blockmodel/blockmodel.hpp): `empty` is
    /// true and it holds no device state; used for the slots of a BlockmodelTriplet.
    Blockmodel() : graph_(nullptr) { empty = true; }
    Blockmodel(Blockmodel&&) = default;
    Blockmodel& operator=(Blockmodel&&) = default;

    /// Blockmodel::copy (src/blockmodel/blockmodel.cpp:139-153), device to device.
    Blockmodel copy() const {
        if (!h_) return Blockmodel();
        sbpgpu_bm* h = nullptr;
        check(sbpgpu_bm_copy(h_.get(), &h), ctx());
        Blockmodel b(graph_, rate_, h);
        b.entropy_ = entropy_;
        b.num_blocks_to_merge_ = num_blocks_to_merge_;
        return b;
    }

    long num_blocks() const { return h_ ? (long)sbpgpu_bm_num_blocks(h_.get()) : 0; }
    const std::vector<long>& block_assignment() const { return view().assignment; }
    long block_assignment(long vertex) const { return view().assignment.at(vertex); }
    const std::vector<long>& degrees_out() const { return view().d_out; }
    const std::vector<long>& degrees_in() const { return view().d_in; }
    const std::vector<long>& degrees() const { return view().d_tot; }
    long degrees_out(long b) const { return view().d_out.at(b); }
    long degrees_in(long b) const { return view().d_in.at(b); }
    long degrees(long b) const { return view().d_tot.at(b); }
    long block_size(long b) const { return view().sizes.at(b); }
    /// The non-zero cells of the blockmatrix, row-major ascending: (row, col, count).
    std::vector<std::tuple<long, long, long>> blockmatrix_cells() const {
        if (!h_) throw std::logic_error("empty blockmodel");
        const int64_t nnz = sbpgpu_bm_nnz(h_.get());
        std::vector<int32_t> r(nnz), c(nnz);
        std::vector<int64_t> v(nnz);
        check(sbpgpu_bm_read(h_.get(), nullptr, nullptr, nullptr, nullptr, nullptr, r.data(), c.data(), v.data()),
              ctx());
        std::vector<std::tuple<long, long, long>> out(nnz);
        for (int64_t i = 0; i < nnz; ++i) out[i] = std::make_tuple((long)r[i], (long)c[i], (long)v[i]);
        return out;
    }
    /// Blockmodel::blockmatrix (include/blockmodel/blockmodel.hpp): a host snapshot of the
    /// current block-edge-count matrix.
    std::shared_ptr<const BlockMatrix> blockmatrix() const {
        return std::make_shared<const BlockMatrix>(num_blocks(), blockmatrix_cells());
    }
    /// Blockmodel::block_size over all blocks (block_sizes()).
    const std::vector<long>& block_sizes() const { return view().sizes; }
    /// true for a Blockmodel slot of a BlockmodelTriplet that holds nothing yet.
    bool empty = false;
    double getOverall_entropy() const { return entropy_; }
    void setOverall_entropy(double e) { entropy_ = e; }
    long getNum_blocks_to_merge() const { return num_blocks_to_merge_; }
    void setNum_blocks_to_merge(long n) { num_blocks_to_merge_ = n; }
    double getBlock_reduction_rate() const { return rate_; }

    sbpgpu_bm* handle() const { return h_.get(); }
    const Graph& graph() const { return *graph_; }
    /// Marks the host copies stale (every device-side mutation calls it).
    void invalidate() { view_.reset(); }

  private:
    struct View {
        std::vector<long> assignment, d_out, d_in, d_tot, sizes;
    };
    struct Deleter {
        void operator()(sbpgpu_bm* b) const { sbpgpu_bm_destroy(b); }
    };
    Blockmodel(const Graph* g, double rate, sbpgpu_bm* h) : graph_(g), rate_(rate), h_(h) {}
    static std::vector<long> range(long n) {
        std::vector<long> a(n);
        for (long i = 0; i < n; ++i) a[i] = i;
        return a;
    }
    sbpgpu_ctx* ctx() const { return graph_->context().get(); }
    const View& view() const {
        if (!h_) throw std::logic_error("empty blockmodel");
        if (!view_) {
            const long n = graph_->num_vertices(), B = num_blocks();
            std::vector<int32_t> a(n);
            std::vector<int64_t> o(B), i(B), t(B), s(B);
            check(sbpgpu_bm_read(h_.get(), a.data(), o.data(), i.data(), t.data(), s.data(), nullptr, nullptr, nullptr),
                  ctx());
            auto v = std::make_shared<View>();
            v->assignment.assign(a.begin(), a.end());
            v->d_out.assign(o.begin(), o.end());
            v->d_in.assign(i.begin(), i.end());
            v->d_tot.assign(t.begin(), t.end());
            v->sizes.assign(s.begin(), s.end());
            view_ = v;
        }
        return *view_;
    }

    const Graph* graph_;
    double rate_ = 0.5;
    std::unique_ptr<sbpgpu_bm, Deleter> h_;
    double entropy_ = std::numeric_limits<double>::max();
    long num_blocks_to_merge_ = 0;
    mutable std::shared_ptr<View> view_;
};

/// VertexMove (include/typedefs.hpp:124-129): the outcome of one proposed vertex move.
struct VertexMove {
    double delta_entropy;
    bool did_move;
    long vertex;
    long proposed_block;
};

namespace utils {
/// utils::ProposalAndEdgeCounts (include/utils.hpp:24-30): a proposed block and the edge
/// counts of the vertex it was drawn for.
struct ProposalAndEdgeCounts {
    long proposal;
    long num_out_neighbor_edges;
    long num_in_neighbor_edges;
    long num_neighbor_edges;
};
}  // namespace utils

/// Delta (include/blockmodel/sparse/delta.hpp:22-148): the change to the cells of the rows
/// and columns of current_block and proposed_block that one vertex move makes.  A cell is
/// kept under the first of (row == current, row == proposed, col == current,
/// col == proposed) that holds, as the reference files it; any other cell is a
/// std::logic_error.  entries() lists the four groups in that order, each ascending.
class Delta {
  public:
    Delta() = default;
    Delta(long current_block, long proposed_block, long /*buckets*/ = 10)
        : current_(current_block), proposed_(proposed_block) {}
    void add(long row, long col, long value) { slot(row, col) += value; }
    void sub(long row, long col, long value) { slot(row, col) -= value; }
    long get(long row, long col) const {
        const std::map<long, long>* m;
        long key;
        route(row, col, m, key);
        const auto it = m->find(key);
        return it == m->end() ? 0 : it->second;
    }
    std::vector<std::tuple<long, long, long>> entries() const {
        std::vector<std::tuple<long, long, long>> out;
        for (const auto& e : cur_row_) out.emplace_back(current_, e.first, e.second);
        for (const auto& e : prop_row_) out.emplace_back(proposed_, e.first, e.second);
        for (const auto& e : cur_col_) out.emplace_back(e.first, current_, e.second);
        for (const auto& e : prop_col_) out.emplace_back(e.first, proposed_, e.second);
        return out;
    }
    long self_edge_weight() const { return self_; }
    void self_edge_weight(long weight) { self_ = weight; }
    long current_block() const { return current_; }
    long proposed_block() const { return proposed_; }

  private:
    void route(long row, long col, const std::map<long, long>*& m, long& key) const {
        if (row == current_) m = &cur_row_, key = col;
        else if (row == proposed_) m = &prop_row_, key = col;
        else if (col == current_) m = &cur_col_, key = row;
        else if (col == proposed_) m = &prop_col_, key = row;
        else throw std::logic_error("Neither the row nor column are current_block or proposed_block.");
    }
    long& slot(long row, long col) {
        const std::map<long, long>* m;
        long key;
        route(row, col, m, key);
        return (*const_cast<std::map<long, long>*>(m))[key];
    }
    long current_ = -1, proposed_ = -1, self_ = 0;
    std::map<long, long> cur_row_, prop_row_, cur_col_, prop_col_;
};

/// BlockmodelTriplet (include/blockmodel/blockmodel_triplet.hpp:12-42,
/// src/blockmodel/blockmodel_triplet.cpp:4-105): the three blockmodels that bracket the
/// golden-section search over block counts, in decreasing number of blocks.
class BlockmodelTriplet {
  public:
    bool optimal_num_blocks_found = false;
    Blockmodel& get(long i) { return blockmodels_[check(i)]; }
    const Blockmodel& get(long i) const { return blockmodels_[check(i)]; }
    /// Puts `blockmodel` (a copy) into its slot: the middle when it has the lowest
    /// description length so far (the old middle moving up or down by block count), else
    /// the upper or lower slot by its block count.
    void update(Blockmodel& blockmodel) {
        long index;
        if (blockmodels_[1].empty) {
            index = 1;
        } else if (blockmodel.getOverall_entropy() <= blockmodels_[1].getOverall_entropy()) {
            const long old_index = blockmodels_[1].num_blocks() > blockmodel.num_blocks() ? 0 : 2;
            blockmodels_[old_index] = blockmodels_[1].copy();
            index = 1;
        } else {
            index = blockmodels_[1].num_blocks() > blockmodel.num_blocks() ? 2 : 0;
        }
        blockmodels_[index] = blockmodel.copy();
    }
    /// true while the lower slot is empty (no bracket yet).
    bool golden_ratio_not_reached() const { return blockmodels_[2].empty; }
    bool is_done() {
        if ((!get(0).empty && get(0).num_blocks() - get(2).num_blocks() == 2) ||
            (get(0).empty && get(1).num_blocks() - get(2).num_blocks() == 1))
            optimal_num_blocks_found = true;
        return optimal_num_blocks_found;
    }
    /// The blockmodel the next merge pass starts from, with its number of blocks to merge:
    /// half the middle's blocks before the bracket exists, else the golden-section point
    /// of the wider side.
    Blockmodel get_next_blockmodel(Blockmodel& old_blockmodel) {
        old_blockmodel.setNum_blocks_to_merge(0);
        update(old_blockmodel);
        if (golden_ratio_not_reached()) {
            Blockmodel next = get(1).copy();
            next.setNum_blocks_to_merge((long)(next.num_blocks() * next.getBlock_reduction_rate()));
            if (next.getNum_blocks_to_merge() == 0) optimal_num_blocks_found = true;
            return next;
        }
        if (is_done()) return get(1).copy();
        long index = 1;
        if (get(0).empty && get(1).num_blocks() > get(2).num_blocks()) index = 1;
        else if (upper_difference() >= lower_difference()) index = 0;
        long next_try = get(index + 1).num_blocks();
        next_try += (long)((get(index).num_blocks() - get(index + 1).num_blocks()) * 0.618);
        Blockmodel next = get(index).copy();
        next.setNum_blocks_to_merge(next.num_blocks() - next_try);
        return next;
    }
    long lower_difference() const { return get(1).num_blocks() - get(2).num_blocks(); }
    long upper_difference() const { return get(0).num_blocks() - get(1).num_blocks(); }

  private:
    static long check(long i) {
        if (i < 0 || i >= 3) throw std::out_of_range("triplet index out of range");
        return i;
    }
    Blockmodel blockmodels_[3];
};

namespace entropy {

namespace nonparametric {

/// nonparametric::mdl (src/entropy.cpp:751-779), directed, not degree-corrected.
inline double mdl(const Blockmodel& blockmodel, const Graph& graph) {
    double out = 0.0;
    check(sbpgpu_np_mdl(blockmodel.handle(), &out), graph.context().get());
    return out;
}

/// nonparametric::delta_mdl (src/entropy.cpp:1146-1178) for the moves vertices[i] -> proposals[i].
inline std::vector<double> delta_mdl(const Blockmodel& blockmodel, const std::vector<long>& vertices,
                                     const std::vector<long>& proposals) {
    if (vertices.size() != proposals.size()) throw std::invalid_argument("vertices and proposals differ in length");
    std::vector<int32_t> v(vertices.begin(), vertices.end()), s(proposals.begin(), proposals.end());
    std::vector<double> out(v.size());
    check(sbpgpu_np_delta_mdl_batch(blockmodel.handle(), (int64_t)v.size(), v.data(), s.data(), out.data()),
          blockmodel.graph().context().get());
    return out;
}

/// nonparametric::block_merge_delta_mdl (src/entropy.cpp:1198-1223).
inline std::vector<double> block_merge_delta_mdl(const Blockmodel& blockmodel, const std::vector<long>& blocks,
                                                 const std::vector<long>& proposals) {
    if (blocks.size() != proposals.size()) throw std::invalid_argument("blocks and proposals differ in length");
    std::vector<int32_t> r(blocks.begin(), blocks.end()), s(proposals.begin(), proposals.end());
    std::vector<double> out(r.size());
    check(sbpgpu_np_merge_delta_mdl_batch(blockmodel.handle(), (int64_t)r.size(), r.data(), s.data(), out.data()),
          blockmodel.graph().context().get());
    return out;
}

}  // namespace nonparametric

/// entropy::mdl (src/entropy.cpp:597-604): the nonparametric form under args.nonparametric.
inline double mdl(const Blockmodel& blockmodel, const Graph& graph) {
    if (args.nonparametric) return nonparametric::mdl(blockmodel, graph);
    double out = 0.0;
    check(sbpgpu_mdl(blockmodel.handle(), &out), graph.context().get());
    return out;
}

/// entropy::delta_mdl (src/entropy.cpp:298-403) for the moves vertices[i] -> proposals[i].
inline std::vector<double> delta_mdl(const Blockmodel& blockmodel, const std::vector<long>& vertices,
                                     const std::vector<long>& proposals) {
    if (vertices.size() != proposals.size()) throw std::invalid_argument("vertices and proposals differ in length");
    std::vector<int32_t> v(vertices.begin(), vertices.end()), s(proposals.begin(), proposals.end());
    std::vector<double> out(v.size());
    check(sbpgpu_delta_mdl_batch(blockmodel.handle(), (int64_t)v.size(), v.data(), s.data(), out.data()),
          blockmodel.graph().context().get());
    return out;
}
inline double delta_mdl(const Blockmodel& blockmodel, long vertex, long proposal) {
    return delta_mdl(blockmodel, std::vector<long>{vertex}, std::vector<long>{proposal})[0];
}

/// entropy::block_merge_delta_mdl (src/entropy.cpp:129-182) for merging blocks[i] into proposals[i].
inline std::vector<double> block_merge_delta_mdl(const Blockmodel& blockmodel, const std::vector<long>& blocks,
                                                 const std::vector<long>& proposals) {
    if (blocks.size() != proposals.size()) throw std::invalid_argument("blocks and proposals differ in length");
    std::vector<int32_t> r(blocks.begin(), blocks.end()), s(proposals.begin(), proposals.end());
    std::vector<double> out(r.size());
    check(sbpgpu_merge_delta_mdl_batch(blockmodel.handle(), (int64_t)r.size(), r.data(), s.data(), out.data()),
          blockmodel.graph().context().get());
    return out;
}
inline double block_merge_delta_mdl(const Blockmodel& blockmodel, long block, long proposal) {
    return block_merge_delta_mdl(blockmodel, std::vector<long>{block}, std::vector<long>{proposal})[0];
}

/// entropy::null_mdl_v1 (src/entropy.cpp:571-585): the one-block model's description length.
inline double null_mdl_v1(const Graph& graph) {
    const double E = (double)graph.num_edges();
    const double log_posterior_p = E * std::log(1.0 / E);
    const double x = 1.0 / E;
    const double h = ((1 + x) * std::log(1 + x)) - (x * std::log(x));
    return (E * h) - log_posterior_p;
}
/// entropy::normalize_mdl_v1 (src/entropy.cpp:563-565).
inline double normalize_mdl_v1(double mdl, const Graph& graph) { return mdl / null_mdl_v1(graph); }

}  // namespace entropy

namespace finetune {

/// finetune::mcmc (src/finetune.cpp:754-771) with the algorithm of sbp_gb300::args.
inline Blockmodel& mcmc(int iteration, const Graph& graph, Blockmodel& blockmodel, bool golden_ratio_not_reached,
                        const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    sbpgpu_stats st;
    check(sbpgpu_mcmc(blockmodel.handle(), &cfg, a.seed, iteration, golden_ratio_not_reached ? 1 : 0, &st),
          graph.context().get());
    blockmodel.invalidate();
    blockmodel.setOverall_entropy(sbpgpu_bm_entropy(blockmodel.handle()));
    return blockmodel;
}
/// finetune::mcmc with a BlockmodelTriplet (src/finetune.cpp:754-771): the golden-ratio flag
/// is the triplet's.
inline Blockmodel& mcmc(int iteration, const Graph& graph, Blockmodel& blockmodel, BlockmodelTriplet& triplet,
                        const Args& a = args) {
    return mcmc(iteration, graph, blockmodel, triplet.golden_ratio_not_reached(), a);
}

/// finetune::accept (src/finetune.cpp:22-32): greedy takes dS < 0; otherwise a uniform
/// draw from a host generator seeded by Args::seed against min(1, e^(-3 dS) H).  The
/// device paths draw from the seeded Philox stream instead.
inline bool accept(double delta_entropy, double hastings_correction, const Args& a = args) {
    if (a.greedy) return delta_entropy < 0.0;
    static std::mt19937_64 generator(a.seed);
    const double p = std::uniform_real_distribution<double>(0.0, 1.0)(generator);
    const double q = std::min(1.0, std::exp(-3.0 * delta_entropy) * hastings_correction);
    return p <= q;
}

/// finetune::early_stop (src/finetune.cpp:265-283): stop on a zero last change, or when the
/// mean of the last three changes falls below 5e-4 (no bracket yet) or 1e-4 of the
/// initial description length.
inline bool early_stop(long iteration, bool golden_ratio_not_reached, double initial_entropy,
                       const std::vector<double>& delta_entropies) {
    const size_t last = delta_entropies.size() - 1;
    if (delta_entropies[last] == 0.0) return true;
    if (iteration < 3) return false;
    const double average = -(delta_entropies[last] + delta_entropies[last - 1] + delta_entropies[last - 2]) / 3.0;
    return average < (golden_ratio_not_reached ? 5e-4 : 1e-4) * initial_entropy;
}
/// finetune::early_stop (src/finetune.cpp:285-294): the 1e-4 rule alone.
inline bool early_stop(long iteration, double initial_entropy, const std::vector<double>& delta_entropies) {
    if (iteration < 3) return false;
    const size_t last = delta_entropies.size() - 1;
    const double average = -(delta_entropies[last] + delta_entropies[last - 1] + delta_entropies[last - 2]) / 3.0;
    return average < 1e-4 * initial_entropy;
}

/// finetune::edge_weights (src/finetune.cpp:419-430): the neighbours of `vertex`, weight 1
/// each (the graph is unweighted).
inline EdgeWeights edge_weights(const NeighborList& neighbors, long vertex, bool ignore_self = false) {
    EdgeWeights w;
    for (long u : neighbors.at(vertex)) {
        if (ignore_self && u == vertex) continue;
        w.indices.push_back(u);
        w.values.push_back(1);
    }
    return w;
}

/// finetune::blockmodel_delta (src/finetune.cpp:201-235): the cell changes of moving
/// `vertex` from current_block to proposed_block, on the host from the blockmodel's
/// assignment.  A self edge counts once per direction into (proposed, proposed).
inline Delta blockmodel_delta(long vertex, long current_block, long proposed_block, const EdgeWeights& out_edges,
                              const EdgeWeights& in_edges, const Blockmodel& blockmodel) {
    Delta delta(current_block, proposed_block);
    const std::vector<long>& assignment = blockmodel.block_assignment();
    for (size_t i = 0; i < out_edges.indices.size(); ++i) {
        const long u = out_edges.indices[i], b = assignment.at(u), w = out_edges.values[i];
        if (u == vertex) {
            delta.add(proposed_block, proposed_block, w);
            delta.self_edge_weight(1);
        } else {
            delta.add(proposed_block, b, w);
        }
        delta.sub(current_block, b, w);
    }
    for (size_t i = 0; i < in_edges.indices.size(); ++i) {
        const long u = in_edges.indices[i], b = assignment.at(u), w = in_edges.values[i];
        if (u == vertex) {
            delta.add(proposed_block, proposed_block, w);
            delta.self_edge_weight(1);
        } else {
            delta.add(b, proposed_block, w);
        }
        delta.sub(b, current_block, w);
    }
    return delta;
}

/// finetune::propose_move (src/finetune.cpp:842-869) on the device: draws the proposal for
/// `vertex` from the seeded stream keyed (vertex, iteration, step) -- the draw the
/// sequential chain makes for it -- and runs move_vertex on it.  A vertex alone in its
/// block gives delta_entropy = DBL_MAX and proposed_block = -1; a proposal equal to the
/// current block gives 0 and -1.
inline VertexMove propose_move(Blockmodel& blockmodel, long vertex, const Graph& graph, int iteration = 0,
                               int step = 0, const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    int32_t proposal = -1, moved = 0;
    double dS = 0.0;
    check(sbpgpu_propose_move(blockmodel.handle(), &cfg, (int32_t)vertex, a.seed, (uint32_t)iteration,
                              (uint32_t)step, &proposal, &dS, &moved),
          graph.context().get());
    if (moved) blockmodel.invalidate();
    return VertexMove{dS, moved != 0, proposal < 0 ? -1 : vertex, (long)proposal};
}

/// finetune::move_vertex (src/finetune.cpp:822-840) on the device: scores the move of
/// `vertex` into proposal.proposal (with the Hastings correction when not greedy), decides
/// with the accept rule on the seeded stream and applies an accepted move.  The vertex's
/// edges are read from the device graph; out_edges and in_edges are accepted for the
/// reference's signature and not read.
inline VertexMove move_vertex(long vertex, long /*current_block*/, utils::ProposalAndEdgeCounts proposal,
                              Blockmodel& blockmodel, const Graph& graph, EdgeWeights& /*out_edges*/,
                              EdgeWeights& /*in_edges*/, int iteration = 0, int step = 0, const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    int32_t moved = 0;
    double dS = 0.0;
    check(sbpgpu_move_vertex(blockmodel.handle(), &cfg, (int32_t)vertex, (int32_t)proposal.proposal, a.seed,
                             (uint32_t)iteration, (uint32_t)step, &dS, &moved),
          graph.context().get());
    if (moved) blockmodel.invalidate();
    return VertexMove{dS, moved != 0, vertex, proposal.proposal};
}

/// finetune::propose_gibbs_move_v3 (src/finetune.cpp:871-901) for many vertices against
/// the current state, nothing applied: the accepted proposal of each, or -1 (the decisions
/// an asynchronous-Gibbs batch applies in vertex-id order).
inline std::vector<long> propose_gibbs_moves(const Blockmodel& blockmodel, const std::vector<long>& vertices,
                                             const Graph& graph, int iteration = 0, int step = 0,
                                             const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    std::vector<int32_t> v(vertices.begin(), vertices.end()), out(vertices.size());
    check(sbpgpu_gibbs_propose(blockmodel.handle(), &cfg, (int64_t)v.size(), v.data(), a.seed, (uint32_t)iteration,
                               (uint32_t)step, out.data()),
          graph.context().get());
    return std::vector<long>(out.begin(), out.end());
}
/// finetune::propose_gibbs_move_v3 for one vertex: did_move tells whether the proposal was
/// accepted (nothing is applied); delta_entropy is its delta-MDL, 0 when nothing was
/// accepted.
inline VertexMove propose_gibbs_move_v3(const Blockmodel& blockmodel, long vertex, const Graph& graph,
                                        int iteration = 0, int step = 0, const Args& a = args) {
    const long s = propose_gibbs_moves(blockmodel, std::vector<long>{vertex}, graph, iteration, step, a)[0];
    double dS = 0.0;
    if (s >= 0) {
        const int32_t vv = (int32_t)vertex, ss = (int32_t)s;
        check(a.nonparametric ? sbpgpu_np_delta_mdl_batch(blockmodel.handle(), 1, &vv, &ss, &dS)
                              : sbpgpu_delta_mdl_batch(blockmodel.handle(), 1, &vv, &ss, &dS),
              graph.context().get());
    }
    return VertexMove{dS, s >= 0, vertex, s};
}

namespace detail {
inline Blockmodel& run(const char* algorithm, Blockmodel& bm, const Graph& g, bool golden, int iteration) {
    Args a = args;
    a.algorithm = algorithm;
    return mcmc(iteration, g, bm, golden, a);
}
}  // namespace detail
/// finetune::asynchronous_gibbs (src/finetune.cpp:34-107).
inline Blockmodel& asynchronous_gibbs(Blockmodel& bm, const Graph& g, bool golden_ratio_not_reached, int iteration = 0) {
    return detail::run("async_gibbs", bm, g, golden_ratio_not_reached, iteration);
}
/// finetune::hybrid_mcmc (src/finetune.cpp:563-646).
inline Blockmodel& hybrid_mcmc(Blockmodel& bm, const Graph& g, bool golden_ratio_not_reached, int iteration = 0) {
    return detail::run("hybrid_mcmc", bm, g, golden_ratio_not_reached, iteration);
}
/// finetune::metropolis_hastings (src/finetune.cpp:773-820).
inline Blockmodel& metropolis_hastings(Blockmodel& bm, const Graph& g, bool golden_ratio_not_reached,
                                       int iteration = 0) {
    return detail::run("metropolis_hastings", bm, g, golden_ratio_not_reached, iteration);
}

}  // namespace finetune

namespace block_merge {

/// block_merge::merge_blocks (src/block_merge.cpp:178-228): merges
/// blockmodel.getNum_blocks_to_merge() blocks; `step` keys the proposal stream.
inline Blockmodel& merge_blocks(Blockmodel& blockmodel, const Graph& graph, long /*num_edges*/, int step = 0,
                                const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    sbpgpu_stats st;
    check(sbpgpu_merge_blocks(blockmodel.handle(), &cfg, a.seed, step, blockmodel.getNum_blocks_to_merge(), &st),
          graph.context().get());
    blockmodel.invalidate();
    blockmodel.setNum_blocks_to_merge((long)(blockmodel.num_blocks() * blockmodel.getBlock_reduction_rate()));
    return blockmodel;
}

/// block_merge::propose_merge_sparse (src/block_merge.cpp:251-285) for every block, as the
/// merge pass draws them (10 proposals per block, src/block_merge.cpp:189-217): each
/// block's best proposal and its delta-MDL.
inline std::pair<std::vector<long>, std::vector<double>> merge_proposals(const Blockmodel& blockmodel,
                                                                         const Graph& graph, int step = 0,
                                                                         const Args& a = args) {
    const long B = blockmodel.num_blocks();
    std::vector<int32_t> best(B);
    std::vector<double> dS(B);
    check(sbpgpu_merge_proposals(blockmodel.handle(), a.seed, step, best.data(), dS.data()), graph.context().get());
    return {std::vector<long>(best.begin(), best.end()), dS};
}

}  // namespace block_merge

namespace sbp {

/// sbp::done_blockmodeling (src/sbp.cpp:74-86).
inline bool done_blockmodeling(Blockmodel& blockmodel, BlockmodelTriplet& triplet, long min_num_blocks = 0) {
    if (min_num_blocks > 0 && (blockmodel.num_blocks() <= min_num_blocks || !triplet.get(2).empty)) return true;
    return triplet.optimal_num_blocks_found;
}

/// sbp::stochastic_block_partition (src/sbp.cpp:16-72): the golden-section search over
/// block counts with merge passes and MCMC, all on the device.
inline Blockmodel stochastic_block_partition(Graph& graph, Args& a, bool divide_and_conquer = false) {
    if (divide_and_conquer)
        throw Error(SBPGPU_EUNSUPPORTED, "divide-and-conquer SBP is outside the device hot path");
    const sbpgpu_config cfg = to_config(a);
    check(sbpgpu_graph_set_undirected(graph.handle(), a.undirected ? 1 : 0), graph.context().get());
    std::vector<int32_t> out(graph.num_vertices());
    int64_t B = 0;
    double mdl = 0.0;
    sbpgpu_stats st;
    check(sbpgpu_sbp(graph.handle(), &cfg, a.seed, out.data(), &B, &mdl, &st), graph.context().get());
    Blockmodel bm(B, graph, 0.5, std::vector<long>(out.begin(), out.end()));
    bm.setOverall_entropy(mdl);
    return bm;
}

}  // namespace sbp

namespace sample {

/// sample::Sample: the sampled graph and mapping[v] = v's id in it, or -1.
struct Sample {
    std::unique_ptr<Graph> graph;
    std::vector<long> mapping;
};

namespace detail {
inline int32_t algorithm(const std::string& name) {
    if (name == "max_degree") return 0;
    if (name == "random") return 1;
    if (name == "degree_product") return 2;
    if (name == "expansion_snowball") return 4;
    if (name == "degree_product_snowball") return 5;
    throw std::invalid_argument(name + " is not a valid sampling algorithm!");
}
// sample::from_vertices (src/sample.cpp:240-253) on the host mirror: edges between sampled
// vertices in source order; the true assignment follows the vertices.
inline Sample from_mapping(const Graph& graph, std::vector<long> mapping, long n) {
    NeighborList out(n), in(n);
    long E = 0;
    for (long v = 0; v < graph.num_vertices(); ++v) {
        if (mapping[v] < 0) continue;
        for (long u : graph.out_neighbors(v))
            if (mapping[u] >= 0) {
                out[mapping[v]].push_back(mapping[u]);
                in[mapping[u]].push_back(mapping[v]);
                ++E;
            }
    }
    Sample s{std::make_unique<Graph>(out, in, n, E, graph.context()), std::move(mapping)};
    for (long v = 0; v < graph.num_vertices(); ++v)
        if (s.mapping[v] >= 0) s.graph->assign(s.mapping[v], graph.assignment(v));
    return s;
}
inline Sample run(const Graph& graph, int32_t alg, double size, uint64_t seed) {
    std::vector<int32_t> m(graph.num_vertices());
    int64_t n = 0;
    check(sbpgpu_sample(graph.handle(), alg, size, seed, m.data(), &n), graph.context().get());
    return from_mapping(graph, std::vector<long>(m.begin(), m.end()), n);
}
inline std::vector<int32_t> narrow(const std::vector<long>& v) { return std::vector<int32_t>(v.begin(), v.end()); }
}  // namespace detail

/// sample::sample (src/sample.cpp:328-341) with args.samplingalg and args.samplesize.
inline Sample sample(const Graph& graph, const Args& a = args) {
    return detail::run(graph, detail::algorithm(a.samplingalg), a.samplesize, a.seed);
}
/// sample::detach (src/sample.cpp:12-26): the vertices of degree above 1.
inline Sample detach(const Graph& graph) { return detail::run(graph, 3, 1.0, 0); }

/// sample::extend (src/sample.cpp:159-199).
inline std::vector<long> extend(const Graph& graph, const Blockmodel& sample_blockmodel, const Sample& s,
                                const Args& a = args) {
    const std::vector<int32_t> sa = detail::narrow(sample_blockmodel.block_assignment());
    const std::vector<int32_t> m = detail::narrow(s.mapping);
    std::vector<int32_t> out(graph.num_vertices());
    check(sbpgpu_extend(graph.handle(), sa.data(), (int64_t)sa.size(), sample_blockmodel.num_blocks(), m.data(), a.seed,
                        out.data()),
          graph.context().get());
    return std::vector<long>(out.begin(), out.end());
}

/// sample::reattach (src/sample.cpp:365-405).
inline Blockmodel reattach(const Graph& graph, const Blockmodel& sample_blockmodel, const Sample& s,
                           const Args& a = args) {
    const std::vector<int32_t> sa = detail::narrow(sample_blockmodel.block_assignment());
    const std::vector<int32_t> m = detail::narrow(s.mapping);
    std::vector<int32_t> out(graph.num_vertices());
    check(sbpgpu_reattach(graph.handle(), sa.data(), (int64_t)sa.size(), sample_blockmodel.num_blocks(), m.data(),
                          a.seed, out.data()),
          graph.context().get());
    return Blockmodel(sample_blockmodel.num_blocks(), graph, 0.5, std::vector<long>(out.begin(), out.end()));
}

}  // namespace sample

namespace finetune {

/// finetune::finetune_assignment (src/finetune.cpp:903-932).
inline Blockmodel& finetune_assignment(Blockmodel& blockmodel, const Graph& graph, const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    sbpgpu_stats st;
    check(sbpgpu_finetune_assignment(blockmodel.handle(), &cfg, a.seed, &st), graph.context().get());
    blockmodel.invalidate();
    blockmodel.setOverall_entropy(sbpgpu_bm_entropy(blockmodel.handle()));
    return blockmodel;
}

}  // namespace finetune

namespace divisive {

/// divisive::split_communities (src/top_down_sbp.cpp:472-530) with --split random.
inline Blockmodel& split_communities(Blockmodel& blockmodel, const Graph& graph, int target_num_communities,
                                     int step = 0, const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    check(sbpgpu_split_communities(blockmodel.handle(), &cfg, a.seed, step, target_num_communities),
          graph.context().get());
    blockmodel.invalidate();
    return blockmodel;
}

/// divisive::run (src/top_down_sbp.cpp:435-470), with args.mix as --mix.
inline Blockmodel run(const Graph& graph, const Args& a = args) {
    const sbpgpu_config cfg = to_config(a);
    std::vector<int32_t> out(graph.num_vertices());
    int64_t B = 0;
    double mdl = 0.0;
    sbpgpu_stats st;
    check(sbpgpu_sbp_top_down(graph.handle(), &cfg, a.seed, a.mix ? 1 : 0, out.data(), &B, &mdl, &st),
          graph.context().get());
    Blockmodel bm(B, graph, 0.5, std::vector<long>(out.begin(), out.end()));
    bm.setOverall_entropy(mdl);
    return bm;
}

}  // namespace divisive

namespace evaluate {

/// evaluate::Eval (include/evaluate.hpp:15-19), with the other figures the reference prints.
struct Eval {
    double f1_score;
    double nmi;
    double true_mdl;
    double precision, recall, rand_index, accuracy;
};

/// evaluate::evaluate_blockmodel (src/evaluate.cpp:100-110) against graph.assignment().
inline Eval evaluate_blockmodel(const Graph& graph, Blockmodel& blockmodel) {
    const std::vector<int32_t> t = sample::detail::narrow(graph.assignment());
    const std::vector<int32_t> a = sample::detail::narrow(blockmodel.block_assignment());
    sbpgpu_eval e;
    check(sbpgpu_evaluate(graph.context().get(), graph.num_vertices(), t.data(), a.data(), &e), graph.context().get());
    // the true blockmodel's MDL (evaluate.cpp:104-108), when every vertex is labelled
    long true_blocks = 0;
    bool labelled = true;
    for (long x : graph.assignment()) {
        true_blocks = std::max(true_blocks, x + 1);
        labelled = labelled && x >= 0;
    }
    double true_mdl = std::numeric_limits<double>::quiet_NaN();
    if (labelled) {
        Blockmodel truth(true_blocks, graph, 0.5, graph.assignment());
        true_mdl = entropy::mdl(truth, graph);
    }
    return Eval{e.f1, e.nmi, true_mdl, e.precision, e.recall, e.rand_index, e.accuracy};
}

}  // namespace evaluate

}  // namespace sbp_gb300

#endif

// The C++ host interface (include/sbp_gb300.hpp) exercised the way the reference's gtest
// suites exercise theirs (test/blockmodel_test.cpp, test/entropy_test.cpp,
// test/block_merge_test.cpp, test/finetune_test.cpp): known answers on the 11-vertex toy
// graph, delta-MDL against MDL differences, copies, error behaviour, and one full
// partition whose result the Python driver compares with its own run.
//
//   test_api <toy.txt> <graph.txt> <seed> <assignment_out.txt>
//
// toy.txt: N E, E edge pairs, B, N assignment entries, MDL, then B out-degrees, B
// in-degrees, B total degrees and the nonparametric MDL.  graph.txt: N E, then E edge pairs.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "sbp_gb300.hpp"

namespace s = sbp_gb300;

static int g_failures = 0;

#define EXPECT(cond)                                                              \
    do {                                                                          \
        if (!(cond)) {                                                            \
            ++g_failures;                                                         \
            std::fprintf(stderr, "%s:%d: expected %s\n", __FILE__, __LINE__, #cond); \
        }                                                                         \
    } while (0)

// EXPECT_FLOAT_EQ: the two values as floats are within 4 units in the last place.
static bool float_eq(double a, double b) {
    const float fa = (float)a, fb = (float)b;
    int32_t ia, ib;
    std::memcpy(&ia, &fa, 4);
    std::memcpy(&ib, &fb, 4);
    if ((ia < 0) != (ib < 0)) return fa == fb;
    return std::abs((long long)ia - (long long)ib) <= 4;
}

struct Toy {
    long n = 0, e = 0, B = 0;
    std::vector<std::pair<long, long>> edges;
    std::vector<long> assignment, dout, din, dtot;
    double mdl = 0.0;
    double np_mdl = 0.0;
};

static Toy read_toy(const char* path) {
    std::ifstream f(path);
    Toy t;
    f >> t.n >> t.e;
    for (long i = 0; i < t.e; ++i) {
        long u, v;
        f >> u >> v;
        t.edges.emplace_back(u, v);
    }
    f >> t.B;
    t.assignment.resize(t.n);
    for (auto& a : t.assignment) f >> a;
    f >> t.mdl;
    for (auto* vec : {&t.dout, &t.din, &t.dtot}) {
        vec->resize(t.B);
        for (auto& x : *vec) f >> x;
    }
    f >> t.np_mdl;
    if (!f) throw std::runtime_error("cannot read the toy fixture");
    return t;
}

static void toy_known_answers(const Toy& t) {
    s::Graph graph(t.n, t.edges);
    s::Blockmodel bm(t.B, graph, 0.5, t.assignment);
    EXPECT(bm.num_blocks() == t.B);
    EXPECT(bm.degrees_out() == t.dout);
    EXPECT(bm.degrees_in() == t.din);
    EXPECT(bm.degrees() == t.dtot);
    EXPECT(bm.getNum_blocks_to_merge() == (long)(t.B * 0.5));
    const double mdl = s::entropy::mdl(bm, graph);
    EXPECT(float_eq(mdl, t.mdl));

    // a vertex move: delta-MDL equals the difference of the two MDLs
    const long v = 7, to = 0;
    const double dS = s::entropy::delta_mdl(bm, v, to);
    std::vector<long> moved = t.assignment;
    moved[v] = to;
    s::Blockmodel bm2(t.B, graph, 0.5, moved);
    EXPECT(std::fabs(dS - (s::entropy::mdl(bm2, graph) - mdl)) < 1e-5);  // float-log rounding of the MDL

    // a block merge, block 0 into block 1: the change of the MDL with block 0 left empty
    // (test/entropy_test.cpp compares with a blockmodel of the same block count)
    const double dM = s::entropy::block_merge_delta_mdl(bm, 0, 1);
    std::vector<long> merged = t.assignment;
    for (auto& a : merged) a = a == 0 ? 1 : a;
    s::Blockmodel bm3(t.B, graph, 0.5, merged);
    EXPECT(std::fabs(dM - (s::entropy::mdl(bm3, graph) - mdl)) < 1e-5);

    // batched scoring agrees with single calls
    const auto batch = s::entropy::delta_mdl(bm, std::vector<long>{v, 1, 9}, std::vector<long>{to, 2, 0});
    EXPECT(batch[0] == dS);

    // a copy is independent of the original
    s::Blockmodel c = bm.copy();
    s::Args a;
    a.seed = 3;
    a.algorithm = "hybrid_mcmc";
    s::finetune::mcmc(0, graph, c, true, a);
    EXPECT(bm.degrees_out() == t.dout);
    EXPECT(bm.block_assignment() == t.assignment);

    // errors surface as the reference's exception types
    bool threw = false;
    try {
        s::entropy::delta_mdl(bm, t.n + 5, 0);
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    EXPECT(threw);
    threw = false;
    try {
        std::vector<long> bad = t.assignment;
        bad[0] = t.B + 3;
        s::Blockmodel b(t.B, graph, 0.5, bad);
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    EXPECT(threw);

    // nonparametric entropy: the toy blockmodel's known answer (nonparametric_entropy_test.cpp:19-27,
    // :57-61) and the vertex-7 move against the MDL difference (:118-133)
    EXPECT(float_eq(s::entropy::nonparametric::mdl(bm, graph), t.np_mdl));
    const double dN = s::entropy::nonparametric::delta_mdl(bm, std::vector<long>{v}, std::vector<long>{to})[0];
    EXPECT(std::fabs(dN - (s::entropy::nonparametric::mdl(bm2, graph) - s::entropy::nonparametric::mdl(bm, graph))) <
           1e-6);
    s::Args na;
    na.nonparametric = true;
    na.seed = 5;
    s::Blockmodel c2 = bm.copy();
    s::finetune::mcmc(0, graph, c2, true, na);
    EXPECT(c2.num_blocks() == t.B);

    // normalize_mdl_v1 divides by the one-block model's length
    EXPECT(std::fabs(s::entropy::normalize_mdl_v1(mdl, graph) * s::entropy::null_mdl_v1(graph) - mdl) < 1e-9 * mdl);
}

// The per-vertex boundary and the host-side types: blockmatrix() snapshot, Delta,
// blockmodel_delta, early_stop, edge_weights, propose_move / move_vertex, BlockmodelTriplet
// and done_blockmodeling (test/finetune_test.cpp, test/blockmodel_triplet_test.cpp).
static void boundary_api(const Toy& t) {
    s::Graph graph(t.n, t.edges);
    s::Blockmodel bm(t.B, graph, 0.5, t.assignment);

    const auto m = bm.blockmatrix();
    EXPECT(m->entries() == bm.blockmatrix_cells());
    EXPECT(m->edges() == t.e);
    EXPECT(m->sum(0) == t.dout);
    EXPECT(m->sum(1) == t.din);
    long cells = 0;
    for (long r = 0; r < t.B; ++r)
        for (long c = 0; c < t.B; ++c) cells += m->get(r, c);
    EXPECT(cells == t.e);

    // Delta of moving vertex 7 to block 0 equals the change of the block matrix
    const long v = 7, to = 0, from = t.assignment[v];
    const s::EdgeWeights out = s::finetune::edge_weights(graph.out_neighbors(), v);
    const s::EdgeWeights in = s::finetune::edge_weights(graph.in_neighbors(), v);
    EXPECT((long)out.indices.size() == (long)graph.out_neighbors(v).size());
    const s::Delta delta = s::finetune::blockmodel_delta(v, from, to, out, in, bm);
    std::vector<long> moved = t.assignment;
    moved[v] = to;
    s::Blockmodel bm2(t.B, graph, 0.5, moved);
    const auto m2 = bm2.blockmatrix();
    long changed = 0;
    for (long r = 0; r < t.B; ++r)
        for (long c = 0; c < t.B; ++c)
            if (m2->get(r, c) != m->get(r, c)) ++changed;
    long listed = 0;
    for (const auto& e : delta.entries()) {
        const long r = std::get<0>(e), c = std::get<1>(e), d = std::get<2>(e);
        EXPECT(m2->get(r, c) - m->get(r, c) == d);
        EXPECT(delta.get(r, c) == d);
        if (d != 0) ++listed;
    }
    EXPECT(listed == changed);
    // the reference's known answers (test/finetune_test.cpp:89-124, :226-238): six keyed cells,
    // zero-valued ones included, summing to zero, also for vertex 10 with its self edge
    const s::Delta k7 = s::finetune::blockmodel_delta(7, from, 0, out, in, bm);
    EXPECT(k7.entries().size() == 6);
    EXPECT(k7.get(0, 0) == 1 && k7.get(0, 1) == 0 && k7.get(0, 2) == 1 && k7.get(1, 0) == 1);
    EXPECT(k7.get(1, 2) == -1 && k7.get(2, 0) == 1 && k7.get(2, 1) == 0 && k7.get(2, 2) == -3);
    for (long u : {7L, 10L}) {
        const s::Delta du = s::finetune::blockmodel_delta(u, t.assignment[u], 0,
                                                          s::finetune::edge_weights(graph.out_neighbors(), u),
                                                          s::finetune::edge_weights(graph.in_neighbors(), u), bm);
        long sum = 0;
        for (const auto& e : du.entries()) sum += std::get<2>(e);
        EXPECT(sum == 0);
    }
    const std::vector<long> assignment3 = {0, 0, 0, 1, 2, 3, 3, 4, 5, 1, 5};
    s::Blockmodel b3(6, graph, 0.5, assignment3);
    // the neighbours of block 1 (test/dict_transpose_matrix_test.cpp:16-34)
    EXPECT(m->neighbors(1) == (std::set<long>{0, 1, 2}));
    EXPECT(b3.blockmatrix()->neighbors(1) == (std::set<long>{0, 3, 4, 5}));
    const s::Delta k6 = s::finetune::blockmodel_delta(6, 3, 0, s::finetune::edge_weights(graph.out_neighbors(), 6),
                                                      s::finetune::edge_weights(graph.in_neighbors(), 6, true), b3);
    EXPECT(k6.entries().size() == 6);
    EXPECT(k6.get(0, 2) == 1 && k6.get(2, 0) == 1 && k6.get(2, 3) == -1 && k6.get(3, 0) == 1);
    EXPECT(k6.get(3, 2) == -1 && k6.get(3, 3) == -1);
    bool threw = false;
    try {
        s::Delta d2(1, 2);
        d2.add(3, 4, 1);
    } catch (const std::logic_error&) {
        threw = true;
    }
    EXPECT(threw);

    // early_stop: zero change stops; three small changes stop; large changes continue
    EXPECT(s::finetune::early_stop(1, true, 100.0, std::vector<double>{-5.0, 0.0}));
    EXPECT(!s::finetune::early_stop(4, true, 100.0, std::vector<double>{-5.0, -5.0, -5.0}));
    EXPECT(s::finetune::early_stop(4, true, 100.0, std::vector<double>{-0.01, -0.01, -0.01}));
    EXPECT(!s::finetune::early_stop(4, 100.0, std::vector<double>{-0.02, -0.02, -0.02}));
    EXPECT(s::finetune::early_stop(4, 100.0, std::vector<double>{-0.005, -0.005, -0.005}));
    s::Args g;
    g.greedy = true;
    EXPECT(s::finetune::accept(-1.0, 1.0, g) && !s::finetune::accept(0.5, 1.0, g));

    // move_vertex on a given proposal: the delta-MDL of the entropy interface, applied iff negative
    s::Blockmodel c = bm.copy();
    const double want = s::entropy::delta_mdl(bm, v, to);
    s::utils::ProposalAndEdgeCounts proposal{to, (long)out.indices.size(), (long)in.indices.size(),
                                             (long)(out.indices.size() + in.indices.size())};
    s::EdgeWeights o2 = out, i2 = in;
    const s::VertexMove mv = s::finetune::move_vertex(v, from, proposal, c, graph, o2, i2, 0, 0, g);
    EXPECT(mv.delta_entropy == want && mv.did_move == (want < 0) && mv.vertex == v && mv.proposed_block == to);
    EXPECT(c.block_assignment(v) == (mv.did_move ? to : from));
    // propose_move over every vertex: each applied move changes the MDL by its delta
    s::Args h;
    h.seed = 11;
    for (long u = 0; u < t.n; ++u) {
        const double before = s::entropy::mdl(c, graph);
        const s::VertexMove pm = s::finetune::propose_move(c, u, graph, 2, 1, h);
        if (pm.did_move) {
            EXPECT(pm.vertex == u && c.block_assignment(u) == pm.proposed_block);
            EXPECT(std::fabs(s::entropy::mdl(c, graph) - before - pm.delta_entropy) < 1e-5);
        } else if (pm.proposed_block == -1) {
            EXPECT(pm.vertex == -1);
        }
    }

    // propose_gibbs_move_v3 applies nothing; merge_proposals gives every block a proposal
    {
        s::Blockmodel d = bm.copy();
        const std::vector<long> before = d.block_assignment();
        const std::vector<long> all = s::finetune::propose_gibbs_moves(d, {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10}, graph,
                                                                       1, 0, h);
        EXPECT(all.size() == 11 && d.block_assignment() == before);
        for (long u = 0; u < t.n; ++u) {
            const s::VertexMove gm = s::finetune::propose_gibbs_move_v3(d, u, graph, 1, 0, h);
            EXPECT(gm.proposed_block == all[u] && gm.did_move == (all[u] >= 0));
            if (gm.did_move) EXPECT(gm.delta_entropy == s::entropy::delta_mdl(d, u, gm.proposed_block));
        }
        const auto mp = s::block_merge::merge_proposals(d, graph, 0, h);
        EXPECT((long)mp.first.size() == d.num_blocks() && (long)mp.second.size() == d.num_blocks());
        for (long b = 0; b < d.num_blocks(); ++b) EXPECT(mp.first[b] < d.num_blocks());
    }

    // BlockmodelTriplet: the bracket forms as blockmodels with fewer blocks arrive
    s::BlockmodelTriplet triplet;
    EXPECT(triplet.golden_ratio_not_reached() && triplet.get(0).empty && triplet.get(1).empty);
    s::Blockmodel b1 = bm.copy();
    b1.setOverall_entropy(100.0);
    s::Blockmodel next = triplet.get_next_blockmodel(b1);
    EXPECT(!triplet.get(1).empty && triplet.get(1).num_blocks() == t.B);
    EXPECT(next.num_blocks() == t.B && next.getNum_blocks_to_merge() == (long)(t.B * 0.5));
    EXPECT(!s::sbp::done_blockmodeling(next, triplet));
    std::vector<long> two = t.assignment;
    for (auto& x : two) x = x % 2;
    s::Blockmodel b2(2, graph, 0.5, two);
    b2.setOverall_entropy(120.0);  // worse than the middle: goes below it
    triplet.update(b2);
    EXPECT(!triplet.golden_ratio_not_reached() && triplet.get(2).num_blocks() == 2);
    EXPECT(triplet.lower_difference() == t.B - 2);
    EXPECT(s::sbp::done_blockmodeling(b2, triplet, 2));
    s::finetune::mcmc(0, graph, b2, triplet, g);
    EXPECT(b2.num_blocks() == 2);
    threw = false;
    try {
        triplet.get(3);
    } catch (const std::out_of_range&) {
        threw = true;
    }
    EXPECT(threw);
}

static void full_partition(const char* graph_path, uint64_t seed, const char* out_path) {
    std::ifstream f(graph_path);
    long n = 0, e = 0;
    f >> n >> e;
    std::vector<std::pair<long, long>> edges(e);
    for (auto& x : edges) f >> x.first >> x.second;
    if (!f) throw std::runtime_error("cannot read the graph");
    s::Graph graph(n, edges);
    s::Args a;
    a.seed = seed;
    a.algorithm = "hybrid_mcmc";
    s::Blockmodel bm = s::sbp::stochastic_block_partition(graph, a);
    EXPECT(bm.num_blocks() >= 1);
    EXPECT((long)bm.block_assignment().size() == n);
    // sampling (src/main.cpp:98-140), top-down partitioning and evaluation entry points
    s::Args sa = a;
    sa.samplesize = 0.5;
    sa.samplingalg = "max_degree";
    s::sample::Sample smp = s::sample::sample(graph, sa);
    EXPECT(smp.graph->num_vertices() == n / 2);
    s::Blockmodel sbm = s::sbp::stochastic_block_partition(*smp.graph, sa);
    const std::vector<long> ext = s::sample::extend(graph, sbm, smp, sa);
    EXPECT((long)ext.size() == n);
    s::Blockmodel ebm(sbm.num_blocks(), graph, 0.5, ext);
    s::finetune::finetune_assignment(ebm, graph, sa);
    EXPECT(ebm.num_blocks() == sbm.num_blocks());
    s::Blockmodel td = s::divisive::run(graph, a);
    EXPECT(td.num_blocks() >= 1);
    graph.assignment(bm.block_assignment());
    const s::evaluate::Eval ev = s::evaluate::evaluate_blockmodel(graph, bm);
    EXPECT(std::fabs(ev.nmi - 1.0) < 1e-6 && ev.f1_score == 1.0 && ev.accuracy == 1.0);
    EXPECT(std::fabs(ev.true_mdl - bm.getOverall_entropy()) < 1e-6 * bm.getOverall_entropy());

    std::ofstream o(out_path);
    o.precision(17);
    o << bm.num_blocks() << " " << bm.getOverall_entropy() << "\n";
    for (long x : bm.block_assignment()) o << x << "\n";
}

int main(int argc, char** argv) {
    if (argc != 5) {
        std::fprintf(stderr, "usage: test_api toy.txt graph.txt seed assignment_out.txt\n");
        return 2;
    }
    try {
        const Toy toy = read_toy(argv[1]);
        toy_known_answers(toy);
        boundary_api(toy);
        full_partition(argv[2], std::stoull(argv[3]), argv[4]);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "unexpected exception: %s\n", ex.what());
        return 1;
    }
    std::printf("%s (%d failures)\n", g_failures ? "FAILED" : "OK", g_failures);
    return g_failures ? 1 : 0;
}

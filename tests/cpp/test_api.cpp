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
        toy_known_answers(read_toy(argv[1]));
        full_partition(argv[2], std::stoull(argv[3]), argv[4]);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "unexpected exception: %s\n", ex.what());
        return 1;
    }
    std::printf("%s (%d failures)\n", g_failures ? "FAILED" : "OK", g_failures);
    return g_failures ? 1 : 0;
}

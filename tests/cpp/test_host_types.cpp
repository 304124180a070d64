// The host-side types of the C++ interface (include/sbp_gb300.hpp) that need no device:
// Delta's routing of cells to the rows and columns of the two blocks (key presence kept for
// zero values, std::logic_error elsewhere, as include/blockmodel/sparse/delta.hpp:55-118),
// the BlockMatrix snapshot's ISparseMatrix queries, edge_weights, early_stop and the greedy
// accept rule.
#include <cstdio>
#include <stdexcept>
#include <tuple>
#include <vector>

#include "sbp_gb300.hpp"

namespace s = sbp_gb300;

static int g_fail = 0;
#define EXPECT(c)                                                              \
    do {                                                                       \
        if (!(c)) {                                                            \
            ++g_fail;                                                          \
            std::fprintf(stderr, "%s:%d: expected %s\n", __FILE__, __LINE__, #c); \
        }                                                                      \
    } while (0)

int main() {
    // Delta: rows of current (2) and proposed (0) first, then their columns
    s::Delta d(2, 0);
    d.add(0, 0, 1);
    d.add(0, 2, 1);
    d.add(1, 0, 1);
    d.add(1, 2, -1);
    d.add(2, 0, 1);
    d.add(2, 2, -3);
    d.add(2, 1, 0);  // a zero change still makes the key present
    EXPECT(d.entries().size() == 7);
    EXPECT(d.get(2, 1) == 0 && d.get(2, 2) == -3 && d.get(1, 2) == -1 && d.get(1, 0) == 1);
    d.sub(2, 2, -3);
    EXPECT(d.get(2, 2) == 0 && d.entries().size() == 7);
    EXPECT(std::get<0>(d.entries()[0]) == 2);  // current block's row first
    EXPECT(d.current_block() == 2 && d.proposed_block() == 0);
    d.self_edge_weight(1);
    EXPECT(d.self_edge_weight() == 1);
    bool threw = false;
    try {
        d.add(1, 1, 1);
    } catch (const std::logic_error&) {
        threw = true;
    }
    EXPECT(threw);
    threw = false;
    try {
        (void)d.get(3, 1);
    } catch (const std::logic_error&) {
        threw = true;
    }
    EXPECT(threw);

    // BlockMatrix: 3 blocks, cells (0,0)=2 (0,2)=1 (1,0)=4 (2,2)=5
    s::BlockMatrix m(3, {{0, 0, 2}, {0, 2, 1}, {1, 0, 4}, {2, 2, 5}});
    EXPECT(m.get(1, 0) == 4 && m.get(0, 1) == 0);
    EXPECT(m.getrow(0) == (std::vector<long>{2, 0, 1}));
    EXPECT(m.getcol(0) == (std::vector<long>{2, 4, 0}));
    EXPECT(m.sum(0) == (std::vector<long>{3, 4, 5}) && m.sum(1) == (std::vector<long>{6, 0, 6}));
    EXPECT(m.edges() == 12 && m.trace() == 7);
    EXPECT(m.neighbors(0) == (std::set<long>{0, 1, 2}) && m.distinct_edges(1) == 1);
    const s::EdgeWeights o = m.outgoing_edges(0);
    EXPECT(o.indices == (std::vector<long>{0, 2}) && o.values == (std::vector<long>{2, 1}));
    EXPECT(m.entries().size() == 4);
    threw = false;
    try {
        (void)m.get(3, 0);
    } catch (const std::out_of_range&) {
        threw = true;
    }
    EXPECT(threw);

    // edge_weights: unit weights, the vertex itself left out on request
    const s::NeighborList nl = {{1, 0, 2}, {}, {2}};
    const s::EdgeWeights w = s::finetune::edge_weights(nl, 0);
    EXPECT(w.indices == (std::vector<long>{1, 0, 2}) && w.values == (std::vector<long>{1, 1, 1}));
    EXPECT(s::finetune::edge_weights(nl, 0, true).indices == (std::vector<long>{1, 2}));

    // early_stop and the greedy accept rule
    EXPECT(s::finetune::early_stop(0, true, 10.0, std::vector<double>{0.0}));
    EXPECT(!s::finetune::early_stop(2, true, 10.0, std::vector<double>{-1.0, -1.0, -1.0}));
    EXPECT(s::finetune::early_stop(3, false, 1e6, std::vector<double>{-1.0, -1.0, -1.0}));
    s::Args g;
    g.greedy = true;
    EXPECT(s::finetune::accept(-1e-9, 1.0, g) && !s::finetune::accept(0.0, 1.0, g));

    std::printf("%s\n", g_fail ? "FAILED" : "OK");
    return g_fail ? 1 : 0;
}

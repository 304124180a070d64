// The search loop of the integration guide, as a caller of the reference writes it
// (src/sbp.cpp:27-44) with the names of include/sbp_gb300.hpp; compiled (not run) by the
// CPU tests so that the guide's example stays valid.
#include "sbp_gb300.hpp"

using namespace sbp_gb300;

Blockmodel partition(Graph& graph) {
    Blockmodel blockmodel(graph.num_vertices(), graph, 0.5);  // every vertex its own block
    BlockmodelTriplet triplet;
    int iteration = 0;
    while (!sbp::done_blockmodeling(blockmodel, triplet)) {
        block_merge::merge_blocks(blockmodel, graph, graph.num_edges(), iteration);
        finetune::mcmc(iteration, graph, blockmodel, triplet);
        blockmodel = triplet.get_next_blockmodel(blockmodel);
        ++iteration;
    }
    return triplet.get(1).copy();
}

/*
 * CPU oracle for the SBP hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, on the CPU and single-address-space, the reference
 * algorithm of vtsynergy/SBP for the MCMC vertex-move sweep (asynchronous Gibbs,
 * hybrid MCMC, Metropolis-Hastings) and the block-merge pass, scored by delta-MDL
 * over the blockmodel.  It is used by the test-suite, by the package's smoke check
 * and by the CPU-baseline leg of the benchmark as the checker; the product never
 * links, imports or executes it.
 *
 * Every function cites the reference file:line it follows.  Where the reference is
 * non-reproducible (std::random_device seeding, robin_map iteration order) the
 * oracle uses the canonical seeded stream that the GPU implementation also uses:
 * Philox4x32-10 counters and ascending-id iteration (see sbp_oracle.cpp).
 */
#ifndef SBP_ORACLE_H
#define SBP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_graph ora_graph;
typedef struct ora_bm ora_bm;

/* Mirrors the hot-path subset of the reference's Args (include/args.hpp:61-212). */
typedef struct ora_config {
    int32_t algorithm;        /* 0 async_gibbs, 1 hybrid_mcmc, 2 metropolis_hastings */
    int32_t batches;          /* --batches */
    float   mh_percent;       /* --mh_percent (float, as in the reference) */
    int32_t greedy;           /* --greedy switch (default true) */
    int32_t ordered;          /* --ordered */
    int32_t approximate;      /* --approximate */
    int32_t asynciterations;  /* --asynciterations */
    int32_t max_iterations;   /* MAX_NUM_ITERATIONS (finetune.hpp:34) = 100 */
    int32_t nonparametric;    /* --nonparametric: entropy::nonparametric::*, greedy forced off (args.hpp:204-207) */
    int32_t split;            /* --split: 0 random, 1 snowball, 2 single-snowball, 3 connectivity-snowball */
    int32_t splitinit;        /* --splitinit: 0 random, 1 degree-weighted, 2 high-degree */
} ora_config;

typedef struct ora_stats {
    int64_t proposals;        /* vertex proposals evaluated (sweep) */
    int64_t merge_proposals;  /* merge proposals evaluated */
    int64_t moves;            /* vertex moves applied */
    int64_t mcmc_iterations;
    int64_t merges;           /* block merges applied */
    int64_t edges_swept;      /* sum of vertex degrees over proposals */
    int64_t outer_steps;
} ora_stats;

/* Philox4x32-10 (Salmon et al., SC'11).  ctr[4], key[2] -> out[4]. */
void ora_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

ora_graph* ora_graph_create(int64_t num_vertices, int64_t num_edges,
                            const int32_t* src, const int32_t* dst);
void ora_graph_destroy(ora_graph* g);

/* Blockmodel(num_blocks, graph, 0.5, assignment) (blockmodel.hpp:82-88). */
ora_bm* ora_bm_create(const ora_graph* g, int64_t num_blocks, const int32_t* assignment);
ora_bm* ora_bm_copy(const ora_bm* bm);
void ora_bm_destroy(ora_bm* bm);
int64_t ora_bm_num_blocks(const ora_bm* bm);
int64_t ora_bm_nnz(const ora_bm* bm);
/* assignment[N]; degrees/sizes[B]; cells (row, col, count) in row-major ascending order. */
void ora_bm_read(const ora_bm* bm, int32_t* assignment, int64_t* d_out, int64_t* d_in,
                 int64_t* d_tot, int64_t* sizes, int32_t* rows, int32_t* cols, int64_t* counts);
int64_t ora_bm_get(const ora_bm* bm, int64_t row, int64_t col);

/* entropy::mdl (entropy.cpp:597-604).  literal = reference arithmetic (glibc logf of the
 * ratio, double sum in row-major order); canonical = exact fixed-point sum of the
 * correctly-rounded float log, the value the device computes. */
void ora_mdl(const ora_bm* bm, double* literal, double* canonical);

/* entropy::delta_mdl(Blockmodel, Delta, proposal) (entropy.cpp:298-403) for moving
 * `vertex` to `proposal`.  literal = reference double arithmetic in ascending order;
 * fixed = the same sum in units of 2^-24 (exact). */
void ora_delta_mdl(const ora_bm* bm, int64_t vertex, int64_t proposal,
                   double* literal, int64_t* fixed);
/* entropy::block_merge_delta_mdl (entropy.cpp:129-182) for merging block into proposal. */
void ora_merge_delta_mdl(const ora_bm* bm, int64_t block, int64_t proposal,
                         double* literal, int64_t* fixed);
/* finetune::blockmodel_delta (finetune.cpp:201-235): writes up to cap entries. Returns count. */
int64_t ora_vertex_delta(const ora_bm* bm, int64_t vertex, int64_t proposal,
                         int32_t* rows, int32_t* cols, int64_t* vals, int64_t cap);
/* block_merge::blockmodel_delta (block_merge.cpp:14-38). */
int64_t ora_merge_delta(const ora_bm* bm, int64_t block, int64_t proposal,
                        int32_t* rows, int32_t* cols, int64_t* vals, int64_t cap);

/* Canonical proposals (common.cpp:138-198) under the seeded stream. */
int64_t ora_propose_vertex(const ora_bm* bm, int64_t vertex, uint64_t seed,
                           uint32_t c1, uint32_t c2, uint32_t c3);
int64_t ora_propose_merge(const ora_bm* bm, int64_t block, uint64_t seed,
                          uint32_t c2, int32_t proposal_index);

/* The proposal loop of block_merge::merge_blocks (block_merge.cpp:188-217) restricted to
 * blocks[0..n): best proposal and delta per listed block; returns the draws made (10 n). */
int64_t ora_merge_proposals(const ora_bm* bm, const int32_t* blocks, int64_t n, uint64_t seed,
                            uint32_t step, int32_t nonparametric, int32_t* best_out, double* dS_out);

/* A bounded sample of one golden-section step for timing: the merge proposals of
 * blocks[0..n), the carry-out of their queue to n / 2 merges, then `sweeps` hybrid sweeps
 * over the vertices of the merged blocks (hub[v]: chain, else one Gibbs batch).  Mutates
 * bm.  counts[0..2] = proposals drawn, merges, vertex proposals. */
void ora_step_sample(ora_bm* bm, const int32_t* blocks, int64_t n, const uint8_t* hub, uint64_t seed,
                     uint32_t step, const ora_config* cfg, int32_t sweeps, int64_t* counts);

/* One parallel-propose + serial-apply batch over vertices[0..n) (finetune.cpp:65-86):
 * proposals against the same snapshot, applied in vertex-id order with the
 * block-size-1 rejection of blockmodel.cpp:437-443. out_moves[i] = proposal or -1. */
int64_t ora_gibbs_batch(ora_bm* bm, const int32_t* vertices, int64_t n, uint64_t seed,
                        uint32_t iteration, uint32_t step, const ora_config* cfg,
                        int32_t* out_moves, double* out_dS);
/* Apply a precomputed move list (vertex-id order, size-1 rule). Returns moves applied. */
int64_t ora_apply_moves(ora_bm* bm, const int32_t* moves_per_vertex);

/* Sequential Metropolis-Hastings over order[0..n) (finetune::propose_move, finetune.cpp:842-869)
 * with draws (vertex, iteration, step, DOM_MH).  Returns the number of applied moves. */
int64_t ora_mh_chain(ora_bm* bm, const int32_t* order, int64_t n, uint64_t seed, uint32_t iteration,
                     uint32_t step, const ora_config* cfg);

/* finetune::mcmc dispatcher (finetune.cpp:754-771); mutates bm. */
int ora_mcmc(ora_bm* bm, const ora_config* cfg, uint64_t seed, int32_t step,
             int32_t golden_ratio_not_reached, ora_stats* stats);
/* block_merge::merge_blocks (block_merge.cpp:178-228); mutates bm.  Merges
 * `num_blocks_to_merge` blocks. */
int ora_merge_blocks(ora_bm* bm, const ora_config* cfg, uint64_t seed, int32_t step,
                     int64_t num_blocks_to_merge, ora_stats* stats);
/* sbp::stochastic_block_partition (sbp.cpp:16-72). Writes the final assignment;
 * returns the number of blocks (<0 on error). */
int64_t ora_sbp(const ora_graph* g, const ora_config* cfg, uint64_t seed,
                int32_t* out_assignment, double* out_mdl, ora_stats* stats);

/* entropy::nonparametric::mdl (entropy.cpp:751-779), directed and not degree-corrected.
 * literal = the reference's double arithmetic; canonical = the value the device computes
 * (lgamma terms rounded to 2^-24, exact integer sums). */
void ora_np_mdl(const ora_bm* bm, double* literal, double* canonical);
/* Its parts in the reference's arithmetic: sparse_entropy (:623-654), get_partition_dl
 * (:656-667), get_deg_dl_dist (:709-743, 0 without degree correction), get_edges_dl (:745-749). */
void ora_np_terms(const ora_bm* bm, double out[4]);
/* entropy::nonparametric::delta_mdl (entropy.cpp:1146-1178) and block_merge_delta_mdl
 * (:1198-1223); fixed = canonical value in units of 2^-24. */
void ora_np_delta_mdl(const ora_bm* bm, int64_t vertex, int64_t proposal, double* literal, int64_t* fixed);
void ora_np_merge_delta_mdl(const ora_bm* bm, int64_t block, int64_t proposal, double* literal, int64_t* fixed);
/* Blockmodel::num_nonempty_blocks as the oracle tracks it. */
int64_t ora_bm_nonempty(const ora_bm* bm);

/* Sampling (sample.cpp).  alg: 0 max_degree, 1 random, 2 degree_product, 3 detach.
 * mapping[v] = the vertex's id in the sample or -1; returns the sample's size. */
int64_t ora_sample(const ora_graph* g, int32_t alg, double samplesize, uint64_t seed, int32_t* mapping);
/* alg 4 expansion_snowball, 5 degree_product_snowball (serial, canonical draws). */
/* sample::reattach (sample.cpp:365-405). */
void ora_reattach(const ora_graph* g, const int32_t* sample_assignment, int64_t sample_n, int64_t num_blocks,
                  const int32_t* mapping, uint64_t seed, int32_t* out_assignment);
/* sample::from_vertices (sample.cpp:240-253). */
ora_graph* ora_subgraph(const ora_graph* g, const int32_t* mapping, int64_t n);
int64_t ora_graph_num_edges(const ora_graph* g);
/* Graph::num_edges (graph.hpp:99) as the description lengths use it: the stored directed
 * edges by default; half of them for an undirected edge list (graph.cpp:145-147). */
int64_t ora_graph_model_edges(const ora_graph* g);
void ora_graph_set_model_edges(ora_graph* g, int64_t num_edges);
/* args.undirected for the nonparametric entropy (entropy.hpp:102-133, entropy.cpp:745). */
void ora_graph_set_undirected(ora_graph* g, int32_t undirected);
/* args.degreecorrected for the nonparametric description length and vertex-move deltas
 * (entropy.hpp:117-133, entropy.cpp:617-764, :994-1110). */
void ora_graph_set_degree_corrected(ora_graph* g, int32_t on);
/* entropy::nonparametric::log_q (entropy.cpp:688-707) and spence (spence.hpp:9-22). */
double ora_log_q(int64_t n, int64_t k);
double ora_spence(double x);
/* The graph's edges, by source vertex, each source's out-neighbours in order. */
void ora_graph_edges(const ora_graph* g, int32_t* src, int32_t* dst);
/* sample::extend (sample.cpp:159-199). */
void ora_extend(const ora_graph* g, const int32_t* sample_assignment, int64_t sample_n, int64_t num_blocks,
                const int32_t* mapping, uint64_t seed, int32_t* out_assignment);
/* finetune::finetune_assignment (finetune.cpp:903-932); mutates bm. */
int ora_finetune_assignment(ora_bm* bm, const ora_config* cfg, uint64_t seed, ora_stats* stats);
/* main.cpp:98-140: sample, partition, extend, finetune.  Returns the number of blocks. */
int64_t ora_sbp_sampled(const ora_graph* g, const ora_config* cfg, uint64_t seed, int32_t alg, double samplesize,
                        int32_t* out_assignment, double* out_mdl, ora_stats* stats);

/* divisive::split_communities (top_down_sbp.cpp:472-530) with random splits toward
 * `target` blocks; mutates bm. */
int ora_split_communities(ora_bm* bm, const ora_config* cfg, uint64_t seed, uint32_t step, int64_t target);
/* divisive::run (top_down_sbp.cpp:435-470); mix: --mix (continue_agglomerative).  Returns
 * the number of blocks. */
int64_t ora_top_down(const ora_graph* g, const ora_config* cfg, uint64_t seed, int32_t mix, int32_t* out_assignment,
                     double* out_mdl, ora_stats* stats);

/* entropy::null_mdl_v1 (entropy.cpp:571-585) for a graph with `num_edges` edges. */
double ora_null_mdl_v1(double num_edges);

#ifdef __cplusplus
}
#endif
#endif

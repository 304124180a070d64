/*
 * sbpgpu -- C ABI of the GB300 (sm_103a) implementation of SBP's data-parallel hot
 * path: the MCMC vertex-move sweep (asynchronous Gibbs, hybrid MCMC,
 * Metropolis-Hastings) and the block-merge pass, scored by delta-MDL.
 *
 * Plain pointers and sizes only; every function returns an sbpgpu_status and the
 * message of the last failure is available from sbpgpu_last_error().  Host arrays are
 * read or written synchronously; device state stays resident between calls.
 *
 * Each entry point names the reference interface it replaces (path:line inside the
 * vtsynergy/SBP project).  A context is not thread-safe: use one per host thread.
 */
#ifndef SBPGPU_H
#define SBPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sbpgpu_status {
    SBPGPU_OK = 0,
    SBPGPU_EINVAL = 1,    /* invalid argument (std::invalid_argument / IndexOutOfBounds in the reference) */
    SBPGPU_ENOMEM = 2,    /* device allocation failed */
    SBPGPU_ETIMEOUT = 3,  /* a bounded device-side wait ran out */
    SBPGPU_EDEVICE = 4,   /* CUDA runtime error or a device-side consistency check failed */
    SBPGPU_EUNSUPPORTED = 5,
    SBPGPU_ECANCELED = 6  /* the call was cancelled (sbpgpu_ctx_set_cancel, sbpgpu_server_cancel) */
} sbpgpu_status;

typedef struct sbpgpu_ctx sbpgpu_ctx;
typedef struct sbpgpu_graph sbpgpu_graph;
typedef struct sbpgpu_bm sbpgpu_bm;

/* Hot-path subset of the reference's Args (include/args.hpp:61-212). */
typedef struct sbpgpu_config {
    int32_t algorithm;        /* 0 async_gibbs, 1 hybrid_mcmc (default), 2 metropolis_hastings (--algorithm) */
    int32_t batches;          /* --batches (default 1) */
    float   mh_percent;       /* --mh_percent (default 0.075) */
    int32_t greedy;           /* --greedy switch (default 1) */
    int32_t ordered;          /* --ordered (default 0) */
    int32_t approximate;      /* --approximate (default 0) */
    int32_t asynciterations;  /* --asynciterations (default INT32_MAX) */
    int32_t max_iterations;   /* MAX_NUM_ITERATIONS, include/finetune.hpp:34 (default 100) */
    int32_t nonparametric;    /* --nonparametric (default 0): entropy::nonparametric::* for every delta and
                                 MDL, in the graph's directed or undirected form, degree-corrected where
                                 the graph is marked so (sbpgpu_graph_set_degree_corrected, evaluation
                                 and single moves only); acceptance is then non-greedy
                                 without the Hastings correction (include/args.hpp:204-207,
                                 src/entropy.cpp:499) whatever `greedy` says */
    int32_t split;            /* --split (top-down): 0 random (default), 1 snowball, 2 single-snowball,
                                 3 connectivity-snowball */
    int32_t splitinit;        /* --splitinit: 0 random (default), 1 degree-weighted, 2 high-degree */
} sbpgpu_config;

typedef struct sbpgpu_stats {
    int64_t proposals;        /* vertex proposals visited by the sweeps */
    int64_t merge_proposals;  /* block-merge proposals */
    int64_t moves;            /* vertex moves applied */
    int64_t mcmc_iterations;
    int64_t merges;           /* block merges applied */
    int64_t edges_swept;      /* sum of k_out + k_in over visited vertex proposals */
    int64_t outer_steps;      /* golden-section iterations */
    int64_t kernel_launches;  /* kernels launched by this library for the call */
    int64_t gibbs_proposals;  /* vertex proposals of the parallel (asynchronous Gibbs) phases */
    int64_t gibbs_edges;      /* sum of k_out + k_in over those proposals */
    int64_t chain_rounds;     /* windows evaluated by the sequential MH chain */
    int64_t carry_rounds;     /* windows evaluated by the merge carry-out */
    int64_t carry_evaluations;  /* merge deltas recomputed by the carry-out */
    int64_t carry_keys;       /* row + column keys walked by those recomputations */
} sbpgpu_stats;

void sbpgpu_default_config(sbpgpu_config* cfg);

/* ---- context ------------------------------------------------------------------ */
sbpgpu_status sbpgpu_ctx_create(int32_t device, sbpgpu_ctx** out);
void sbpgpu_ctx_destroy(sbpgpu_ctx* ctx);
const char* sbpgpu_last_error(const sbpgpu_ctx* ctx);
/* Blocks the host until all work of the context has finished. */
sbpgpu_status sbpgpu_ctx_synchronize(sbpgpu_ctx* ctx);
/* The CUDA stream (cudaStream_t) all work of the context is issued on. */
void* sbpgpu_ctx_stream(sbpgpu_ctx* ctx);
/* Device memory (bytes) the sequential phases (merge carry-out, windowed MH chain) may hold
 * for dense num_blocks^2 int32 matrices of cell counts; larger blockmodels use the hashed
 * cell store.  Default 64 GiB (a GB300 holds about 280 GB); 0 always uses the hash.
 * Results do not depend on it.  No counterpart in the reference. */
sbpgpu_status sbpgpu_ctx_set_cells_budget(sbpgpu_ctx* ctx, int64_t bytes);
/* Smallest block count at which the sequential phases -- the Metropolis-Hastings chain and
 * the exact merge carry-out -- are evaluated in wide windows spread over a thread-block
 * cluster instead of one CTA; sets both thresholds (defaults: 65536 for the carry-out, 129
 * for the chain; 0: always, for the chain once the blockmodel has more than 128 blocks).
 * Results do not depend on them.  No counterpart in the reference. */
sbpgpu_status sbpgpu_ctx_set_cluster_blocks(sbpgpu_ctx* ctx, int64_t min_blocks);
/* The chain's threshold alone (default 129).  The partition server's workers set it to
 * 65536, so that concurrent jobs keep their chains on one SM each below that size. */
sbpgpu_status sbpgpu_ctx_set_chain_cluster_blocks(sbpgpu_ctx* ctx, int64_t min_blocks);
/* Requests (requested != 0) or withdraws cancellation of the context's running
 * sbpgpu_sbp; safe to call from another thread.  The partition checks the request between
 * golden-section steps, when none of its work is in flight on the device, withdraws it and
 * returns SBPGPU_ECANCELED; the context stays usable.  A request made while no partition
 * runs cancels the next one at its first step.  No counterpart in the reference. */
sbpgpu_status sbpgpu_ctx_set_cancel(sbpgpu_ctx* ctx, int32_t requested);
/* Failure injection for tests of the error paths: after `after` more device allocations
 * through the context, the next one fails as a failed cudaMallocAsync does (the call
 * returns SBPGPU_ENOMEM and the context stays usable); negative: no injection (default).
 * Nothing reaches the device.  No counterpart in the reference. */
sbpgpu_status sbpgpu_ctx_inject_alloc_failure(sbpgpu_ctx* ctx, int64_t after);

/* ---- graph: replaces Graph(out_neighbors, in_neighbors, ...) (include/graph.hpp:29-60)
 * and Graph::add_edge (src/graph.cpp:10-18).  Directed edges in input order; self-loops
 * and duplicate edges are kept.  Requires num_edges < 2^31. */
sbpgpu_status sbpgpu_graph_create(sbpgpu_ctx* ctx, int64_t num_vertices, int64_t num_edges,
                                  const int32_t* src, const int32_t* dst, sbpgpu_graph** out);
/* Same, with src/dst already resident in device memory. */
sbpgpu_status sbpgpu_graph_create_device(sbpgpu_ctx* ctx, int64_t num_vertices, int64_t num_edges,
                                         const int32_t* d_src, const int32_t* d_dst, sbpgpu_graph** out);
/* Graph::load (src/graph.cpp:33-233): a TSV edge list ("from to [weight]" per line, 1-based
 * ids; tabs, spaces or commas; lines starting with '%' or '#' skipped) or a Matrix Market
 * coordinate file (a "symmetric" one is read as undirected), parsed on the device.  With
 * `undirected`, or for symmetric Matrix Market, each edge u-v (u != v) is followed by v-u,
 * as the reference inserts it, so neighbour lists keep the reference's order.  The vertex
 * count is the largest id (at least the Matrix Market size).  The stored edge count
 * (sbpgpu_graph_num_edges) is the directed one; the model edge count is half of it for
 * undirected TSV input, as the reference's Graph reports it (graph.cpp:145-147). */
sbpgpu_status sbpgpu_graph_load(sbpgpu_ctx* ctx, const char* path, int32_t undirected, sbpgpu_graph** out);
void sbpgpu_graph_destroy(sbpgpu_graph* g);
int64_t sbpgpu_graph_num_vertices(const sbpgpu_graph* g);
/* The directed edges stored (the length of the edge arrays). */
int64_t sbpgpu_graph_num_edges(const sbpgpu_graph* g);
/* Graph::num_edges (include/graph.hpp:99) as the description lengths use it: entropy::mdl
 * (src/entropy.cpp:597-604), null_mdl_v1 and the nonparametric get_edges_dl
 * (:745-749).  It is the stored count, except for an undirected edge list, whose
 * reference Graph counts each stored pair once (src/graph.cpp:145-147).  The setter gives
 * the count of a graph built from arrays that hold both directions of each edge; EINVAL
 * for a count below 1. */
int64_t sbpgpu_graph_model_edges(const sbpgpu_graph* g);
sbpgpu_status sbpgpu_graph_set_model_edges(sbpgpu_graph* g, int64_t num_edges);
/* args.undirected (include/args.hpp:55) as the nonparametric entropy reads it
 * (include/entropy.hpp:102-133, src/entropy.cpp:745-749): a diagonal cell's eterm carries
 * -w log 2, a block's vertex term counts its out-degree only, and get_edges_dl spreads the
 * edges over B (B + 1) / 2 block pairs.  Set by sbpgpu_graph_load for undirected or
 * symmetric input and inherited by sampled subgraphs; off for graphs built from arrays
 * until set.  The parametric entropy does not read it. */
int32_t sbpgpu_graph_undirected(const sbpgpu_graph* g);
sbpgpu_status sbpgpu_graph_set_undirected(sbpgpu_graph* g, int32_t undirected);
/* args.degreecorrected (include/args.hpp:24) as the nonparametric description length reads
 * it: vertex terms become lgamma of the block degrees (include/entropy.hpp:117-133) and the
 * degree prior get_deg_entropy + get_deg_dl_dist (src/entropy.cpp:617-743) is added, with
 * per-block degree histograms of the current assignment (blockmodel.cpp:209-235) and
 * log_q, the partition-count asymptotic through the dilogarithm (:677-707).  Applies to
 * sbpgpu_np_mdl, sbpgpu_np_delta_mdl_batch (get_delta_deg_dl, :1072-1109) and the
 * nonparametric sbpgpu_move_vertex / sbpgpu_propose_move; sweeps, merges, splits and
 * partitions of a degree-corrected graph with the nonparametric entropy return
 * SBPGPU_EUNSUPPORTED, as does sbpgpu_np_merge_delta_mdl_batch. */
int32_t sbpgpu_graph_degree_corrected(const sbpgpu_graph* g);
sbpgpu_status sbpgpu_graph_set_degree_corrected(sbpgpu_graph* g, int32_t on);

/* ---- blockmodel: replaces Blockmodel(num_blocks, graph, rate, assignment) and
 * Blockmodel::initialize_edge_counts (src/blockmodel/blockmodel.cpp:193-276).
 * assignment == NULL means the identity assignment (B = N, src/sbp.cpp:23). */
sbpgpu_status sbpgpu_bm_create(sbpgpu_graph* g, int64_t num_blocks, const int32_t* assignment,
                               sbpgpu_bm** out);
/* Blockmodel::copy (src/blockmodel/blockmodel.cpp:139-153): device-to-device. */
sbpgpu_status sbpgpu_bm_copy(const sbpgpu_bm* bm, sbpgpu_bm** out);
void sbpgpu_bm_destroy(sbpgpu_bm* bm);
int64_t sbpgpu_bm_num_blocks(const sbpgpu_bm* bm);
int64_t sbpgpu_bm_nnz(const sbpgpu_bm* bm);
/* Blockmodel accessors (include/blockmodel/blockmodel.hpp:90-200): any pointer may be NULL.
 * degrees/sizes hold num_blocks values; rows/cols/counts hold nnz cells in row-major,
 * ascending order (the blockmatrix). */
sbpgpu_status sbpgpu_bm_read(const sbpgpu_bm* bm, int32_t* assignment, int64_t* d_out, int64_t* d_in,
                             int64_t* d_tot, int64_t* sizes, int32_t* rows, int32_t* cols, int64_t* counts);
/* Blockmodel::getOverall_entropy / setOverall_entropy */
double sbpgpu_bm_entropy(const sbpgpu_bm* bm);

/* ---- entropy ------------------------------------------------------------------- */
/* entropy::mdl (src/entropy.cpp:597-604). */
sbpgpu_status sbpgpu_mdl(sbpgpu_bm* bm, double* out);
/* entropy::delta_mdl(Blockmodel, Delta, proposal) (src/entropy.cpp:298-403) for n moves
 * vertex[i] -> proposal[i] against the current blockmodel. */
sbpgpu_status sbpgpu_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* vertex,
                                     const int32_t* proposal, double* out_delta);
/* The same as sbpgpu_delta_mdl_batch, for callers that must not allocate device memory
 * while they score moves (a cudaMalloc can synchronise the device, or fail when the GPU's
 * memory is committed elsewhere).  No counterpart in the reference.  The ids, proposals
 * and results are staged in a fixed 1 MiB device array built into the library, so n is at
 * most 65536; larger batches return SBPGPU_EINVAL.  The first call on a device looks the
 * array up (cudaGetSymbolAddress); make that first call before any stream capture.
 * Nothing needs zeroing beforehand.  Calls that overlap in time on the same device, from
 * any thread or context, share the array and race: serialise them.  The array's address is
 * kept for the life of the process: a cudaDeviceReset between calls is not supported. */
sbpgpu_status sbpgpu_delta_mdl_batch_noalloc(sbpgpu_bm* bm, int64_t n, const int32_t* vertex,
                                             const int32_t* proposal, double* out_delta);
/* entropy::block_merge_delta_mdl (src/entropy.cpp:129-182) for n merges block[i] -> proposal[i]. */
sbpgpu_status sbpgpu_merge_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* block,
                                           const int32_t* proposal, double* out_delta);
/* entropy::nonparametric (src/entropy.cpp:617-1225), directed, without degree correction:
 * mdl (:751-779), delta_mdl (:1146-1178) and block_merge_delta_mdl (:1198-1223).  The
 * lgamma(x + 1) terms are rounded to multiples of 2^-24 and summed exactly, so a delta
 * equals the difference of the two MDLs it connects up to one rounding of the terms that
 * depend on the number of non-empty blocks.  The graph's lgamma table is built on the
 * first call. */
sbpgpu_status sbpgpu_np_mdl(sbpgpu_bm* bm, double* out);
sbpgpu_status sbpgpu_np_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* vertex,
                                        const int32_t* proposal, double* out_delta);
sbpgpu_status sbpgpu_np_merge_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* block,
                                              const int32_t* proposal, double* out_delta);

/* ---- finetune ------------------------------------------------------------------ */
/* common::propose_new_block under the canonical seeded stream (src/common.cpp:138-198):
 * proposal for vertex[i] drawn with counter (vertex, c1, c2, c3). */
sbpgpu_status sbpgpu_propose_batch(sbpgpu_bm* bm, int64_t n, const int32_t* vertex, uint64_t seed,
                                   uint32_t c1, uint32_t c2, uint32_t c3, int32_t* out_proposal);
/* One asynchronous-Gibbs batch: propose for vertex[0..n) against one snapshot
 * (finetune::propose_gibbs_move_v3, src/finetune.cpp:871-901) and apply the accepted
 * moves in vertex-id order (Blockmodel::move_vertex(VertexMove_v3),
 * src/blockmodel/blockmodel.cpp:437-494).  out_moves[i] = accepted proposal or -1
 * (before the block-size-1 rule); returns the number of applied moves in *applied. */
sbpgpu_status sbpgpu_gibbs_batch(sbpgpu_bm* bm, const sbpgpu_config* cfg, int64_t n, const int32_t* vertex,
                                 uint64_t seed, uint32_t iteration, uint32_t step, int32_t* out_moves,
                                 int64_t* applied);
/* finetune::propose_gibbs_move_v3 (src/finetune.cpp:871-901) for vertex[0..n) against the
 * current blockmodel, with nothing applied: out_moves[i] = the accepted proposal or -1 --
 * the decisions sbpgpu_gibbs_batch takes before it applies them. */
sbpgpu_status sbpgpu_gibbs_propose(sbpgpu_bm* bm, const sbpgpu_config* cfg, int64_t n, const int32_t* vertex,
                                   uint64_t seed, uint32_t iteration, uint32_t step, int32_t* out_moves);
/* Sequential Metropolis-Hastings over vertex[0..n) in order, each accepted move applied
 * before the next proposal (finetune::propose_move / move_vertex, src/finetune.cpp:822-869). */
sbpgpu_status sbpgpu_mh_chain(sbpgpu_bm* bm, const sbpgpu_config* cfg, int64_t n, const int32_t* vertex,
                              uint64_t seed, uint32_t iteration, uint32_t step, int64_t* applied);
/* finetune::propose_move (src/finetune.cpp:842-869) for one vertex: the proposal drawn from
 * the canonical stream (vertex, iteration, step, MH domain) -- the draw the chain above
 * makes for that vertex -- then finetune::move_vertex on it.  *out_proposal is -1 when the
 * vertex's block is a singleton (*out_dS = DBL_MAX) or the proposal is its own block
 * (*out_dS = 0); *out_moved tells whether the move was applied.  Calling it for a sequence
 * of vertices gives the same state as sbpgpu_mh_chain on that sequence. */
sbpgpu_status sbpgpu_propose_move(sbpgpu_bm* bm, const sbpgpu_config* cfg, int32_t vertex, uint64_t seed,
                                  uint32_t iteration, uint32_t step, int32_t* out_proposal, double* out_dS,
                                  int32_t* out_moved);
/* finetune::move_vertex (src/finetune.cpp:822-840): scores moving `vertex` into `proposal`
 * against the current state (entropy::delta_mdl or its nonparametric form; the Hastings
 * correction when not greedy), decides with finetune::accept -- greedy: dS < 0; otherwise
 * the uniform draw of (vertex, iteration, step, MH domain) against min(1, e^(-3 dS) H) --
 * and, when accepted, applies the move (Blockmodel::move_vertex) and rebuilds. */
sbpgpu_status sbpgpu_move_vertex(sbpgpu_bm* bm, const sbpgpu_config* cfg, int32_t vertex, int32_t proposal,
                                 uint64_t seed, uint32_t iteration, uint32_t step, double* out_dS,
                                 int32_t* out_moved);
/* finetune::mcmc (src/finetune.cpp:754-771) dispatching to asynchronous_gibbs (:34-107),
 * hybrid_mcmc (:563-646) or metropolis_hastings (:773-820). */
sbpgpu_status sbpgpu_mcmc(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed, int32_t step,
                          int32_t golden_ratio_not_reached, sbpgpu_stats* stats);

/* ---- block merge --------------------------------------------------------------- */
/* block_merge::merge_blocks (src/block_merge.cpp:178-228): 10 proposals per block,
 * carry_out_best_merges_advanced (:40-117) or, with cfg->approximate,
 * Blockmodel::carry_out_best_merges (src/blockmodel/blockmodel.cpp:55-122); then the
 * blockmodel is rebuilt with num_blocks - num_blocks_to_merge blocks. */
sbpgpu_status sbpgpu_merge_blocks(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed, int32_t step,
                                  int64_t num_blocks_to_merge, sbpgpu_stats* stats);
/* The per-block best merge proposals only (block_merge.cpp:189-217). */
sbpgpu_status sbpgpu_merge_proposals(sbpgpu_bm* bm, uint64_t seed, int32_t step, int32_t* best_proposal,
                                     double* best_delta);

/* ---- full partition ------------------------------------------------------------ */
/* sbp::stochastic_block_partition (src/sbp.cpp:16-72) with the golden-section search of
 * BlockmodelTriplet (src/blockmodel/blockmodel_triplet.cpp:4-105).  Writes the final
 * assignment (num_vertices values) and returns the number of blocks in *num_blocks. */
sbpgpu_status sbpgpu_sbp(sbpgpu_graph* g, const sbpgpu_config* cfg, uint64_t seed, int32_t* out_assignment,
                         int64_t* num_blocks, double* out_mdl, sbpgpu_stats* stats);

/* ---- sampling (src/sample.cpp, src/main.cpp:98-140) ------------------------------ */
/* A vertex sample: algorithm 0 max_degree (sample.cpp:255-270), 1 random (:272-284, the
 * seeded stream), 2 degree_product (:28-49), 3 detach (:12-26, vertices of degree above 1;
 * sample_size unused), 4 expansion_snowball (:125-157), 5 degree_product_snowball (:51-101;
 * the two snowballs grow one vertex at a time and run on the host).  mapping[N] receives each vertex's id in the sample or -1;
 * sample_n the sample's size (long(sample_size * N) vertices, or as the algorithm gives). */
sbpgpu_status sbpgpu_sample(sbpgpu_graph* g, int32_t algorithm, double sample_size, uint64_t seed,
                            int32_t* mapping, int64_t* sample_n);
/* sample::from_vertices (sample.cpp:240-253): the graph of the sampled vertices. */
sbpgpu_status sbpgpu_graph_subgraph(sbpgpu_graph* g, const int32_t* mapping, int64_t sample_n,
                                    sbpgpu_graph** out);
/* sample::extend (sample.cpp:159-199): sampled vertices keep their sample block; the others,
 * in vertex order, take the block most of their assigned neighbours are in (ties to the
 * smallest block), or a block drawn from the seeded stream. */
sbpgpu_status sbpgpu_extend(sbpgpu_graph* g, const int32_t* sample_assignment, int64_t sample_n,
                            int64_t num_blocks, const int32_t* mapping, uint64_t seed, int32_t* out_assignment);
/* sample::reattach (sample.cpp:365-405) after a detach: a detached vertex takes its one
 * neighbour's block, or (alone, or paired with another detached vertex) a block drawn from
 * the seeded stream.  Every unsampled vertex must have degree 0 or 1. */
sbpgpu_status sbpgpu_reattach(sbpgpu_graph* g, const int32_t* sample_assignment, int64_t sample_n,
                              int64_t num_blocks, const int32_t* mapping, uint64_t seed, int32_t* out_assignment);
/* finetune::finetune_assignment (src/finetune.cpp:903-932). */
sbpgpu_status sbpgpu_finetune_assignment(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed,
                                         sbpgpu_stats* stats);
/* The --samplesize < 1 path of main.cpp:98-140: sample, sbpgpu_sbp on the sample, extend,
 * then finetune_assignment on the full graph. */
sbpgpu_status sbpgpu_sbp_sampled(sbpgpu_graph* g, const sbpgpu_config* cfg, uint64_t seed, int32_t algorithm,
                                 double sample_size, int32_t* out_assignment, int64_t* num_blocks,
                                 double* out_mdl, sbpgpu_stats* stats);

/* ---- top-down (divisive) partitioning (src/top_down_sbp.cpp) --------------------- */
/* divisive::split_communities (top_down_sbp.cpp:472-530) with --split random: every cluster
 * of at least 0.001 N vertices gets 10 random two-way splits scored by the nonparametric
 * description length of its subgraph against entropy::null_mdl_v1; the clusters are split
 * in ascending order of their best delta until the block count reaches the target. */
sbpgpu_status sbpgpu_split_communities(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed, int32_t step,
                                       int64_t target_num_blocks);
/* divisive::run (top_down_sbp.cpp:435-470): from one block, split toward ceil(1.5 B)
 * blocks and finetune until the golden-section bracket of TopDownBlockmodelTriplet closes;
 * with mix (--mix) until the bracket forms, then continue_agglomerative (:67-98). */
sbpgpu_status sbpgpu_sbp_top_down(sbpgpu_graph* g, const sbpgpu_config* cfg, uint64_t seed, int32_t mix,
                                  int32_t* out_assignment, int64_t* num_blocks, double* out_mdl,
                                  sbpgpu_stats* stats);

/* ---- evaluation ------------------------------------------------------------------ */
/* evaluate::evaluate_blockmodel (src/evaluate.cpp:9-180) against a true partition: the
 * contingency table is counted on the device; NMI (float-log marginal entropies as the
 * reference), pair-counting F1 / precision / recall / Rand index and the accuracy of the
 * best one-to-one matching of communities follow on the host.  truth[i] < 0 marks an
 * unlabelled vertex (left out of the table); assignment values are blocks >= 0. */
typedef struct sbpgpu_eval {
    double nmi, f1, precision, recall, rand_index, accuracy;
    int64_t true_blocks, found_blocks;
} sbpgpu_eval;
sbpgpu_status sbpgpu_evaluate(sbpgpu_ctx* ctx, int64_t n, const int32_t* truth, const int32_t* assignment,
                              sbpgpu_eval* out);
/* evaluate::calculate_f1_score and evaluate::calculate_nmi (src/evaluate.cpp:9-98) of a
 * contingency table given row-major, nrows x ncols, as the reference's Hungarian::Matrix:
 * F1, precision, recall and Rand index by pair counting and NMI, over num_vertices.  A host
 * computation that needs no device; accuracy is left 0, true_blocks = ncols and
 * found_blocks = nrows. */
sbpgpu_status sbpgpu_partition_scores(int64_t num_vertices, int64_t nrows, int64_t ncols, const int64_t* table,
                                      sbpgpu_eval* out);

/* ---- batched and served partitioning ----------------------------------------------
 * No counterpart in the reference (its plain driver partitions one graph per process).  A
 * server partitions many independent graphs at once on one device: `workers` host threads,
 * each with its own context and stream, take jobs in submission order and run
 * sbpgpu_sbp on them concurrently.  A job is admitted while the estimated device footprint
 * (sbpgpu_job_footprint) of the jobs in flight plus its own stays within hbm_budget_bytes;
 * a job whose own footprint exceeds the budget is refused at submission (SBPGPU_ENOMEM).  Each worker's context uses
 * cells_budget_bytes for dense cell counts (sbpgpu_ctx_set_cells_budget).  A job's result
 * equals sbpgpu_sbp of the same graph, configuration and seed run alone.  The job's host
 * arrays must stay valid until sbpgpu_server_wait returns for it.  Set the environment
 * variable CUDA_DEVICE_MAX_CONNECTIONS=32 before CUDA starts in the process: with the
 * default 8 hardware queues the workers' streams share queues and wait on one another. */
typedef struct sbpgpu_server sbpgpu_server;
typedef struct sbpgpu_job {
    int64_t num_vertices;
    int64_t num_edges;
    const int32_t* src;          /* host edge arrays, as sbpgpu_graph_create */
    const int32_t* dst;
    sbpgpu_config config;
    uint64_t seed;
    int32_t* out_assignment;     /* host, num_vertices entries, written by the job */
} sbpgpu_job;
typedef struct sbpgpu_job_result {
    sbpgpu_status status;
    int64_t num_blocks;
    double mdl;
    double queued_ms;            /* submission to start */
    double run_ms;               /* start to finish (graph upload, partition, result read) */
    sbpgpu_stats stats;
    char error[256];             /* message of a failed job */
} sbpgpu_job_result;

/* Estimated device bytes of one job (graph, work buffers, blockmodels, dense cells). */
int64_t sbpgpu_job_footprint(int64_t num_vertices, int64_t num_edges, int64_t cells_budget_bytes);
sbpgpu_status sbpgpu_server_create(int32_t device, int32_t workers, int64_t hbm_budget_bytes,
                                   int64_t cells_budget_bytes, sbpgpu_server** out);
sbpgpu_status sbpgpu_server_submit(sbpgpu_server* server, const sbpgpu_job* job, int64_t* ticket);
/* Blocks until the job is done and returns its result (once per ticket). */
sbpgpu_status sbpgpu_server_wait(sbpgpu_server* server, int64_t ticket, sbpgpu_job_result* result);
/* As sbpgpu_server_wait, but returns SBPGPU_ETIMEOUT when the job is not done within
 * timeout_ms; the ticket stays valid. */
sbpgpu_status sbpgpu_server_wait_for(sbpgpu_server* server, int64_t ticket, int64_t timeout_ms,
                                     sbpgpu_job_result* result);
/* Cancels a job: a queued job is removed at once; a running one stops at its next
 * golden-section step (sbpgpu_ctx_set_cancel).  Its result then has status
 * SBPGPU_ECANCELED; a job that finishes first keeps its result.  SBPGPU_EINVAL for an
 * unknown ticket. */
sbpgpu_status sbpgpu_server_cancel(sbpgpu_server* server, int64_t ticket);
/* Pauses (paused != 0) or resumes the start of queued jobs; running jobs go on.
 * Destroying a paused server still finishes every submitted job. */
sbpgpu_status sbpgpu_server_pause(sbpgpu_server* server, int32_t paused);
/* Failure injection for tests: the queued job's worker context fails its device
 * allocation number `after` + 1 (sbpgpu_ctx_inject_alloc_failure).  SBPGPU_EINVAL once the
 * job has started. */
sbpgpu_status sbpgpu_server_inject_alloc_failure(sbpgpu_server* server, int64_t ticket, int64_t after);
/* Finishes every submitted job, then stops the workers. */
void sbpgpu_server_destroy(sbpgpu_server* server);
/* The batched form: n jobs through a server, results in job order. */
sbpgpu_status sbpgpu_sbp_batch(int32_t device, int32_t workers, int64_t hbm_budget_bytes, int64_t cells_budget_bytes,
                               int64_t n, const sbpgpu_job* jobs, sbpgpu_job_result* results);

/* ---- timing of the dominant kernels (CUDA events on the context's stream) --------- */
typedef struct sbpgpu_kernel_timing {
    double gibbs_propose_ms;  int64_t gibbs_propose_launches;  int64_t gibbs_propose_bytes;
    double mh_chain_ms;       int64_t mh_chain_launches;
    double merge_propose_ms;  int64_t merge_propose_launches;  int64_t merge_propose_bytes;
    double carry_out_ms;      int64_t carry_out_launches;
    double rebuild_ms;        int64_t rebuild_launches;       int64_t rebuild_bytes;
} sbpgpu_kernel_timing;
/* Enables (1) or disables (0) event timing; reading resets the accumulators. */
void sbpgpu_set_timing(sbpgpu_ctx* ctx, int32_t enabled);
sbpgpu_status sbpgpu_read_timing(sbpgpu_ctx* ctx, sbpgpu_kernel_timing* out);

#ifdef __cplusplus
}
#endif
#endif

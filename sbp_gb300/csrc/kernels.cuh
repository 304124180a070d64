// Host-side launchers of the sbpgpu kernels (implemented in blockmodel.cu, sweep.cu,
// merge.cu).  All work is issued on the given stream.
#pragma once

#include <string>
#include <vector>

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sbp {

// Device buffers shared by the phases of one graph (sized for B <= N, nnz <= E).
struct Work {
    // sort / rebuild
    uint64_t* keys = nullptr;
    uint64_t* keys_alt = nullptr;
    int32_t* vals = nullptr;
    int32_t* vals_alt = nullptr;
    int32_t* flags = nullptr;
    void* temp = nullptr;
    size_t temp_bytes = 0;
    int32_t* d_scalar = nullptr;       // [8] small device scalars
    unsigned long long* d_acc = nullptr;  // [4] device accumulators
    // sweeps
    int32_t* moves = nullptr;          // [N] accepted proposal per vertex or -1
    int32_t* m_out = nullptr;          // [N]
    int32_t* last = nullptr;           // [N]
    int32_t* acc = nullptr;            // [N]
    int32_t* dep = nullptr;            // [2N]
    int32_t* list_small = nullptr;     // [N]
    int32_t* list_big = nullptr;       // [N]
    int32_t* list_tmp = nullptr;       // [N]
    int32_t* ghash = nullptr;          // global group hash for huge vertices [3 << ghash_log2]
    int ghash_log2 = 0;
    // chain state
    DevChain chain{};
    ulonglong2* chain_slots = nullptr;
    uint64_t chain_cap = 0;            // allocated slots (power of two)
    int32_t* pool = nullptr;
    int64_t pool_words = 0;
    int32_t* row_head = nullptr;       // [N]
    int32_t* col_head = nullptr;       // [N]
    // merge
    int32_t* best = nullptr;           // [N]
    double* best_dS = nullptr;         // [N]
    double* heap_dS = nullptr;         // [N]
    int32_t* heap_blk = nullptr;       // [N]
    int32_t* parent = nullptr;         // [N]
    int32_t* root = nullptr;           // [N]
    int32_t* used = nullptr;           // [N]
    DevFlags* flags_dev = nullptr;
    int32_t* dense_M = nullptr;        // [kDenseGlobalMax^2] (allocated when N allows)
    int32_t* dense_MT = nullptr;
    int32_t dense_cap = 0;             // largest B the dense matrices hold
    // neighbour hashes of the windowed chain's high-degree vertices [16 warps x 4 x 8192]
    int32_t* win_hash = nullptr;
    // the cluster chain's per-warp neighbour hashes and row scratch (allocated on first use)
    int32_t* cl_hash = nullptr;
    int32_t* cl_scratch = nullptr;
    // the cluster carry-out's per-block candidate (or -1) and staged new keys of the merges'
    // targets (allocated on first use)
    int32_t* cc_head = nullptr;        // [N]
    int32_t* cc_stage = nullptr;
    // dense B x B cell values of the merge carry-out (allocated on demand within a budget)
    int32_t* cells = nullptr;
    uint64_t cells_elems = 0;
};

int ceil_log2(uint64_t x);

// ---- blockmodel.cu
// Blockmodel::initialize_edge_counts: rebuilds degrees, sizes and the sorted CSR / CSC
// of the blockmatrix from bm.asg.  Updates bm.nnz (read back to the host).
void rebuild(const DevGraph& g, DevBM& bm, Work& w, cudaStream_t st);
// Sum of v * canonical_log(v / (d_out * d_in)) in units of 2^-24 into w.d_acc[0].
void launch_mdl(const DevGraph& g, const DevBM& bm, Work& w, cudaStream_t st);
// The table terms of nonparametric::mdl (entropy.cpp:751-779) in units of 2^-24 into
// w.d_acc[0]: -sum LG[cell] + sum over blocks (vterm - LG[size]).
void launch_np_mdl(const DevGraph& g, const DevBM& bm, Work& w, cudaStream_t st);
// Degree-corrected additions (degcorr.cu): to the description length, added into *acc in
// units of 2^-24; and to each vertex move's delta out[i] (units of 2^-24).
void launch_dc_mdl(const DevGraph& g, const DevBM& bm, unsigned long long* acc, cudaStream_t st);
void launch_dc_vertex_deltas(const DevGraph& g, const DevBM& bm, const int32_t* v, const int32_t* s, int64_t n,
                             long long* out, cudaStream_t st);
// np: nonparametric deltas (the graph's nonparametric tables must exist).
// hastings (optional, not with np): entropy::hastings_correction of each pair.
void launch_vertex_dS_batch(const DevGraph& g, const DevBM& bm, const int32_t* v, const int32_t* s, int64_t n,
                            int32_t max_k, long long* out, Work& w, cudaStream_t st, bool np = false,
                            double* hastings = nullptr);
void launch_merge_dS_batch(const DevGraph& g, const DevBM& bm, const int32_t* r, const int32_t* s, int64_t n,
                           long long* out, Work& w, cudaStream_t st, bool np = false);
void launch_propose_batch(const DevGraph& g, const DevBM& bm, const int32_t* v, int64_t n, uint64_t seed,
                          uint32_t c1, uint32_t c2, uint32_t c3, int32_t* out, cudaStream_t st);
// Initialises the chain cell store from the current CSR (capacity for extra new keys).
void chain_init(const DevBM& bm, Work& w, uint64_t extra_keys, cudaStream_t st);
// Initialises only the chain's row / column key lists (empty appended chunks).
void lists_init(const DevBM& bm, Work& w, cudaStream_t st);

// ---- sweep.cu
// Proposals for vlist[0..n) against the current snapshot (moves[v] = s or -1), then the
// vertex-id-order apply with the block-size-1 rule; asg updated (no rebuild).
// mode: ACC_GREEDY, ACC_HASTINGS or ACC_NP.
void gibbs_propose(const DevGraph& g, const DevBM& bm, const int32_t* vlist, int32_t n, int32_t small_k,
                   uint64_t seed, uint32_t iter, uint32_t step, int mode, Work& w, cudaStream_t st);
void gibbs_apply(const DevBM& bm, const int32_t* vlist, int32_t n, Work& w, cudaStream_t st);
void mh_chain(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, int32_t max_k, uint64_t seed,
              uint32_t iter, uint32_t step, int greedy, Work& w, cudaStream_t st);
// The same chain with the whole blockmatrix in shared memory (B <= kDenseMax).
constexpr int32_t kDenseMax = 192;
constexpr int32_t kDenseGlobalMax = 4096;
size_t mh_chain_dense_smem(int32_t B);
void mh_chain_dense(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, uint64_t seed, uint32_t iter,
                    uint32_t step, Work& w, cudaStream_t st);
// The chain evaluated in windows of upcoming vertices (chain_window.cu): cells dense in
// shared memory for B <= kWinSharedMax, else dense M, its transpose and their row tile
// sums in w.cells (mh_window_cells(B) int32).
constexpr int32_t kWinSharedMax = 128;
struct WindowPlan {
    int nw;        // warps, one window entry each
    int mode;      // 0 shared cells; 1 global cells, shared degrees; 2 all global
    int log2cap;   // neighbour-hash size for the largest vertex
    int64_t ld;    // leading dimension of the dense cells
};
uint64_t mh_window_cells(int32_t B);
// False when the windowed chain does not apply (a vertex needs a hash over 2^13 slots, or
// no dense buffer holds the matrices).
bool mh_window_plan(int32_t B, int32_t max_k, const Work& w, WindowPlan* p);
void mh_chain_window(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, const WindowPlan& p,
                     uint64_t seed, uint32_t iter, uint32_t step, int mode, Work& w, cudaStream_t st);
// The chain evaluated in windows spread over a thread-block cluster (chain_cluster.cu), for
// blockmodels with many blocks: cells dense in w.cells (as the windowed chain's global mode)
// or, when hashed is set, in the chain hash (chain_init first).  mh_cluster_size() is the
// cluster size the device holds (0: none); the buffers w.cl_hash and w.cl_scratch hold
// mh_cluster_hash_ints / mh_cluster_scratch_ints int32 for it.
int mh_cluster_size();
size_t mh_cluster_hash_ints(int cs);
size_t mh_cluster_scratch_ints(int cs);
void mh_chain_cluster(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, int32_t max_k, bool hashed,
                      uint64_t seed, uint32_t iter, uint32_t step, int mode, Work& w, cudaStream_t st);
// order[i] = base[perm(i)] with the canonical shuffle keyed by (i, iter, step, dom).
void shuffle(const int32_t* base, int32_t n, uint64_t seed, uint32_t iter, uint32_t step, uint32_t dom,
             int32_t* order, Work& w, cudaStream_t st);

// ---- merge.cu
// np: score with nonparametric::block_merge_delta_mdl.
void merge_propose(const DevGraph& g, const DevBM& bm, uint64_t seed, uint32_t step, Work& w, cudaStream_t st,
                   bool np = false);
// Carries out merges; writes the number done to w.d_scalar[1].  Leaves asg relabelled
// to dense block ids (B - merges blocks); the caller rebuilds.
// cluster: the exact carry-out on a thread-block cluster (carry_cluster.cu).
void carry_out(const DevGraph& g, DevBM& bm, int64_t num_to_merge, int approximate, Work& w, cudaStream_t st,
               bool np = false, bool cluster = false);

// ---- carry.cu
// carry_out_best_merges_advanced over the queue (w.keys, w.vals) sorted by (delta, block)
// with the union-find block map in w.parent (identity on entry).  Uses the dense cells
// w.cells when B * B <= w.cells_elems, the chain hash otherwise.
void carry_out_exact(const DevGraph& g, DevBM& bm, int64_t num_to_merge, Work& w, cudaStream_t st, bool np = false);
// The same on a thread-block cluster of carry_cluster_size() CTAs (0: the device holds
// none); needs w.cc_head and w.cc_stage.
int carry_cluster_size();
size_t carry_cluster_stage_ints(int cs);
void carry_out_cluster(const DevGraph& g, DevBM& bm, int64_t num_to_merge, Work& w, cudaStream_t st, bool np);

// Blocks the calling thread, sleeping rather than spinning, until the work queued on st so
// far is done (many host threads may each drive a context of their own).
void host_wait(cudaStream_t st);
// 256 bytes of pinned host memory belonging to the calling thread, for scalar read-backs.
void* host_scratch();

// Raises `func`'s dynamic shared-memory limit to the most the device allows, once per
// kernel.  Every launcher uses the same limit, so host threads that launch concurrently
// (the partition server's workers) never lower it under one another.
void allow_max_dynamic_smem(const void* func);

// ---- ingest.cu
// Parses edge lines ("from to [weight]", 1-based) held in device memory into 0-based device
// edge arrays in file order, with each reverse edge right after its edge when undirected.
// *max_id is the largest 1-based id seen.  The arrays are allocated on st (cudaMallocAsync).
bool parse_edges_device(const char* d_text, int64_t n, int undirected, int32_t** d_src, int32_t** d_dst, int64_t* E,
                        int64_t* max_id, std::string* err, cudaStream_t st);

// ---- sample.cu
// Philox4x32-10 on the host: the device stream's words for the same counter and key.
void philox_host(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint64_t seed, uint32_t w[4]);
// A host copy of the adjacency: out-lists in input order, in-lists with each self-loop as
// the vertex itself, and Graph::degrees (out + in - has a self-loop).
struct HostAdjacency {
    std::vector<int32_t> out_off, out_nbr, in_off, in_nbr, deg;
};
HostAdjacency host_adjacency(const DevGraph& g, cudaStream_t st);
// Vertex sample (alg 0 max_degree, 1 random, 2 degree_product, 3 detach) into the device
// array mapping[N] (sample id or -1); returns the sample's size.
int64_t sample_vertices(const DevGraph& g, int alg, double samplesize, uint64_t seed, int32_t* mapping, Work& w,
                        cudaStream_t st);
// Edges between sampled vertices, relabelled, in out-CSR order (cudaMallocAsync'd; the
// caller frees them).
void subgraph_edges(const DevGraph& g, const int32_t* mapping, int32_t** d_src, int32_t** d_dst, int64_t* E,
                    Work& w, cudaStream_t st);
// sample::extend into asg[N] (device), from the sample's assignment (device).
void extend_assignment(const DevGraph& g, const int32_t* mapping, const int32_t* sample_asg, int32_t B,
                       int32_t max_k, uint64_t seed, int32_t* asg, cudaStream_t st);

// sample::reattach into asg[N] for a mapping whose unsampled vertices have degree <= 1.
void reattach_assignment(const DevGraph& g, const int32_t* mapping, const int32_t* sample_asg, int32_t B, uint64_t seed,
                         int32_t* asg, cudaStream_t st);

// ---- split.cu
// Buffers of one split pass over B clusters (10 proposals each) and N vertices.
struct SplitBuffers {
    long long* split_size;       // [B * 10] side-0 size, or -1 when the cluster is not split
    int32_t* eligible;           // [B] cluster of at least 0.001 N vertices
    uint16_t* mask;              // [N] bit i: the vertex's side in proposal i
    int32_t* n1;                 // [B * 10] vertices on side 1
    int32_t* cells;              // [B * 10 * 4] 2 x 2 blockmatrix of the cluster's edges
    unsigned long long* ecount;  // [B] edges inside the cluster
    int32_t* new_block;          // [B] block receiving the cluster's side 1, or -1
    int32_t* proposal;           // [B] the proposal applied
};
// Counts every cluster's 10 random two-way splits (divisive::split_communities,
// top_down_sbp.cpp:472-530; propose_random_split :248-260).
void split_count(const DevGraph& g, const DevBM& bm, uint64_t seed, uint32_t step, SplitBuffers& b, cudaStream_t st);
// Moves side-1 vertices of the chosen clusters into their new blocks (apply_best_splits).
void split_apply(const DevGraph& g, DevBM& bm, const SplitBuffers& b, cudaStream_t st);
// The edge counts alone, for sides (b.mask) and eligibility (b.eligible) set by the host.
void split_count_edges(const DevGraph& g, const DevBM& bm, SplitBuffers& b, cudaStream_t st);
// Snowball splits (propose_snowball_split, propose_single_snowball_split,
// propose_connectivity_snowball_split, top_down_sbp.cpp:262-426) of every eligible cluster:
// split 1 snowball, 2 single-snowball, 3 connectivity-snowball; init (split_init) 0 random,
// 1 degree-weighted, 2 high-degree.  Fills mask[N] (bit i: side in proposal i) and
// n1[B * 10].
void snowball_split_masks(const HostAdjacency& a, const std::vector<int32_t>& asg, const std::vector<int32_t>& sizes,
                          const std::vector<int32_t>& eligible, int32_t B, int split, int init, uint64_t seed,
                          uint32_t step, std::vector<uint16_t>& mask, std::vector<int32_t>& n1);

// ---- evaluate.cu
struct PartitionQuality {
    double nmi, f1, precision, recall, rand_index, accuracy;
    int64_t true_blocks, found_blocks;
};
// table[t * ncols + f] += 1 for every vertex with truth t >= 0 and found block f.
void launch_contingency(const int32_t* truth, const int32_t* found, int64_t n, int32_t ncols,
                        unsigned long long* table, cudaStream_t st);
// Metrics of evaluate::evaluate_blockmodel from the nt x nb table (rows = true).
PartitionQuality quality_from_table(const std::vector<unsigned long long>& table, int64_t nt, int64_t nb,
                                    int64_t num_vertices);
// calculate_f1_score and calculate_nmi (evaluate.cpp:9-98) of a contingency table given as
// the reference passes it (rows x columns), and the best one-to-one matching's accuracy
// when with_accuracy is set.
PartitionQuality scores_from_matrix(const std::vector<std::vector<long long>>& m, int64_t num_vertices,
                                    bool with_accuracy);

// Streaming multiprocessors of the current device (queried once per device and cached);
// grids of grid-stride kernels are capped at a multiple of it.
int device_sms();

// Launch accounting.
int64_t kernel_launches();
void count_launches(int64_t n);

}  // namespace sbp

// Host side of libsbpgpu: the C ABI (include/sbpgpu.h), device allocations and the
// drivers that sequence the kernels like the reference's host loops:
//   finetune::mcmc / asynchronous_gibbs / hybrid_mcmc / metropolis_hastings
//     (reference src/finetune.cpp:34-107, 563-646, 754-820),
//   block_merge::merge_blocks (src/block_merge.cpp:178-228),
//   sbp::stochastic_block_partition + BlockmodelTriplet (src/sbp.cpp:16-86,
//     src/blockmodel/blockmodel_triplet.cpp:4-105).
// Every entry point catches exceptions and reports them as status codes.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/sbpgpu.h"
#include "host_csr.h"
#include "kernels.cuh"
#include "noalloc.cuh"
#include "prims.cuh"

using namespace sbp;

namespace {

struct CudaError : std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t c, const char* what) : std::runtime_error(what), code(c) {}
};
struct ApiError : std::runtime_error {
    sbpgpu_status code;
    ApiError(sbpgpu_status c, const std::string& what) : std::runtime_error(what), code(c) {}
};

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);         \
            throw CudaError(e_, m_.c_str());                                              \
        }                                                                                 \
    } while (0)

// Device memory is allocated and freed in stream order on the stream of the context whose
// call is in progress on this thread (cudaMallocAsync / cudaFreeAsync from the device's
// pool): freeing does not wait for the whole device, so contexts that run concurrently
// (the partition server's workers) do not stall one another.
thread_local cudaStream_t tls_stream = nullptr;
// Allocations left before an injected allocation failure on this thread's current context
// (sbpgpu_ctx_inject_alloc_failure); null or negative: none injected.
thread_local int64_t* tls_fail_after = nullptr;

struct StreamScope {
    cudaStream_t prev;
    int64_t* prev_fail;
    StreamScope(cudaStream_t s, int64_t* fail_after) : prev(tls_stream), prev_fail(tls_fail_after) {
        tls_stream = s;
        tls_fail_after = fail_after;
    }
    ~StreamScope() {
        tls_stream = prev;
        tls_fail_after = prev_fail;
    }
};

template <typename T>
T* dalloc(std::vector<void*>& owned, size_t n) {
    void* p = nullptr;
    const size_t bytes = (n ? n : 1) * sizeof(T);
    if (tls_fail_after && *tls_fail_after >= 0 && (*tls_fail_after)-- == 0)
        throw ApiError(SBPGPU_ENOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed (injected)");
    const cudaError_t e = cudaMallocAsync(&p, bytes, tls_stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw ApiError(SBPGPU_ENOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed");
    }
    owned.push_back(p);
    return static_cast<T*>(p);
}

double early_threshold(bool golden, double initial) { return golden ? 5e-4 * initial : 1e-4 * initial; }

/* finetune::early_stop (reference src/finetune.cpp:265-283). */
bool early_stop(int64_t iteration, bool golden, double initial, const std::vector<double>& d) {
    const size_t last = d.size() - 1;
    if (d[last] == 0.0) return true;
    if (iteration < 3) return false;
    double average = d[last] + d[last - 1] + d[last - 2];
    average /= -3.0;
    return average < early_threshold(golden, initial);
}

// finetune::early_stop(iteration, initial_entropy, deltas) (finetune.cpp:285-294), used by
// finetune_assignment: no zero test, threshold 1e-4.
bool early_stop_finetune(int64_t iteration, double initial, const std::vector<double>& d) {
    if (iteration < 3) return false;
    const size_t last = d.size() - 1;
    double average = d[last] + d[last - 1] + d[last - 2];
    average /= -3.0;
    return average < 1e-4 * initial;
}

}  // namespace

struct TimedSpan {
    cudaEvent_t a, b;
    int kind;
};

struct sbpgpu_ctx {
    int device = 0;
    int refs = 0;          // live graphs
    bool dead = false;     // destroy requested
    cudaStream_t stream = nullptr;
    std::string err;
    bool timing = false;
    int64_t cells_budget = int64_t(64) << 30;  // dense cells of the sequential phases, bytes
    int64_t cluster_blocks = 65536;             // smallest B whose carry-out runs on a cluster
    // smallest B whose MH chain runs on a cluster (it always does when B > 128 by default:
    // over the golden-section steps of a 1,000,000-vertex, 20M-edge DCSBM graph from 62,500
    // down to 245 blocks, the cluster chain took 17.6 s where the one-CTA window took 21.0 s)
    int64_t chain_cluster_blocks = 129;
    DevFlags* flags_host = nullptr;            // pinned staging of the device flags
    std::vector<TimedSpan> pending;
    std::vector<cudaEvent_t> free_events;
    sbpgpu_kernel_timing tm{};
    std::atomic<int32_t> cancel{0};  // cancellation requested (sbpgpu_ctx_set_cancel)
    int64_t fail_alloc_after = -1;   // injected allocation failure (sbpgpu_ctx_inject_alloc_failure)

    cudaEvent_t ev() {
        if (!free_events.empty()) {
            cudaEvent_t e = free_events.back();
            free_events.pop_back();
            return e;
        }
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        return e;
    }
    void collect() {
        for (auto& s : pending) {
            float ms = 0.f;
            CK(cudaEventSynchronize(s.b));
            CK(cudaEventElapsedTime(&ms, s.a, s.b));
            switch (s.kind) {
                case 0: tm.gibbs_propose_ms += ms; tm.gibbs_propose_launches++; break;
                case 1: tm.mh_chain_ms += ms; tm.mh_chain_launches++; break;
                case 2: tm.merge_propose_ms += ms; tm.merge_propose_launches++; break;
                case 3: tm.carry_out_ms += ms; tm.carry_out_launches++; break;
                case 4: tm.rebuild_ms += ms; tm.rebuild_launches++; break;
                default: break;
            }
            free_events.push_back(s.a);
            free_events.push_back(s.b);
        }
        pending.clear();
    }
};

// RAII span recorded only when timing is enabled.
struct Span {
    sbpgpu_ctx* c;
    int kind;
    cudaEvent_t a = nullptr;
    Span(sbpgpu_ctx* ctx, int k) : c(ctx), kind(k) {
        if (c->timing) {
            a = c->ev();
            CK(cudaEventRecord(a, c->stream));
        }
    }
    ~Span() {
        if (c->timing && a) {
            cudaEvent_t b = c->ev();
            cudaEventRecord(b, c->stream);
            c->pending.push_back({a, b, kind});
        }
    }
};

struct sbpgpu_graph {
    sbpgpu_ctx* ctx = nullptr;
    int refs = 0;          // live blockmodels
    bool dead = false;     // destroy requested
    int64_t N = 0, E = 0;
    // Graph::num_edges (graph.hpp:99), the count the description lengths use: the stored
    // directed edges, or half of them for an undirected edge list (graph.cpp:145-147)
    int64_t Em = 0;
    // args.undirected for the nonparametric entropy (entropy.hpp:102-133, entropy.cpp:745)
    int32_t und = 0;
    int32_t dc = 0;       // args.degreecorrected for the nonparametric description length
    int64_t np_Em = -1;   // the count the nonparametric Dm / Dp tables were built for
    int32_t np_und = -1;  // and the form
    DevGraph dg{};
    std::vector<void*> owned;
    std::vector<int32_t> deg;   // Graph::degrees (graph.cpp:24-31): out + in - self
    std::vector<int32_t> kdeg;  // out + in without self (proposal neighbour count)
    int32_t max_k = 0;
    Work w;
    DevFlags* flags_host = nullptr;  // pinned
    int32_t* d_all = nullptr;        // identity vertex list
    int32_t* d_order = nullptr;      // scratch order [N]
    int32_t* d_order2 = nullptr;     // scratch order [N]
    // hdv / ldv split for one mh_percent (Graph::sort_vertices, graph.cpp:235-268)
    float split_mh = -1.f;
    int32_t* d_hdv = nullptr;
    int32_t* d_ldv = nullptr;
    int32_t n_hdv = 0, n_ldv = 0, max_k_hdv = 0;
    int64_t hdv_k_sum = 0;
    long long np_lg_N = 0;  // lgamma(N + 1) in units of 2^-24 (nonparametric partition term)
    std::vector<long long> np_lg;  // host copy of the lgamma table
    sbpgpu_stats st{};
};

struct sbpgpu_bm {
    sbpgpu_graph* g = nullptr;
    DevBM d{};
    std::vector<void*> owned;
    double entropy = DBL_MAX;
    int64_t num_blocks_to_merge = 0;
};

namespace {

sbpgpu_status fail(sbpgpu_ctx* ctx, sbpgpu_status code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

template <typename F>
sbpgpu_status guarded(sbpgpu_ctx* ctx, F f) {
    StreamScope scope(ctx ? ctx->stream : nullptr, ctx ? &ctx->fail_alloc_after : nullptr);
    try {
        return f();
    } catch (const ApiError& e) {
        return fail(ctx, e.code, e.what());
    } catch (const CudaError& e) {
        return fail(ctx, SBPGPU_EDEVICE, e.what());
    } catch (const std::bad_alloc&) {
        return fail(ctx, SBPGPU_ENOMEM, "host allocation failed");
    } catch (const std::invalid_argument& e) {
        return fail(ctx, SBPGPU_EINVAL, e.what());
    } catch (const std::exception& e) {
        return fail(ctx, SBPGPU_EDEVICE, e.what());
    }
}

void check_flags(sbpgpu_graph* g) {
    CK(cudaMemcpyAsync(g->flags_host, g->w.flags_dev, sizeof(DevFlags), cudaMemcpyDeviceToHost, g->ctx->stream));
    host_wait(g->ctx->stream);
    CK(cudaGetLastError());
    const int32_t err = g->flags_host->err;
    if (err) {
        g->flags_host->err = 0;
        CK(cudaMemsetAsync(g->w.flags_dev, 0, sizeof(DevFlags), g->ctx->stream));
        host_wait(g->ctx->stream);
        std::string m = "device check failed (flags 0x" + std::to_string(err) + "):";
        if (err & ERR_DEGREE) m += " a vertex or block row exceeds the supported neighbour count;";
        if (err & ERR_HASH_FULL) m += " chain cell store full;";
        if (err & ERR_POOL_FULL) m += " chain list pool full;";
        if (err & ERR_STATE) m += " blockmodel consistency check failed;";
        if (err & ERR_SELECT) m += " cumulative search out of range;";
        throw ApiError(SBPGPU_EDEVICE, m);
    }
}

void alloc_work(sbpgpu_graph* g) {
    Work& w = g->w;
    auto& o = g->owned;
    const int64_t N = g->N, E = g->E;
    const int64_t KE = std::max<int64_t>(E, 2 * N + 16);
    w.keys = dalloc<uint64_t>(o, KE);
    w.keys_alt = dalloc<uint64_t>(o, KE);
    w.vals = dalloc<int32_t>(o, KE);
    w.vals_alt = dalloc<int32_t>(o, KE);
    w.flags = dalloc<int32_t>(o, KE);
    w.temp_bytes = std::max(radix_temp_bytes(KE), scan_temp_bytes(KE)) + 4096;
    w.temp = dalloc<char>(o, w.temp_bytes);
    w.d_scalar = dalloc<int32_t>(o, 16);
    w.d_acc = dalloc<unsigned long long>(o, 4);
    w.moves = dalloc<int32_t>(o, N);
    w.m_out = dalloc<int32_t>(o, N);
    w.last = dalloc<int32_t>(o, N);
    w.acc = dalloc<int32_t>(o, N);
    w.dep = dalloc<int32_t>(o, 2 * N + 16);
    w.list_small = dalloc<int32_t>(o, 2 * N + 16);
    w.list_big = dalloc<int32_t>(o, 2 * N + 16);
    w.list_tmp = dalloc<int32_t>(o, N);
    // chain cell store: capacity for every cell plus the new cells of one phase.
    w.chain_cap = 1ull << ceil_log2((uint64_t)(8 * (uint64_t)E + 4096));
    w.chain_slots = dalloc<ulonglong2>(o, w.chain_cap);
    // list pool: every list's chunks at most double, so 16 words per block plus three
    // times the new keys of a phase bound it
    w.pool_words = std::min<int64_t>(16 * N + 24 * E + 4096, (int64_t)INT32_MAX - (1 << 20));
    w.pool = dalloc<int32_t>(o, (size_t)w.pool_words);
    w.row_head = dalloc<int32_t>(o, N);
    w.col_head = dalloc<int32_t>(o, N);
    w.best = dalloc<int32_t>(o, N);
    w.best_dS = dalloc<double>(o, N);
    w.heap_dS = dalloc<double>(o, N);
    w.heap_blk = dalloc<int32_t>(o, N);
    w.parent = dalloc<int32_t>(o, N);
    w.root = dalloc<int32_t>(o, N);
    w.used = dalloc<int32_t>(o, N);
    w.flags_dev = dalloc<DevFlags>(o, 1);
    w.win_hash = dalloc<int32_t>(o, (size_t)16 * 4 * 8192);
    // dense M / transpose of the one-vertex-at-a-time chain: allocated when first needed
    w.dense_cap = (int32_t)std::min<int64_t>(N, kDenseGlobalMax);
}

// fastlbinom (include/entropy.hpp:144-148) with fastlgamma(x) = lgamma((double)x)
// (include/fastlgamma.hpp:19-27).
double np_lbinom(int64_t n, int64_t k) {
    if (n == 0 || k == 0 || k > n) return 0.0;
    return (std::lgamma((double)(n + 1)) - std::lgamma((double)(k + 1))) - std::lgamma((double)(n - k + 1));
}
// get_edges_dl (entropy.cpp:745-749) for a directed graph: NB = B * B.
// get_edges_dl (entropy.cpp:745-749): NB = B * B, or B (B + 1) / 2 when undirected.
double np_edges_dl(int64_t b, int64_t E, bool und) { return np_lbinom((und ? b * (b + 1) / 2 : b * b) + E - 1, E); }
// log 2 in units of 2^-24, rounded: the undirected diagonal eterm's w log 2 is w times this.
const long long kLn2Fix = std::llrint(0.69314718055994530942 * 16777216.0);

// Runs f(i) for i in [lo, hi) on the host's cores.
template <class F>
void parallel_for(int64_t lo, int64_t hi, F f) {
    const int64_t n = hi - lo;
    const int64_t nt = std::max<int64_t>(1, std::min<int64_t>(std::thread::hardware_concurrency(), n / 65536));
    if (nt <= 1) {
        for (int64_t i = lo; i < hi; ++i) f(i);
        return;
    }
    std::vector<std::thread> ts;
    for (int64_t t = 0; t < nt; ++t)
        ts.emplace_back([=] {
            for (int64_t i = lo + n * t / nt; i < lo + n * (t + 1) / nt; ++i) f(i);
        });
    for (auto& t : ts) t.join();
}

// The nonparametric tables (entropy::nonparametric), built on first use: LG[x] =
// lgamma(x + 1) in units of 2^-24 over the range of Lq, and the rounded change of
// lbinom(N - 1, b - 1) + edges_dl(b) (get_delta_partition_dl, entropy.cpp:933-940;
// get_delta_edges_dl, :1111-1143) when the non-empty block count steps from b to b - 1
// (Dm) or b + 1 (Dp).  Dm and Dp are rebuilt when the graph's model edge count changes.
void ensure_np(sbpgpu_graph* g) {
    if (g->dg.LG && g->np_Em == g->Em && g->np_und == g->und) return;
    const bool und = g->und != 0;
    const int64_t n = (int64_t)g->dg.nlq + 1, N = g->N, E = g->Em;
    const bool have_lg = g->dg.LG != nullptr;
    std::vector<long long> LG(have_lg ? 0 : n), Dm(N + 2, 0), Dp(N + 2, 0);
    if (!have_lg)
        parallel_for(0, n, [&](int64_t x) { LG[x] = std::llrint(std::lgamma((double)(x + 1)) * 16777216.0); });
    auto step = [&](int64_t b, int dB) {
        const double part = np_lbinom(N - 1, b + dB - 1) - np_lbinom(N - 1, b - 1);
        const double edges = np_edges_dl(b + dB, E, und) - np_edges_dl(b, E, und);
        return std::llrint((part + edges) * 16777216.0);
    };
    parallel_for(1, N + 2, [&](int64_t b) {
        if (b >= 2) Dm[b] = step(b, -1);
        if (b <= N) Dp[b] = step(b, +1);
    });
    cudaStream_t st = g->ctx->stream;
    if (!have_lg) {
        long long* d_LG = dalloc<long long>(g->owned, n);
        CK(cudaMemcpyAsync(d_LG, LG.data(), n * sizeof(long long), cudaMemcpyHostToDevice, st));
        g->dg.Dm = dalloc<long long>(g->owned, N + 2);
        g->dg.Dp = dalloc<long long>(g->owned, N + 2);
        g->dg.LG = d_LG;
        g->np_lg_N = LG[N];
        g->np_lg = std::move(LG);
    }
    // the graph owns the tables; the device view holds them read-only
    CK(cudaMemcpyAsync(const_cast<long long*>(g->dg.Dm), Dm.data(), (N + 2) * sizeof(long long),
                       cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(const_cast<long long*>(g->dg.Dp), Dp.data(), (N + 2) * sizeof(long long),
                       cudaMemcpyHostToDevice, st));
    host_wait(st);
    g->np_Em = g->Em;
    g->np_und = g->und;
    g->dg.np_und = g->und;
    g->dg.ln2q = kLn2Fix;
}

// The sweeps, chains, merges and splits score moves without the degree-corrected terms:
// the reference's block-merge form of them (entropy.cpp:1180-1196) reads a block's total
// degree as a key of its vertex-degree histograms and evaluates lgamma at non-positive
// arguments, so there is no consistent merge score to reproduce, and the device paths do
// not carry the degree histograms through their moves.
void ensure_np_sweeps(sbpgpu_graph* g) {
    if (g->dc)
        throw ApiError(SBPGPU_EUNSUPPORTED,
                       "degree-corrected description lengths are evaluated (np_mdl, np_delta_mdl_batch, "
                       "move_vertex), not used by sweeps, merges or splits");
    ensure_np(g);
}

void ensure_split(sbpgpu_graph* g, float mh_percent) {
    if (g->split_mh == mh_percent) return;
    const std::vector<int32_t> idx = order_by_degree_desc(g->deg);  // a stable sort by descending degree
    const float limit = mh_percent * (float)g->N;  // float arithmetic as in graph.cpp:252
    std::vector<int32_t> hdv, ldv;
    for (int64_t i = 0; i < g->N; ++i) ((float)i < limit ? hdv : ldv).push_back(idx[i]);
    if (!g->d_hdv) {
        g->d_hdv = dalloc<int32_t>(g->owned, g->N);
        g->d_ldv = dalloc<int32_t>(g->owned, g->N);
    }
    g->n_hdv = (int32_t)hdv.size();
    g->n_ldv = (int32_t)ldv.size();
    g->max_k_hdv = 0;
    g->hdv_k_sum = 0;
    for (int32_t v : hdv) {
        g->max_k_hdv = std::max(g->max_k_hdv, g->kdeg[v]);
        g->hdv_k_sum += g->kdeg[v];
    }
    if (!hdv.empty())
        CK(cudaMemcpyAsync(g->d_hdv, hdv.data(), hdv.size() * 4, cudaMemcpyHostToDevice, g->ctx->stream));
    if (!ldv.empty())
        CK(cudaMemcpyAsync(g->d_ldv, ldv.data(), ldv.size() * 4, cudaMemcpyHostToDevice, g->ctx->stream));
    host_wait(g->ctx->stream);
    g->split_mh = mh_percent;
}

void do_rebuild(sbpgpu_bm* bm) {
    sbpgpu_graph* g = bm->g;
    Span sp(g->ctx, 4);
    rebuild(g->dg, bm->d, g->w, g->ctx->stream);
}

// How a configuration scores and accepts vertex moves.
int accept_mode(const sbpgpu_config& c) { return c.nonparametric ? ACC_NP : c.greedy ? ACC_GREEDY : ACC_HASTINGS; }

double do_mdl(sbpgpu_bm* bm, bool np = false) {
    sbpgpu_graph* g = bm->g;
    if (np) ensure_np(g);
    if (np) launch_np_mdl(g->dg, bm->d, g->w, g->ctx->stream);
    else launch_mdl(g->dg, bm->d, g->w, g->ctx->stream);
    if (np && g->dc) launch_dc_mdl(g->dg, bm->d, g->w.d_acc, g->ctx->stream);
    unsigned long long* h_acc = static_cast<unsigned long long*>(host_scratch());
    int32_t* h_ne = reinterpret_cast<int32_t*>(h_acc + 1);
    CK(cudaMemcpyAsync(h_acc, g->w.d_acc, sizeof(*h_acc), cudaMemcpyDeviceToHost, g->ctx->stream));
    if (np) CK(cudaMemcpyAsync(h_ne, bm->d.nonempty, sizeof(int32_t), cudaMemcpyDeviceToHost, g->ctx->stream));
    check_flags(g);
    const unsigned long long acc = *h_acc;
    g->ctx->collect();
    if (np) {
        // nonparametric::mdl (entropy.cpp:751-779): the table terms, lgamma(N + 1) and
        // fastlog(N) of get_partition_dl, then the two terms of the non-empty block count
        const int64_t N = g->N, E = g->Em, ne = *h_ne;
        const long long lqN = (long long)(int32_t)((double)logf((float)N) * 16777216.0);
        const long long fixed = (long long)acc + g->np_lg_N + lqN;
        return (double)fixed * (1.0 / 16777216.0) + (np_lbinom(N - 1, ne - 1) + np_edges_dl(ne, E, g->und != 0));
    }
    const long long lpq = (long long)acc;
    const double E = (double)g->Em;
    const double B = (double)bm->d.B;
    const double x = pow(B, 2) / E;
    const double h = ((1 + x) * log(1 + x)) - (x * log(x));
    return (E * h) + ((double)g->N * log(B)) - (double)lpq * (1.0 / 16777216.0);
}

void reset_counters(sbpgpu_graph* g) {
    CK(cudaMemsetAsync(g->w.flags_dev, 0, sizeof(DevFlags), g->ctx->stream));
}

// Reads the device counters into the graph's running statistics.
void harvest_counters(sbpgpu_graph* g) {
    CK(cudaMemcpyAsync(g->flags_host, g->w.flags_dev, sizeof(DevFlags), cudaMemcpyDeviceToHost, g->ctx->stream));
    check_flags(g);
    const DevFlags& f = *g->flags_host;
    g->st.moves += (int64_t)f.counters[2] + (int64_t)f.counters[5];
    g->st.edges_swept += (int64_t)f.counters[3] + (int64_t)f.counters[4];
    g->st.gibbs_edges += (int64_t)f.counters[3];
    g->st.merge_proposals += (int64_t)f.counters[6];
    g->st.chain_rounds += (int64_t)f.counters[8];
    g->st.carry_rounds += (int64_t)f.counters[0];
    g->st.carry_evaluations += (int64_t)f.counters[10];
    g->st.carry_keys += (int64_t)f.counters[9];
    reset_counters(g);
}

void gibbs_batch_dev(sbpgpu_bm* bm, const int32_t* list, int32_t n, uint64_t seed, uint32_t it, uint32_t step,
                     int mode) {
    sbpgpu_graph* g = bm->g;
    if (mode == ACC_NP) ensure_np_sweeps(g);
    {
        Span sp(g->ctx, 0);
        gibbs_propose(g->dg, bm->d, list, n, g->max_k, seed, it, step, mode, g->w, g->ctx->stream);
    }
    gibbs_apply(bm->d, list, n, g->w, g->ctx->stream);
    g->st.proposals += n;
    g->st.gibbs_proposals += n;
    do_rebuild(bm);
}

// At least `need` int32 of dense cells (the carry-out's B x B counts, or the windowed
// chain's matrix and transpose) when they fit the context's budget; otherwise, or when the
// allocation fails, the callers use the chain hash.
void ensure_cells(sbpgpu_graph* g, uint64_t need) {
    Work& w = g->w;
    const uint64_t budget = (uint64_t)std::max<int64_t>(g->ctx->cells_budget, 0) / sizeof(int32_t);
    if (w.cells && (w.cells_elems > budget || (need <= budget && w.cells_elems < need))) {
        CK(cudaFreeAsync(w.cells, g->ctx->stream));
        w.cells = nullptr;
        w.cells_elems = 0;
    }
    if (need > budget || w.cells) return;
    void* p = nullptr;
    if (cudaMallocAsync(&p, need * sizeof(int32_t), g->ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    w.cells = static_cast<int32_t*>(p);
    w.cells_elems = need;
}

// The cluster chain's buffers (per-warp neighbour hashes and row scratch), allocated on
// first use.  False when the device holds no cluster.
bool ensure_cluster(sbpgpu_graph* g) {
    const int cs = mh_cluster_size();
    if (cs <= 0) return false;
    Work& w = g->w;
    if (!w.cl_hash) w.cl_hash = dalloc<int32_t>(g->owned, mh_cluster_hash_ints(cs));
    if (!w.cl_scratch) w.cl_scratch = dalloc<int32_t>(g->owned, mh_cluster_scratch_ints(cs));
    return true;
}

// The cluster carry-out's per-block candidate array and staging buffer, allocated on first
// use.  False when the device
// holds no cluster.
bool ensure_cluster_carry(sbpgpu_graph* g) {
    if (carry_cluster_size() <= 0) return false;
    Work& w = g->w;
    if (!w.cc_head) {
        w.cc_head = dalloc<int32_t>(g->owned, g->N);
        w.cc_stage = dalloc<int32_t>(g->owned, carry_cluster_stage_ints(carry_cluster_size()));
    }
    return true;
}

void chain_run(sbpgpu_bm* bm, const int32_t* order, int32_t n, int32_t max_k, int64_t k_sum, uint64_t seed,
               uint32_t it, uint32_t step, int mode) {
    sbpgpu_graph* g = bm->g;
    if (mode == ACC_NP) ensure_np_sweeps(g);
    const int64_t B = bm->d.B;
    if (B > kWinSharedMax) ensure_cells(g, mh_window_cells((int32_t)B));
    WindowPlan plan{};
    const bool window = mh_window_plan(bm->d.B, max_k, g->w, &plan);
    // Many blocks, or a blockmodel whose dense cells exceed the budget: the window spread
    // over a thread-block cluster, cells dense when the budget holds them, else hashed.
    if ((B >= g->ctx->chain_cluster_blocks || !window) && B > kWinSharedMax && max_k <= 4096 && ensure_cluster(g)) {
        const bool hashed = !g->w.cells || mh_window_cells((int32_t)B) > g->w.cells_elems;
        if (hashed) chain_init(bm->d, g->w, (uint64_t)(2 * k_sum + 4 * (int64_t)n), g->ctx->stream);
        {
            Span sp(g->ctx, 1);
            mh_chain_cluster(g->dg, bm->d, order, n, max_k, hashed, seed, it, step, mode, g->w, g->ctx->stream);
        }
        g->st.proposals += n;
        do_rebuild(bm);
        return;
    }
    if (window) {
        Span sp(g->ctx, 1);
        mh_chain_window(g->dg, bm->d, order, n, plan, seed, it, step, mode, g->w, g->ctx->stream);
    } else if (mode != ACC_GREEDY) {
        throw ApiError(SBPGPU_EUNSUPPORTED,
                       "non-greedy or nonparametric acceptance needs the windowed chain (vertex degree <= 4096 and the dense "
                       "cell budget holding the blockmodel)");
    } else if (bm->d.B <= kDenseMax || bm->d.B <= g->w.dense_cap) {
        if (bm->d.B > kDenseMax && !g->w.dense_M) {
            g->w.dense_M = dalloc<int32_t>(g->owned, (size_t)g->w.dense_cap * g->w.dense_cap);
            g->w.dense_MT = dalloc<int32_t>(g->owned, (size_t)g->w.dense_cap * g->w.dense_cap);
        }
        Span sp(g->ctx, 1);
        mh_chain_dense(g->dg, bm->d, order, n, seed, it, step, g->w, g->ctx->stream);
    } else {
        if (max_k * 2 > (1 << 13))
            throw ApiError(SBPGPU_EUNSUPPORTED, "sequential MH supports vertices with k <= 4096");
        chain_init(bm->d, g->w, (uint64_t)(2 * k_sum + 4 * (int64_t)n), g->ctx->stream);
        Span sp(g->ctx, 1);
        mh_chain(g->dg, bm->d, order, n, max_k, seed, it, step, 1, g->w, g->ctx->stream);
    }
    g->st.proposals += n;
    do_rebuild(bm);
}

void async_gibbs(sbpgpu_bm* bm, const sbpgpu_config& cfg, uint64_t seed, int32_t step, bool golden) {
    sbpgpu_graph* g = bm->g;
    if (bm->d.B == 1) return;
    std::vector<double> deltas;
    const double initial = do_mdl(bm, cfg.nonparametric != 0);
    bm->entropy = initial;
    double last = initial;
    const int64_t N = g->N;
    const int64_t batch_size = (int64_t)ceil((double)N / (double)cfg.batches);
    for (int it = 0; it < cfg.max_iterations; ++it) {
        const int32_t* list = g->d_all;
        if (!cfg.ordered && cfg.batches > 1) {
            shuffle(g->d_all, (int32_t)N, seed, (uint32_t)it, (uint32_t)step, DOM_SHUFFLE_ALL, g->d_order, g->w,
                    g->ctx->stream);
            list = g->d_order;
        }
        for (int64_t b = 0; batch_size > 0 && b < N / batch_size; ++b) {
            const int64_t s0 = b * batch_size, s1 = std::min(N, (b + 1) * batch_size);
            gibbs_batch_dev(bm, list + s0, (int32_t)(s1 - s0), seed, (uint32_t)it, (uint32_t)step, accept_mode(cfg));
        }
        const double e = do_mdl(bm, cfg.nonparametric != 0);
        harvest_counters(g);
        deltas.push_back(e - last);
        last = e;
        g->st.mcmc_iterations++;
        if (early_stop(it, golden, initial, deltas)) break;
    }
    bm->entropy = last;
}

void hybrid_mcmc(sbpgpu_bm* bm, const sbpgpu_config& cfg, uint64_t seed, int32_t step, bool golden) {
    sbpgpu_graph* g = bm->g;
    if (bm->d.B == 1) return;
    ensure_split(g, cfg.mh_percent);
    std::vector<double> deltas;
    const double initial = do_mdl(bm, cfg.nonparametric != 0);
    bm->entropy = initial;
    double last = initial;
    const int64_t nlow = g->n_ldv;
    const int64_t batch_size = (int64_t)ceil((double)nlow / (double)cfg.batches);
    for (int it = 0; it < cfg.max_iterations; ++it) {
        if (g->n_hdv > 0) {
            const int32_t* order = g->d_hdv;
            if (!cfg.ordered) {
                shuffle(g->d_hdv, g->n_hdv, seed, (uint32_t)it, (uint32_t)step, DOM_SHUFFLE_HDV, g->d_order, g->w,
                        g->ctx->stream);
                order = g->d_order;
            }
            chain_run(bm, order, g->n_hdv, g->max_k_hdv, g->hdv_k_sum, seed, (uint32_t)it, (uint32_t)step, accept_mode(cfg));
        }
        const int32_t* list = g->d_ldv;
        if (!cfg.ordered && cfg.batches > 1) {
            shuffle(g->d_ldv, (int32_t)nlow, seed, (uint32_t)it, (uint32_t)step, DOM_SHUFFLE_ALL, g->d_order2, g->w,
                    g->ctx->stream);
            list = g->d_order2;
        }
        for (int64_t b = 0; batch_size > 0 && b < nlow / batch_size; ++b) {
            const int64_t s0 = b * batch_size, s1 = std::min(nlow, (b + 1) * batch_size);
            gibbs_batch_dev(bm, list + s0, (int32_t)(s1 - s0), seed, (uint32_t)it, (uint32_t)step, accept_mode(cfg));
        }
        const double e = do_mdl(bm, cfg.nonparametric != 0);
        harvest_counters(g);
        deltas.push_back(e - last);
        last = e;
        g->st.mcmc_iterations++;
        if (early_stop(it, golden, initial, deltas)) break;
    }
    bm->entropy = last;
}

void metropolis_hastings(sbpgpu_bm* bm, const sbpgpu_config& cfg, uint64_t seed, int32_t step, bool golden) {
    sbpgpu_graph* g = bm->g;
    if (bm->d.B == 1) return;
    std::vector<double> deltas;
    bm->entropy = do_mdl(bm, cfg.nonparametric != 0);
    int64_t ksum = 0;
    for (int64_t v = 0; v < g->N; ++v) ksum += g->kdeg[v];
    for (int it = 0; it < cfg.max_iterations; ++it) {
        const int32_t* order = g->d_all;
        if (!cfg.ordered) {
            shuffle(g->d_all, (int32_t)g->N, seed, (uint32_t)it, (uint32_t)step, DOM_SHUFFLE_ALL, g->d_order, g->w,
                    g->ctx->stream);
            order = g->d_order;
        }
        chain_run(bm, order, (int32_t)g->N, g->max_k, ksum, seed, (uint32_t)it, (uint32_t)step, accept_mode(cfg));
        CK(cudaMemcpyAsync(g->flags_host, g->w.flags_dev, sizeof(DevFlags), cudaMemcpyDeviceToHost, g->ctx->stream));
        check_flags(g);
        const double dsum = (double)(long long)g->flags_host->counters[7] * (1.0 / 16777216.0);
        harvest_counters(g);
        deltas.push_back(dsum);
        g->st.mcmc_iterations++;
        if (early_stop(it, golden, bm->entropy, deltas)) break;
    }
    bm->entropy = do_mdl(bm, cfg.nonparametric != 0);
}

// finetune::finetune_assignment (finetune.cpp:903-932): the sequential MH chain over every
// vertex in id order (draws keyed by step 0xffffffff), stopped by the three-iteration
// average against 1e-4 of the entropy.
constexpr uint32_t kFinetuneStep = 0xffffffffu;

void finetune_assignment_impl(sbpgpu_bm* bm, const sbpgpu_config& cfg, uint64_t seed) {
    sbpgpu_graph* g = bm->g;
    const bool np = cfg.nonparametric != 0;
    if (bm->d.B < 2) {
        bm->entropy = do_mdl(bm, np);
        return;
    }
    bm->entropy = do_mdl(bm, np);
    int64_t ksum = 0;
    for (int64_t v = 0; v < g->N; ++v) ksum += g->kdeg[v];
    std::vector<double> deltas;
    for (int it = 0; it < cfg.max_iterations; ++it) {
        chain_run(bm, g->d_all, (int32_t)g->N, g->max_k, ksum, seed, (uint32_t)it, kFinetuneStep, accept_mode(cfg));
        CK(cudaMemcpyAsync(g->flags_host, g->w.flags_dev, sizeof(DevFlags), cudaMemcpyDeviceToHost, g->ctx->stream));
        check_flags(g);
        const double dsum = (double)(long long)g->flags_host->counters[7] * (1.0 / 16777216.0);
        harvest_counters(g);
        deltas.push_back(dsum);
        g->st.mcmc_iterations++;
        if (early_stop_finetune(it, bm->entropy, deltas)) break;
    }
    bm->entropy = do_mdl(bm, np);
}

void free_all(std::vector<void*>& owned, cudaStream_t st) {
    for (void* p : owned) cudaFreeAsync(p, st);
    owned.clear();
}

// fastlog(x) in units of 2^-24 (the Lq table's values).
long long lq_of(int64_t x) { return x <= 0 ? 0 : (long long)(int32_t)((double)logf((float)x) * 16777216.0); }

// nonparametric::mdl (entropy.cpp:751-779) of a two-block model of a subgraph of n vertices
// and E edges (sizes, row-major cells M), in the canonical arithmetic of the device deltas.
double np_mdl_two_blocks(const sbpgpu_graph* g, int64_t n, int64_t E, const int64_t sizes[2], const int64_t M[4]) {
    const std::vector<long long>& LG = g->np_lg;
    const bool und = g->und != 0;
    long long fixed = 0;
    for (int k = 0; k < 4; ++k) fixed -= LG[M[k]] + (und && (k == 0 || k == 3) ? M[k] * kLn2Fix : 0);
    for (int b = 0; b < 2; ++b) {
        const int64_t dout = M[2 * b] + M[2 * b + 1], din = M[b] + M[2 + b];
        fixed += (sizes[b] == 0 ? 0 : (und ? dout : dout + din) * lq_of(sizes[b])) - LG[sizes[b]];
    }
    fixed += LG[n] + lq_of(n);
    const int64_t ne = (sizes[0] > 0) + (sizes[1] > 0);
    return (double)fixed * (1.0 / 16777216.0) + (np_lbinom(n - 1, ne - 1) + np_edges_dl(ne, E, und));
}

// entropy::null_mdl_v1 (entropy.cpp:571-585) of a subgraph: the one-block nonparametric MDL
// under --nonparametric, else the parametric formula.
double split_null_mdl(const sbpgpu_graph* g, int64_t n, int64_t E, bool np) {
    if (np) {
        const int64_t sizes[2] = {n, 0}, M[4] = {E, 0, 0, 0};
        return np_mdl_two_blocks(g, n, E, sizes, M);
    }
    const double e = (double)E;
    const double log_posterior_p = e * log(1.0 / e);
    const double x = 1.0 / e;
    const double h = ((1 + x) * log(1 + x)) - (x * log(x));
    return (e * h) - log_posterior_p;
}

// divisive::split_communities (top_down_sbp.cpp:472-530) with random splits, then
// apply_best_splits (:30-65): the clusters in ascending order of their best split's
// delta are split until the block count reaches `target`.
void split_impl(sbpgpu_bm* bm, const sbpgpu_config& cfg, uint64_t seed, uint32_t step, int64_t target) {
    sbpgpu_graph* g = bm->g;
    ensure_np_sweeps(g);
    cudaStream_t st = g->ctx->stream;
    const int64_t B = bm->d.B, N = g->N, P = 10;
    std::vector<void*> tmp;
    SplitBuffers b{};
    b.split_size = dalloc<long long>(tmp, B * P);
    b.eligible = dalloc<int32_t>(tmp, B);
    b.mask = dalloc<uint16_t>(tmp, N);
    b.n1 = dalloc<int32_t>(tmp, B * P);
    b.cells = dalloc<int32_t>(tmp, B * P * 4);
    b.ecount = dalloc<unsigned long long>(tmp, B);
    b.new_block = dalloc<int32_t>(tmp, B);
    b.proposal = dalloc<int32_t>(tmp, B);
    try {
        if (cfg.split == 0) {
            split_count(g->dg, bm->d, seed, step, b, st);
        } else {
            // snowball splits: serial frontier processes on the host, counted on the device
            std::vector<int32_t> asg(N), hsizes(B), helig(B);
            CK(cudaMemcpyAsync(asg.data(), bm->d.asg, N * 4, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(hsizes.data(), bm->d.sizes, B * 4, cudaMemcpyDeviceToHost, st));
            host_wait(st);
            for (int64_t c = 0; c < B; ++c) helig[c] = (double)hsizes[c] < 0.001 * (double)N ? 0 : 1;
            std::vector<uint16_t> mask;
            std::vector<int32_t> hn1;
            snowball_split_masks(host_adjacency(g->dg, st), asg, hsizes, helig, (int32_t)B, cfg.split, cfg.splitinit, seed,
                                 step, mask, hn1);
            CK(cudaMemcpyAsync(b.mask, mask.data(), N * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(b.n1, hn1.data(), hn1.size() * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(b.eligible, helig.data(), B * 4, cudaMemcpyHostToDevice, st));
            split_count_edges(g->dg, bm->d, b, st);
            host_wait(st);
        }
        std::vector<int32_t> n1(B * P), cells(B * P * 4), elig(B), sizes(B);
        std::vector<unsigned long long> ecount(B);
        CK(cudaMemcpyAsync(n1.data(), b.n1, n1.size() * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(cells.data(), b.cells, cells.size() * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(elig.data(), b.eligible, B * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(sizes.data(), bm->d.sizes, B * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(ecount.data(), b.ecount, B * 8, cudaMemcpyDeviceToHost, st));
        host_wait(st);
        CK(cudaGetLastError());
        std::vector<double> best(B, DBL_MAX);
        std::vector<int32_t> best_i(B, -1);
        for (int64_t c = 0; c < B; ++c) {
            if (!elig[c]) continue;
            const int64_t n = sizes[c], E = (int64_t)ecount[c];
            const double old_entropy = split_null_mdl(g, n, E, cfg.nonparametric != 0);
            for (int64_t i = 0; i < P; ++i) {
                const int64_t s2[2] = {n - n1[c * P + i], n1[c * P + i]};
                int64_t M[4];
                for (int k = 0; k < 4; ++k) M[k] = cells[(c * P + i) * 4 + k];
                const double delta = np_mdl_two_blocks(g, n, E, s2, M) - old_entropy;
                if (delta < best[c]) {
                    best[c] = delta;
                    best_i[c] = (int32_t)i;
                }
            }
        }
        // utils::argsort<double> is a stable descending sort; apply_best_splits walks it from the end
        std::vector<int64_t> order(B);
        for (int64_t c = 0; c < B; ++c) order[c] = c;
        std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return best[x] > best[y]; });
        std::vector<int32_t> new_block(B, -1), prop(B, 0);
        int64_t num_blocks = B;
        for (int64_t k = B - 1; k >= 0; --k) {
            const int64_t c = order[k];
            if (best_i[c] < 0) continue;  // no split was proposed (small cluster)
            new_block[c] = (int32_t)num_blocks;
            prop[c] = best_i[c];
            num_blocks++;
            if (num_blocks >= target) break;
        }
        if (num_blocks > N) throw ApiError(SBPGPU_EINVAL, "splits would exceed one block per vertex");
        CK(cudaMemcpyAsync(b.new_block, new_block.data(), B * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(b.proposal, prop.data(), B * 4, cudaMemcpyHostToDevice, st));
        split_apply(g->dg, bm->d, b, st);
        host_wait(st);
        bm->d.B = (int32_t)num_blocks;
    } catch (...) {
        free_all(tmp, st);
        throw;
    }
    free_all(tmp, st);
    do_rebuild(bm);
}

void mcmc_impl(sbpgpu_bm* bm, const sbpgpu_config& cfg, uint64_t seed, int32_t step, bool golden) {
    if (cfg.nonparametric) ensure_np_sweeps(bm->g);
    if (cfg.algorithm == 0 && step < cfg.asynciterations) async_gibbs(bm, cfg, seed, step, golden);
    else if (cfg.algorithm == 1) hybrid_mcmc(bm, cfg, seed, step, golden);
    else metropolis_hastings(bm, cfg, seed, step, golden);
}

void merge_impl(sbpgpu_bm* bm, const sbpgpu_config& cfg, uint64_t seed, int32_t step, int64_t num_to_merge) {
    sbpgpu_graph* g = bm->g;
    if (num_to_merge <= 0) return;  // nothing is merged; the rebuild would reproduce the same state
    const int32_t B = bm->d.B;
    if (num_to_merge >= B) throw ApiError(SBPGPU_EINVAL, "num_blocks_to_merge must be < num_blocks");
    {
        Span sp(g->ctx, 2);
        if (cfg.nonparametric) ensure_np_sweeps(g);
        merge_propose(g->dg, bm->d, seed, (uint32_t)step, g->w, g->ctx->stream, cfg.nonparametric != 0);
    }
    if (!cfg.approximate) ensure_cells(g, (uint64_t)B * (uint64_t)B);
    const bool cluster = !cfg.approximate && B >= g->ctx->cluster_blocks && ensure_cluster_carry(g);
    {
        Span sp(g->ctx, 3);
        carry_out(g->dg, bm->d, num_to_merge, cfg.approximate, g->w, g->ctx->stream, cfg.nonparametric != 0,
                  cluster);
    }
    int32_t sc[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(sc, g->w.d_scalar, sizeof(sc), cudaMemcpyDeviceToHost, g->ctx->stream));
    harvest_counters(g);
    // build_mapping numbers the blocks that still hold vertices densely and the blockmodel
    // keeps B - num_to_merge blocks (block_merge.cpp:109-115), so blocks that were empty
    // before the pass end up as empty trailing blocks
    if (sc[1] != num_to_merge || sc[2] > B - num_to_merge)
        throw ApiError(SBPGPU_EDEVICE, "merge pass carried out " + std::to_string(sc[1]) + " of " +
                                           std::to_string(num_to_merge) + " merges (" + std::to_string(sc[2]) +
                                           " blocks left)");
    g->st.merges += sc[1];
    bm->d.B = (int32_t)(B - num_to_merge);
    do_rebuild(bm);
}

void upload_graph(sbpgpu_graph* g, const int32_t* src, const int32_t* dst) {
    const int64_t N = g->N, E = g->E;
    // stable: neighbour lists keep input order (graph.cpp:10-18); built by several threads
    HostCsr csr;
    try {
        build_host_csr(N, E, src, dst, csr);
    } catch (const std::invalid_argument& e) {
        throw ApiError(SBPGPU_EINVAL, e.what());
    }
    const std::vector<int32_t>&out_off = csr.out_off, &inns_off = csr.inns_off, &selfcnt = csr.selfcnt,
                            &indeg = csr.indeg, &out_nbr = csr.out_nbr, &esrc = csr.esrc, &inns_nbr = csr.inns_nbr;
    g->deg.resize(N);
    g->kdeg.resize(N);
    g->max_k = 0;
    for (int64_t v = 0; v < N; ++v) {
        const int32_t outd = out_off[v + 1] - out_off[v];
        g->deg[v] = outd + indeg[v] - (selfcnt[v] > 0 ? 1 : 0);
        g->kdeg[v] = outd + (inns_off[v + 1] - inns_off[v]);
        g->max_k = std::max(g->max_k, g->kdeg[v]);
    }
    // fastlog table (fastlog.hpp:21-30): logf((float)x) is a multiple of 2^-24 for x >= 1;
    // up to max(E, N) + 1 so that block sizes index it too (nonparametric vterm)
    const int64_t nlq = std::max(E, N) + 2;
    std::vector<int32_t> Lq(nlq);
    Lq[0] = 0;
    parallel_for(1, nlq, [&](int64_t x) { Lq[x] = (int32_t)((double)logf((float)x) * 16777216.0); });
    cudaStream_t st = g->ctx->stream;
    auto& o = g->owned;
    int32_t* d_out_off = dalloc<int32_t>(o, N + 1);
    int32_t* d_out_nbr = dalloc<int32_t>(o, E);
    int32_t* d_inns_off = dalloc<int32_t>(o, N + 1);
    int32_t* d_inns_nbr = dalloc<int32_t>(o, inns_nbr.size());
    int32_t* d_self = dalloc<int32_t>(o, N);
    int32_t* d_esrc = dalloc<int32_t>(o, E);
    int32_t* d_Lq = dalloc<int32_t>(o, nlq);
    CK(cudaMemcpyAsync(d_out_off, out_off.data(), (N + 1) * 4, cudaMemcpyHostToDevice, st));
    if (E) CK(cudaMemcpyAsync(d_out_nbr, out_nbr.data(), E * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_inns_off, inns_off.data(), (N + 1) * 4, cudaMemcpyHostToDevice, st));
    if (!inns_nbr.empty())
        CK(cudaMemcpyAsync(d_inns_nbr, inns_nbr.data(), inns_nbr.size() * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_self, selfcnt.data(), N * 4, cudaMemcpyHostToDevice, st));
    if (E) CK(cudaMemcpyAsync(d_esrc, esrc.data(), E * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_Lq, Lq.data(), nlq * 4, cudaMemcpyHostToDevice, st));
    g->dg = DevGraph{(int32_t)N, (int32_t)E, d_out_off, d_out_nbr, d_inns_off, d_inns_nbr, d_self, d_esrc, d_Lq};
    g->dg.nlq = (int32_t)(nlq - 1);
    alloc_work(g);
    std::vector<int32_t> iota(N);
    for (int64_t v = 0; v < N; ++v) iota[v] = (int32_t)v;
    g->d_all = dalloc<int32_t>(o, N);
    g->d_order = dalloc<int32_t>(o, N);
    g->d_order2 = dalloc<int32_t>(o, N);
    CK(cudaMemcpyAsync(g->d_all, iota.data(), N * 4, cudaMemcpyHostToDevice, st));
    g->flags_host = g->ctx->flags_host;
    reset_counters(g);
    host_wait(st);
}

sbpgpu_bm* new_bm(sbpgpu_graph* g, int64_t B) {
    auto* bm = new sbpgpu_bm();
    bm->g = g;
    const int64_t N = g->N, E = g->E;
    auto& o = bm->owned;
    DevBM& d = bm->d;
    d.B = (int32_t)B;
    d.asg = dalloc<int32_t>(o, N);
    d.d_out = dalloc<int32_t>(o, N);
    d.d_in = dalloc<int32_t>(o, N);
    d.d_tot = dalloc<int32_t>(o, N);
    d.sizes = dalloc<int32_t>(o, N);
    d.diag = dalloc<int32_t>(o, N);
    d.row_off = dalloc<int32_t>(o, N + 1);
    d.col_off = dalloc<int32_t>(o, N + 1);
    d.row_col = dalloc<int32_t>(o, E);
    d.row_cnt = dalloc<int32_t>(o, E);
    d.row_cum = dalloc<int32_t>(o, E);
    d.row_of = dalloc<int32_t>(o, E);
    d.col_row = dalloc<int32_t>(o, E);
    d.col_cnt = dalloc<int32_t>(o, E);
    d.col_cum = dalloc<int32_t>(o, E);
    d.nonempty = dalloc<int32_t>(o, 1);
    return bm;
}

// Destruction is reference counted so that handles may be destroyed in any order: a
// graph is freed once it was destroyed and its last blockmodel is gone, a context once
// it was destroyed and its last graph is gone.
void release_ctx(sbpgpu_ctx* ctx) {
    if (!ctx->dead || ctx->refs > 0) return;
    cudaStreamSynchronize(ctx->stream);
    for (auto& s : ctx->pending) {
        cudaEventDestroy(s.a);
        cudaEventDestroy(s.b);
    }
    for (auto e : ctx->free_events) cudaEventDestroy(e);
    if (ctx->flags_host) cudaFreeHost(ctx->flags_host);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

void release_graph(sbpgpu_graph* g) {
    if (!g->dead || g->refs > 0) return;
    sbpgpu_ctx* ctx = g->ctx;
    free_all(g->owned, ctx->stream);
    if (g->w.cells) cudaFreeAsync(g->w.cells, ctx->stream);
    delete g;
    ctx->refs--;
    release_ctx(ctx);
}

sbpgpu_status delta_batch_impl(sbpgpu_bm* bm, int64_t n, const int32_t* vertex, const int32_t* proposal, double* out,
                               bool np) {
    if (!bm || n < 0 || (n && (!vertex || !proposal || !out))) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (n == 0) return SBPGPU_OK;
        int32_t max_k = 0;
        for (int64_t i = 0; i < n; ++i) {
            if (vertex[i] < 0 || vertex[i] >= g->N || proposal[i] < 0 || proposal[i] >= bm->d.B)
                throw ApiError(SBPGPU_EINVAL, "vertex or proposal out of range");
            max_k = std::max(max_k, g->kdeg[vertex[i]]);
        }
        if (max_k > 8192) throw ApiError(SBPGPU_EUNSUPPORTED, "vertex degree above 8192");
        if (np) ensure_np(g);
        std::vector<void*> tmp;
        int32_t* dv = dalloc<int32_t>(tmp, n);
        int32_t* ds = dalloc<int32_t>(tmp, n);
        long long* dout = dalloc<long long>(tmp, n);
        cudaStream_t st = g->ctx->stream;
        std::vector<long long> h(n);
        try {
            CK(cudaMemcpyAsync(dv, vertex, n * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(ds, proposal, n * 4, cudaMemcpyHostToDevice, st));
            launch_vertex_dS_batch(g->dg, bm->d, dv, ds, n, max_k, dout, g->w, st, np);
            if (np && g->dc) launch_dc_vertex_deltas(g->dg, bm->d, dv, ds, n, dout, st);
            CK(cudaMemcpyAsync(h.data(), dout, n * 8, cudaMemcpyDeviceToHost, st));
            check_flags(g);
        } catch (...) {
            free_all(tmp, g->ctx->stream);
            throw;
        }
        free_all(tmp, g->ctx->stream);
        for (int64_t i = 0; i < n; ++i) out[i] = (double)h[i] * (1.0 / 16777216.0);
        return SBPGPU_OK;
    });
}

sbpgpu_status merge_delta_batch_impl(sbpgpu_bm* bm, int64_t n, const int32_t* block, const int32_t* proposal,
                                     double* out, bool np) {
    if (!bm || n < 0 || (n && (!block || !proposal || !out))) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (n == 0) return SBPGPU_OK;
        for (int64_t i = 0; i < n; ++i)
            if (block[i] < 0 || block[i] >= bm->d.B || proposal[i] < 0 || proposal[i] >= bm->d.B ||
                block[i] == proposal[i])
                throw ApiError(SBPGPU_EINVAL, "block or proposal out of range");
        if (np) ensure_np_sweeps(g);
        std::vector<void*> tmp;
        int32_t* dr = dalloc<int32_t>(tmp, n);
        int32_t* ds = dalloc<int32_t>(tmp, n);
        long long* dout = dalloc<long long>(tmp, n);
        cudaStream_t st = g->ctx->stream;
        std::vector<long long> h(n);
        try {
            CK(cudaMemcpyAsync(dr, block, n * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(ds, proposal, n * 4, cudaMemcpyHostToDevice, st));
            launch_merge_dS_batch(g->dg, bm->d, dr, ds, n, dout, g->w, st, np);
            CK(cudaMemcpyAsync(h.data(), dout, n * 8, cudaMemcpyDeviceToHost, st));
            check_flags(g);
        } catch (...) {
            free_all(tmp, g->ctx->stream);
            throw;
        }
        free_all(tmp, g->ctx->stream);
        for (int64_t i = 0; i < n; ++i) out[i] = (double)h[i] * (1.0 / 16777216.0);
        return SBPGPU_OK;
    });
}

// finetune::move_vertex (finetune.cpp:822-840) for one vertex and a given proposal: the delta
// (and, non-greedy, the Hastings correction) against the current state, finetune::accept
// with the canonical draw of (vertex, iteration, step, DOM_MH) -- word 3, as the chains use
// it -- and, when accepted, the move applied and the blockmodel rebuilt.
void move_one(sbpgpu_bm* bm, const sbpgpu_config& cfg, int32_t v, int32_t s, uint64_t seed, uint32_t iteration,
              uint32_t step, double* out_dS, int32_t* out_moved) {
    sbpgpu_graph* g = bm->g;
    const bool np = cfg.nonparametric != 0, greedy = cfg.greedy != 0 && !np;
    if (np) ensure_np(g);
    const int32_t max_k = g->kdeg[v];
    if (max_k > 8192) throw ApiError(SBPGPU_EUNSUPPORTED, "vertex degree above 8192");
    cudaStream_t st = g->ctx->stream;
    std::vector<void*> tmp;
    int32_t* dv = dalloc<int32_t>(tmp, 2);
    long long* ddS = dalloc<long long>(tmp, 1);
    double* dH = dalloc<double>(tmp, 1);
    long long dS_fixed = 0;
    double H = 1.0;
    try {
        const int32_t pair[2] = {v, s};
        CK(cudaMemcpyAsync(dv, pair, 8, cudaMemcpyHostToDevice, st));
        launch_vertex_dS_batch(g->dg, bm->d, dv, dv + 1, 1, max_k, ddS, g->w, st, np, greedy || np ? nullptr : dH);
        if (np && g->dc) launch_dc_vertex_deltas(g->dg, bm->d, dv, dv + 1, 1, ddS, st);
        CK(cudaMemcpyAsync(&dS_fixed, ddS, 8, cudaMemcpyDeviceToHost, st));
        if (!greedy && !np) CK(cudaMemcpyAsync(&H, dH, 8, cudaMemcpyDeviceToHost, st));
        check_flags(g);
    } catch (...) {
        free_all(tmp, st);
        throw;
    }
    free_all(tmp, st);
    const double dS = (double)dS_fixed * (1.0 / 16777216.0);
    bool accepted;
    if (greedy) {
        accepted = dS_fixed < 0;
    } else {
        uint32_t w[4];
        philox_host((uint32_t)v, iteration, step, DOM_MH, seed, w);
        const double u = (double)w[3] * (1.0 / 4294967296.0);
        double p = std::exp(-3.0 * dS) * H;
        p = p >= 1.0 ? 1.0 : p;
        accepted = u <= p;
    }
    if (accepted) {
        CK(cudaMemcpyAsync(bm->d.asg + v, &s, 4, cudaMemcpyHostToDevice, st));
        do_rebuild(bm);
        host_wait(st);
    }
    if (out_dS) *out_dS = dS;
    if (out_moved) *out_moved = accepted ? 1 : 0;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

void sbpgpu_default_config(sbpgpu_config* cfg) {
    cfg->algorithm = 1;
    cfg->batches = 1;
    cfg->mh_percent = 0.075f;
    cfg->greedy = 1;
    cfg->ordered = 0;
    cfg->approximate = 0;
    cfg->asynciterations = INT32_MAX;
    cfg->max_iterations = 100;
    cfg->nonparametric = 0;
    cfg->split = 0;
    cfg->splitinit = 0;
}

sbpgpu_status sbpgpu_ctx_create(int32_t device, sbpgpu_ctx** out) {
    if (!out) return SBPGPU_EINVAL;
    *out = nullptr;
    auto* ctx = new sbpgpu_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->flags_host, sizeof(DevFlags));
    if (e == cudaSuccess) {
        memset(ctx->flags_host, 0, sizeof(DevFlags));
        // keep memory freed by one partition in the device pool for the next one
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (e != cudaSuccess) {
        if (ctx->flags_host) cudaFreeHost(ctx->flags_host);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        cudaGetLastError();
        return SBPGPU_EDEVICE;
    }
    *out = ctx;
    return SBPGPU_OK;
}

void sbpgpu_ctx_destroy(sbpgpu_ctx* ctx) {
    if (!ctx || ctx->dead) return;
    ctx->dead = true;
    release_ctx(ctx);
}

const char* sbpgpu_last_error(const sbpgpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

sbpgpu_status sbpgpu_ctx_synchronize(sbpgpu_ctx* ctx) {
    return guarded(ctx, [&] {
        host_wait(ctx->stream);
        return SBPGPU_OK;
    });
}

void* sbpgpu_ctx_stream(sbpgpu_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

sbpgpu_status sbpgpu_ctx_set_cluster_blocks(sbpgpu_ctx* ctx, int64_t min_blocks) {
    if (!ctx || min_blocks < 0) return SBPGPU_EINVAL;
    ctx->cluster_blocks = min_blocks;
    ctx->chain_cluster_blocks = min_blocks;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_ctx_set_chain_cluster_blocks(sbpgpu_ctx* ctx, int64_t min_blocks) {
    if (!ctx || min_blocks < 0) return SBPGPU_EINVAL;
    ctx->chain_cluster_blocks = min_blocks;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_ctx_set_cancel(sbpgpu_ctx* ctx, int32_t requested) {
    if (!ctx) return SBPGPU_EINVAL;
    ctx->cancel.store(requested ? 1 : 0);
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_ctx_inject_alloc_failure(sbpgpu_ctx* ctx, int64_t after) {
    if (!ctx) return SBPGPU_EINVAL;
    ctx->fail_alloc_after = after < 0 ? -1 : after;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_ctx_set_cells_budget(sbpgpu_ctx* ctx, int64_t bytes) {
    if (!ctx) return SBPGPU_EINVAL;
    if (bytes < 0) return fail(ctx, SBPGPU_EINVAL, "cells budget must be >= 0");
    ctx->cells_budget = bytes;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_graph_create(sbpgpu_ctx* ctx, int64_t N, int64_t E, const int32_t* src, const int32_t* dst,
                                  sbpgpu_graph** out) {
    if (!ctx || !out) return SBPGPU_EINVAL;
    *out = nullptr;
    if (N <= 0 || E < 0 || E >= (int64_t)INT32_MAX - 2 || N >= INT32_MAX / 2 || (E > 0 && (!src || !dst)))
        return fail(ctx, SBPGPU_EINVAL, "graph needs 0 < N < 2^30, 0 <= E < 2^31 - 2 and edge arrays");
    auto* g = new sbpgpu_graph();
    g->ctx = ctx;
    g->N = N;
    g->E = E;
    g->Em = E;
    const sbpgpu_status rc = guarded(ctx, [&] {
        CK(cudaSetDevice(ctx->device));
        upload_graph(g, src, dst);
        return SBPGPU_OK;
    });
    if (rc != SBPGPU_OK) {
        free_all(g->owned, ctx->stream);
        delete g;
        return rc;
    }
    ctx->refs++;
    *out = g;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_graph_create_device(sbpgpu_ctx* ctx, int64_t N, int64_t E, const int32_t* d_src,
                                         const int32_t* d_dst, sbpgpu_graph** out) {
    if (!ctx || !out) return SBPGPU_EINVAL;
    std::vector<int32_t> src(E), dst(E);
    const sbpgpu_status rc = guarded(ctx, [&] {
        if (E) {
            CK(cudaMemcpy(src.data(), d_src, E * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(dst.data(), d_dst, E * 4, cudaMemcpyDeviceToHost));
        }
        return SBPGPU_OK;
    });
    if (rc != SBPGPU_OK) return rc;
    return sbpgpu_graph_create(ctx, N, E, src.data(), dst.data(), out);
}

sbpgpu_status sbpgpu_graph_load(sbpgpu_ctx* ctx, const char* path, int32_t undirected, sbpgpu_graph** out) {
    if (!ctx || !path || !out) return SBPGPU_EINVAL;
    *out = nullptr;
    std::string data;
    {
        FILE* f = std::fopen(path, "rb");
        if (!f) return fail(ctx, SBPGPU_EINVAL, std::string("cannot open ") + path);
        char buf[1 << 16];
        size_t got;
        while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.append(buf, got);
        std::fclose(f);
    }
    // Matrix Market: banner, comment lines, then "rows cols entries" (graph.cpp:75-103)
    size_t offset = 0;
    int64_t header_n = 0;
    bool symmetric = false, matrix_market = false;
    auto next_line = [&](size_t at) {
        const size_t e = data.find('\n', at);
        return e == std::string::npos ? data.size() : e + 1;
    };
    if (data.compare(0, 14, "%%MatrixMarket") == 0) {
        matrix_market = true;
        const size_t e = next_line(0);
        std::vector<std::string> tok;
        {
            std::string cur;
            for (size_t i = 0; i < e; ++i) {
                const char c = data[i];
                if (c == ' ' || c == '\t' || c == '\n' || c == '\r') {
                    if (!cur.empty()) tok.push_back(cur);
                    cur.clear();
                } else {
                    cur += c;
                }
            }
            if (!cur.empty()) tok.push_back(cur);
        }
        if (tok.size() < 5 || tok[2] != "coordinate")
            return fail(ctx, SBPGPU_EINVAL, "only coordinate Matrix Market files hold graphs");
        symmetric = tok[4] == "symmetric";
        size_t at = e;
        while (at < data.size() && data[at] == '%') at = next_line(at);
        long long rows = 0, cols = 0, nnz = 0;
        if (std::sscanf(data.c_str() + at, "%lld %lld %lld", &rows, &cols, &nnz) != 3)
            return fail(ctx, SBPGPU_EINVAL, "missing Matrix Market size line");
        if (rows != cols) return fail(ctx, SBPGPU_EINVAL, "rectangular matrices are not graphs");
        header_n = rows;
        offset = next_line(at);
    }
    const int un = (undirected || symmetric) ? 1 : 0;
    int32_t *d_src = nullptr, *d_dst = nullptr;
    int64_t E = 0, max_id = 0;
    const sbpgpu_status rc = guarded(ctx, [&] {
        CK(cudaSetDevice(ctx->device));
        const int64_t n = (int64_t)(data.size() - offset);
        char* d_text = nullptr;
        if (n > 0) {
            CK(cudaMallocAsync(&d_text, (size_t)n, ctx->stream));
            CK(cudaMemcpyAsync(d_text, data.data() + offset, (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
        }
        std::string err;
        const bool ok = parse_edges_device(d_text, n, un, &d_src, &d_dst, &E, &max_id, &err, ctx->stream);
        if (d_text) cudaFreeAsync(d_text, ctx->stream);
        if (!ok) throw ApiError(SBPGPU_EINVAL, err);
        return SBPGPU_OK;
    });
    if (rc != SBPGPU_OK) return rc;
    const int64_t N = std::max<int64_t>(max_id, header_n);
    sbpgpu_status rc2 = N > 0 ? sbpgpu_graph_create_device(ctx, N, E, d_src, d_dst, out)
                              : fail(ctx, SBPGPU_EINVAL, "the file holds no vertices");
    // an undirected edge list counts each stored pair once (graph.cpp:145-147); a Matrix
    // Market file counts its header entries plus the reverse edges added (graph.cpp:96-116)
    if (rc2 == SBPGPU_OK && un && !matrix_market) (*out)->Em = E / 2;
    if (rc2 == SBPGPU_OK) (*out)->und = un;
    if (d_src) cudaFreeAsync(d_src, ctx->stream);
    if (d_dst) cudaFreeAsync(d_dst, ctx->stream);
    return rc2;
}

sbpgpu_status sbpgpu_sample(sbpgpu_graph* g, int32_t algorithm, double sample_size, uint64_t seed, int32_t* mapping,
                            int64_t* sample_n) {
    if (!g || !mapping || !sample_n || algorithm < 0 || algorithm > 5 || !(sample_size > 0.0)) return SBPGPU_EINVAL;
    return guarded(g->ctx, [&] {
        cudaStream_t st = g->ctx->stream;
        std::vector<void*> tmp;
        int32_t* d_map = dalloc<int32_t>(tmp, g->N);
        try {
            *sample_n = sample_vertices(g->dg, algorithm, sample_size, seed, d_map, g->w, st);
            CK(cudaMemcpyAsync(mapping, d_map, g->N * 4, cudaMemcpyDeviceToHost, st));
            host_wait(st);
            CK(cudaGetLastError());
        } catch (...) {
            free_all(tmp, st);
            throw;
        }
        free_all(tmp, st);
        return SBPGPU_OK;
    });
}

namespace {

// The sampled subgraph of g for the device mapping d_map (n sampled vertices).
sbpgpu_graph* make_subgraph(sbpgpu_graph* g, const int32_t* d_map, int64_t n) {
    cudaStream_t st = g->ctx->stream;
    int32_t *d_src = nullptr, *d_dst = nullptr;
    int64_t E2 = 0;
    subgraph_edges(g->dg, d_map, &d_src, &d_dst, &E2, g->w, st);
    sbpgpu_graph* sub = nullptr;
    const sbpgpu_status rc = sbpgpu_graph_create_device(g->ctx, n, E2, d_src, d_dst, &sub);
    if (d_src) cudaFreeAsync(d_src, st);
    if (d_dst) cudaFreeAsync(d_dst, st);
    if (rc != SBPGPU_OK) throw ApiError(rc, std::string("sample graph: ") + sbpgpu_last_error(g->ctx));
    sub->und = g->und;  // args.undirected is global in the reference
    return sub;
}

// Checks a host mapping: every entry in [-1, n) and each sample id used exactly once.
void check_mapping(const sbpgpu_graph* g, const int32_t* mapping, int64_t n) {
    std::vector<char> seen(n, 0);
    for (int64_t v = 0; v < g->N; ++v) {
        const int32_t m = mapping[v];
        if (m < -1 || m >= n || (m >= 0 && seen[m]++)) throw ApiError(SBPGPU_EINVAL, "invalid sample mapping");
    }
    for (int64_t i = 0; i < n; ++i)
        if (!seen[i]) throw ApiError(SBPGPU_EINVAL, "sample mapping misses a sample id");
}

}  // namespace

sbpgpu_status sbpgpu_graph_subgraph(sbpgpu_graph* g, const int32_t* mapping, int64_t n, sbpgpu_graph** out) {
    if (!g || !mapping || !out || n <= 0) return SBPGPU_EINVAL;
    *out = nullptr;
    return guarded(g->ctx, [&] {
        check_mapping(g, mapping, n);
        cudaStream_t st = g->ctx->stream;
        std::vector<void*> tmp;
        int32_t* d_map = dalloc<int32_t>(tmp, g->N);
        try {
            CK(cudaMemcpyAsync(d_map, mapping, g->N * 4, cudaMemcpyHostToDevice, st));
            *out = make_subgraph(g, d_map, n);
        } catch (...) {
            free_all(tmp, st);
            throw;
        }
        free_all(tmp, st);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_extend(sbpgpu_graph* g, const int32_t* sample_assignment, int64_t sample_n, int64_t num_blocks,
                            const int32_t* mapping, uint64_t seed, int32_t* out) {
    if (!g || !sample_assignment || !mapping || !out || sample_n <= 0 || num_blocks <= 0) return SBPGPU_EINVAL;
    return guarded(g->ctx, [&] {
        check_mapping(g, mapping, sample_n);
        for (int64_t i = 0; i < sample_n; ++i)
            if (sample_assignment[i] < 0 || sample_assignment[i] >= num_blocks)
                throw ApiError(SBPGPU_EINVAL, "sample assignment out of range");
        cudaStream_t st = g->ctx->stream;
        std::vector<void*> tmp;
        int32_t* d_map = dalloc<int32_t>(tmp, g->N);
        int32_t* d_sasg = dalloc<int32_t>(tmp, sample_n);
        int32_t* d_asg = dalloc<int32_t>(tmp, g->N);
        try {
            CK(cudaMemcpyAsync(d_map, mapping, g->N * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(d_sasg, sample_assignment, sample_n * 4, cudaMemcpyHostToDevice, st));
            extend_assignment(g->dg, d_map, d_sasg, (int32_t)num_blocks, g->max_k, seed, d_asg, st);
            CK(cudaMemcpyAsync(out, d_asg, g->N * 4, cudaMemcpyDeviceToHost, st));
            host_wait(st);
            CK(cudaGetLastError());
        } catch (...) {
            free_all(tmp, st);
            throw;
        }
        free_all(tmp, st);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_reattach(sbpgpu_graph* g, const int32_t* sample_assignment, int64_t sample_n, int64_t num_blocks,
                              const int32_t* mapping, uint64_t seed, int32_t* out) {
    if (!g || !sample_assignment || !mapping || !out || sample_n <= 0 || num_blocks <= 0) return SBPGPU_EINVAL;
    return guarded(g->ctx, [&] {
        check_mapping(g, mapping, sample_n);
        for (int64_t i = 0; i < sample_n; ++i)
            if (sample_assignment[i] < 0 || sample_assignment[i] >= num_blocks)
                throw ApiError(SBPGPU_EINVAL, "sample assignment out of range");
        cudaStream_t st = g->ctx->stream;
        std::vector<void*> tmp;
        int32_t* d_map = dalloc<int32_t>(tmp, g->N);
        int32_t* d_sasg = dalloc<int32_t>(tmp, sample_n);
        int32_t* d_asg = dalloc<int32_t>(tmp, g->N);
        try {
            CK(cudaMemcpyAsync(d_map, mapping, g->N * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(d_sasg, sample_assignment, sample_n * 4, cudaMemcpyHostToDevice, st));
            try {
                reattach_assignment(g->dg, d_map, d_sasg, (int32_t)num_blocks, seed, d_asg, st);
            } catch (const std::invalid_argument& e) {
                throw ApiError(SBPGPU_EINVAL, e.what());
            }
            CK(cudaMemcpyAsync(out, d_asg, g->N * 4, cudaMemcpyDeviceToHost, st));
            host_wait(st);
            CK(cudaGetLastError());
        } catch (...) {
            free_all(tmp, st);
            throw;
        }
        free_all(tmp, st);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_finetune_assignment(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed,
                                         sbpgpu_stats* stats) {
    if (!bm || !cfg) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        g->st = sbpgpu_stats{};
        const int64_t l0 = kernel_launches();
        reset_counters(g);
        finetune_assignment_impl(bm, *cfg, seed);
        harvest_counters(g);
        g->st.kernel_launches = kernel_launches() - l0;
        if (stats) *stats = g->st;
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_sbp_sampled(sbpgpu_graph* g, const sbpgpu_config* cfg, uint64_t seed, int32_t algorithm,
                                 double sample_size, int32_t* out_assignment, int64_t* num_blocks, double* out_mdl,
                                 sbpgpu_stats* stats) {
    if (!g || !cfg || algorithm < 0 || algorithm > 5 || !(sample_size > 0.0)) return SBPGPU_EINVAL;
    sbpgpu_graph* sub = nullptr;
    sbpgpu_bm* bm = nullptr;
    const sbpgpu_status rc = guarded(g->ctx, [&] {
        cudaStream_t st = g->ctx->stream;
        const int64_t l0 = kernel_launches();
        std::vector<void*> tmp;
        int32_t* d_map = dalloc<int32_t>(tmp, g->N);
        int32_t* d_asg = dalloc<int32_t>(tmp, g->N);
        sbpgpu_stats st1{};
        int64_t B = 0;
        try {
            // sample, then the partition of the sample (main.cpp:98-121)
            const int64_t n = sample_vertices(g->dg, algorithm, sample_size, seed, d_map, g->w, st);
            if (n <= 0) throw ApiError(SBPGPU_EINVAL, "the sample is empty");
            sub = make_subgraph(g, d_map, n);
            std::vector<int32_t> sasg(n);
            double smdl = 0.0;
            const sbpgpu_status r1 = sbpgpu_sbp(sub, cfg, seed, sasg.data(), &B, &smdl, &st1);
            if (r1 != SBPGPU_OK) throw ApiError(r1, std::string("sample partition: ") + sbpgpu_last_error(g->ctx));
            // extend to the full graph, then finetune_assignment (main.cpp:122-140)
            int32_t* d_sasg = dalloc<int32_t>(tmp, n);
            CK(cudaMemcpyAsync(d_sasg, sasg.data(), n * 4, cudaMemcpyHostToDevice, st));
            extend_assignment(g->dg, d_map, d_sasg, (int32_t)B, g->max_k, seed, d_asg, st);
            std::vector<int32_t> asg(g->N);
            CK(cudaMemcpyAsync(asg.data(), d_asg, g->N * 4, cudaMemcpyDeviceToHost, st));
            host_wait(st);
            const sbpgpu_status r2 = sbpgpu_bm_create(g, B, asg.data(), &bm);
            if (r2 != SBPGPU_OK) throw ApiError(r2, std::string("extended blockmodel: ") + sbpgpu_last_error(g->ctx));
        } catch (...) {
            free_all(tmp, st);
            throw;
        }
        free_all(tmp, st);
        g->st = sbpgpu_stats{};
        reset_counters(g);
        finetune_assignment_impl(bm, *cfg, seed);
        harvest_counters(g);
        if (out_assignment) CK(cudaMemcpyAsync(out_assignment, bm->d.asg, g->N * 4, cudaMemcpyDeviceToHost, st));
        host_wait(st);
        if (num_blocks) *num_blocks = B;
        if (out_mdl) *out_mdl = bm->entropy;
        if (stats) {
            sbpgpu_stats s = st1;
            s.proposals += g->st.proposals;
            s.moves += g->st.moves;
            s.mcmc_iterations += g->st.mcmc_iterations;
            s.edges_swept += g->st.edges_swept;
            s.chain_rounds += g->st.chain_rounds;
            s.kernel_launches = kernel_launches() - l0;
            *stats = s;
        }
        return SBPGPU_OK;
    });
    if (bm) sbpgpu_bm_destroy(bm);
    if (sub) sbpgpu_graph_destroy(sub);
    return rc;
}

sbpgpu_status sbpgpu_partition_scores(int64_t num_vertices, int64_t nrows, int64_t ncols, const int64_t* table,
                                      sbpgpu_eval* out) {
    if (!table || !out || num_vertices < 2 || nrows <= 0 || ncols <= 0 || nrows * ncols > (int64_t(1) << 28))
        return SBPGPU_EINVAL;
    try {
        std::vector<std::vector<long long>> m(nrows, std::vector<long long>(ncols));
        for (int64_t r = 0; r < nrows; ++r)
            for (int64_t c = 0; c < ncols; ++c) m[r][c] = table[r * ncols + c];
        const PartitionQuality q = scores_from_matrix(m, num_vertices, false);
        *out = sbpgpu_eval{q.nmi, q.f1, q.precision, q.recall, q.rand_index, 0.0, q.true_blocks, q.found_blocks};
    } catch (const std::bad_alloc&) {
        return SBPGPU_ENOMEM;
    }
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_evaluate(sbpgpu_ctx* ctx, int64_t n, const int32_t* truth, const int32_t* assignment,
                              sbpgpu_eval* out) {
    if (!ctx || !out || n <= 0 || !truth || !assignment) return SBPGPU_EINVAL;
    return guarded(ctx, [&] {
        // true communities renumbered in order of first appearance (evaluate.cpp:103-113)
        std::unordered_map<int32_t, int32_t> ids;
        std::vector<int32_t> t(n);
        int64_t nb = 0;
        for (int64_t i = 0; i < n; ++i) {
            if (assignment[i] < 0) throw ApiError(SBPGPU_EINVAL, "negative block in the assignment");
            nb = std::max<int64_t>(nb, (int64_t)assignment[i] + 1);
            if (truth[i] < 0) {
                t[i] = -1;
                continue;
            }
            auto it = ids.emplace(truth[i], (int32_t)ids.size()).first;
            t[i] = it->second;
        }
        const int64_t nt = (int64_t)ids.size();
        if (nt == 0) throw ApiError(SBPGPU_EINVAL, "no vertex of the true partition is labelled");
        if (nt * nb > (int64_t(1) << 28)) throw ApiError(SBPGPU_EINVAL, "contingency table above 2^28 cells");
        cudaStream_t st = ctx->stream;
        std::vector<void*> tmp;
        int32_t* dt = dalloc<int32_t>(tmp, n);
        int32_t* da = dalloc<int32_t>(tmp, n);
        auto* table = dalloc<unsigned long long>(tmp, (size_t)(nt * nb));
        std::vector<unsigned long long> h((size_t)(nt * nb));
        try {
            CK(cudaMemcpyAsync(dt, t.data(), n * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(da, assignment, n * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemsetAsync(table, 0, h.size() * sizeof(unsigned long long), st));
            launch_contingency(dt, da, n, (int32_t)nb, table, st);
            CK(cudaMemcpyAsync(h.data(), table, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
            host_wait(st);
            CK(cudaGetLastError());
        } catch (...) {
            free_all(tmp, st);
            throw;
        }
        free_all(tmp, st);
        const PartitionQuality q = quality_from_table(h, nt, nb, n);
        *out = sbpgpu_eval{q.nmi, q.f1, q.precision, q.recall, q.rand_index, q.accuracy, q.true_blocks,
                           q.found_blocks};
        return SBPGPU_OK;
    });
}

void sbpgpu_graph_destroy(sbpgpu_graph* g) {
    if (!g || g->dead) return;
    g->dead = true;
    release_graph(g);
}

int64_t sbpgpu_graph_num_vertices(const sbpgpu_graph* g) { return g ? g->N : 0; }
int64_t sbpgpu_graph_num_edges(const sbpgpu_graph* g) { return g ? g->E : 0; }
int64_t sbpgpu_graph_model_edges(const sbpgpu_graph* g) { return g ? g->Em : 0; }

int32_t sbpgpu_graph_undirected(const sbpgpu_graph* g) { return g ? g->und : 0; }

int32_t sbpgpu_graph_degree_corrected(const sbpgpu_graph* g) { return g ? g->dc : 0; }

sbpgpu_status sbpgpu_graph_set_degree_corrected(sbpgpu_graph* g, int32_t on) {
    if (!g) return SBPGPU_EINVAL;
    g->dc = on ? 1 : 0;
    g->dg.dc = g->dc;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_graph_set_undirected(sbpgpu_graph* g, int32_t undirected) {
    if (!g) return SBPGPU_EINVAL;
    g->und = undirected ? 1 : 0;  // the nonparametric tables follow on their next use
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_graph_set_model_edges(sbpgpu_graph* g, int64_t num_edges) {
    if (!g) return SBPGPU_EINVAL;
    if (num_edges <= 0) return fail(g->ctx, SBPGPU_EINVAL, "the model edge count must be positive");
    g->Em = num_edges;  // the nonparametric tables follow on their next use
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_bm_create(sbpgpu_graph* g, int64_t B, const int32_t* assignment, sbpgpu_bm** out) {
    if (!g || !out) return SBPGPU_EINVAL;
    *out = nullptr;
    sbpgpu_ctx* ctx = g->ctx;
    if (B <= 0 || B > g->N) return fail(ctx, SBPGPU_EINVAL, "num_blocks must be in [1, N]");
    if (assignment)
        for (int64_t v = 0; v < g->N; ++v)
            if (assignment[v] < 0 || assignment[v] >= B)
                return fail(ctx, SBPGPU_EINVAL, "assignment value out of range");
    sbpgpu_bm* bm = nullptr;
    const sbpgpu_status rc = guarded(ctx, [&] {
        bm = new_bm(g, B);
        if (assignment) {
            CK(cudaMemcpyAsync(bm->d.asg, assignment, g->N * 4, cudaMemcpyHostToDevice, ctx->stream));
        } else {
            CK(cudaMemcpyAsync(bm->d.asg, g->d_all, g->N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        }
        bm->num_blocks_to_merge = (int64_t)((double)B * 0.5);
        do_rebuild(bm);
        check_flags(g);
        return SBPGPU_OK;
    });
    if (rc != SBPGPU_OK) {
        if (bm) {
            free_all(bm->owned, bm->g->ctx->stream);
            delete bm;
        }
        return rc;
    }
    g->refs++;
    *out = bm;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_bm_copy(const sbpgpu_bm* src, sbpgpu_bm** out) {
    if (!src || !out) return SBPGPU_EINVAL;
    sbpgpu_graph* g = src->g;
    sbpgpu_bm* bm = nullptr;
    const sbpgpu_status rc = guarded(g->ctx, [&] {
        bm = new_bm(g, src->d.B);
        cudaStream_t st = g->ctx->stream;
        const int64_t N = g->N;
        const int64_t nnz = src->d.nnz;
        const DevBM& a = src->d;
        DevBM& b = bm->d;
        CK(cudaMemcpyAsync(b.asg, a.asg, N * 4, cudaMemcpyDeviceToDevice, st));
        for (auto pr : {std::make_pair(b.d_out, a.d_out), std::make_pair(b.d_in, a.d_in),
                        std::make_pair(b.d_tot, a.d_tot), std::make_pair(b.sizes, a.sizes),
                        std::make_pair(b.diag, a.diag)})
            CK(cudaMemcpyAsync(pr.first, pr.second, a.B * 4, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(b.row_off, a.row_off, (a.B + 1) * 4, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(b.col_off, a.col_off, (a.B + 1) * 4, cudaMemcpyDeviceToDevice, st));
        if (nnz)
            for (auto pr : {std::make_pair(b.row_col, a.row_col), std::make_pair(b.row_cnt, a.row_cnt),
                            std::make_pair(b.row_cum, a.row_cum), std::make_pair(b.row_of, a.row_of),
                            std::make_pair(b.col_row, a.col_row), std::make_pair(b.col_cnt, a.col_cnt),
                            std::make_pair(b.col_cum, a.col_cum)})
                CK(cudaMemcpyAsync(pr.first, pr.second, nnz * 4, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(b.nonempty, a.nonempty, 4, cudaMemcpyDeviceToDevice, st));
        b.nnz = a.nnz;
        bm->entropy = src->entropy;
        bm->num_blocks_to_merge = 0;  // Blockmodel::copy (blockmodel.cpp:151)
        host_wait(st);
        return SBPGPU_OK;
    });
    if (rc != SBPGPU_OK) {
        if (bm) {
            free_all(bm->owned, bm->g->ctx->stream);
            delete bm;
        }
        return rc;
    }
    g->refs++;
    *out = bm;
    return SBPGPU_OK;
}

void sbpgpu_bm_destroy(sbpgpu_bm* bm) {
    if (!bm) return;
    sbpgpu_graph* g = bm->g;
    host_wait(g->ctx->stream);
    free_all(bm->owned, bm->g->ctx->stream);
    delete bm;
    g->refs--;
    release_graph(g);
}

int64_t sbpgpu_bm_num_blocks(const sbpgpu_bm* bm) { return bm ? bm->d.B : 0; }
int64_t sbpgpu_bm_nnz(const sbpgpu_bm* bm) { return bm ? bm->d.nnz : 0; }
double sbpgpu_bm_entropy(const sbpgpu_bm* bm) { return bm ? bm->entropy : 0.0; }

sbpgpu_status sbpgpu_bm_read(const sbpgpu_bm* bm, int32_t* assignment, int64_t* d_out, int64_t* d_in, int64_t* d_tot,
                             int64_t* sizes, int32_t* rows, int32_t* cols, int64_t* counts) {
    if (!bm) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        cudaStream_t st = g->ctx->stream;
        const int64_t B = bm->d.B, nnz = bm->d.nnz;
        if (assignment) CK(cudaMemcpyAsync(assignment, bm->d.asg, g->N * 4, cudaMemcpyDeviceToHost, st));
        std::vector<int32_t> tmp;
        auto widen = [&](const int32_t* src, int64_t* dst, int64_t n) {
            if (!dst) return;
            tmp.resize(n);
            CK(cudaMemcpyAsync(tmp.data(), src, n * 4, cudaMemcpyDeviceToHost, st));
            host_wait(st);
            for (int64_t i = 0; i < n; ++i) dst[i] = tmp[i];
        };
        widen(bm->d.d_out, d_out, B);
        widen(bm->d.d_in, d_in, B);
        widen(bm->d.d_tot, d_tot, B);
        widen(bm->d.sizes, sizes, B);
        if (rows) CK(cudaMemcpyAsync(rows, bm->d.row_of, nnz * 4, cudaMemcpyDeviceToHost, st));
        if (cols) CK(cudaMemcpyAsync(cols, bm->d.row_col, nnz * 4, cudaMemcpyDeviceToHost, st));
        widen(bm->d.row_cnt, counts, nnz);
        host_wait(st);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_mdl(sbpgpu_bm* bm, double* out) {
    if (!bm || !out) return SBPGPU_EINVAL;
    return guarded(bm->g->ctx, [&] {
        *out = do_mdl(bm);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_np_mdl(sbpgpu_bm* bm, double* out) {
    if (!bm || !out) return SBPGPU_EINVAL;
    return guarded(bm->g->ctx, [&] {
        *out = do_mdl(bm, true);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* vertex, const int32_t* proposal,
                                     double* out) {
    return delta_batch_impl(bm, n, vertex, proposal, out, false);
}

sbpgpu_status sbpgpu_np_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* vertex, const int32_t* proposal,
                                        double* out) {
    return delta_batch_impl(bm, n, vertex, proposal, out, true);
}

sbpgpu_status sbpgpu_merge_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* block, const int32_t* proposal,
                                           double* out) {
    return merge_delta_batch_impl(bm, n, block, proposal, out, false);
}

sbpgpu_status sbpgpu_np_merge_delta_mdl_batch(sbpgpu_bm* bm, int64_t n, const int32_t* block,
                                              const int32_t* proposal, double* out) {
    return merge_delta_batch_impl(bm, n, block, proposal, out, true);
}


sbpgpu_status sbpgpu_delta_mdl_batch_noalloc(sbpgpu_bm* bm, int64_t n, const int32_t* vertex,
                                             const int32_t* proposal, double* out) {
    if (!bm || n < 0 || (n && (!vertex || !proposal || !out))) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (n == 0) return SBPGPU_OK;
        if (n > kNoAllocMaxBatch)
            throw ApiError(SBPGPU_EINVAL, "batch of " + std::to_string(n) + " exceeds the allocation-free limit of " +
                                              std::to_string(kNoAllocMaxBatch) + " entries");
        int32_t max_k = 0;
        for (int64_t i = 0; i < n; ++i) {
            if (vertex[i] < 0 || vertex[i] >= g->N || proposal[i] < 0 || proposal[i] >= bm->d.B)
                throw ApiError(SBPGPU_EINVAL, "vertex or proposal out of range");
            max_k = std::max(max_k, g->kdeg[vertex[i]]);
        }
        if (max_k > 8192) throw ApiError(SBPGPU_EUNSUPPORTED, "vertex degree above 8192");
        NoAllocScratch sc{};
        std::string err;
        if (!noalloc_scratch(g->ctx->device, &sc, &err)) throw ApiError(SBPGPU_EDEVICE, err);
        cudaStream_t st = g->ctx->stream;
        CK(cudaMemcpyAsync(sc.vertex, vertex, n * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(sc.proposal, proposal, n * 4, cudaMemcpyHostToDevice, st));
        launch_vertex_dS_batch(g->dg, bm->d, sc.vertex, sc.proposal, n, max_k, sc.result, g->w, st);
        launch_fixed_to_double(sc.result, n, st);
        CK(cudaMemcpyAsync(out, sc.result, n * 8, cudaMemcpyDeviceToHost, st));
        check_flags(g);
        return SBPGPU_OK;
    });
}


sbpgpu_status sbpgpu_propose_batch(sbpgpu_bm* bm, int64_t n, const int32_t* vertex, uint64_t seed, uint32_t c1,
                                   uint32_t c2, uint32_t c3, int32_t* out) {
    if (!bm || n < 0 || (n && (!vertex || !out))) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (n == 0) return SBPGPU_OK;
        for (int64_t i = 0; i < n; ++i)
            if (vertex[i] < 0 || vertex[i] >= g->N) throw ApiError(SBPGPU_EINVAL, "vertex out of range");
        if (bm->d.B < 2) throw ApiError(SBPGPU_EINVAL, "proposals need at least two blocks");
        std::vector<void*> tmp;
        int32_t* dv = dalloc<int32_t>(tmp, n);
        int32_t* dout = dalloc<int32_t>(tmp, n);
        cudaStream_t st = g->ctx->stream;
        try {
            CK(cudaMemcpyAsync(dv, vertex, n * 4, cudaMemcpyHostToDevice, st));
            launch_propose_batch(g->dg, bm->d, dv, n, seed, c1, c2, c3, dout, st);
            CK(cudaMemcpyAsync(out, dout, n * 4, cudaMemcpyDeviceToHost, st));
            check_flags(g);
        } catch (...) {
            free_all(tmp, g->ctx->stream);
            throw;
        }
        free_all(tmp, g->ctx->stream);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_gibbs_batch(sbpgpu_bm* bm, const sbpgpu_config* cfg, int64_t n, const int32_t* vertex,
                                 uint64_t seed, uint32_t iteration, uint32_t step, int32_t* out_moves,
                                 int64_t* applied) {
    if (!bm || !cfg || n < 0 || (n && !vertex)) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (bm->d.B < 2) throw ApiError(SBPGPU_EINVAL, "proposals need at least two blocks");
        if (n > g->N) throw ApiError(SBPGPU_EINVAL, "a batch holds at most num_vertices vertices");
        for (int64_t i = 0; i < n; ++i)
            if (vertex[i] < 0 || vertex[i] >= g->N) throw ApiError(SBPGPU_EINVAL, "vertex out of range");
        cudaStream_t st = g->ctx->stream;
        CK(cudaMemcpyAsync(g->w.list_tmp, vertex, n * 4, cudaMemcpyHostToDevice, st));
        reset_counters(g);
        gibbs_batch_dev(bm, g->w.list_tmp, (int32_t)n, seed, iteration, step, accept_mode(*cfg));
        if (out_moves) {
            std::vector<int32_t> mv(g->N);
            CK(cudaMemcpyAsync(mv.data(), g->w.moves, g->N * 4, cudaMemcpyDeviceToHost, st));
            host_wait(st);
            for (int64_t i = 0; i < n; ++i) out_moves[i] = mv[vertex[i]];
        }
        CK(cudaMemcpyAsync(g->flags_host, g->w.flags_dev, sizeof(DevFlags), cudaMemcpyDeviceToHost, st));
        check_flags(g);
        if (applied) *applied = (int64_t)g->flags_host->counters[2];
        reset_counters(g);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_gibbs_propose(sbpgpu_bm* bm, const sbpgpu_config* cfg, int64_t n, const int32_t* vertex,
                                   uint64_t seed, uint32_t iteration, uint32_t step, int32_t* out_moves) {
    if (!bm || !cfg || n < 0 || (n && (!vertex || !out_moves))) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (bm->d.B < 2) throw ApiError(SBPGPU_EINVAL, "proposals need at least two blocks");
        if (n > g->N) throw ApiError(SBPGPU_EINVAL, "a batch holds at most num_vertices vertices");
        for (int64_t i = 0; i < n; ++i)
            if (vertex[i] < 0 || vertex[i] >= g->N) throw ApiError(SBPGPU_EINVAL, "vertex out of range");
        if (n == 0) return SBPGPU_OK;
        const int mode = accept_mode(*cfg);
        if (mode == ACC_NP) ensure_np_sweeps(g);
        cudaStream_t st = g->ctx->stream;
        CK(cudaMemcpyAsync(g->w.list_tmp, vertex, n * 4, cudaMemcpyHostToDevice, st));
        reset_counters(g);
        gibbs_propose(g->dg, bm->d, g->w.list_tmp, (int32_t)n, g->max_k, seed, iteration, step, mode, g->w, st);
        std::vector<int32_t> mv(g->N);
        CK(cudaMemcpyAsync(mv.data(), g->w.moves, g->N * 4, cudaMemcpyDeviceToHost, st));
        check_flags(g);
        for (int64_t i = 0; i < n; ++i) out_moves[i] = mv[vertex[i]];
        reset_counters(g);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_mh_chain(sbpgpu_bm* bm, const sbpgpu_config* cfg, int64_t n, const int32_t* vertex,
                              uint64_t seed, uint32_t iteration, uint32_t step, int64_t* applied) {
    if (!bm || !cfg || n < 0 || (n && !vertex)) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (bm->d.B < 2) throw ApiError(SBPGPU_EINVAL, "proposals need at least two blocks");
        if (n > g->N) throw ApiError(SBPGPU_EINVAL, "the chain visits at most num_vertices vertices per call");
        int32_t max_k = 0;
        int64_t ksum = 0;
        for (int64_t i = 0; i < n; ++i) {
            if (vertex[i] < 0 || vertex[i] >= g->N) throw ApiError(SBPGPU_EINVAL, "vertex out of range");
            max_k = std::max(max_k, g->kdeg[vertex[i]]);
            ksum += g->kdeg[vertex[i]];
        }
        cudaStream_t st = g->ctx->stream;
        CK(cudaMemcpyAsync(g->w.list_tmp, vertex, n * 4, cudaMemcpyHostToDevice, st));
        reset_counters(g);
        chain_run(bm, g->w.list_tmp, (int32_t)n, max_k, ksum, seed, iteration, step, accept_mode(*cfg));
        CK(cudaMemcpyAsync(g->flags_host, g->w.flags_dev, sizeof(DevFlags), cudaMemcpyDeviceToHost, st));
        check_flags(g);
        if (applied) *applied = (int64_t)g->flags_host->counters[5];
        reset_counters(g);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_move_vertex(sbpgpu_bm* bm, const sbpgpu_config* cfg, int32_t vertex, int32_t proposal,
                                 uint64_t seed, uint32_t iteration, uint32_t step, double* out_dS,
                                 int32_t* out_moved) {
    if (!bm || !cfg) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (vertex < 0 || vertex >= g->N || proposal < 0 || proposal >= bm->d.B)
            throw ApiError(SBPGPU_EINVAL, "vertex or proposal out of range");
        reset_counters(g);
        move_one(bm, *cfg, vertex, proposal, seed, iteration, step, out_dS, out_moved);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_propose_move(sbpgpu_bm* bm, const sbpgpu_config* cfg, int32_t vertex, uint64_t seed,
                                  uint32_t iteration, uint32_t step, int32_t* out_proposal, double* out_dS,
                                  int32_t* out_moved) {
    if (!bm || !cfg) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (vertex < 0 || vertex >= g->N) throw ApiError(SBPGPU_EINVAL, "vertex out of range");
        if (bm->d.B < 2) throw ApiError(SBPGPU_EINVAL, "proposals need at least two blocks");
        cudaStream_t st = g->ctx->stream;
        int32_t r = 0, size = 0;
        CK(cudaMemcpyAsync(&r, bm->d.asg + vertex, 4, cudaMemcpyDeviceToHost, st));
        host_wait(st);
        CK(cudaMemcpyAsync(&size, bm->d.sizes + r, 4, cudaMemcpyDeviceToHost, st));
        host_wait(st);
        int32_t s = -1;
        double dS = 0.0;
        int32_t moved = 0;
        if (size == 1) {  // a singleton block never moves (finetune.cpp:845-847)
            dS = DBL_MAX;
        } else {
            std::vector<void*> tmp;
            int32_t* dv = dalloc<int32_t>(tmp, 1);
            int32_t* dp = dalloc<int32_t>(tmp, 1);
            try {
                CK(cudaMemcpyAsync(dv, &vertex, 4, cudaMemcpyHostToDevice, st));
                launch_propose_batch(g->dg, bm->d, dv, 1, seed, iteration, step, DOM_MH, dp, st);
                CK(cudaMemcpyAsync(&s, dp, 4, cudaMemcpyDeviceToHost, st));
                check_flags(g);
            } catch (...) {
                free_all(tmp, st);
                throw;
            }
            free_all(tmp, st);
            if (s == r) s = -1;  // proposal equal to the current block: no move (finetune.cpp:863-865)
            else move_one(bm, *cfg, vertex, s, seed, iteration, step, &dS, &moved);
        }
        if (out_proposal) *out_proposal = s;
        if (out_dS) *out_dS = dS;
        if (out_moved) *out_moved = moved;
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_mcmc(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed, int32_t step,
                          int32_t golden_ratio_not_reached, sbpgpu_stats* stats) {
    if (!bm || !cfg) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        g->st = sbpgpu_stats{};
        const int64_t l0 = kernel_launches();
        reset_counters(g);
        mcmc_impl(bm, *cfg, seed, step, golden_ratio_not_reached != 0);
        harvest_counters(g);
        g->st.kernel_launches = kernel_launches() - l0;
        if (stats) *stats = g->st;
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_merge_blocks(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed, int32_t step,
                                  int64_t num_blocks_to_merge, sbpgpu_stats* stats) {
    if (!bm || !cfg || num_blocks_to_merge < 0) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        g->st = sbpgpu_stats{};
        const int64_t l0 = kernel_launches();
        reset_counters(g);
        merge_impl(bm, *cfg, seed, step, num_blocks_to_merge);
        g->st.kernel_launches = kernel_launches() - l0;
        if (stats) *stats = g->st;
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_merge_proposals(sbpgpu_bm* bm, uint64_t seed, int32_t step, int32_t* best_proposal,
                                     double* best_delta) {
    if (!bm) return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (bm->d.B < 2) throw ApiError(SBPGPU_EINVAL, "merge proposals need at least two blocks");
        cudaStream_t st = g->ctx->stream;
        reset_counters(g);
        merge_propose(g->dg, bm->d, seed, (uint32_t)step, g->w, st);
        if (best_proposal) CK(cudaMemcpyAsync(best_proposal, g->w.best, bm->d.B * 4, cudaMemcpyDeviceToHost, st));
        if (best_delta) CK(cudaMemcpyAsync(best_delta, g->w.best_dS, bm->d.B * 8, cudaMemcpyDeviceToHost, st));
        check_flags(g);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_sbp(sbpgpu_graph* g, const sbpgpu_config* cfg_in, uint64_t seed, int32_t* out_assignment,
                         int64_t* num_blocks, double* out_mdl, sbpgpu_stats* stats) {
    if (!g || !cfg_in) return SBPGPU_EINVAL;
    sbpgpu_ctx* ctx = g->ctx;
    sbpgpu_bm* bm = nullptr;
    std::vector<void*> slots_mem;
    const sbpgpu_status rc = guarded(ctx, [&] {
        const sbpgpu_config cfg = *cfg_in;
        g->st = sbpgpu_stats{};
        const int64_t l0 = kernel_launches();
        reset_counters(g);
        cudaStream_t st = ctx->stream;
        const int64_t N = g->N;
        // Blockmodel(N, graph, 0.5) (sbp.cpp:23): identity assignment, B = N.
        bm = new_bm(g, N);
        CK(cudaMemcpyAsync(bm->d.asg, g->d_all, N * 4, cudaMemcpyDeviceToDevice, st));
        do_rebuild(bm);
        bm->num_blocks_to_merge = (int64_t)((double)N * 0.5);
        bm->entropy = DBL_MAX;
        struct Slot {
            bool empty = true;
            int64_t B = 0;
            double entropy = DBL_MAX;
            int32_t* asg = nullptr;
        } s[3];
        for (auto& sl : s) sl.asg = dalloc<int32_t>(slots_mem, N);
        bool optimal = false;
        int32_t step = 0;
        while (!optimal) {
            // between golden-section steps nothing of this call is in flight on the device
            if (ctx->cancel.exchange(0)) throw ApiError(SBPGPU_ECANCELED, "partition cancelled");
            merge_impl(bm, cfg, seed, step, bm->num_blocks_to_merge);
            mcmc_impl(bm, cfg, seed, step, s[2].empty);
            ++step;
            g->st.outer_steps++;
            // BlockmodelTriplet::update (blockmodel_triplet.cpp:82-105)
            int idx;
            if (s[1].empty) {
                idx = 1;
            } else if (bm->entropy <= s[1].entropy) {
                const int old = (s[1].B > bm->d.B) ? 0 : 2;
                std::swap(s[old], s[1]);
                idx = 1;
            } else {
                idx = (s[1].B > bm->d.B) ? 2 : 0;
            }
            s[idx].empty = false;
            s[idx].B = bm->d.B;
            s[idx].entropy = bm->entropy;
            CK(cudaMemcpyAsync(s[idx].asg, bm->d.asg, N * 4, cudaMemcpyDeviceToDevice, st));
            // BlockmodelTriplet::get_next_blockmodel (blockmodel_triplet.cpp:4-37)
            const Slot* src;
            int64_t next_merge;
            if (s[2].empty) {
                src = &s[1];
                next_merge = (int64_t)((double)src->B * 0.5);
                if (next_merge == 0) optimal = true;
            } else {
                if ((!s[0].empty && s[0].B - s[2].B == 2) || (s[0].empty && s[1].B - s[2].B == 1)) optimal = true;
                if (optimal) {
                    src = &s[1];
                    next_merge = 0;
                } else {
                    int index;
                    if (s[0].empty && s[1].B > s[2].B) index = 1;
                    else if ((s[0].B - s[1].B) >= (s[1].B - s[2].B)) index = 0;
                    else index = 1;
                    int64_t next_try = s[index + 1].B;
                    next_try += (int64_t)((double)(s[index].B - s[index + 1].B) * 0.618);
                    src = &s[index];
                    next_merge = src->B - next_try;
                }
            }
            CK(cudaMemcpyAsync(bm->d.asg, src->asg, N * 4, cudaMemcpyDeviceToDevice, st));
            bm->d.B = (int32_t)src->B;
            bm->entropy = src->entropy;
            bm->num_blocks_to_merge = next_merge;
            do_rebuild(bm);
        }
        if (out_assignment) CK(cudaMemcpyAsync(out_assignment, bm->d.asg, N * 4, cudaMemcpyDeviceToHost, st));
        harvest_counters(g);
        if (num_blocks) *num_blocks = bm->d.B;
        if (out_mdl) *out_mdl = bm->entropy;
        g->st.kernel_launches = kernel_launches() - l0;
        if (stats) *stats = g->st;
        return SBPGPU_OK;
    });
    free_all(slots_mem, ctx->stream);
    if (bm) {
        free_all(bm->owned, bm->g->ctx->stream);
        delete bm;
    }
    return rc;
}

sbpgpu_status sbpgpu_split_communities(sbpgpu_bm* bm, const sbpgpu_config* cfg, uint64_t seed, int32_t step,
                                       int64_t target_num_blocks) {
    if (!bm || !cfg || target_num_blocks < 1 || cfg->split < 0 || cfg->split > 3 || cfg->splitinit < 0 ||
        cfg->splitinit > 2)
        return SBPGPU_EINVAL;
    sbpgpu_graph* g = bm->g;
    return guarded(g->ctx, [&] {
        if (target_num_blocks > g->N) throw ApiError(SBPGPU_EINVAL, "target above one block per vertex");
        split_impl(bm, *cfg, seed, (uint32_t)step, target_num_blocks);
        return SBPGPU_OK;
    });
}

sbpgpu_status sbpgpu_sbp_top_down(sbpgpu_graph* g, const sbpgpu_config* cfg_in, uint64_t seed, int32_t mix,
                                  int32_t* out_assignment, int64_t* num_blocks, double* out_mdl,
                                  sbpgpu_stats* stats) {
    if (!g || !cfg_in || cfg_in->split < 0 || cfg_in->split > 3 || cfg_in->splitinit < 0 || cfg_in->splitinit > 2)
        return SBPGPU_EINVAL;
    sbpgpu_ctx* ctx = g->ctx;
    sbpgpu_bm* bm = nullptr;
    std::vector<void*> slots_mem;
    const sbpgpu_status rc = guarded(ctx, [&] {
        const sbpgpu_config cfg = *cfg_in;
        g->st = sbpgpu_stats{};
        const int64_t l0 = kernel_launches();
        reset_counters(g);
        cudaStream_t st = ctx->stream;
        const int64_t N = g->N;
        // Blockmodel(1, graph, 1.5, zeros) (top_down_sbp.cpp:440-442)
        bm = new_bm(g, N);
        CK(cudaMemsetAsync(bm->d.asg, 0, N * 4, st));
        bm->d.B = 1;
        do_rebuild(bm);
        bm->entropy = DBL_MAX;
        struct Slot {
            bool empty = true;
            int64_t B = 0;
            double entropy = DBL_MAX;
            int32_t* asg = nullptr;
        } s[3];
        for (auto& sl : s) sl.asg = dalloc<int32_t>(slots_mem, N);
        bool optimal = false;
        // TopDownBlockmodelTriplet::update and get_next_blockmodel (blockmodel_triplet.cpp:107-193)
        auto next = [&](int64_t* target) -> const Slot* {
            int idx;
            if (s[1].empty) {
                idx = 1;
            } else if (bm->entropy <= s[1].entropy && std::labs(bm->d.B - s[1].B) > 0.1 * (double)s[1].B) {
                const int old = s[1].B < bm->d.B ? 0 : 2;
                std::swap(s[old], s[1]);
                idx = 1;
            } else {
                idx = s[1].B < bm->d.B ? 2 : 0;
            }
            s[idx].empty = false;
            s[idx].B = bm->d.B;
            s[idx].entropy = bm->entropy;
            CK(cudaMemcpyAsync(s[idx].asg, bm->d.asg, N * 4, cudaMemcpyDeviceToDevice, st));
            if (s[2].empty) {
                *target = (int64_t)ceil((double)s[1].B * 1.5);
                if (*target == 0 || *target >= N) optimal = true;
                return &s[1];
            }
            if ((!s[0].empty && s[2].B - s[0].B <= 2) || (s[0].empty && s[2].B - s[1].B <= 1)) optimal = true;
            if (optimal) return &s[1];
            int index;
            if (s[0].empty && s[1].B < s[2].B) index = 1;
            else if ((s[1].B - s[0].B) <= (s[2].B - s[1].B)) index = 1;
            else index = 0;
            *target = s[index + 1].B + (int64_t)((double)(s[index].B - s[index + 1].B) * 0.618);
            return &s[index];
        };
        int64_t target = 0;
        int32_t step = 0;
        const Slot* src = next(&target);
        // end_condition_not_reached (top_down_sbp.cpp:428-433): with --mix, until the bracket forms
        while (mix ? s[2].empty : !optimal) {
            CK(cudaMemcpyAsync(bm->d.asg, src->asg, N * 4, cudaMemcpyDeviceToDevice, st));
            bm->d.B = (int32_t)src->B;
            bm->entropy = src->entropy;
            do_rebuild(bm);
            split_impl(bm, cfg, seed, (uint32_t)step, target);
            mcmc_impl(bm, cfg, seed, step, s[2].empty);
            ++step;
            g->st.outer_steps++;
            src = next(&target);
        }
        if (mix) {
            // continue_agglomerative (top_down_sbp.cpp:67-98): an agglomerative triplet fed the
            // three top-down blockmodels in slot order, then merges and finetuning until done;
            // the finetuning keeps the top-down triplet's (reached) golden-ratio state
            Slot gs[3];
            for (auto& sl : gs) sl.asg = dalloc<int32_t>(slots_mem, N);
            bool gopt = false;
            int64_t next_merge = 0;
            // BlockmodelTriplet::update and get_next_blockmodel (blockmodel_triplet.cpp:4-37, :82-105)
            auto agg_next = [&](int64_t B, double entropy, const int32_t* asg) -> const Slot* {
                int idx;
                if (gs[1].empty) {
                    idx = 1;
                } else if (entropy <= gs[1].entropy) {
                    const int old = (gs[1].B > B) ? 0 : 2;
                    std::swap(gs[old], gs[1]);
                    idx = 1;
                } else {
                    idx = (gs[1].B > B) ? 2 : 0;
                }
                gs[idx].empty = false;
                gs[idx].B = B;
                gs[idx].entropy = entropy;
                CK(cudaMemcpyAsync(gs[idx].asg, asg, N * 4, cudaMemcpyDeviceToDevice, st));
                if (gs[2].empty) {
                    next_merge = (int64_t)((double)gs[1].B * 0.5);
                    if (next_merge == 0) gopt = true;
                    return &gs[1];
                }
                if ((!gs[0].empty && gs[0].B - gs[2].B == 2) || (gs[0].empty && gs[1].B - gs[2].B == 1)) gopt = true;
                if (gopt) {
                    next_merge = 0;
                    return &gs[1];
                }
                int index;
                if (gs[0].empty && gs[1].B > gs[2].B) index = 1;
                else if ((gs[0].B - gs[1].B) >= (gs[1].B - gs[2].B)) index = 0;
                else index = 1;
                int64_t next_try = gs[index + 1].B;
                next_try += (int64_t)((double)(gs[index].B - gs[index + 1].B) * 0.618);
                next_merge = gs[index].B - next_try;
                return &gs[index];
            };
            const Slot* gsrc = nullptr;
            for (int k = 0; k < 3; ++k) gsrc = agg_next(s[k].B, s[k].entropy, s[k].asg);
            while (!gopt) {
                CK(cudaMemcpyAsync(bm->d.asg, gsrc->asg, N * 4, cudaMemcpyDeviceToDevice, st));
                bm->d.B = (int32_t)gsrc->B;
                bm->entropy = gsrc->entropy;
                do_rebuild(bm);
                merge_impl(bm, cfg, seed, step, next_merge);
                mcmc_impl(bm, cfg, seed, step, s[2].empty);
                ++step;
                g->st.outer_steps++;
                gsrc = agg_next(bm->d.B, bm->entropy, bm->d.asg);
            }
            src = gsrc;
        }
        if (out_assignment) CK(cudaMemcpyAsync(out_assignment, src->asg, N * 4, cudaMemcpyDeviceToHost, st));
        harvest_counters(g);
        if (num_blocks) *num_blocks = src->B;
        if (out_mdl) *out_mdl = src->entropy;
        g->st.kernel_launches = kernel_launches() - l0;
        if (stats) *stats = g->st;
        return SBPGPU_OK;
    });
    free_all(slots_mem, ctx->stream);
    if (bm) {
        free_all(bm->owned, bm->g->ctx->stream);
        delete bm;
    }
    return rc;
}

void sbpgpu_set_timing(sbpgpu_ctx* ctx, int32_t enabled) {
    if (ctx) ctx->timing = enabled != 0;
}

sbpgpu_status sbpgpu_read_timing(sbpgpu_ctx* ctx, sbpgpu_kernel_timing* out) {
    if (!ctx || !out) return SBPGPU_EINVAL;
    return guarded(ctx, [&] {
        ctx->collect();
        *out = ctx->tm;
        ctx->tm = sbpgpu_kernel_timing{};
        return SBPGPU_OK;
    });
}

}  // extern "C"

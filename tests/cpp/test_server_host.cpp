// The partition server's host logic (sbp_gb300/csrc/server.cu) without a GPU: server.cu is
// compiled as plain C++ against stand-ins for the library calls it makes, whose
// "partition" is a loop of short sleeps that honours the context's cancellation flag and
// whose graph upload can be made to fail as an allocation failure does.  Checked:
// admission by footprint (never more jobs in flight than the budget holds), refusal of a
// job that can never fit, pause and bounded waits, cancellation of a queued and of a
// running job, an injected allocation failure failing its job alone, and results routed
// to the right tickets.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "sbpgpu.h"

// ---- stand-ins for the library calls server.cu makes
struct sbpgpu_ctx {
    std::atomic<int32_t> cancel{0};
    int64_t fail_after = -1;
    std::string err;
};
struct sbpgpu_graph {
    sbpgpu_ctx* ctx;
    int64_t n;
};

static std::atomic<int> g_running{0}, g_max_running{0}, g_started{0};

extern "C" {
void sbpgpu_default_config(sbpgpu_config* cfg) { std::memset(cfg, 0, sizeof(*cfg)); }
sbpgpu_status sbpgpu_ctx_create(int32_t, sbpgpu_ctx** out) {
    *out = new sbpgpu_ctx();
    return SBPGPU_OK;
}
void sbpgpu_ctx_destroy(sbpgpu_ctx* ctx) { delete ctx; }
const char* sbpgpu_last_error(const sbpgpu_ctx* ctx) { return ctx->err.c_str(); }
sbpgpu_status sbpgpu_ctx_set_cells_budget(sbpgpu_ctx*, int64_t) { return SBPGPU_OK; }
sbpgpu_status sbpgpu_ctx_set_chain_cluster_blocks(sbpgpu_ctx*, int64_t) { return SBPGPU_OK; }
sbpgpu_status sbpgpu_ctx_set_cancel(sbpgpu_ctx* ctx, int32_t requested) {
    ctx->cancel.store(requested ? 1 : 0);
    return SBPGPU_OK;
}
sbpgpu_status sbpgpu_ctx_inject_alloc_failure(sbpgpu_ctx* ctx, int64_t after) {
    ctx->fail_after = after < 0 ? -1 : after;
    return SBPGPU_OK;
}
sbpgpu_status sbpgpu_graph_create(sbpgpu_ctx* ctx, int64_t n, int64_t, const int32_t*, const int32_t*,
                                  sbpgpu_graph** out) {
    if (ctx->fail_after == 0) {
        ctx->err = "device allocation failed (injected)";
        return SBPGPU_ENOMEM;
    }
    *out = new sbpgpu_graph{ctx, n};
    return SBPGPU_OK;
}
void sbpgpu_graph_destroy(sbpgpu_graph* g) { delete g; }
// A "partition" of n / 100 steps of 1 ms (2,000 steps for seed 99); the assignment is
// (v + seed) % 3, the block count 3 and the description length n, so each result names its
// job.
sbpgpu_status sbpgpu_sbp(sbpgpu_graph* g, const sbpgpu_config*, uint64_t seed, int32_t* out, int64_t* B,
                         double* mdl, sbpgpu_stats*) {
    const int now = ++g_running;
    int prev = g_max_running.load();
    while (now > prev && !g_max_running.compare_exchange_weak(prev, now)) {
    }
    ++g_started;
    sbpgpu_status st = SBPGPU_OK;
    const int64_t steps = seed == 99 ? 2000 : g->n / 100;
    for (int64_t s = 0; s < steps; ++s) {
        if (g->ctx->cancel.exchange(0)) {
            g->ctx->err = "partition cancelled";
            st = SBPGPU_ECANCELED;
            break;
        }
        std::this_thread::sleep_for(std::chrono::milliseconds(1));
    }
    if (st == SBPGPU_OK) {
        for (int64_t v = 0; v < g->n; ++v) out[v] = (int32_t)((v + (int64_t)seed) % 3);
        *B = 3;
        *mdl = (double)g->n;
    }
    --g_running;
    return st;
}
}

// ---- the checks
static int g_fail = 0;
#define EXPECT(c)                                                          \
    do {                                                                   \
        if (!(c)) {                                                        \
            ++g_fail;                                                      \
            std::fprintf(stderr, "%s:%d: expected %s\n", __FILE__, __LINE__, #c); \
        }                                                                  \
    } while (0)

struct Job {
    std::vector<int32_t> src, dst, out;
    sbpgpu_job job{};
    Job(int64_t n, uint64_t seed) : src{0}, dst{1}, out(n, -1) {
        job.num_vertices = n;
        job.num_edges = 1;
        job.src = src.data();
        job.dst = dst.data();
        sbpgpu_default_config(&job.config);
        job.seed = seed;
        job.out_assignment = out.data();
    }
};

int main() {
    const int64_t n = 2000;  // 20 ms a job
    const int64_t fp = sbpgpu_job_footprint(n, 1, 0);
    sbpgpu_server* s = nullptr;
    // a budget for two jobs at once, four workers
    EXPECT(sbpgpu_server_create(0, 4, 2 * fp + fp / 2, 0, &s) == SBPGPU_OK);

    // admission: eight jobs, never more than two in flight; results to the right tickets
    std::vector<Job*> jobs;
    std::vector<int64_t> t(8);
    for (int i = 0; i < 8; ++i) {
        jobs.push_back(new Job(n, (uint64_t)i));
        EXPECT(sbpgpu_server_submit(s, &jobs[i]->job, &t[i]) == SBPGPU_OK);
    }
    for (int i = 0; i < 8; ++i) {
        sbpgpu_job_result r;
        EXPECT(sbpgpu_server_wait(s, t[i], &r) == SBPGPU_OK);
        EXPECT(r.status == SBPGPU_OK && r.num_blocks == 3 && r.mdl == (double)n);
        EXPECT(jobs[i]->out[1] == (int32_t)((1 + i) % 3));
    }
    EXPECT(g_max_running.load() <= 2 && g_max_running.load() >= 1);

    // a job that can never fit is refused at submission
    Job huge(n * 1000, 0);
    int64_t th = 0;
    EXPECT(sbpgpu_server_submit(s, &huge.job, &th) == SBPGPU_ENOMEM);

    // pause: nothing starts, a bounded wait runs out and the ticket stays valid
    EXPECT(sbpgpu_server_pause(s, 1) == SBPGPU_OK);
    Job a(n, 11), b(n, 12), c(n, 13);
    int64_t ta = 0, tb = 0, tc = 0;
    EXPECT(sbpgpu_server_submit(s, &a.job, &ta) == SBPGPU_OK);
    EXPECT(sbpgpu_server_submit(s, &b.job, &tb) == SBPGPU_OK);
    EXPECT(sbpgpu_server_submit(s, &c.job, &tc) == SBPGPU_OK);
    sbpgpu_job_result r;
    EXPECT(sbpgpu_server_wait_for(s, ta, 30, &r) == SBPGPU_ETIMEOUT);
    // a queued job cancelled at once; an injected allocation failure fails its job alone
    EXPECT(sbpgpu_server_cancel(s, tb) == SBPGPU_OK);
    EXPECT(sbpgpu_server_wait_for(s, tb, 0, &r) == SBPGPU_OK && r.status == SBPGPU_ECANCELED);
    EXPECT(sbpgpu_server_inject_alloc_failure(s, tc, 0) == SBPGPU_OK);
    EXPECT(sbpgpu_server_pause(s, 0) == SBPGPU_OK);
    EXPECT(sbpgpu_server_wait(s, ta, &r) == SBPGPU_OK && r.status == SBPGPU_OK && a.out[1] == (1 + 11) % 3);
    EXPECT(sbpgpu_server_wait(s, tc, &r) == SBPGPU_OK && r.status == SBPGPU_ENOMEM);
    EXPECT(std::strstr(r.error, "injected") != nullptr);

    // a running job stops at its next step when cancelled
    Job longjob(n, 99);  // 2 s if left alone
    int64_t tl = 0;
    const int started0 = g_started.load();
    EXPECT(sbpgpu_server_submit(s, &longjob.job, &tl) == SBPGPU_OK);
    for (int i = 0; i < 2000 && g_started.load() == started0; ++i) std::this_thread::sleep_for(std::chrono::milliseconds(1));
    EXPECT(sbpgpu_server_inject_alloc_failure(s, tl, 0) == SBPGPU_EINVAL);  // too late: started
    EXPECT(sbpgpu_server_cancel(s, tl) == SBPGPU_OK);
    const auto t0 = std::chrono::steady_clock::now();
    EXPECT(sbpgpu_server_wait(s, tl, &r) == SBPGPU_OK && r.status == SBPGPU_ECANCELED);
    EXPECT(std::chrono::steady_clock::now() - t0 < std::chrono::milliseconds(1000));

    // and the server keeps serving; unknown tickets are refused
    Job after(n, 7);
    int64_t tn = 0;
    EXPECT(sbpgpu_server_submit(s, &after.job, &tn) == SBPGPU_OK);
    EXPECT(sbpgpu_server_wait(s, tn, &r) == SBPGPU_OK && r.status == SBPGPU_OK);
    EXPECT(sbpgpu_server_wait(s, tn, &r) == SBPGPU_EINVAL);
    EXPECT(sbpgpu_server_cancel(s, 999999) == SBPGPU_EINVAL);
    sbpgpu_server_destroy(s);
    for (Job* j : jobs) delete j;
    std::printf("%s\n", g_fail ? "FAILED" : "OK");
    return g_fail ? 1 : 0;
}

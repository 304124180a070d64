// Batched and served partitioning: many independent graphs partitioned at once on one GPU.
//
// A plain partition spends most of its time in the sequential phases (the hybrid MH chain
// and the merge carry-out), each a single CTA on one SM, so one graph at a time leaves most
// of the GPU's SMs idle.  A server runs several partitions concurrently: worker threads, each
// with its own context and stream, take jobs in submission order and run the same host
// loop as sbpgpu_sbp; their kernels share the device.  A job is admitted only while the
// estimated device footprint of the jobs in flight plus its own stays within the server's
// HBM budget (a job that could never fit is refused at submission), and its graph,
// blockmodels and work buffers stay on the device until it finishes.  A job can be
// cancelled: a queued one leaves the queue, a running one stops between golden-section
// steps through its worker context's cancellation flag.  Every job's result equals
// sbpgpu_sbp of the same graph, configuration and seed run alone: jobs share no device
// state, and the proposal stream depends only on the seed.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/sbpgpu.h"

namespace {

using Clock = std::chrono::steady_clock;

struct JobState {
    sbpgpu_job job{};
    sbpgpu_job_result result{};
    int64_t footprint = 0;
    Clock::time_point t_submit, t_start;
    bool started = false;
    bool done = false;
    sbpgpu_ctx* ctx = nullptr;  // the worker context while running
    int64_t inject_after = -1;  // injected allocation failure for the run
};

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

int64_t pow2_at_least(int64_t x) {
    int64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

}  // namespace

struct sbpgpu_server {
    int32_t device = 0;
    int64_t hbm_budget = 0;
    int64_t cells_budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> pending;
    std::unordered_map<int64_t, std::unique_ptr<JobState>> jobs;
    int64_t next_ticket = 1;
    int64_t inflight_bytes = 0;
    int32_t running = 0;
    bool stop = false;
    bool paused = false;  // workers start no new job
    std::vector<std::thread> threads;
    std::string err;
};

namespace {

bool admissible(const sbpgpu_server* s) {
    if (s->pending.empty() || (s->paused && !s->stop)) return false;
    const JobState* st = s->jobs.at(s->pending.front()).get();
    return s->inflight_bytes + st->footprint <= s->hbm_budget;
}

void finish(sbpgpu_server* s, JobState* st, sbpgpu_status status, const char* msg) {
    st->result.status = status;
    std::strncpy(st->result.error, msg, sizeof(st->result.error) - 1);
    st->done = true;
    s->cv_done.notify_all();
}

void run_job(sbpgpu_ctx* ctx, JobState* st) {
    const sbpgpu_job& j = st->job;
    sbpgpu_job_result& r = st->result;
    sbpgpu_graph* g = nullptr;
    r.status = sbpgpu_graph_create(ctx, j.num_vertices, j.num_edges, j.src, j.dst, &g);
    if (r.status == SBPGPU_OK) {
        r.status = sbpgpu_sbp(g, &j.config, j.seed, j.out_assignment, &r.num_blocks, &r.mdl, &r.stats);
        sbpgpu_graph_destroy(g);
    }
    if (r.status != SBPGPU_OK) std::strncpy(r.error, sbpgpu_last_error(ctx), sizeof(r.error) - 1);
}

void worker(sbpgpu_server* s) {
    sbpgpu_ctx* ctx = nullptr;
    const sbpgpu_status cs = sbpgpu_ctx_create(s->device, &ctx);
    if (cs == SBPGPU_OK) {
        sbpgpu_ctx_set_cells_budget(ctx, s->cells_budget);
        // many jobs share the device: their chains stay on one SM each below 65,536 blocks
        sbpgpu_ctx_set_chain_cluster_blocks(ctx, 65536);
    }
    while (true) {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_work.wait(lk, [&] { return admissible(s) || (s->stop && s->pending.empty()); });
        if (s->pending.empty()) break;  // stopping and drained
        const int64_t t = s->pending.front();
        s->pending.pop_front();
        JobState* st = s->jobs.at(t).get();
        s->inflight_bytes += st->footprint;
        s->running++;
        st->t_start = Clock::now();
        st->started = true;
        st->ctx = ctx;
        lk.unlock();
        if (cs == SBPGPU_OK) {
            sbpgpu_ctx_inject_alloc_failure(ctx, st->inject_after);
            run_job(ctx, st);
            sbpgpu_ctx_inject_alloc_failure(ctx, -1);
        } else {
            st->result.status = cs;
            std::strncpy(st->result.error, "cannot create a CUDA context for a worker", sizeof(st->result.error) - 1);
        }
        const auto t_end = Clock::now();
        lk.lock();
        // a cancellation that arrived after the job's last step must not reach the next job
        if (ctx) sbpgpu_ctx_set_cancel(ctx, 0);
        st->ctx = nullptr;
        s->inflight_bytes -= st->footprint;
        s->running--;
        st->result.queued_ms = ms_between(st->t_submit, st->t_start);
        st->result.run_ms = ms_between(st->t_start, t_end);
        st->done = true;
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
    if (ctx) sbpgpu_ctx_destroy(ctx);
}

}  // namespace

extern "C" {

int64_t sbpgpu_job_footprint(int64_t N, int64_t E, int64_t cells_budget_bytes) {
    if (N <= 0 || E < 0) return 0;
    const int64_t KE = std::max<int64_t>(E, 2 * N + 16);
    int64_t b = 0;
    b += 4 * (4 * E + 12 * N);                      // graph CSR, log table, vertex lists
    b += KE * (8 + 8 + 4 + 4 + 4) + 8 * KE + 4096;  // sort keys / values, flags, sort temporaries
    b += 4 * 16 * N;                                // per-vertex and per-block work arrays
    b += 16 * pow2_at_least(8 * E + 4096);          // chain cell hash
    b += 4 * (16 * N + 24 * E + 4096);              // chain list pool
    b += 16 * 4 * 8192 * 4;                         // windowed chain's high-degree hashes
    b += 4 * 4 * (8 * N + 7 * E);                   // up to four blockmodels (search triplet + current)
    b += std::max<int64_t>(cells_budget_bytes, 0);  // dense cells, when a blockmodel fits them
    return b;
}

sbpgpu_status sbpgpu_server_create(int32_t device, int32_t workers, int64_t hbm_budget_bytes,
                                   int64_t cells_budget_bytes, sbpgpu_server** out) {
    if (!out || workers < 1 || workers > 1024 || hbm_budget_bytes <= 0 || cells_budget_bytes < 0)
        return SBPGPU_EINVAL;
    *out = nullptr;
    auto* s = new sbpgpu_server();
    s->device = device;
    s->hbm_budget = hbm_budget_bytes;
    s->cells_budget = cells_budget_bytes;
    try {
        for (int32_t i = 0; i < workers; ++i) s->threads.emplace_back(worker, s);
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        for (auto& t : s->threads) t.join();
        delete s;
        return SBPGPU_ENOMEM;
    }
    *out = s;
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_server_submit(sbpgpu_server* s, const sbpgpu_job* job, int64_t* ticket) {
    if (!s || !job || !ticket || job->num_vertices <= 0 || job->num_edges < 0 ||
        (job->num_edges > 0 && (!job->src || !job->dst)) || !job->out_assignment)
        return SBPGPU_EINVAL;
    auto st = std::make_unique<JobState>();
    st->job = *job;
    st->footprint = sbpgpu_job_footprint(job->num_vertices, job->num_edges, s->cells_budget);
    if (job->config.nonparametric)  // lgamma table and the non-empty-count steps (int64)
        st->footprint += 8 * (std::max(job->num_vertices, job->num_edges) + 2) + 16 * (job->num_vertices + 2);
    if (st->footprint > s->hbm_budget) return SBPGPU_ENOMEM;  // could never be admitted
    st->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return SBPGPU_EINVAL;
        const int64_t t = s->next_ticket++;
        s->jobs.emplace(t, std::move(st));
        s->pending.push_back(t);
        *ticket = t;
    }
    s->cv_work.notify_all();
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_server_wait(sbpgpu_server* s, int64_t ticket, sbpgpu_job_result* result) {
    return sbpgpu_server_wait_for(s, ticket, -1, result);
}

sbpgpu_status sbpgpu_server_wait_for(sbpgpu_server* s, int64_t ticket, int64_t timeout_ms,
                                     sbpgpu_job_result* result) {
    if (!s || !result) return SBPGPU_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return SBPGPU_EINVAL;
    JobState* st = it->second.get();
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, [&] { return st->done; });
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return st->done; })) {
        return SBPGPU_ETIMEOUT;
    }
    *result = st->result;
    s->jobs.erase(it);
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_server_cancel(sbpgpu_server* s, int64_t ticket) {
    if (!s) return SBPGPU_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return SBPGPU_EINVAL;
    JobState* st = it->second.get();
    if (st->done) return SBPGPU_OK;
    if (!st->started) {
        s->pending.erase(std::find(s->pending.begin(), s->pending.end(), ticket));
        st->t_start = Clock::now();
        st->result.queued_ms = ms_between(st->t_submit, st->t_start);
        finish(s, st, SBPGPU_ECANCELED, "job cancelled before it started");
        s->cv_work.notify_all();  // the queue head may have changed
    } else if (st->ctx) {
        sbpgpu_ctx_set_cancel(st->ctx, 1);
    }
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_server_pause(sbpgpu_server* s, int32_t paused) {
    if (!s) return SBPGPU_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->paused = paused != 0;
    }
    s->cv_work.notify_all();
    return SBPGPU_OK;
}

sbpgpu_status sbpgpu_server_inject_alloc_failure(sbpgpu_server* s, int64_t ticket, int64_t after) {
    if (!s) return SBPGPU_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end() || it->second->started) return SBPGPU_EINVAL;
    it->second->inject_after = after;
    return SBPGPU_OK;
}

void sbpgpu_server_destroy(sbpgpu_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->threads) t.join();
    delete s;
}

sbpgpu_status sbpgpu_sbp_batch(int32_t device, int32_t workers, int64_t hbm_budget_bytes, int64_t cells_budget_bytes,
                               int64_t n, const sbpgpu_job* jobs, sbpgpu_job_result* results) {
    if (n < 0 || (n > 0 && (!jobs || !results))) return SBPGPU_EINVAL;
    sbpgpu_server* s = nullptr;
    sbpgpu_status rc = sbpgpu_server_create(device, workers, hbm_budget_bytes, cells_budget_bytes, &s);
    if (rc != SBPGPU_OK) return rc;
    std::vector<int64_t> tickets(n, 0);
    for (int64_t i = 0; i < n && rc == SBPGPU_OK; ++i) rc = sbpgpu_server_submit(s, &jobs[i], &tickets[i]);
    for (int64_t i = 0; i < n; ++i)
        if (tickets[i] > 0) sbpgpu_server_wait(s, tickets[i], &results[i]);
    sbpgpu_server_destroy(s);
    return rc;
}

}  // extern "C"

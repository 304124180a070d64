// Host-side helpers of graph upload.
//
// Stable compressed adjacency of a directed edge list, built on the host with several
// threads: the out-neighbour lists (with each edge's source, for the edge-ordered
// kernels) and the in-neighbour lists without self-loops, every list in input order as
// Graph::add_edge leaves it (reference src/graph.cpp:10-18), plus per-vertex self-loop and
// in-degree counts.  Plain C++ (no CUDA), so that it is tested on its own.
//
// The edges are cut into T contiguous chunks.  Each thread counts its chunk's edges per
// source and per destination; the counts are turned into per-chunk starting positions
// (vertex by vertex, chunks in order); then each thread scatters its chunk in order.  The
// lists come out exactly as one pass over the edges in order would write them.
#pragma once

#include <algorithm>
#include <atomic>
#include <new>
#include <cstdint>
#include <stdexcept>
#include <thread>
#include <vector>

namespace sbp {

struct HostCsr {
    std::vector<int32_t> out_off, out_nbr, esrc;  // out lists, the source of each entry
    std::vector<int32_t> inns_off, inns_nbr;      // in lists without self-loops
    std::vector<int32_t> selfcnt, indeg;          // self-loops; in-degree with self-loops
};

namespace host_csr_detail {

// Runs f(0) .. f(t - 1) on t threads; an exception in any of them is rethrown here as
// std::bad_alloc (the only one the bodies below can raise).
template <class F>
void run_threads(int t, F f) {
    if (t <= 1) {
        f(0);
        return;
    }
    std::atomic<bool> failed{false};
    std::vector<std::thread> ts;
    ts.reserve(t);
    for (int i = 0; i < t; ++i)
        ts.emplace_back([=, &f, &failed] {
            try {
                f(i);
            } catch (...) {
                failed = true;
            }
        });
    for (auto& x : ts) x.join();
    if (failed) throw std::bad_alloc();
}

}  // namespace host_csr_detail

// Throws std::invalid_argument for an endpoint outside [0, N).  threads <= 0: choose.
inline void build_host_csr(int64_t N, int64_t E, const int32_t* src, const int32_t* dst, HostCsr& c,
                           int threads = 0) {
    using host_csr_detail::run_threads;
    int T = threads > 0 ? threads : (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
    T = (int)std::max<int64_t>(1, std::min<int64_t>(T, E / (1 << 20) + 1));  // about 1M edges a thread at least
    while (T > 1 && (int64_t)T * N * 12 > ((int64_t)1 << 30)) --T;            // per-chunk counts within 1 GiB
    std::vector<std::vector<int32_t>> co(T), ci(T), cs(T);
    std::atomic<bool> bad{false};
    run_threads(T, [&](int t) {
        co[t].assign(N, 0);
        ci[t].assign(N, 0);
        cs[t].assign(N, 0);
        const int64_t lo = E * t / T, hi = E * (t + 1) / T;
        for (int64_t e = lo; e < hi; ++e) {
            const int32_t u = src[e], v = dst[e];
            if (u < 0 || u >= N || v < 0 || v >= N) {
                bad = true;
                return;
            }
            co[t][u]++;
            if (u == v) cs[t][u]++;
            else ci[t][v]++;
        }
    });
    if (bad) throw std::invalid_argument("edge endpoint out of range");
    c.out_off.assign(N + 1, 0);
    c.inns_off.assign(N + 1, 0);
    c.selfcnt.assign(N, 0);
    c.indeg.assign(N, 0);
    run_threads(T, [&](int t) {  // per-vertex totals over the chunks
        const int64_t lo = N * t / T, hi = N * (t + 1) / T;
        for (int64_t v = lo; v < hi; ++v) {
            int32_t o = 0, i = 0, s = 0;
            for (int q = 0; q < T; ++q) {
                o += co[q][v];
                i += ci[q][v];
                s += cs[q][v];
            }
            c.out_off[v + 1] = o;
            c.inns_off[v + 1] = i;
            c.selfcnt[v] = s;
            c.indeg[v] = i + s;
        }
    });
    for (int64_t v = 0; v < N; ++v) {
        c.out_off[v + 1] += c.out_off[v];
        c.inns_off[v + 1] += c.inns_off[v];
    }
    // per-chunk starting positions, chunks in order within each vertex's list
    run_threads(T, [&](int t) {
        const int64_t lo = N * t / T, hi = N * (t + 1) / T;
        for (int64_t v = lo; v < hi; ++v) {
            int32_t ro = c.out_off[v], ri = c.inns_off[v];
            for (int q = 0; q < T; ++q) {
                const int32_t a = co[q][v], b = ci[q][v];
                co[q][v] = ro;
                ci[q][v] = ri;
                ro += a;
                ri += b;
            }
        }
    });
    c.out_nbr.assign(E, 0);
    c.esrc.assign(E, 0);
    c.inns_nbr.assign(c.inns_off[N], 0);
    run_threads(T, [&](int t) {
        const int64_t lo = E * t / T, hi = E * (t + 1) / T;
        int32_t* po = co[t].data();
        int32_t* pi = ci[t].data();
        for (int64_t e = lo; e < hi; ++e) {
            const int32_t u = src[e], v = dst[e];
            const int32_t p = po[u]++;
            c.esrc[p] = u;
            c.out_nbr[p] = v;
            if (u != v) c.inns_nbr[pi[v]++] = u;
        }
    });
}

// The vertices in order of descending degree, ties by ascending id: what a stable sort of
// 0..N-1 by descending degree gives (Graph::sort_vertices, src/graph.cpp:235-268), by one
// counting pass over the degrees (a comparison sort when the degrees span far more values
// than there are vertices).
inline std::vector<int32_t> order_by_degree_desc(const std::vector<int32_t>& deg) {
    const int64_t N = (int64_t)deg.size();
    std::vector<int32_t> order(N);
    int32_t mx = 0;
    for (int32_t d : deg) mx = std::max(mx, d);
    if ((int64_t)mx > 16 * N + 1024) {
        for (int64_t v = 0; v < N; ++v) order[v] = (int32_t)v;
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return deg[a] > deg[b]; });
        return order;
    }
    std::vector<int64_t> start((size_t)mx + 2, 0);
    for (int32_t d : deg) start[d]++;
    int64_t run = 0;
    for (int64_t d = mx; d >= 0; --d) {  // higher degrees first
        const int64_t c = start[d];
        start[d] = run;
        run += c;
    }
    for (int64_t v = 0; v < N; ++v) order[start[deg[v]]++] = (int32_t)v;
    return order;
}

}  // namespace sbp

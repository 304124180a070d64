// The threaded host adjacency build (sbp_gb300/csrc/host_csr.h) against one sequential pass
// over the edges in order, on random graphs with self-loops, repeated edges and vertices
// without edges, at thread counts 1 to 16; and the counting-pass degree order against a
// stable sort.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "../../sbp_gb300/csrc/host_csr.h"

static int check(int64_t N, int64_t E, uint32_t seed, int threads) {
    std::mt19937 rng(seed);
    std::vector<int32_t> src(E), dst(E);
    for (int64_t e = 0; e < E; ++e) {
        src[e] = (int32_t)(rng() % (uint32_t)(N - N / 10));  // the last tenth has no out-edges
        dst[e] = rng() % 7 == 0 ? src[e] : (int32_t)(rng() % (uint32_t)N);
    }
    sbp::HostCsr c;
    sbp::build_host_csr(N, E, src.data(), dst.data(), c, threads);
    // the sequential reference
    std::vector<int32_t> oo(N + 1, 0), io(N + 1, 0), sc(N, 0), ind(N, 0);
    for (int64_t e = 0; e < E; ++e) {
        oo[src[e] + 1]++;
        ind[dst[e]]++;
        if (src[e] == dst[e]) sc[src[e]]++;
        else io[dst[e] + 1]++;
    }
    for (int64_t v = 0; v < N; ++v) {
        oo[v + 1] += oo[v];
        io[v + 1] += io[v];
    }
    std::vector<int32_t> on(E), es(E), in(io[N]);
    std::vector<int32_t> po(oo.begin(), oo.end() - 1), pi(io.begin(), io.end() - 1);
    for (int64_t e = 0; e < E; ++e) {
        es[po[src[e]]] = src[e];
        on[po[src[e]]++] = dst[e];
        if (src[e] != dst[e]) in[pi[dst[e]]++] = src[e];
    }
    const bool ok = c.out_off == oo && c.inns_off == io && c.selfcnt == sc && c.indeg == ind && c.out_nbr == on &&
                    c.esrc == es && c.inns_nbr == in;
    if (!ok) std::fprintf(stderr, "mismatch N=%lld E=%lld threads=%d\n", (long long)N, (long long)E, threads);
    return ok ? 0 : 1;
}

static int check_order(int64_t N, int32_t maxdeg, uint32_t seed) {
    std::mt19937 rng(seed);
    std::vector<int32_t> deg(N);
    for (auto& d : deg) d = (int32_t)(rng() % (uint32_t)(maxdeg + 1));
    std::vector<int32_t> want(N);
    for (int64_t v = 0; v < N; ++v) want[v] = (int32_t)v;
    std::stable_sort(want.begin(), want.end(), [&](int32_t a, int32_t b) { return deg[a] > deg[b]; });
    const bool ok = sbp::order_by_degree_desc(deg) == want;
    if (!ok) std::fprintf(stderr, "order mismatch N=%lld maxdeg=%d\n", (long long)N, maxdeg);
    return ok ? 0 : 1;
}

int main() {
    int bad = 0;
    for (auto nd : {std::pair<int64_t, int32_t>{0, 0}, {1, 0}, {1000, 3}, {1000, 5000}, {100000, 700},
                    {1000, 2000000000}})
        bad += check_order(nd.first, nd.second, 5u + (uint32_t)nd.first);
    for (int threads : {1, 2, 3, 7, 16, 0})
        for (auto ne : {std::pair<int64_t, int64_t>{50, 0}, {50, 400}, {1000, 20000}, {200000, 3000000}})
            bad += check(ne.first, ne.second, 11u + (uint32_t)threads, threads);
    bool threw = false;
    try {
        sbp::HostCsr c;
        const int32_t s[2] = {0, 9}, d[2] = {1, 2};
        sbp::build_host_csr(5, 2, s, d, c, 2);
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    bad += !threw;
    std::printf("%s\n", bad ? "FAILED" : "OK");
    return bad ? 1 : 0;
}

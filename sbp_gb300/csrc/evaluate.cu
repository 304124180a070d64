// Partition quality against a true partition (reference src/evaluate.cpp:9-180): the
// contingency table of (true community, found block) is counted on the device; NMI, the
// pair-counting F1 / precision / recall / Rand index and the matched accuracy follow on
// the host from the table, with the reference's formulas.
//
// The reference matches communities with a Hungarian solver from a dependency that is not
// part of its tree; only its printed accuracy depends on the matching (NMI and the pair
// counts are invariant under permuting columns).  Here the matching is a maximum-weight
// assignment computed with the shortest-augmenting-path Hungarian method with vertex
// potentials (Kuhn-Munkres, O(r^2 c) for r <= c).
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "kernels.cuh"

namespace sbp {

namespace {

__global__ void k_contingency(const int32_t* __restrict__ truth, const int32_t* __restrict__ found, int64_t n,
                              int32_t ncols, unsigned long long* __restrict__ table) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (truth[i] >= 0) atomicAdd(table + (int64_t)truth[i] * ncols + found[i], 1ull);
}

// Minimum-cost assignment of every row to a distinct column (rows <= cols); returns, per
// row, its column.
std::vector<int64_t> min_cost_assignment(const std::vector<std::vector<long long>>& cost, int64_t rows, int64_t cols) {
    const long long INF = LLONG_MAX / 4;
    std::vector<long long> u(rows + 1, 0), v(cols + 1, 0);
    std::vector<int64_t> match(cols + 1, 0), way(cols + 1, 0);  // match[j]: row (1-based) on column j
    for (int64_t i = 1; i <= rows; ++i) {
        match[0] = i;
        int64_t j0 = 0;
        std::vector<long long> minv(cols + 1, INF);
        std::vector<char> used(cols + 1, 0);
        do {
            used[j0] = 1;
            const int64_t i0 = match[j0];
            long long delta = INF;
            int64_t j1 = 0;
            for (int64_t j = 1; j <= cols; ++j) {
                if (used[j]) continue;
                const long long cur = cost[i0 - 1][j - 1] - u[i0] - v[j];
                if (cur < minv[j]) {
                    minv[j] = cur;
                    way[j] = j0;
                }
                if (minv[j] < delta) {
                    delta = minv[j];
                    j1 = j;
                }
            }
            for (int64_t j = 0; j <= cols; ++j) {
                if (used[j]) {
                    u[match[j]] += delta;
                    v[j] -= delta;
                } else {
                    minv[j] -= delta;
                }
            }
            j0 = j1;
        } while (match[j0] != 0);
        do {
            const int64_t j1 = way[j0];
            match[j0] = match[j1];
            j0 = j1;
        } while (j0);
    }
    std::vector<int64_t> col_of(rows, -1);
    for (int64_t j = 1; j <= cols; ++j)
        if (match[j]) col_of[match[j] - 1] = j - 1;
    return col_of;
}

}  // namespace

void launch_contingency(const int32_t* truth, const int32_t* found, int64_t n, int32_t ncols,
                        unsigned long long* table, cudaStream_t st) {
    if (n <= 0) return;
    int64_t blocks = (n + 255) / 256;
    if (blocks > (int64_t)device_sms() * 16) blocks = (int64_t)device_sms() * 16;
    k_contingency<<<(unsigned)blocks, 256, 0, st>>>(truth, found, n, ncols, table);
    count_launches(1);
}

PartitionQuality quality_from_table(const std::vector<unsigned long long>& t, int64_t nt, int64_t nb,
                                    int64_t num_vertices) {
    // orient as the reference reports it: rows = found blocks, columns = true communities
    std::vector<std::vector<long long>> m(nb, std::vector<long long>(nt, 0));
    for (int64_t i = 0; i < nt; ++i)
        for (int64_t j = 0; j < nb; ++j) m[j][i] = (long long)t[i * nb + j];
    PartitionQuality q = scores_from_matrix(m, num_vertices, true);
    q.true_blocks = nt;
    q.found_blocks = nb;
    return q;
}

PartitionQuality scores_from_matrix(const std::vector<std::vector<long long>>& m, int64_t num_vertices,
                                    bool with_accuracy) {
    const int64_t nrows = (int64_t)m.size(), ncols = nrows ? (int64_t)m[0].size() : 0;
    PartitionQuality q{};
    q.true_blocks = ncols;
    q.found_blocks = nrows;
    // F1 (calculate_f1_score, evaluate.cpp:9-61): pair counts from the table
    const double V = (double)num_vertices;
    const double num_pairs = (V * (V - 1.0)) / 2.0;
    std::vector<double> rowsums(nrows, 0.0), colsums(ncols, 0.0);
    double cell_pairs = 0, cells_squared = 0;
    for (int64_t r = 0; r < nrows; ++r)
        for (int64_t c = 0; c < ncols; ++c) {
            const double x = (double)m[r][c];
            rowsums[r] += x;
            colsums[c] += x;
            cell_pairs += x * (x - 1);
            cells_squared += x * x;
        }
    cell_pairs /= 2.0;
    double row_pairs = 0, col_pairs = 0, rs2 = 0, cs2 = 0;
    for (double s : rowsums) {
        row_pairs += s * (s - 1);
        rs2 += s * s;
    }
    for (double s : colsums) {
        col_pairs += s * (s - 1);
        cs2 += s * s;
    }
    row_pairs /= 2.0;
    col_pairs /= 2.0;
    const double agree_diff = (V * V + cells_squared - (rs2 + cs2)) / 2.0;
    q.rand_index = (cell_pairs + agree_diff) / num_pairs;
    q.recall = cell_pairs / row_pairs;
    q.precision = cell_pairs / col_pairs;
    q.f1 = (2.0 * q.precision * q.recall) / (q.precision + q.recall);
    // NMI (calculate_nmi, evaluate.cpp:63-98): marginal entropies with float logs
    // (utils::nat_log), mutual information with double logs, all over num_vertices
    std::vector<double> p1(nrows, 0.0), p2(ncols, 0.0);
    for (int64_t r = 0; r < nrows; ++r)
        for (int64_t c = 0; c < ncols; ++c) {
            const double p = (double)m[r][c] / V;
            p1[r] += p;
            p2[c] += p;
        }
    double h1 = 0, h2 = 0;
    for (double p : p1) h1 += p * (double)logf((float)p);
    for (double p : p2) h2 += p * (double)logf((float)p);
    h1 = -h1;
    h2 = -h2;
    double mi = 0.0;
    for (int64_t r = 0; r < nrows; ++r)
        for (int64_t c = 0; c < ncols; ++c) {
            const double p = (double)m[r][c] / V;
            if (p == 0.0) continue;
            mi += p * std::log(p / (p1[r] * p2[c]));
        }
    q.nmi = mi / std::sqrt(h1 * h2);
    if (!with_accuracy) return q;
    // accuracy: the best one-to-one matching of the smaller side into the larger
    const bool by_rows = nrows <= ncols;
    const int64_t a = by_rows ? nrows : ncols, b = by_rows ? ncols : nrows;
    long long maxv = 0;
    for (const auto& row : m)
        for (long long x : row) maxv = std::max(maxv, x);
    std::vector<std::vector<long long>> cost(a, std::vector<long long>(b, 0));
    for (int64_t i = 0; i < a; ++i)
        for (int64_t j = 0; j < b; ++j) cost[i][j] = maxv - (by_rows ? m[i][j] : m[j][i]);
    const std::vector<int64_t> col_of = min_cost_assignment(cost, a, b);
    double correct = 0;
    for (int64_t i = 0; i < a; ++i) correct += (double)(by_rows ? m[i][col_of[i]] : m[col_of[i]][i]);
    q.accuracy = correct / V;
    return q;
}

}  // namespace sbp

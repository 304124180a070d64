// Graph ingest on the device: a TSV edge list or a Matrix Market coordinate file parsed
// straight into the device edge arrays (reference Graph::load, load_text, parse_directed,
// parse_undirected, load_matrix_market: src/graph.cpp:33-233).
//
// The host reads the file and, for Matrix Market, its header (banner, comment lines and
// the size line); the bytes of the edge lines go to the device, where
//   1. every byte that starts a line is flagged and the flags are scanned into line offsets,
//   2. one thread per line parses "from to [weight]" (1-based ids, separated by tabs,
//      spaces or commas; blank lines and lines starting with '%' or '#' carry no edge) and
//      counts the edges it emits: 1, or 2 when the graph is undirected and from != to (the
//      reverse edge follows its edge, as the reference inserts it),
//   3. the counts are scanned into output positions and the edges written 0-based,
//   4. the largest id gives the vertex count (at least the Matrix Market size).
// The edge order therefore equals the reference's insertion order, so every vertex's out-
// and in-neighbour lists come out in the reference's order.
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "prims.cuh"

namespace sbp {

namespace {

__global__ void k_line_starts(const char* __restrict__ text, int64_t n, int32_t* __restrict__ flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = (i == 0 || text[i - 1] == '\n') ? 1 : 0;
}

__global__ void k_line_offsets(const int32_t* __restrict__ flag, const int32_t* __restrict__ pos, int64_t n,
                               int32_t* __restrict__ starts) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) starts[pos[i]] = (int32_t)i;
}

__device__ __forceinline__ bool is_sep(char c) { return c == ' ' || c == '\t' || c == ',' || c == '\r'; }

// Parses a non-negative decimal at text[*p], advancing *p; false when there is none.
__device__ __forceinline__ bool parse_id(const char* text, int64_t end, int64_t* p, long long* v) {
    int64_t i = *p;
    while (i < end && is_sep(text[i])) ++i;
    if (i >= end || text[i] < '0' || text[i] > '9') return false;
    long long x = 0;
    while (i < end && text[i] >= '0' && text[i] <= '9') {
        x = x * 10 + (text[i] - '0');
        if (x > (1ll << 40)) return false;
        ++i;
    }
    *p = i;
    *v = x;
    return true;
}

// Per line: the edge it holds (0-based) and how many edges it emits; flags bad lines.
__global__ void k_parse_lines(const char* __restrict__ text, int64_t n, const int32_t* __restrict__ starts,
                              int32_t lines, int undirected, int32_t* __restrict__ from, int32_t* __restrict__ to,
                              int32_t* __restrict__ emit, unsigned long long* __restrict__ max_id,
                              int32_t* __restrict__ bad) {
    for (int32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < lines; l += gridDim.x * blockDim.x) {
        const int64_t b = starts[l], e = l + 1 < lines ? starts[l + 1] : n;
        int64_t p = b;
        while (p < e && is_sep(text[p])) ++p;
        emit[l] = 0;
        if (p >= e || text[p] == '\n' || text[p] == '%' || text[p] == '#') continue;
        long long f = 0, t = 0;
        if (!parse_id(text, e, &p, &f) || !parse_id(text, e, &p, &t) || f < 1 || t < 1 || f > INT32_MAX / 2 ||
            t > INT32_MAX / 2) {
            atomicAdd(bad, 1);
            continue;
        }
        from[l] = (int32_t)(f - 1);
        to[l] = (int32_t)(t - 1);
        emit[l] = (undirected && f != t) ? 2 : 1;
        atomicMax(max_id, (unsigned long long)(f > t ? f : t));
    }
}

__global__ void k_emit_edges(const int32_t* __restrict__ from, const int32_t* __restrict__ to,
                             const int32_t* __restrict__ emit, const int32_t* __restrict__ pos, int32_t lines,
                             int32_t* __restrict__ src, int32_t* __restrict__ dst) {
    for (int32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < lines; l += gridDim.x * blockDim.x) {
        const int32_t k = emit[l];
        if (k == 0) continue;
        const int32_t o = pos[l];
        src[o] = from[l];
        dst[o] = to[l];
        if (k == 2) {  // the reverse edge right after its edge (parse_undirected, graph.cpp:207-215)
            src[o + 1] = to[l];
            dst[o + 1] = from[l];
        }
    }
}

unsigned grid_of(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > (int64_t)device_sms() * 16) b = (int64_t)device_sms() * 16;
    return (unsigned)b;
}

}  // namespace

bool parse_edges_device(const char* d_text, int64_t n, int undirected, int32_t** d_src, int32_t** d_dst, int64_t* E,
                        int64_t* max_id, std::string* err, cudaStream_t st) {
    *d_src = *d_dst = nullptr;
    if (n <= 0) {
        *E = 0;
        *max_id = 0;
        return true;
    }
    if (n >= (int64_t)INT32_MAX) {
        *err = "edge text above 2 GiB";
        return false;
    }
    int32_t *flag = nullptr, *pos = nullptr, *starts = nullptr, *from = nullptr, *to = nullptr, *emit = nullptr,
            *epos = nullptr, *scal = nullptr;
    unsigned long long* d_max = nullptr;
    void* temp = nullptr;
    bool ok = false;
    int32_t h[4] = {0, 0, 0, 0};
    unsigned long long hmax = 0;
    const size_t tb = scan_temp_bytes(n) + 1024;
    do {
        if (cudaMallocAsync(&flag, 4 * n, st) || cudaMallocAsync(&pos, 4 * n, st) || cudaMallocAsync(&temp, tb, st) ||
            cudaMallocAsync(&scal, 16, st) || cudaMallocAsync(&d_max, 8, st)) {
            *err = "device allocation failed";
            break;
        }
        cudaMemsetAsync(scal, 0, 16, st);
        cudaMemsetAsync(d_max, 0, 8, st);
        k_line_starts<<<grid_of(n), 256, 0, st>>>(d_text, n, flag);
        scan_i32(flag, pos, n, false, scal, temp, st);
        cudaMemcpyAsync(h, scal, 4, cudaMemcpyDeviceToHost, st);
        host_wait(st);
        const int32_t lines = h[0];
        if (cudaMallocAsync(&starts, 4 * (size_t)lines + 4, st) || cudaMallocAsync(&from, 4 * (size_t)lines + 4, st) ||
            cudaMallocAsync(&to, 4 * (size_t)lines + 4, st) || cudaMallocAsync(&emit, 4 * (size_t)lines + 4, st) ||
            cudaMallocAsync(&epos, 4 * (size_t)lines + 4, st)) {
            *err = "device allocation failed";
            break;
        }
        k_line_offsets<<<grid_of(n), 256, 0, st>>>(flag, pos, n, starts);
        k_parse_lines<<<grid_of(lines), 256, 0, st>>>(d_text, n, starts, lines, undirected, from, to, emit, d_max,
                                                      scal + 1);
        scan_i32(emit, epos, lines, false, scal + 2, temp, st);
        cudaMemcpyAsync(h, scal, 16, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&hmax, d_max, 8, cudaMemcpyDeviceToHost, st);
        host_wait(st);
        if (h[1] > 0) {
            *err = std::to_string(h[1]) + " edge lines could not be parsed";
            break;
        }
        *E = h[2];
        *max_id = (int64_t)hmax;
        if (cudaMallocAsync(d_src, 4 * (size_t)h[2] + 4, st) || cudaMallocAsync(d_dst, 4 * (size_t)h[2] + 4, st)) {
            *err = "device allocation failed";
            break;
        }
        k_emit_edges<<<grid_of(lines), 256, 0, st>>>(from, to, emit, epos, lines, *d_src, *d_dst);
        count_launches(6);
        ok = true;
    } while (0);
    for (void* p : {(void*)flag, (void*)pos, (void*)temp, (void*)scal, (void*)d_max, (void*)starts, (void*)from,
                    (void*)to, (void*)emit, (void*)epos})
        if (p) cudaFreeAsync(p, st);
    if (!ok) {
        if (*d_src) cudaFreeAsync(*d_src, st);
        if (*d_dst) cudaFreeAsync(*d_dst, st);
        *d_src = *d_dst = nullptr;
        cudaGetLastError();
    }
    return ok;
}

}  // namespace sbp

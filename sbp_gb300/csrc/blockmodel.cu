// Blockmodel construction (Blockmodel::initialize_edge_counts, reference
// src/blockmodel/blockmodel.cpp:193-276), MDL (entropy::mdl, src/entropy.cpp:597-604),
// batch delta-MDL / proposal kernels and chain-state initialisation.
//
// Rebuild: every edge (u -> v) becomes the key (asg[u] << nb | asg[v]); a stable LSD
// radix sort groups equal cells, a head-flag scan compacts them into the sorted CSR
// (row-major, ascending columns) and the same is done on (col << nb | row) for the CSC.
// Traffic per rebuild is O(E) and independent of how many vertices moved.
#include <mutex>
#include <unordered_map>
#include <unordered_set>

#include <stdexcept>

#include "kernels.cuh"
#include "delta.cuh"
#include "prims.cuh"

namespace sbp {

namespace {
thread_local int64_t g_launch_count = 0;  // per host thread: each thread drives its own context
constexpr int kT = 256;

inline unsigned grid_for(int64_t n, int per = kT) {
    int64_t b = (n + per - 1) / per;
    if (b < 1) b = 1;
    if (b > (int64_t)device_sms() * 64) b = (int64_t)device_sms() * 64;
    return (unsigned)b;
}

__global__ void k_edge_keys(DevGraph g, const int32_t* __restrict__ asg, int nb, uint64_t* __restrict__ keys) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.E; e += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)asg[__ldg(g.esrc + e)];
        const uint32_t b = (uint32_t)asg[__ldg(g.out_nbr + e)];
        keys[e] = ((uint64_t)a << nb) | b;
    }
}

__global__ void k_head_flags(const uint64_t* __restrict__ keys, int64_t n, int32_t* __restrict__ flags) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

// Compacts run heads: ukeys[pos] = key, ustart[pos] = i (flags hold exclusive positions
// after the scan; heads are recomputed from the keys).
__global__ void k_compact_heads(const uint64_t* __restrict__ keys, int64_t n, const int32_t* __restrict__ pos,
                                uint64_t* __restrict__ ukeys, int32_t* __restrict__ ustart) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i == 0 || keys[i] != keys[i - 1]) {
            ukeys[pos[i]] = keys[i];
            ustart[pos[i]] = (int32_t)i;
        }
    }
}

// From sorted unique keys (major << nb | minor) and run starts: minor index, count,
// major-of-entry and the offsets of every major id (empty majors included).
__global__ void k_fill_segments(const uint64_t* __restrict__ ukeys, const int32_t* __restrict__ ustart, int32_t nnz,
                                int32_t total, int nb, int32_t B, int32_t* __restrict__ off, int32_t* __restrict__ idx,
                                int32_t* __restrict__ cnt, int32_t* __restrict__ major_of) {
    const uint64_t mask = (1ull << nb) - 1ull;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = ukeys[j];
        const int32_t maj = (int32_t)(k >> nb);
        idx[j] = (int32_t)(k & mask);
        if (cnt) cnt[j] = (j + 1 < nnz ? ustart[j + 1] : total) - ustart[j];
        if (major_of) major_of[j] = maj;
        const int32_t prev = j == 0 ? -1 : (int32_t)(ukeys[j - 1] >> nb);
        for (int32_t b = prev + 1; b <= maj; ++b) off[b] = (int32_t)j;
        if (j == nnz - 1)
            for (int32_t b = maj + 1; b <= B; ++b) off[b] = nnz;
    }
}

__global__ void k_cnt_from_vals(const int32_t* __restrict__ vals_sorted, int32_t nnz, int32_t* __restrict__ cnt) {
    // CSC counts: the value carried through the sort is the cell count.
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        cnt[j] = vals_sorted[j];
}

__global__ void k_csc_keys(const int32_t* __restrict__ row_of, const int32_t* __restrict__ row_col, int32_t nnz,
                           int nb, uint64_t* __restrict__ keys, const int32_t* __restrict__ row_cnt,
                           int32_t* __restrict__ vals) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        keys[j] = ((uint64_t)(uint32_t)row_col[j] << nb) | (uint32_t)row_of[j];
        vals[j] = row_cnt[j];
    }
}

__global__ void k_degrees(DevBM bm, bool with_cells) {
    for (int32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < bm.B; b += gridDim.x * blockDim.x) {
        if (bm.sizes[b] > 0) atomicAdd(bm.nonempty, 1);  // blockmodel.cpp:194, :231
        if (!with_cells) continue;
        const int32_t dout = (int32_t)(cum_before(bm.row_cum, bm.row_off[b + 1]) - cum_before(bm.row_cum, bm.row_off[b]));
        const int32_t din = (int32_t)(cum_before(bm.col_cum, bm.col_off[b + 1]) - cum_before(bm.col_cum, bm.col_off[b]));
        const int32_t dg = csr_get(bm.row_off, bm.row_col, bm.row_cnt, b, b);
        bm.d_out[b] = dout;
        bm.d_in[b] = din;
        bm.diag[b] = dg;
        bm.d_tot[b] = dout + din - dg;
    }
}

__global__ void k_sizes(const int32_t* __restrict__ asg, int32_t N, int32_t* __restrict__ sizes) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x)
        atomicAdd(sizes + asg[v], 1);
}

__global__ void k_mdl(DevBM bm, unsigned long long* __restrict__ out) {
    long long acc = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < bm.nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = bm.row_cnt[j];
        const double ratio = (double)v / ((double)bm.d_out[bm.row_of[j]] * (double)bm.d_in[bm.row_col[j]]);
        const float lf = (float)log((double)(float)ratio);
        acc += (long long)v * (long long)((double)lf * 16777216.0);
    }
    acc = warp_sum_ll(acc);
    __shared__ long long ws[kT / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int i = 0; i < kT / 32; ++i) t += ws[i];
        atomicAdd(out, (unsigned long long)t);
    }
}

__global__ void k_np_mdl(DevGraph g, DevBM bm, unsigned long long* __restrict__ out) {
    long long acc = 0;
    const int64_t n = bm.nnz > bm.B ? bm.nnz : bm.B;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        if (j < bm.nnz)  // eterm_exact (entropy.hpp:103-113)
            acc += bm.row_of[j] == bm.row_col[j] ? -np_cell_diag(g, bm.row_cnt[j], -bm.row_cnt[j])
                                                 : -np_lg(g, bm.row_cnt[j]);
        if (j < bm.B) acc += np_vterm(g, bm.d_out[j], bm.d_in[j], bm.sizes[j]) - np_lg(g, bm.sizes[j]);
    }
    acc = warp_sum_ll(acc);
    __shared__ long long ws[kT / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int i = 0; i < kT / 32; ++i) t += ws[i];
        atomicAdd(out, (unsigned long long)t);
    }
}

template <bool kNP>
__global__ void k_vertex_dS_batch(DevGraph g, DevBM bm, const int32_t* __restrict__ vs, const int32_t* __restrict__ ss,
                                  int64_t n, int log2cap, long long* __restrict__ out, double* __restrict__ hout) {
    extern __shared__ int32_t sh[];
    __shared__ long long red[32][8];
    const int cap = 1 << log2cap;
    int32_t* hk = sh;
    int32_t* hO = sh + cap;
    int32_t* hI = sh + 2 * cap;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const int32_t v = vs[i], s = ss[i], r = bm.asg[v];
        long long d = 0;
        if (s != r)
            d = vertex_delta_fixed<kT, CsrAcc, kNP>(g, bm.asg, bm.d_out, bm.d_in, CsrAcc{bm}, v, r, s, hk, hO, hI,
                                                    log2cap, red, bm.sizes, kNP ? *bm.nonempty : 0);
        if (threadIdx.x == 0) out[i] = d;
        if (hout && !kNP) {  // entropy::hastings_correction over the neighbour hash just filled
            double H = 1.0;
            const int32_t o0 = __ldg(g.out_off + v), i0 = __ldg(g.inns_off + v);
            const int32_t kout = __ldg(g.out_off + v + 1) - o0, kin = __ldg(g.inns_off + v + 1) - i0;
            if (s != r && kout + kin > 0)
                H = hastings_fixed<kT>(CsrAcc{bm}, [&](int32_t b) { return bm.d_tot[b]; }, bm.d_out, bm.d_in, bm.B, r,
                                       s, kout, kin, __ldg(g.selfcnt + v), hk, hO, hI, log2cap, red);
            if (threadIdx.x == 0) hout[i] = H;
        }
        __syncthreads();
    }
}

template <bool kNP>
__global__ void k_merge_dS_batch(DevGraph g, DevBM bm, const int32_t* __restrict__ rs, const int32_t* __restrict__ ss,
                                 int64_t n, long long* __restrict__ out) {
    __shared__ long long red[32][8];
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const long long d = kNP ? np_merge_delta_csr<kT>(g, bm, rs[i], ss[i], *bm.nonempty, red)
                                : merge_delta_fixed_csr<kT>(g, bm, rs[i], ss[i], red);
        if (threadIdx.x == 0) out[i] = d;
        __syncthreads();
    }
}

__global__ void k_propose_batch(DevGraph g, DevBM bm, const int32_t* __restrict__ vs, int64_t n, uint64_t seed,
                                uint32_t c1, uint32_t c2, uint32_t c3, int32_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = vs[i];
        uint32_t w[4];
        philox4x32_10((uint32_t)v, c1, c2, c3, seed, w);
        out[i] = sample_vertex_proposal(g, bm, v, bm.asg[v], w);
    }
}

__global__ void k_chain_fill(DevBM bm, DevChain ch, DevFlags* flags) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < bm.nnz; j += (int64_t)gridDim.x * blockDim.x) {
        bool ins;
        const int32_t slot = chain_slot(ch, bm.row_of[j], bm.row_col[j], &ins, flags);
        if (slot >= 0) *slot_val(ch, slot) = bm.row_cnt[j];
    }
}

__global__ void k_fill_slots(ulonglong2* p, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = make_ulonglong2(kEmptyKey, 0ull);  // a key inserted later starts from zero
}

}  // namespace

int64_t kernel_launches() { return g_launch_count + prims_launch_count(); }
void count_launches(int64_t n) { g_launch_count += n; }

void host_wait(cudaStream_t st) {
    thread_local cudaEvent_t ev = nullptr;
    thread_local int ev_dev = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!ev || ev_dev != dev) {
        if (ev) cudaEventDestroy(ev);
        cudaEventCreateWithFlags(&ev, cudaEventBlockingSync | cudaEventDisableTiming);
        ev_dev = dev;
    }
    cudaEventRecord(ev, st);
    cudaEventSynchronize(ev);
}

void allow_max_dynamic_smem(const void* func) {
    static std::mutex mu;
    static std::unordered_set<const void*> done;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(func)) return;
    cudaFuncAttributes a;
    int dev = 0, optin = 0;
    if (cudaFuncGetAttributes(&a, func) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes);
    done.insert(func);
}

int device_sms() {
    static std::mutex mu;
    static std::unordered_map<int, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 1;
    }
    cache[dev] = n;
    return n;
}

void* host_scratch() {
    thread_local void* p = nullptr;
    if (!p && cudaMallocHost(&p, 256) != cudaSuccess) p = nullptr;
    return p;
}

int ceil_log2(uint64_t x) {
    int l = 0;
    while ((1ull << l) < x) ++l;
    return l;
}

void rebuild(const DevGraph& g, DevBM& bm, Work& w, cudaStream_t st) {
    const int nb = ceil_log2((uint64_t)(bm.B > 1 ? bm.B : 2));
    const int64_t E = g.E;
    cudaMemsetAsync(bm.sizes, 0, sizeof(int32_t) * bm.B, st);
    cudaMemsetAsync(bm.nonempty, 0, sizeof(int32_t), st);
    k_sizes<<<grid_for(g.N), kT, 0, st>>>(bm.asg, g.N, bm.sizes);
    count_launches(1);
    if (E == 0) {
        cudaMemsetAsync(bm.row_off, 0, sizeof(int32_t) * (bm.B + 1), st);
        cudaMemsetAsync(bm.col_off, 0, sizeof(int32_t) * (bm.B + 1), st);
        cudaMemsetAsync(bm.d_out, 0, sizeof(int32_t) * bm.B, st);
        cudaMemsetAsync(bm.d_in, 0, sizeof(int32_t) * bm.B, st);
        cudaMemsetAsync(bm.d_tot, 0, sizeof(int32_t) * bm.B, st);
        cudaMemsetAsync(bm.diag, 0, sizeof(int32_t) * bm.B, st);
        k_degrees<<<grid_for(bm.B), kT, 0, st>>>(bm, false);
        count_launches(1);
        bm.nnz = 0;
        return;
    }
    // rows
    k_edge_keys<<<grid_for(E), kT, 0, st>>>(g, bm.asg, nb, w.keys);
    radix_sort_u64(w.keys, w.keys_alt, nullptr, nullptr, E, 2 * nb, w.temp, st);
    k_head_flags<<<grid_for(E), kT, 0, st>>>(w.keys, E, w.flags);
    scan_i32(w.flags, w.flags, E, false, w.d_scalar, w.temp, st);
    int32_t* h_nnz = static_cast<int32_t*>(host_scratch());
    cudaMemcpyAsync(h_nnz, w.d_scalar, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    k_compact_heads<<<grid_for(E), kT, 0, st>>>(w.keys, E, w.flags, w.keys_alt, w.vals);
    host_wait(st);
    const int32_t nnz = *h_nnz;
    bm.nnz = nnz;
    k_fill_segments<<<grid_for(nnz), kT, 0, st>>>(w.keys_alt, w.vals, nnz, (int32_t)E, nb, bm.B, bm.row_off, bm.row_col,
                                                   bm.row_cnt, bm.row_of);
    scan_i32(bm.row_cnt, bm.row_cum, nnz, true, nullptr, w.temp, st);
    // columns
    k_csc_keys<<<grid_for(nnz), kT, 0, st>>>(bm.row_of, bm.row_col, nnz, nb, w.keys, bm.row_cnt, w.vals);
    radix_sort_u64(w.keys, w.keys_alt, w.vals, w.vals_alt, nnz, 2 * nb, w.temp, st);
    k_fill_segments<<<grid_for(nnz), kT, 0, st>>>(w.keys, nullptr, nnz, 0, nb, bm.B, bm.col_off, bm.col_row, nullptr,
                                                   nullptr);
    k_cnt_from_vals<<<grid_for(nnz), kT, 0, st>>>(w.vals, nnz, bm.col_cnt);
    scan_i32(bm.col_cnt, bm.col_cum, nnz, true, nullptr, w.temp, st);
    k_degrees<<<grid_for(bm.B), kT, 0, st>>>(bm, true);
    count_launches(8);
}

void launch_mdl(const DevGraph& g, const DevBM& bm, Work& w, cudaStream_t st) {
    cudaMemsetAsync(w.d_acc, 0, sizeof(unsigned long long), st);
    k_mdl<<<grid_for(bm.nnz), kT, 0, st>>>(bm, w.d_acc);
    count_launches(1);
}

void launch_np_mdl(const DevGraph& g, const DevBM& bm, Work& w, cudaStream_t st) {
    if (!g.LG || !g.Dm || !g.Dp) throw std::logic_error("nonparametric tables missing");
    cudaMemsetAsync(w.d_acc, 0, sizeof(unsigned long long), st);
    k_np_mdl<<<grid_for(bm.nnz > bm.B ? bm.nnz : bm.B), kT, 0, st>>>(g, bm, w.d_acc);
    count_launches(1);
}

void launch_vertex_dS_batch(const DevGraph& g, const DevBM& bm, const int32_t* v, const int32_t* s, int64_t n,
                            int32_t max_k, long long* out, Work& w, cudaStream_t st, bool np, double* hastings) {
    if (n <= 0) return;
    if (np && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    int log2cap = ceil_log2((uint64_t)(2 * (max_k > 16 ? max_k : 16)));
    const size_t smem = (size_t)3 * sizeof(int32_t) << log2cap;
    if (smem > 200 * 1024)
        throw std::invalid_argument("a vertex of degree " + std::to_string(max_k) +
                                    " needs more shared memory for its neighbour hash than a block has");
    if (np) {
        allow_max_dynamic_smem((const void*)k_vertex_dS_batch<true>);
        k_vertex_dS_batch<true><<<grid_for(n, 1), kT, smem, st>>>(g, bm, v, s, n, log2cap, out, nullptr);
    } else {
        allow_max_dynamic_smem((const void*)k_vertex_dS_batch<false>);
        k_vertex_dS_batch<false><<<grid_for(n, 1), kT, smem, st>>>(g, bm, v, s, n, log2cap, out, hastings);
    }
    count_launches(1);
}

void launch_merge_dS_batch(const DevGraph& g, const DevBM& bm, const int32_t* r, const int32_t* s, int64_t n,
                           long long* out, Work& w, cudaStream_t st, bool np) {
    if (n <= 0) return;
    if (np && (!g.LG || !g.Dm || !g.Dp)) throw std::logic_error("nonparametric tables missing");
    if (np) k_merge_dS_batch<true><<<grid_for(n, 1), kT, 0, st>>>(g, bm, r, s, n, out);
    else k_merge_dS_batch<false><<<grid_for(n, 1), kT, 0, st>>>(g, bm, r, s, n, out);
    count_launches(1);
}

void launch_propose_batch(const DevGraph& g, const DevBM& bm, const int32_t* v, int64_t n, uint64_t seed, uint32_t c1,
                          uint32_t c2, uint32_t c3, int32_t* out, cudaStream_t st) {
    if (n <= 0) return;
    k_propose_batch<<<grid_for(n), kT, 0, st>>>(g, bm, v, n, seed, c1, c2, c3, out);
    count_launches(1);
}

void lists_init(const DevBM& bm, Work& w, cudaStream_t st) {
    w.chain.slots = w.chain_slots;
    w.chain.n_keys = (uint32_t*)(w.d_scalar + 4);
    w.chain.row_head = w.row_head;
    w.chain.col_head = w.col_head;
    w.chain.pool = w.pool;
    w.chain.pool_words = w.pool_words;
    w.chain.pool_used = w.d_scalar + 5;
    cudaMemsetAsync(w.d_scalar + 4, 0, 2 * sizeof(int32_t), st);
    cudaMemsetAsync(w.row_head, 0xff, sizeof(int32_t) * bm.B, st);
    cudaMemsetAsync(w.col_head, 0xff, sizeof(int32_t) * bm.B, st);
}

void chain_init(const DevBM& bm, Work& w, uint64_t extra_keys, cudaStream_t st) {
    uint64_t need = (uint64_t)bm.nnz + extra_keys + 1024;
    uint64_t cap = 1ull << ceil_log2(need * 2);
    if (cap > w.chain_cap) cap = w.chain_cap;
    lists_init(bm, w, st);
    w.chain.mask = (uint32_t)(cap - 1);
    w.chain.load_limit = (uint32_t)(cap * 0.85);
    k_fill_slots<<<grid_for((int64_t)cap), kT, 0, st>>>(w.chain_slots, cap);
    k_chain_fill<<<grid_for(bm.nnz), kT, 0, st>>>(bm, w.chain, w.flags_dev);
    count_launches(2);
}

}  // namespace sbp

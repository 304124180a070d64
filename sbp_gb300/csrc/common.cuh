// Shared device definitions of the sbpgpu library (sm_103a).
//
// Data layout in HBM (all int32 unless noted; E < 2^31 so every count fits):
//   graph   : out CSR (out_off[N+1], out_nbr[E]), in CSR without self-loops
//             (inns_off[N+1], inns_nbr[E-L]), selfcnt[N], edge source esrc[E]
//             (the vertex owning each out-CSR slot), Lq[max(E,N)+2] = logf((float)x) * 2^24;
//             for the nonparametric entropy LG[max(E,N)+2] = lgamma(x+1) * 2^24 (int64) and
//             the non-empty-block-count steps Dm, Dp [N+2] (int64), built on first use.
//   blockmodel: asg[N]; d_out, d_in, d_tot, sizes, diag[B];
//             blockmatrix as sorted CSR (row_off[B+1], row_col/row_cnt/row_cum[nnz])
//             and sorted CSC (col_off[B+1], col_row/col_cnt/col_cum[nnz]); row_of[nnz].
//             *_cum are global inclusive prefix sums of the counts (a block's row is
//             a contiguous, ascending segment, so cumulative searches are binary searches).
//   chain state (sequential phases): open-addressing cell hash keyed (row << 32 | col)
//             plus per-row / per-column key lists (snapshot CSR segment + appended chunks).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define SBP_FULL_MASK 0xffffffffu

namespace sbp {

// Philox counter domains (word 3 of the counter) -- the canonical proposal stream.
enum : uint32_t {
    DOM_GIBBS = 1,
    DOM_MH = 2,
    DOM_MERGE = 3,
    DOM_SHUFFLE_HDV = 4,
    DOM_SHUFFLE_ALL = 5,
};

// Device error flags (OR-ed into DevFlags::err).
enum : int32_t {
    ERR_NONE = 0,
    ERR_DEGREE = 1,      // a vertex exceeds the supported neighbour count
    ERR_HASH_FULL = 2,   // chain cell hash exceeded its load limit
    ERR_POOL_FULL = 4,   // chain list pool exhausted
    ERR_STATE = 8,       // blockmodel consistency check failed
    ERR_SELECT = 16,     // cumulative search fell outside its segment
};

struct DevGraph {
    int32_t N;
    int32_t E;
    const int32_t* out_off;
    const int32_t* out_nbr;
    const int32_t* inns_off;
    const int32_t* inns_nbr;
    const int32_t* selfcnt;
    const int32_t* esrc;
    const int32_t* Lq;
    const long long* LG;  // nonparametric tables (null until first used)
    const long long* Dm;
    const long long* Dp;
    int32_t nlq;          // last index of Lq and LG
    // args.undirected for the nonparametric entropy: diagonal cells carry -w log 2 (ln2q =
    // log 2 in units of 2^-24, rounded), vertex terms count out-degrees only
    int32_t np_und;
    long long ln2q;
    // args.degreecorrected: vertex terms are lgamma of the block degrees, and the degree
    // prior's terms are added by degcorr.cu
    int32_t dc;
};

struct DevBM {
    int32_t B;
    int32_t nnz;
    int32_t* asg;
    int32_t* d_out;
    int32_t* d_in;
    int32_t* d_tot;
    int32_t* sizes;
    int32_t* diag;
    int32_t* row_off;
    int32_t* row_col;
    int32_t* row_cnt;
    int32_t* row_cum;
    int32_t* row_of;
    int32_t* col_off;
    int32_t* col_row;
    int32_t* col_cnt;
    int32_t* col_cum;
    int32_t* nonempty;  // device scalar: blocks with at least one vertex (recounted by rebuild)
};

// Mutable cell store used by the sequential phases (MH chain, merge carry-out): an
// open-addressing table of 16-byte slots (.x = key row << 32 | col, .y low word = count;
// one vector load per probe) and per-row / per-column key lists made of the snapshot
// CSR / CSC segment plus appended chunks [next, count, capacity, items...] in a pool.
struct DevChain {
    ulonglong2* slots;          // key EMPTY = ~0ull
    uint32_t mask;              // capacity - 1
    uint32_t load_limit;        // maximum number of keys
    uint32_t* n_keys;           // device counter
    int32_t* row_head;          // [B] newest appended chunk of row b or -1
    int32_t* col_head;          // [B]
    int32_t* pool;              // int32 words
    int64_t pool_words;
    int32_t* pool_used;         // device counter (words)
};

struct DevFlags {
    int32_t err;
    int32_t pad;
    // 0 carry-out rounds, 1 Gibbs accepted, 2 Gibbs applied, 3 Gibbs edges, 4 chain edges,
    // 5 chain moves, 6 merge proposals, 7 chain delta sum (2^-24 units), 8 chain rounds,
    // 9 carry-out keys walked, 10 carry-out evaluations
    unsigned long long counters[12];
};

constexpr unsigned long long kEmptyKey = ~0ull;

// How proposals are scored and accepted (finetune::accept, reference src/finetune.cpp:22-32):
// greedy (dS < 0); Metropolis-Hastings with the Hastings correction; or the nonparametric
// entropy, which the reference always runs non-greedy and without the correction
// (include/args.hpp:204-207, src/entropy.cpp:499).
enum : int { ACC_GREEDY = 0, ACC_HASTINGS = 1, ACC_NP = 2 };

// ------------------------------------------------------------------ Philox4x32-10
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint64_t seed, uint32_t w[4]) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    w[0] = c0;
    w[1] = c1;
    w[2] = c2;
    w[3] = c3;
}

__device__ __forceinline__ uint32_t u32_below(uint32_t w, uint32_t n) {
    return (uint32_t)(((uint64_t)w * n) >> 32);
}
__device__ __forceinline__ uint64_t u64_below(uint32_t hi, uint32_t lo, uint64_t n) {
    return __umul64hi(((uint64_t)hi << 32) | lo, n);
}
// common::propose_random_block (reference src/common.cpp:200-209).
__device__ __forceinline__ int32_t random_block(int32_t current, int32_t B, uint32_t w) {
    int32_t x = (int32_t)u32_below(w, (uint32_t)(B - 1));
    if (x >= current) x++;
    return x;
}

// ------------------------------------------------------------------ entropy terms
// fastlog table in units of 2^-24 with its last valid index; indices are clamped so
// an inconsistent state can never read outside the table.
struct LogTab {
    const int32_t* q;
    int32_t hi;
};
__device__ __forceinline__ long long Lx(const LogTab& t, long long x) {
    x = x < 0 ? 0 : (x > t.hi ? t.hi : x);
    return (long long)__ldg(t.q + x);
}
// The same table with its first sn entries also in shared memory (sq).
struct LogTabCached {
    const int32_t* q;
    int32_t hi;
    const int32_t* sq;
    int32_t sn;
};
__device__ __forceinline__ long long Lx(const LogTabCached& t, long long x) {
    x = x < 0 ? 0 : (x > t.hi ? t.hi : x);
    if (x < t.sn) return (long long)t.sq[x];
    return (long long)__ldg(t.q + x);
}
// common::cell_entropy (reference include/common.hpp:39-50) in units of 2^-24:
// v * (L[v] - L[d_in] - L[d_out]); zero for an empty cell; L[0] = 0 (fastlog(0)).
template <class Tab>
__device__ __forceinline__ long long ce_fixed(const Tab& L, long long v, long long din, long long dout) {
    if (v == 0) return 0;
    return v * (Lx(L, v) - Lx(L, din) - Lx(L, dout));
}
// Change of an unchanged cell's term when only degrees move: old - new.
template <class Tab>
__device__ __forceinline__ long long ce_delta(const Tab& L, long long v, long long din, long long dout,
                                              long long din2, long long dout2) {
    if (v == 0) return 0;
    return v * (Lx(L, din2) - Lx(L, din) + Lx(L, dout2) - Lx(L, dout));
}

__device__ __forceinline__ double fixed_to_double(long long q) { return (double)q * (1.0 / 16777216.0); }

// ------------------------------------------------------------------ warp helpers
__device__ __forceinline__ long long warp_sum_ll(long long x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(SBP_FULL_MASK, x, o);
    return x;
}
__device__ __forceinline__ int warp_sum_i(int x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(SBP_FULL_MASK, x, o);
    return x;
}
__device__ __forceinline__ int warp_max_i(int x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(SBP_FULL_MASK, x, o));
    return x;
}
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------------------------ CSR lookups
// Count of cell (row, col) via binary search in the row's ascending column segment.
__device__ __forceinline__ int32_t csr_get(const int32_t* __restrict__ off, const int32_t* __restrict__ idx,
                                           const int32_t* __restrict__ cnt, int32_t row, int32_t key) {
    int32_t lo = __ldg(off + row), hi = __ldg(off + row + 1);
    while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (__ldg(idx + mid) < key) lo = mid + 1;
        else hi = mid;
    }
    if (lo < __ldg(off + row + 1) && __ldg(idx + lo) == key) return __ldg(cnt + lo);
    return 0;
}
// Position of key in the segment or -1.
__device__ __forceinline__ int32_t csr_find(const int32_t* __restrict__ off, const int32_t* __restrict__ idx,
                                            int32_t row, int32_t key) {
    int32_t lo = __ldg(off + row), hi = __ldg(off + row + 1);
    const int32_t end = hi;
    while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (__ldg(idx + mid) < key) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && __ldg(idx + lo) == key) ? lo : -1;
}
// Inclusive prefix up to (excluding) position i of a global cumulative array.
__device__ __forceinline__ long long cum_before(const int32_t* __restrict__ cum, int32_t i) {
    return i > 0 ? (long long)__ldg(cum + i - 1) : 0ll;
}
// First position j in [lo, hi) with cum[j] > target (target < cum[hi-1]).
__device__ __forceinline__ int32_t cum_upper(const int32_t* __restrict__ cum, int32_t lo, int32_t hi,
                                             long long target) {
    while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if ((long long)__ldg(cum + mid) <= target) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Selects the entry at cumulative unit t of segment [lo, hi) of a (idx, cum) array,
// skipping up to two positions p1 < p2 (or -1) whose weights are w1, w2.
__device__ __forceinline__ int32_t seg_select(const int32_t* __restrict__ idx, const int32_t* __restrict__ cum,
                                              int32_t lo, int32_t hi, long long t, int32_t p1, long long w1,
                                              int32_t p2, long long w2) {
    const long long base = cum_before(cum, lo);
    long long u = t;
    if (p1 >= 0 && u >= cum_before(cum, p1) - base) u += w1;
    if (p2 >= 0 && u >= cum_before(cum, p2) - base) u += w2;
    const int32_t j = cum_upper(cum, lo, hi, base + u);
    return j < hi ? __ldg(idx + j) : -1;
}

// ------------------------------------------------------------------ chain cell hash
__device__ __forceinline__ unsigned long long cell_key(int32_t r, int32_t c) {
    return ((unsigned long long)(uint32_t)r << 32) | (uint32_t)c;
}
__device__ __forceinline__ uint32_t cell_slot(unsigned long long k, uint32_t mask) {
    return (uint32_t)((k * 0x9E3779B97F4A7C15ull) >> 32) & mask;
}
// A 32-bit load with acquire semantics at device scope.
__device__ __forceinline__ int32_t ld_acquire_gpu(const int32_t* p) {
    int32_t v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ ulonglong2 ld_slot(const ulonglong2* p) {
    ulonglong2 v;
    asm volatile("ld.volatile.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ int32_t* slot_val(const DevChain& ch, int32_t s) {
    return reinterpret_cast<int32_t*>(&ch.slots[s].y);
}
__device__ __forceinline__ int32_t chain_get(const DevChain& ch, int32_t r, int32_t c) {
    const unsigned long long k = cell_key(r, c);
    uint32_t s = cell_slot(k, ch.mask);
    for (uint32_t probe = 0; probe <= ch.mask; ++probe) {
        const ulonglong2 v = ld_slot(ch.slots + s);
        if (v.x == k) return (int32_t)(uint32_t)v.y;
        if (v.x == kEmptyKey) return 0;
        s = (s + 1) & ch.mask;
    }
    return 0;
}
// Finds or inserts the cell; returns its slot; *inserted tells whether the key is new.
__device__ __forceinline__ int32_t chain_slot(const DevChain& ch, int32_t r, int32_t c, bool* inserted,
                                              DevFlags* flags) {
    const unsigned long long k = cell_key(r, c);
    uint32_t s = cell_slot(k, ch.mask);
    *inserted = false;
    for (uint32_t probe = 0; probe <= ch.mask; ++probe) {
        const unsigned long long kk = ((volatile unsigned long long*)&ch.slots[s].x)[0];
        if (kk == k) return (int32_t)s;
        if (kk == kEmptyKey) {
            const unsigned long long prev = atomicCAS(&ch.slots[s].x, kEmptyKey, k);
            if (prev == kEmptyKey) {
                *inserted = true;
                const uint32_t n = atomicAdd(ch.n_keys, 1u);
                if (n >= ch.load_limit) atomicOr(&flags->err, ERR_HASH_FULL);
                return (int32_t)s;
            }
            if (prev == k) return (int32_t)s;
        }
        s = (s + 1) & ch.mask;
    }
    atomicOr(&flags->err, ERR_HASH_FULL);
    return -1;
}

}  // namespace sbp

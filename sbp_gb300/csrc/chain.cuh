// Single-CTA helpers for the sequential phases (the hybrid MH chain and the merge
// carry-out).  The current blockmatrix is held in a DevChain: an open-addressing cell
// hash (exact counts, zero counts kept as keys) plus per-row / per-column key lists made
// of the snapshot CSR / CSC segment and appended chunks.  A key appears in a list once.
#pragma once

#include "common.cuh"

namespace sbp {

constexpr int kChainThreads = 512;

// Appends item to list b (one thread per list at a time).
__device__ __forceinline__ void list_append(int32_t* head, const DevChain& ch, int32_t b, int32_t item,
                                            DevFlags* flags) {
    int32_t c = head[b];
    if (c < 0 || ch.pool[c * 32 + 1] >= kChunkItems) {
        const int32_t nc = atomicAdd(ch.pool_used, 1);
        if (nc >= ch.pool_cap) {
            atomicOr(&flags->err, ERR_POOL_FULL);
            return;
        }
        ch.pool[nc * 32] = c;
        ch.pool[nc * 32 + 1] = 0;
        head[b] = nc;
        c = nc;
    }
    const int32_t n = ch.pool[c * 32 + 1];
    ch.pool[c * 32 + 2 + n] = item;
    ch.pool[c * 32 + 1] = n + 1;
}

// Warp 0 appends new cells (rows[i], cols[i]) to the row and column lists.  Lanes that
// share a list are grouped and their leader appends the group's items in order.
__device__ __forceinline__ void append_new_keys(const DevChain& ch, const int32_t* rows, const int32_t* cols, int n,
                                                DevFlags* flags) {
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    for (int base = 0; base < n; base += 32) {
        const int j = base + lane;
        const bool valid = j < n;
        for (int pass = 0; pass < 2; ++pass) {
            const int32_t key = valid ? (pass == 0 ? rows[j] : cols[j]) : -1;
            const unsigned peers = __match_any_sync(SBP_FULL_MASK, key);
            if (valid && lane == __ffs(peers) - 1) {
                int32_t* head = pass == 0 ? ch.row_head : ch.col_head;
                unsigned m = peers;
                while (m) {
                    const int l = __ffs(m) - 1;
                    m &= m - 1;
                    const int jj = base + l;
                    list_append(head, ch, key, pass == 0 ? cols[jj] : rows[jj], flags);
                }
            }
            __syncwarp();
        }
    }
}

// Adds d to cell (r, c); new keys are recorded for list appends.
__device__ __forceinline__ void chain_add(const DevChain& ch, int32_t r, int32_t c, int32_t d, int32_t* new_rows,
                                          int32_t* new_cols, int* new_n, int new_cap, DevFlags* flags) {
    if (d == 0) return;
    bool ins;
    const int32_t slot = chain_slot(ch, r, c, &ins, flags);
    if (slot < 0) return;
    atomicAdd(ch.vals + slot, d);
    if (ins) {
        const int p = atomicAdd(new_n, 1);
        if (p < new_cap) {
            new_rows[p] = r;
            new_cols[p] = c;
        } else {
            atomicOr(&flags->err, ERR_POOL_FULL);
        }
    }
}

// Calls f(key) for every key of row (is_row) or column b: snapshot segment
// [lo, hi) of seg_idx and the appended chunks.  Thread-strided; every thread returns.
template <typename F>
__device__ __forceinline__ void chain_for_each(const int32_t* seg_idx, int32_t lo, int32_t hi, int32_t head,
                                               const DevChain& ch, F f) {
    for (int32_t j = lo + threadIdx.x; j < hi; j += blockDim.x) f(seg_idx[j]);
    int32_t c = head;
    int guard = 0;
    while (c >= 0 && guard < (1 << 26)) {
        const int32_t n = ((volatile int32_t*)ch.pool)[c * 32 + 1];
        for (int i = threadIdx.x; i < n; i += blockDim.x) f(((volatile int32_t*)ch.pool)[c * 32 + 2 + i]);
        c = ((volatile int32_t*)ch.pool)[c * 32];
        ++guard;
    }
}

// CTA exclusive scan of 1024 ints in shared memory (blockDim.x == 512); finds the
// bucket d with ex[d] <= t < ex[d] + h[d].  Returns d and reduces *t by ex[d].
__device__ __forceinline__ int cta_find_bucket(int32_t* h, long long* t, int* s_bucket, long long* s_t) {
    __shared__ int32_t wsum[16];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int a = h[2 * tid], b = h[2 * tid + 1];
    int x = a + b, incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    int off = 0;
    for (int i = 0; i < w; ++i) off += wsum[i];
    const long long ex0 = (long long)off + incl - x;
    const long long ex1 = ex0 + a;
    const long long tt = *t;
    if (a > 0 && tt >= ex0 && tt < ex0 + a) {
        *s_bucket = 2 * tid;
        *s_t = tt - ex0;
    }
    if (b > 0 && tt >= ex1 && tt < ex1 + b) {
        *s_bucket = 2 * tid + 1;
        *s_t = tt - ex1;
    }
    __syncthreads();
    *t = *s_t;
    const int d = *s_bucket;
    __syncthreads();
    return d;
}

// Key at cumulative unit t, in ascending key order, over (keys[i], vals[i]) i < n,
// ignoring keys skip1 / skip2.  nbits = bits of the key range.  -1 if t is out of range.
__device__ __forceinline__ int32_t cta_radix_select(const int32_t* keys, const int32_t* vals, int n, long long t,
                                                    int nbits, int32_t skip1, int32_t skip2, int32_t* hist,
                                                    int* s_bucket, long long* s_t) {
    const int levels = nbits <= 10 ? 1 : (nbits <= 20 ? 2 : 3);
    int32_t prefix = 0;
    if (threadIdx.x == 0) {
        *s_bucket = -1;
        *s_t = 0;
    }
    for (int lv = levels - 1; lv >= 0; --lv) {
        const int shift = 10 * lv;
        for (int i = threadIdx.x; i < 1024; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int32_t k = keys[i];
            if (k == skip1 || k == skip2) continue;
            if (lv < levels - 1 && (k >> (shift + 10)) != prefix) continue;
            atomicAdd(hist + ((k >> shift) & 1023), vals[i]);
        }
        __syncthreads();
        const int d = cta_find_bucket(hist, &t, s_bucket, s_t);
        if (d < 0) return -1;
        prefix = (prefix << 10) | d;
        if (threadIdx.x == 0) *s_bucket = -1;
        __syncthreads();
    }
    return prefix;
}

}  // namespace sbp

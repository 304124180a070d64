// Single-CTA helpers for the sequential phases (the hybrid MH chain and the merge
// carry-out).  The current blockmatrix is held in a DevChain: an open-addressing cell
// table (exact counts; a cell that drops to zero keeps its key) plus per-row /
// per-column key lists made of the snapshot CSR / CSC segment and appended chunks.  A
// key appears in a list once.
//
// A list that receives keys from many threads of one move or merge (row / column of the
// target block) is appended in bulk -- keys are staged, one thread reserves room for all
// of them, every thread copies.  Any other list receives keys from a single owning thread
// (list_push1) or, when several merges are applied together, through list_push1_shared.
// Lists are never read while they are appended to.
#pragma once

#include "common.cuh"

namespace sbp {

constexpr int kChainThreads = 512;

// Reserves g item slots at the head of list b; returns the pool word index of the first
// slot or -1 when the pool is full.  One thread per list at a time.
__device__ __forceinline__ int32_t list_reserve(int32_t* head, const DevChain& ch, int32_t b, int32_t g,
                                                DevFlags* flags) {
    const int32_t c = head[b];
    if (c >= 0) {
        const int32_t cnt = ch.pool[c + 1], cap = ch.pool[c + 2];
        if (cnt + g <= cap) {
            ch.pool[c + 1] = cnt + g;
            return c + 3 + cnt;
        }
    }
    int32_t cap = c >= 0 ? min(2 * ch.pool[c + 2], 1 << 16) : 13;
    if (cap < g) cap = g;
    const int32_t words = 3 + cap;
    const int32_t nc = atomicAdd(ch.pool_used, words);
    if ((int64_t)nc + words > ch.pool_words) {
        atomicOr(&flags->err, ERR_POOL_FULL);
        return -1;
    }
    ch.pool[nc] = c;
    ch.pool[nc + 1] = g;
    ch.pool[nc + 2] = cap;
    head[b] = nc;
    return nc + 3;
}

__device__ __forceinline__ void list_push1(int32_t* head, const DevChain& ch, int32_t b, int32_t item,
                                           DevFlags* flags) {
    const int32_t p = list_reserve(head, ch, b, 1, flags);
    if (p >= 0) ch.pool[p] = item;
}

// Appends one item to list b when other threads may append to the same list at the same
// time: a slot of the head chunk is claimed with an atomic increment of its count (a count
// past the capacity means the chunk is full; readers clamp it), and a full or missing head
// is replaced by a new chunk published with a compare-and-swap.  A chunk whose publication
// loses the race is left unused.  No thread may read the list concurrently.  The appending
// threads may sit in different CTAs of a cluster: a new chunk's header is published with a
// device-scope fence before the swap, and the head is read with acquire semantics, so a
// thread that finds the chunk also sees its count and capacity.
__device__ __forceinline__ void list_push1_shared(int32_t* head, const DevChain& ch, int32_t b, int32_t item,
                                                  DevFlags* flags) {
    volatile int32_t* vpool = ch.pool;
    for (int tries = 0; tries < 64; ++tries) {
        const int32_t c = ld_acquire_gpu(head + b);
        if (c >= 0) {
            const int32_t pos = atomicAdd(ch.pool + c + 1, 1);
            if (pos < vpool[c + 2]) {
                ch.pool[c + 3 + pos] = item;
                return;
            }
        }
        const int32_t cap = c >= 0 ? min(2 * vpool[c + 2], 1 << 16) : 13;
        const int32_t nc = atomicAdd(ch.pool_used, 3 + cap);
        if ((int64_t)nc + 3 + cap > ch.pool_words) {
            atomicOr(&flags->err, ERR_POOL_FULL);
            return;
        }
        ch.pool[nc] = c;
        ch.pool[nc + 1] = 1;
        ch.pool[nc + 2] = cap;
        ch.pool[nc + 3] = item;
        __threadfence();
        if (atomicCAS(head + b, c, nc) == c) return;
    }
    atomicOr(&flags->err, ERR_STATE);
}

// Adds d to cell (r, c); returns true when the key was inserted by this call.
__device__ __forceinline__ bool chain_add(const DevChain& ch, int32_t r, int32_t c, int32_t d, DevFlags* flags) {
    if (d == 0) return false;
    bool ins;
    const int32_t slot = chain_slot(ch, r, c, &ins, flags);
    if (slot < 0) return false;
    atomicAdd(slot_val(ch, slot), d);
    return ins;
}

// Stages one item of a bulk-appended list (shared or global staging buffer).
__device__ __forceinline__ void stage(int32_t* buf, int* count, int cap, int32_t item, DevFlags* flags) {
    const int p = atomicAdd(count, 1);
    if (p < cap) buf[p] = item;
    else atomicOr(&flags->err, ERR_POOL_FULL);
}

// Thread `leader` reserves room for n staged items in list b (result in *slot); after a
// barrier every thread copies.  Must be called by the whole CTA.
__device__ __forceinline__ void bulk_append(int32_t* head, const DevChain& ch, int32_t b, const int32_t* buf, int n,
                                            int leader, int32_t* slot, DevFlags* flags) {
    if (threadIdx.x == leader) *slot = n > 0 ? list_reserve(head, ch, b, n, flags) : -1;
    __syncthreads();
    const int32_t p = *slot;
    if (p >= 0)
        for (int i = threadIdx.x; i < n; i += blockDim.x) ch.pool[p + i] = buf[i];
}

// Number of keys in the appended chunks of a list starting at head (chunk headers only).
__device__ __forceinline__ int32_t list_chunk_keys(int32_t head, const DevChain& ch) {
    int32_t n = 0, c = head;
    int guard = 0;
    while (c >= 0 && guard++ < (1 << 20)) {
        n += min(((volatile int32_t*)ch.pool)[c + 1], ((volatile int32_t*)ch.pool)[c + 2]);
        c = ((volatile int32_t*)ch.pool)[c];
    }
    return n;
}

// Calls f(key) for every key held in the appended chunks of a list starting at head,
// strided over threads t = 0..nt-1 of a team.
template <typename F>
__device__ __forceinline__ void chunks_for_each(int32_t head, const DevChain& ch, int t, int nt, F f) {
    int32_t c = head;
    int guard = 0;
    while (c >= 0 && guard < (1 << 26)) {
        const int32_t n = min(((volatile int32_t*)ch.pool)[c + 1], ((volatile int32_t*)ch.pool)[c + 2]);
        for (int i = t; i < n; i += nt) f(((volatile int32_t*)ch.pool)[c + 3 + i]);
        c = ((volatile int32_t*)ch.pool)[c];
        ++guard;
    }
}

// Calls f(key) for every key of a row (or column): snapshot segment [lo, hi) of seg_idx
// and the appended chunks starting at head, strided over threads t = 0..nt-1.
template <typename F>
__device__ __forceinline__ void list_for_each(const int32_t* seg_idx, int32_t lo, int32_t hi, int32_t head,
                                              const DevChain& ch, int t, int nt, F f) {
    for (int32_t j = lo + t; j < hi; j += nt) f(seg_idx[j]);
    chunks_for_each(head, ch, t, nt, f);
}

// The same over all threads of the CTA.
template <typename F>
__device__ __forceinline__ void chain_for_each(const int32_t* seg_idx, int32_t lo, int32_t hi, int32_t head,
                                               const DevChain& ch, F f) {
    list_for_each(seg_idx, lo, hi, head, ch, threadIdx.x, blockDim.x, f);
}

// Block-wide sum of N int64 values (blockDim.x == kChainThreads); every thread gets the totals.
template <int N>
__device__ __forceinline__ void cta_sum(long long v[N], long long (*red)[8]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = warp_sum_ll(v[j]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < N; ++j) red[w][j] = v[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < N; ++j) {
        long long t = 0;
        for (int i = 0; i < kChainThreads / 32; ++i) t += red[i][j];
        v[j] = t;
    }
    __syncthreads();
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

// Sequential Metropolis-Hastings chain of hybrid MCMC (reference src/finetune.cpp:589-594,
// propose_move :842-869, move_vertex :822-840) for blockmodels with few blocks.
//
// For B <= kDenseMax the whole blockmatrix (B x B counts), the block degrees and sizes
// fit in one CTA's shared memory; for B <= kDenseGlobalMax the matrix and its transpose
// are dense arrays in global memory (rows and columns are then both contiguous) and the
// degrees, sizes and per-vertex counts stay in shared memory.  One CTA walks the
// high-degree vertices in order; per vertex it gathers the neighbours' blocks once, then
// the proposal (ascending-id multinomial over nb's row then column), the delta-MDL and
// the apply use O(1) cell accesses.  Only the assignment is written back: the caller
// rebuilds the blockmatrix from it afterwards.  Semantics and the proposal stream are
// identical to the hash-based chain used for larger B.
#include "delta.cuh"
#include "kernels.cuh"

namespace sbp {

namespace {

constexpr int kT = 512;

// Block-wide sum of five int64 values; every thread receives the totals.
__device__ __forceinline__ void block_sum5(long long v[5], long long (*red)[5]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 5; ++j) v[j] = warp_sum_ll(v[j]);
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < 5; ++j) red[w][j] = v[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        long long t = 0;
        for (int i = 0; i < kT / 32; ++i) t += red[i][j];
        v[j] = t;
    }
    __syncthreads();
}

// kGlobal: M (row-major) and MT (its transpose) in global memory; otherwise M in shared.
template <bool kGlobal>
__global__ void __launch_bounds__(kT, 1) k_mh_chain_dense(DevGraph g, DevBM bm, const int32_t* __restrict__ order,
                                                          int32_t n, uint64_t seed, uint32_t iter, uint32_t step,
                                                          int32_t* gM, int32_t* gMT, DevFlags* flags) {
    extern __shared__ int32_t sm[];
    const int32_t B = bm.B;
    int32_t* M = kGlobal ? gM : sm;  // B * B
    int32_t* dout = kGlobal ? sm : M + B * B;  // B
    int32_t* din = dout + B;         // B
    int32_t* size = din + B;         // B
    int32_t* O = size + B;           // B
    int32_t* I = O + B;              // B
    __shared__ long long wsum64[kT / 32];
    __shared__ long long red[kT / 32][5];
    __shared__ int32_t s_v, s_r, s_go, s_nb, s_s;
    const int tid = threadIdx.x;
    const LogTab Lq{g.Lq, g.E + 1};

    if (!kGlobal) {  // the global matrices are filled by k_dense_fill before the launch
        for (int i = tid; i < B * B; i += kT) M[i] = 0;
        __syncthreads();
        for (int32_t j = tid; j < bm.nnz; j += kT) M[bm.row_of[j] * B + bm.row_col[j]] = bm.row_cnt[j];
    }
    for (int b = tid; b < B; b += kT) {
        dout[b] = bm.d_out[b];
        din[b] = bm.d_in[b];
        size[b] = bm.sizes[b];
    }
    __syncthreads();

    unsigned long long edges = 0, moved = 0;
    long long dsum = 0;
    for (int32_t it = 0; it < n; ++it) {
        if (tid == 0) {
            const int32_t v = order[it];
            const int32_t r = bm.asg[v];
            s_v = v;
            s_r = r;
            s_go = size[r] == 1 ? 0 : 1;  // a singleton block never moves (finetune.cpp:845)
            s_nb = -1;
        }
        for (int b = tid; b < B; b += kT) {
            O[b] = 0;
            I[b] = 0;
        }
        __syncthreads();
        const int32_t v = s_v, r = s_r;
        const int32_t o0 = __ldg(g.out_off + v), o1 = __ldg(g.out_off + v + 1);
        const int32_t i0 = __ldg(g.inns_off + v), i1 = __ldg(g.inns_off + v + 1);
        const int32_t kout = o1 - o0, kin = i1 - i0, k = kout + kin;
        edges += k;
        do {  // every exit is uniform across the CTA; one barrier closes each iteration
        if (!s_go) break;
        uint32_t w[4];
        philox4x32_10((uint32_t)v, iter, step, DOM_MH, seed, w);
        const int32_t idx = k > 0 ? (int32_t)u32_below(w[0], (uint32_t)k) : -1;
        for (int32_t j = tid; j < kout; j += kT) {
            const int32_t u = __ldg(g.out_nbr + o0 + j);
            const int32_t b = bm.asg[u];
            if (j == idx) s_nb = b;
            if (u != v) atomicAdd(O + b, 1);
        }
        for (int32_t j = tid; j < kin; j += kT) {
            const int32_t b = bm.asg[__ldg(g.inns_nbr + i0 + j)];
            if (kout + j == idx) s_nb = b;
            atomicAdd(I + b, 1);
        }
        __syncthreads();
        int32_t s;
        if (k == 0) {
            s = random_block(r, B, w[1]);
        } else {
            // multinomial over nb's row (ascending column) then column without the diagonal
            const int32_t nb = s_nb;
            const long long R = dout[nb];
            const long long C = (long long)din[nb] - M[(int64_t)nb * B + nb];
            long long t = (long long)u64_below(w[1], w[2], (uint64_t)(R + C));
            const bool in_row = t < R;
            if (!in_row) t -= R;
            // ascending-id prefix search: thread tid owns blocks [tid*per, tid*per + per)
            const int lane = tid & 31, wid = tid >> 5;
            const int per = (B + kT - 1) / kT;
            const int32_t b0 = tid * per;
            const int32_t* rowp = kGlobal ? (in_row ? gM + (int64_t)nb * B : gMT + (int64_t)nb * B)
                                          : nullptr;
            long long local = 0;
            for (int q = 0; q < per; ++q) {
                const int32_t b = b0 + q;
                if (b >= B) break;
                int32_t x;
                if (kGlobal) x = (!in_row && b == nb) ? 0 : rowp[b];
                else x = in_row ? M[nb * B + b] : (b == nb ? 0 : M[b * B + nb]);
                local += x;
            }
            long long incl = local;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(SBP_FULL_MASK, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) wsum64[wid] = incl;
            if (tid == 0) s_s = -1;
            __syncthreads();
            long long off = 0;
            for (int q = 0; q < wid; ++q) off += wsum64[q];
            long long run = off + incl - local;
            if (local > 0 && t >= run && t < run + local) {
                for (int q = 0; q < per; ++q) {
                    const int32_t b = b0 + q;
                    int32_t x;
                    if (kGlobal) x = (!in_row && b == nb) ? 0 : rowp[b];
                    else x = in_row ? M[nb * B + b] : (b == nb ? 0 : M[b * B + nb]);
                    if (t < run + x) {
                        s_s = b;
                        break;
                    }
                    run += x;
                }
            }
            __syncthreads();
            s = s_s;
        }
        if (s < 0) {
            if (tid == 0) atomicOr(&flags->err, ERR_SELECT);
            break;
        }
        if (s == r) break;
        // delta-MDL (same terms as vertex_delta_fixed, with every lookup in shared memory)
        const int32_t L = __ldg(g.selfcnt + v), selfw = L > 0 ? 1 : 0;
        const int32_t dout_r = dout[r], dout_s = dout[s], din_r = din[r], din_s = din[s];
        const int32_t dout_r2 = dout_r - kout, dout_s2 = dout_s + kout;
        const int32_t din_r2 = din_r - (kin + selfw), din_s2 = din_s + (kin + selfw);
        long long acc[5] = {0, 0, 0, 0, 0};  // terms, sRo, sSo, sRi, sSi
        for (int32_t b = tid; b < B; b += kT) {
            if (b == r || b == s) continue;
            const int32_t Ob = O[b], Ib = I[b];
            if (Ob > 0) {
                const int32_t Mrb = M[(int64_t)r * B + b], Msb = M[(int64_t)s * B + b], dinb = din[b];
                acc[0] += ce_fixed(Lq, Mrb, dinb, dout_r) - ce_fixed(Lq, Mrb - Ob, dinb, dout_r2);
                acc[0] += ce_fixed(Lq, Msb, dinb, dout_s) - ce_fixed(Lq, Msb + Ob, dinb, dout_s2);
                acc[1] += Mrb;
                acc[2] += Msb;
            }
            if (Ib > 0) {
                const int32_t Mbr = kGlobal ? gMT[(int64_t)r * B + b] : M[b * B + r];
                const int32_t Mbs = kGlobal ? gMT[(int64_t)s * B + b] : M[b * B + s];
                const int32_t doutb = dout[b];
                acc[0] += ce_fixed(Lq, Mbr, din_r, doutb) - ce_fixed(Lq, Mbr - Ib, din_r2, doutb);
                acc[0] += ce_fixed(Lq, Mbs, din_s, doutb) - ce_fixed(Lq, Mbs + Ib, din_s2, doutb);
                acc[3] += Mbr;
                acc[4] += Mbs;
            }
        }
        block_sum5(acc, red);
        const int32_t Or = O[r], Ir = I[r], Os = O[s], Is = I[s];
        const int32_t Mrr = M[(int64_t)r * B + r], Mrs = M[(int64_t)r * B + s], Msr = M[(int64_t)s * B + r],
                      Mss = M[(int64_t)s * B + s];
        long long tot = acc[0];
        {
            const int32_t d = -Or - Ir - L;
            if (Or | Ir | L) tot += ce_fixed(Lq, Mrr, din_r, dout_r) - ce_fixed(Lq, Mrr + d, din_r2, dout_r2);
            else tot += ce_delta(Lq, Mrr, din_r, dout_r, din_r2, dout_r2);
        }
        {
            const int32_t d = Ir - Os;
            if (Os | Ir) tot += ce_fixed(Lq, Mrs, din_s, dout_r) - ce_fixed(Lq, Mrs + d, din_s2, dout_r2);
            if (d == 0) tot += ce_delta(Lq, Mrs, din_s, dout_r, din_s2, dout_r2);
        }
        {
            const int32_t d = Or - Is;
            if (Or | Is) tot += ce_fixed(Lq, Msr, din_r, dout_s) - ce_fixed(Lq, Msr + d, din_r2, dout_s2);
            if (d == 0) tot += ce_delta(Lq, Msr, din_r, dout_s, din_r2, dout_s2);
        }
        {
            const int32_t d = Os + Is + L;
            if (Os | Is | L) tot += ce_fixed(Lq, Mss, din_s, dout_s) - ce_fixed(Lq, Mss + d, din_s2, dout_s2);
            else tot += ce_delta(Lq, Mss, din_s, dout_s, din_s2, dout_s2);
        }
        tot += ((long long)dout_r - Mrr - Mrs - acc[1]) * (Lx(Lq, dout_r2) - Lx(Lq, dout_r));
        tot += ((long long)dout_s - Msr - Mss - acc[2]) * (Lx(Lq, dout_s2) - Lx(Lq, dout_s));
        tot += ((long long)din_r - Mrr - Msr - acc[3]) * (Lx(Lq, din_r2) - Lx(Lq, din_r));
        tot += ((long long)din_s - Mrs - Mss - acc[4]) * (Lx(Lq, din_s2) - Lx(Lq, din_s));
        if (!(tot < 0)) break;  // greedy acceptance; uniform
        // Blockmodel::move_vertex(Vertex, Delta, proposal) (blockmodel.cpp:408-435)
        for (int32_t b = tid; b < B; b += kT) {
            if (b == r || b == s) continue;
            const int32_t Ob = O[b], Ib = I[b];
            if (Ob) {
                M[(int64_t)r * B + b] -= Ob;
                M[(int64_t)s * B + b] += Ob;
                if (kGlobal) {
                    gMT[(int64_t)b * B + r] -= Ob;
                    gMT[(int64_t)b * B + s] += Ob;
                }
            }
            if (Ib) {
                M[(int64_t)b * B + r] -= Ib;
                M[(int64_t)b * B + s] += Ib;
                if (kGlobal) {
                    gMT[(int64_t)r * B + b] -= Ib;
                    gMT[(int64_t)s * B + b] += Ib;
                }
            }
        }
        if (tid == 0) {
            M[(int64_t)r * B + r] += -Or - Ir - L;
            M[(int64_t)r * B + s] += Ir - Os;
            M[(int64_t)s * B + r] += Or - Is;
            M[(int64_t)s * B + s] += Os + Is + L;
            if (kGlobal) {
                gMT[(int64_t)r * B + r] += -Or - Ir - L;
                gMT[(int64_t)s * B + r] += Ir - Os;
                gMT[(int64_t)r * B + s] += Or - Is;
                gMT[(int64_t)s * B + s] += Os + Is + L;
            }
            dout[r] -= kout;
            dout[s] += kout;
            din[r] -= kin + selfw;
            din[s] += kin + selfw;
            size[r] -= 1;
            size[s] += 1;
            bm.asg[v] = s;
            moved++;
            dsum += tot;
        }
        } while (0);
        __syncthreads();
    }
    if (tid == 0) {
        atomicAdd(&flags->counters[4], edges);
        atomicAdd(&flags->counters[5], moved);
        atomicAdd(&flags->counters[7], (unsigned long long)dsum);
    }
}

__global__ void k_dense_fill(DevBM bm, int32_t* M, int32_t* MT) {
    const int32_t B = bm.B;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < bm.nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = bm.row_of[j], c = bm.row_col[j], v = bm.row_cnt[j];
        M[(int64_t)r * B + c] = v;
        MT[(int64_t)c * B + r] = v;
    }
}

}  // namespace

size_t mh_chain_dense_smem(int32_t B) {
    if (B <= kDenseMax) return sizeof(int32_t) * ((size_t)B * B + 5 * (size_t)B);
    return sizeof(int32_t) * 5 * (size_t)B;
}

void mh_chain_dense(const DevGraph& g, DevBM& bm, const int32_t* order, int32_t n, uint64_t seed, uint32_t iter,
                    uint32_t step, Work& w, cudaStream_t st) {
    if (n <= 0) return;
    const size_t smem = mh_chain_dense_smem(bm.B);
    if (bm.B <= kDenseMax) {
        allow_max_dynamic_smem((const void*)k_mh_chain_dense<false>);
        k_mh_chain_dense<false><<<1, kT, smem, st>>>(g, bm, order, n, seed, iter, step, nullptr, nullptr, w.flags_dev);
        count_launches(1);
        return;
    }
    const size_t cells = (size_t)bm.B * bm.B;
    cudaMemsetAsync(w.dense_M, 0, cells * sizeof(int32_t), st);
    cudaMemsetAsync(w.dense_MT, 0, cells * sizeof(int32_t), st);
    int64_t blocks = ((int64_t)bm.nnz + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > (int64_t)device_sms() * 16) blocks = (int64_t)device_sms() * 16;
    k_dense_fill<<<(unsigned)blocks, 256, 0, st>>>(bm, w.dense_M, w.dense_MT);
    allow_max_dynamic_smem((const void*)k_mh_chain_dense<true>);
    k_mh_chain_dense<true><<<1, kT, smem, st>>>(g, bm, order, n, seed, iter, step, w.dense_M, w.dense_MT,
                                               w.flags_dev);
    count_launches(2);
}

}  // namespace sbp

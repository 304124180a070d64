"""Seeded directed degree-corrected SBM generator for the synthetic benchmark graphs.

The reference benchmarks on Graph Challenge TSV graphs; these seeded synthetic graphs
stand in for them with the configured shapes:
  1. block sizes ~ Dirichlet(alpha) * N (every block non-empty);
  2. out- and in-degree propensities theta ~ power law (exponent gamma) truncated to
     [dmin, dmax], normalised within each block;
  3. `ratio` is the within:between ratio of edge totals (as in the Graph Challenge
     generators' ratio_within_over_between): ratio/(1+ratio) of the expected edges fall
     inside blocks and 1/(1+ratio) between blocks; within each part the expected count
     of a block pair is proportional to n_a * n_b;
  4. Poisson edge counts per block pair; endpoints drawn proportional to theta.
Duplicate edges are kept (a multigraph, as the reference accepts without
--noduplicates); a vertex keeps at most one self-loop.  Vertex ids are a random
permutation of the planted order and edges are in random order.
"""
import numpy as np

CONFIGS = {
    # N, E, blocks, alpha, dmin, dmax, ratio
    "C1": dict(num_vertices=1000, num_edges=8000, num_blocks=11, alpha=2.0, dmin=10, dmax=100, ratio=2.5),
    "C2": dict(num_vertices=50000, num_edges=1000000, num_blocks=33, alpha=2.0, dmin=10, dmax=100, ratio=2.5),
    "C3": dict(num_vertices=1000000, num_edges=20000000, num_blocks=100, alpha=0.5, dmin=5, dmax=500, ratio=1.5),
    # the C3 shape at a fifth of its size: the case profiler captures run on (a full-set
    # capture saves and restores device memory on every pass)
    "C3S": dict(num_vertices=200000, num_edges=4000000, num_blocks=100, alpha=0.5, dmin=5, dmax=500, ratio=1.5),
}


def _power_law(rng, n, gamma, lo, hi):
    u = rng.random(n)
    a = 1.0 - gamma
    return (lo ** a + u * (hi ** a - lo ** a)) ** (1.0 / a)


def generate(num_vertices, num_edges, num_blocks, alpha=2.0, dmin=10, dmax=100, ratio=2.5, gamma=2.1, seed=0):
    """Returns (src int32[E], dst int32[E], planted int32[N])."""
    rng = np.random.default_rng(seed)
    N, B = int(num_vertices), int(num_blocks)
    if B > N:
        raise ValueError("more blocks than vertices")
    p = rng.dirichlet(np.full(B, alpha))
    sizes = np.maximum(1, np.floor(p * N).astype(np.int64))
    while sizes.sum() > N:
        sizes[np.argmax(sizes)] -= 1
    sizes[np.argmax(p)] += N - sizes.sum()
    planted_sorted = np.repeat(np.arange(B, dtype=np.int64), sizes)
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    th_out = _power_law(rng, N, gamma, dmin, dmax)
    th_in = _power_law(rng, N, gamma, dmin, dmax)
    # normalised cumulative propensities within each block
    cum_out = np.empty(N)
    cum_in = np.empty(N)
    for b in range(B):
        s, e = starts[b], starts[b] + sizes[b]
        co = np.cumsum(th_out[s:e])
        ci = np.cumsum(th_in[s:e])
        cum_out[s:e] = co / co[-1]
        cum_in[s:e] = ci / ci[-1]
    w = np.outer(sizes, sizes).astype(np.float64)
    diag = np.diag(w).copy()
    off = w.copy()
    off[np.diag_indices(B)] = 0.0
    lam = np.zeros_like(w)
    if B > 1:
        lam += off / off.sum() * (num_edges / (1.0 + ratio))
        lam[np.diag_indices(B)] = diag / diag.sum() * (num_edges * ratio / (1.0 + ratio))
    else:
        lam[0, 0] = num_edges
    counts = rng.poisson(lam)
    ea, eb = np.nonzero(counts)
    reps = counts[ea, eb]
    src_block = np.repeat(ea, reps)
    dst_block = np.repeat(eb, reps)
    E = src_block.size
    u = rng.random(E)
    v = rng.random(E)
    src = np.empty(E, np.int64)
    dst = np.empty(E, np.int64)
    for b in range(B):
        s, n = starts[b], sizes[b]
        m = src_block == b
        src[m] = s + np.minimum(np.searchsorted(cum_out[s:s + n], u[m], side="right"), n - 1)
        m = dst_block == b
        dst[m] = s + np.minimum(np.searchsorted(cum_in[s:s + n], v[m], side="right"), n - 1)
    # at most one self-loop per vertex
    loop = src == dst
    if loop.any():
        idx = np.nonzero(loop)[0]
        _, first = np.unique(src[idx], return_index=True)
        keep = np.ones(E, bool)
        keep[idx] = False
        keep[idx[first]] = True
        src, dst = src[keep], dst[keep]
    perm = rng.permutation(N)
    src = perm[src]
    dst = perm[dst]
    order = rng.permutation(src.size)
    src, dst = src[order], dst[order]
    planted = np.empty(N, np.int64)
    planted[perm] = planted_sorted
    return src.astype(np.int32), dst.astype(np.int32), planted.astype(np.int32)


def generate_config(name, seed=0, scale=1.0):
    c = dict(CONFIGS[name])
    if scale != 1.0:
        c["num_vertices"] = max(c["num_blocks"] * 4, int(c["num_vertices"] * scale))
        c["num_edges"] = int(c["num_edges"] * scale)
    return generate(seed=seed, **c)

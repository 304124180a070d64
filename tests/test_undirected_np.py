"""The undirected form of the nonparametric entropy (args.undirected; reference
include/entropy.hpp:102-133, src/entropy.cpp:745-749), not degree-corrected.

Against the directed form: a diagonal cell's eterm carries -w log 2, a block's vertex term
counts its out-degree only (the stored graph holds both directions of every edge), and the
edge description length spreads the edges over B (B + 1) / 2 block pairs.  The CPU tests
pin the oracle on these formulas, computed here independently from the cells; the GPU tests
hold the library's deltas, sweeps, merges and partitions to the oracle's, exactly as for
the directed form (test_gpu_nonparametric.py)."""
import math

import numpy as np
import pytest

from test_gpu_parity import same_state
from test_ingest import _edges

MDL_REL_TOL_CANONICAL = 1e-12


def _lbinom(n, k):
    if n == 0 or k == 0 or k > n:
        return 0.0
    return (math.lgamma(n + 1) - math.lgamma(k + 1)) - math.lgamma(n - k + 1)


def _symmetric(n, e, blocks, seed, isolated=0):
    from sbp_gb300 import dcsbm
    src, dst, planted = dcsbm.generate(n, e, blocks, seed=seed)
    s2, d2 = _edges(True, src, dst)
    return s2, d2, s2.size // 2, n + isolated, planted


def _terms(s2, d2, N, a, B, Em):
    """The four parts of nonparametric::mdl for an undirected graph, from the cells."""
    M = np.zeros((B, B), np.int64)
    np.add.at(M, (a[s2], a[d2]), 1)
    dout = M.sum(axis=1)
    sizes = np.bincount(a, minlength=B)
    S = 0.0
    for r, c in zip(*np.nonzero(M)):
        w = int(M[r, c])
        S += -math.lgamma(w + 1) - (w * math.log(2) if r == c else 0.0)
    flog = lambda x: float(np.log(np.float32(x)))  # fastlog: logf of the float
    S += sum(float(dout[b]) * flog(sizes[b]) for b in range(B) if sizes[b] > 0)
    ne = int((sizes > 0).sum())
    P = _lbinom(N - 1, ne - 1) + math.lgamma(N + 1) - sum(math.lgamma(int(x) + 1) for x in sizes) + flog(N)
    # numpy's float32 log and the C library's logf may differ by an ulp (< 1e-6 here), which
    # the vertex terms multiply by the block out-degrees
    slack = 1e-6 * float(dout.sum()) + 1e-9 * abs(S)
    return S, P, _lbinom(ne * (ne + 1) // 2 + Em - 1, Em), slack


def test_oracle_undirected_terms(oracle):
    s2, d2, Em, N, planted = _symmetric(500, 3000, 5, seed=51, isolated=10)
    rng = np.random.default_rng(3)
    B = 12
    a = rng.integers(0, B - 1, N).astype(np.int32)  # block B - 1 empty
    O = oracle.Graph(N, s2, d2, num_edges=Em, undirected=True)
    t = oracle.Blockmodel(O, B, a).np_terms()
    S, P, Edl, slack = _terms(s2, d2, N, a, B, Em)
    assert abs(t["sparse_entropy"] - S) <= slack
    assert t["partition_dl"] == pytest.approx(P, rel=1e-9)
    assert t["edges_dl"] == pytest.approx(Edl, rel=1e-12)
    # the directed form of the same cells differs by exactly these terms
    td = oracle.Blockmodel(oracle.Graph(N, s2, d2, num_edges=Em), B, a).np_terms()
    assert td["edges_dl"] == pytest.approx(_lbinom(11 * 11 + Em - 1, Em), rel=1e-12)


def test_oracle_undirected_deltas_match_mdl_differences(oracle):
    """A vertex move's and a block merge's canonical delta equal the change of the
    canonical MDL, with moves onto and off the diagonal and into an empty block."""
    s2, d2, Em, N, planted = _symmetric(400, 2500, 4, seed=52)
    rng = np.random.default_rng(4)
    B = 10
    a = rng.integers(0, B - 1, N).astype(np.int32)
    O = oracle.Graph(N, s2, d2, num_edges=Em, undirected=True)
    before = oracle.Blockmodel(O, B, a).np_mdl()[1]
    for v, s in [(0, int((a[0] + 1) % (B - 1))), (5, B - 1), (7, int(a[8]))]:
        if s == a[v]:
            continue
        d = oracle.Blockmodel(O, B, a).np_delta_mdl(v, s)[1] / 2**24
        a2 = a.copy()
        a2[v] = s
        after = oracle.Blockmodel(O, B, a2).np_mdl()[1]
        assert abs((after - before) - d) <= 1e-6, (v, s)
    r, t = 1, 2
    d = oracle.Blockmodel(O, B, a).np_merge_delta_mdl(r, t)[1] / 2**24
    a2 = np.where(a == r, t, a).astype(np.int32)
    after = oracle.Blockmodel(O, B, a2).np_mdl()[1]
    assert abs((after - before) - d) <= 1e-6


def _pair(gpu, oracle, n, e, blocks, B, seed, isolated=0, empty=0, assignment=None):
    s2, d2, Em, N, planted = _symmetric(n, e, blocks, seed, isolated)
    rng = np.random.default_rng(seed)
    if assignment is None:
        live = B - empty
        a = rng.integers(0, live - 1, N).astype(np.int32)
        a[: live - 1] = np.arange(live - 1)
        a[N - 1] = live - 1  # a singleton block
    else:
        a = np.asarray(assignment, np.int32)
    G = gpu.Graph(N, s2, d2, num_edges=Em, undirected=True)
    O = oracle.Graph(N, s2, d2, num_edges=Em, undirected=True)
    return G, O, gpu.Blockmodel(B, G, 0.5, a), oracle.Blockmodel(O, B, a), a


@pytest.mark.gpu
@pytest.mark.parametrize("B", [5, 300])
def test_gpu_undirected_np_mdl_and_deltas_exact(gpu, oracle, B):
    G, O, gb, ob, a = _pair(gpu, oracle, 1200, 9000, 6, B, seed=260 + B, isolated=20, empty=2)
    assert G.undirected()
    assert abs(gpu.entropy.nonparametric.mdl(gb) - ob.np_mdl()[1]) <= MDL_REL_TOL_CANONICAL * abs(ob.np_mdl()[1])
    N = a.size
    rng = np.random.default_rng(B)
    v = np.concatenate([rng.integers(0, N, 1500), [N - 1] * 2]).astype(np.int32)
    s = np.concatenate([rng.integers(0, B, 1500), [0, B - 1]]).astype(np.int32)
    keep = s != a[v]
    v, s = v[keep], s[keep]
    got = gpu.entropy.nonparametric.delta_mdl(gb, v, s)
    for i in range(v.size):
        assert got[i] == ob.np_delta_mdl(int(v[i]), int(s[i]))[1] / 2**24, (i, v[i], s[i])
    r = rng.integers(0, B, 800).astype(np.int32)
    t = rng.integers(0, B, 800).astype(np.int32)
    keep = r != t
    r, t = r[keep], t[keep]
    got = gpu.entropy.nonparametric.block_merge_delta_mdl(gb, r, t)
    for i in range(r.size):
        assert got[i] == ob.np_merge_delta_mdl(int(r[i]), int(t[i]))[1] / 2**24, (i, r[i], t[i])


@pytest.mark.gpu
@pytest.mark.parametrize("alg", ["async_gibbs", "hybrid_mcmc"])
def test_gpu_undirected_np_mcmc_identical(gpu, oracle, alg):
    G, O, gb, ob, a = _pair(gpu, oracle, 1500, 12000, 6, 120, seed=270, isolated=30, empty=2)
    gpu.finetune.mcmc(2, G, gb, True, gpu.Args(algorithm=alg, seed=17, max_iterations=5, nonparametric=True))
    ob.mcmc(oracle.make_config(alg, max_iterations=5, nonparametric=True), seed=17, step=2,
            golden_ratio_not_reached=True)
    same_state(gb, ob)


@pytest.mark.gpu
@pytest.mark.parametrize("cells", ["dense", "hash"])
def test_gpu_undirected_np_merges_identical(gpu, oracle, cells):
    ctx = gpu.core.default_context()
    ctx.set_cells_budget(0 if cells == "hash" else 16 << 30)
    try:
        G, O, gb, ob, a = _pair(gpu, oracle, 2000, 14000, 6, 400, seed=280, empty=3)
        gpu.block_merge.merge_blocks(gb, G, args=gpu.Args(seed=23, nonparametric=True), step=5,
                                     num_blocks_to_merge=200)
        ob.merge_blocks(oracle.make_config(nonparametric=True), seed=23, step=5, num_to_merge=200)
        same_state(gb, ob)
    finally:
        ctx.set_cells_budget(16 << 30)


@pytest.mark.gpu
def test_gpu_undirected_np_partition_identical(gpu, oracle):
    src, dst, _ = gpu.dcsbm.generate_config("C1", seed=0)
    s2, d2 = _edges(True, src, dst)
    G = gpu.Graph(1000, s2, d2, num_edges=s2.size // 2, undirected=True)
    O = oracle.Graph(1000, s2, d2, num_edges=s2.size // 2, undirected=True)
    a_g, B_g, mdl_g, st = gpu.sbp.stochastic_block_partition(
        G, gpu.Args(algorithm="hybrid_mcmc", seed=6, nonparametric=True))
    a_o, B_o, mdl_o, ost = oracle.sbp(O, oracle.make_config("hybrid_mcmc", nonparametric=True), seed=6)
    assert B_g == B_o
    assert np.array_equal(a_g, a_o)
    assert abs(mdl_g - mdl_o) <= MDL_REL_TOL_CANONICAL * abs(mdl_o)

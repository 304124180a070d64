"""Graph::num_edges as the description lengths use it (reference include/graph.hpp:99).

For an undirected edge list the reference stores both directions of every edge but its
Graph reports half of the stored count (src/graph.cpp:145-147), and entropy::mdl
(src/entropy.cpp:597-604), null_mdl_v1 and the nonparametric get_edges_dl (:745-749) take
that count.  The CPU tests pin the oracle: changing the count moves the parametric MDL by
exactly the change of E * h(B^2 / E) and the nonparametric one by the change of
get_edges_dl, nothing else.  The GPU tests check that the library follows the same count,
from arrays and from an undirected TSV load."""
import math

import numpy as np
import pytest

from test_ingest import _edges, _write_tsv


def _undirected_pair(src, dst):
    """Both directions of each edge, as the reference's parse_undirected inserts them."""
    s2, d2 = _edges(True, src, dst)
    return s2, d2, s2.size // 2


def _model_term(E, B):
    x = B * B / E
    return E * (((1 + x) * math.log(1 + x)) - (x * math.log(x)))


def _lbinom(n, k):
    if n == 0 or k == 0 or k > n:
        return 0.0
    return (math.lgamma(n + 1) - math.lgamma(k + 1)) - math.lgamma(n - k + 1)


def _graph(seed=41):
    from sbp_gb300 import dcsbm
    return dcsbm.generate(600, 4000, 6, seed=seed)


def test_oracle_mdl_follows_model_edges(oracle):
    src, dst, planted = _graph()
    s2, d2, Em = _undirected_pair(src, dst)
    n = int(max(src.max(), dst.max())) + 1
    full = oracle.Graph(n, s2, d2)
    half = oracle.Graph(n, s2, d2, num_edges=Em)
    assert full.model_edges() == s2.size and half.model_edges() == Em
    a = planted[:n].astype(np.int32)
    B = int(a.max()) + 1
    bf, bh = oracle.Blockmodel(full, B, a), oracle.Blockmodel(half, B, a)
    want = _model_term(Em, B) - _model_term(s2.size, B)
    for k in (0, 1):  # literal and canonical
        assert abs((bh.mdl()[k] - bf.mdl()[k]) - want) <= 1e-9 * abs(bf.mdl()[k])
    ne = B
    want_np = _lbinom(ne * ne + Em - 1, Em) - _lbinom(ne * ne + s2.size - 1, s2.size)
    assert abs((bh.np_mdl()[1] - bf.np_mdl()[1]) - want_np) <= 1e-9 * abs(bf.np_mdl()[1])
    assert bh.np_terms()["edges_dl"] == pytest.approx(_lbinom(ne * ne + Em - 1, Em), rel=1e-12)
    # the deltas do not depend on the count (the block count does not change here)
    assert bh.delta_mdl(0, int((a[0] + 1) % B)) == bf.delta_mdl(0, int((a[0] + 1) % B))


@pytest.mark.gpu
def test_gpu_mdl_follows_model_edges(gpu, oracle):
    src, dst, planted = _graph()
    s2, d2, Em = _undirected_pair(src, dst)
    n = int(max(src.max(), dst.max())) + 1
    G = gpu.Graph(n, s2, d2, num_edges=Em)
    assert G.num_edges() == Em and G.num_stored_edges() == s2.size
    O = oracle.Graph(n, s2, d2, num_edges=Em)
    a = planted[:n].astype(np.int32)
    B = int(a.max()) + 1
    gb, ob = gpu.Blockmodel(B, G, 0.5, a), oracle.Blockmodel(O, B, a)
    assert abs(gpu.entropy.mdl(gb, G) - ob.mdl()[1]) <= 1e-12 * abs(ob.mdl()[1])
    assert abs(gpu.entropy.nonparametric.mdl(gb) - ob.np_mdl()[1]) <= 1e-12 * abs(ob.np_mdl()[1])


@pytest.mark.gpu
@pytest.mark.parametrize("nonparametric", [False, True])
def test_gpu_partition_with_model_edges_identical(gpu, oracle, nonparametric):
    """The golden-section search compares MDLs, so the count steers the whole partition;
    the nonparametric merges read it through the non-empty-count tables."""
    src, dst, _ = gpu.dcsbm.generate_config("C1", seed=0)
    s2, d2, Em = _undirected_pair(src, dst)
    G = gpu.Graph(1000, s2, d2, num_edges=Em)
    O = oracle.Graph(1000, s2, d2, num_edges=Em)
    a_g, B_g, mdl_g, st = gpu.sbp.stochastic_block_partition(
        G, gpu.Args(algorithm="hybrid_mcmc", seed=5, nonparametric=nonparametric))
    a_o, B_o, mdl_o, ost = oracle.sbp(O, oracle.make_config("hybrid_mcmc", nonparametric=nonparametric), seed=5)
    assert B_g == B_o
    assert np.array_equal(a_g, a_o)
    assert abs(mdl_g - mdl_o) <= 1e-12 * abs(mdl_o)


@pytest.mark.gpu
def test_gpu_model_edges_reset_nonparametric_tables(gpu, oracle):
    """The non-empty-count tables are built on first use and rebuilt when the count changes."""
    src, dst, planted = _graph(seed=43)
    s2, d2, Em = _undirected_pair(src, dst)
    n = int(max(src.max(), dst.max())) + 1
    G = gpu.Graph(n, s2, d2)
    a = planted[:n].astype(np.int32)
    B = int(a.max()) + 2  # one empty block: merges into it change the non-empty count
    gb = gpu.Blockmodel(B, G, 0.5, a)
    r, t = np.array([0, 1], np.int32), np.array([1, 2], np.int32)
    before = gpu.entropy.nonparametric.block_merge_delta_mdl(gb, r, t)
    G.ctx.check(G.ctx.lib.sbpgpu_graph_set_model_edges(G.h, Em))
    after = gpu.entropy.nonparametric.block_merge_delta_mdl(gb, r, t)
    ob = oracle.Blockmodel(oracle.Graph(n, s2, d2, num_edges=Em), B, a)
    for i in range(r.size):
        assert after[i] == ob.np_merge_delta_mdl(int(r[i]), int(t[i]))[1] / 2**24
    assert not np.array_equal(before, after)


@pytest.mark.gpu
def test_tsv_undirected_load_counts_each_pair_once(gpu, tmp_path):
    src, dst, _ = gpu.dcsbm.generate(500, 3000, 5, seed=44)
    path = tmp_path / "g.tsv"
    _write_tsv(path, src, dst)
    G = gpu.Graph.load(str(path), undirected=True)
    s2, d2, Em = _undirected_pair(src, dst)
    assert G.num_stored_edges() == s2.size and G.num_edges() == Em

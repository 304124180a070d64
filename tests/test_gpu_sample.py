"""GPU parity of sampling and the sampled partition (reference src/sample.cpp,
src/main.cpp:98-140): the device's sample mappings, sampled subgraphs, extended
assignments, finetune_assignment and the whole sample -> partition -> extend -> finetune
flow are identical to the oracle's on the same seeded inputs."""
import numpy as np
import pytest

from test_gpu_parity import same_state

pytestmark = pytest.mark.gpu


def graphs(gpu, oracle, n, e, k, seed, isolated=0):
    src, dst, planted = gpu.dcsbm.generate(n, e, k, seed=seed)
    N = n + isolated
    return gpu.Graph(N, src, dst), oracle.Graph(N, src, dst), src, dst, planted


@pytest.mark.parametrize("alg", ["max_degree", "random", "degree_product", "detach", "expansion_snowball",
                                 "degree_product_snowball"])
@pytest.mark.parametrize("size", [0.001, 0.3, 0.75])
def test_sample_mapping_identical(gpu, oracle, alg, size):
    G, O, *_ = graphs(gpu, oracle, 3000, 30000, 9, seed=300, isolated=60)
    m_g, n_g = gpu.sample.sample_mapping(G, alg, size, seed=4)
    m_o, n_o = oracle.sample(O, alg, size, 4)
    assert n_g == n_o
    assert np.array_equal(m_g, m_o)


def test_degree_product_beyond_the_vertices_with_edges(gpu, oracle):
    # 40% of the vertices have no edges: a sample of 90% takes every vertex with an edge
    G, O, *_ = graphs(gpu, oracle, 600, 5000, 4, seed=301, isolated=400)
    m_g, n_g = gpu.sample.sample_mapping(G, "degree_product", 0.9, seed=1)
    m_o, n_o = oracle.sample(O, "degree_product", 0.9, 1)
    assert n_g == n_o and np.array_equal(m_g, m_o)


@pytest.mark.parametrize("alg", ["max_degree", "random", "degree_product"])
def test_subgraph_identical(gpu, oracle, alg):
    """The sampled graph: same vertices and edges in the same per-vertex order, checked
    through identical blockmodels and an identical MH chain on it."""
    G, O, src, dst, _ = graphs(gpu, oracle, 2500, 25000, 9, seed=310)
    m, n = gpu.sample.sample_mapping(G, alg, 0.4, seed=2)
    S = gpu.sample.from_vertices(G, m)
    n_o, s_o, d_o = oracle.subgraph_edges(O, m)
    # the reference's insertion order: by original source id, each source's edges in order
    keep = np.argsort(src, kind="stable")
    keep = keep[(m[src[keep]] >= 0) & (m[dst[keep]] >= 0)]
    s_w, d_w = m[src[keep]], m[dst[keep]]
    assert sorted(zip(s_o.tolist(), d_o.tolist())) == sorted(zip(s_w.tolist(), d_w.tolist()))
    assert S.num_vertices() == n == n_o and S.num_edges() == s_w.size
    SO = oracle.Graph(n, s_w, d_w)
    rng = np.random.default_rng(1)
    B = 40
    a = rng.integers(0, B, n).astype(np.int32)
    a[:B] = np.arange(B)
    gb, ob = gpu.Blockmodel(B, S, 0.5, a), oracle.Blockmodel(SO, B, a)
    same_state(gb, ob)
    order = rng.permutation(n).astype(np.int32)
    assert gpu.finetune.mh_chain(gb, order, seed=3, iteration=0, step=1) == \
        ob.mh_chain(order, 3, 0, 1, oracle.make_config("hybrid_mcmc"))
    same_state(gb, ob)


@pytest.mark.parametrize("B", [1, 7, 300])
def test_extend_identical(gpu, oracle, B):
    G, O, *_ = graphs(gpu, oracle, 4000, 36000, 9, seed=320 + B, isolated=50)
    m, n = gpu.sample.sample_mapping(G, "random", 0.35, seed=B)
    rng = np.random.default_rng(B)
    sa = rng.integers(0, B, n).astype(np.int32)
    smp = gpu.sample.Sample(None, m)
    got = gpu.sample.extend(G, sa, B, smp, seed=7)
    want = oracle.extend(O, sa, B, m, 7)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("greedy", [True, False])
def test_finetune_assignment_identical(gpu, oracle, greedy):
    G, O, src, dst, planted = graphs(gpu, oracle, 2500, 30000, 9, seed=330)
    rng = np.random.default_rng(5)
    a = np.where(rng.random(2500) < 0.7, planted, rng.integers(0, 9, 2500)).astype(np.int32)
    gb, ob = gpu.Blockmodel(9, G, 0.5, a), oracle.Blockmodel(O, 9, a)
    args = gpu.Args(seed=11, greedy=greedy)
    st = gpu.sample.finetune_assignment(gb, G, args)
    ost = ob.finetune_assignment(oracle.make_config(greedy=greedy), 11)
    same_state(gb, ob)
    assert st["mcmc_iterations"] == ost.mcmc_iterations
    assert abs(gb.getOverall_entropy() - ob.mdl()[1]) <= 1e-12 * ob.mdl()[1]


@pytest.mark.parametrize("alg,size,np_", [("max_degree", 0.5, False), ("random", 0.4, False),
                                          ("degree_product", 0.5, False), ("random", 0.5, True)])
def test_sampled_partition_identical_c1(gpu, oracle, alg, size, np_):
    src, dst, planted = gpu.dcsbm.generate_config("C1", seed=0)
    G, O = gpu.Graph(1000, src, dst), oracle.Graph(1000, src, dst)
    args = gpu.Args(algorithm="hybrid_mcmc", seed=2, samplesize=size, samplingalg=alg, nonparametric=np_)
    a_g, B_g, mdl_g, st = gpu.sample.partition(G, args)
    a_o, B_o, mdl_o, ost = oracle.sbp_sampled(O, oracle.make_config("hybrid_mcmc", nonparametric=np_), 2, alg, size)
    assert B_g == B_o
    assert np.array_equal(a_g, a_o)
    assert abs(mdl_g - mdl_o) <= 1e-12 * abs(mdl_o)


def _detach_graph(gpu, oracle):
    src, dst, planted = gpu.dcsbm.generate(2000, 16000, 6, seed=340)
    extra_s = [2000, 2002, 2003, 2005, 2006]
    extra_d = [2001, 2002, 7, 2004, 9]
    src = np.concatenate([src, extra_s]).astype(np.int32)
    dst = np.concatenate([dst, extra_d]).astype(np.int32)
    N = 2010  # 2007..2009 isolated
    return gpu.Graph(N, src, dst), oracle.Graph(N, src, dst), src, dst, N


def test_reattach_identical(gpu, oracle):
    G, O, src, dst, N = _detach_graph(gpu, oracle)
    m, n = gpu.sample.sample_mapping(G, "detach", 1.0)
    m_o, n_o = oracle.sample(O, "detach", 1.0, 0)
    assert n == n_o and np.array_equal(m, m_o)
    sa = (np.arange(n) * 7 % 11).astype(np.int32)
    got = gpu.sample.reattach(G, sa, 11, gpu.sample.Sample(None, m), seed=5)
    assert np.array_equal(got, oracle.reattach(O, sa, 11, m, 5))


def test_detached_partition_identical(gpu, oracle):
    """main.cpp with --detach: partition the graph of degree > 1 vertices, then reattach."""
    G, O, src, dst, N = _detach_graph(gpu, oracle)
    args = gpu.Args(algorithm="hybrid_mcmc", seed=4, detach=True)
    a_g, B_g, mdl_g, st = gpu.sample.partition(G, args)
    m, n = oracle.sample(O, "detach", 1.0, 0)
    n2, s2, d2 = oracle.subgraph_edges(O, m)
    keep = np.argsort(src, kind="stable")
    keep = keep[(m[src[keep]] >= 0) & (m[dst[keep]] >= 0)]
    SO = oracle.Graph(n, m[src[keep]], m[dst[keep]])
    sa, B_o, _, _ = oracle.sbp(SO, oracle.make_config("hybrid_mcmc"), 4)
    a_o = oracle.reattach(O, sa, B_o, m, 4)
    assert B_g == B_o and np.array_equal(a_g, a_o)
    assert abs(mdl_g - oracle.Blockmodel(O, B_o, a_o).mdl()[1]) <= 1e-12 * abs(mdl_g)


def test_max_degree_sample_of_the_toy_graph(gpu, oracle, golden):
    """sample_test.cpp's known answer (pinned on the oracle): the device draws the same
    4-vertex sample of the toy graph."""
    e = np.array(golden["edges"], np.int32)
    G, O = gpu.Graph(11, e[:, 0], e[:, 1]), oracle.Graph(11, e[:, 0], e[:, 1])
    size = golden["sample_max_degree"]["sample_size"]
    m_g, n_g = gpu.sample.sample_mapping(G, "max_degree", size, seed=0)
    m_o, n_o = oracle.sample(O, "max_degree", size, 0)
    assert n_g == n_o == golden["sample_max_degree"]["num_vertices"]
    assert np.array_equal(m_g, m_o)

"""GPU parity of the top-down (divisive) partition (reference src/top_down_sbp.cpp): the
random splits of every cluster, their nonparametric scores, the clusters chosen for
splitting and the whole divisive run equal the oracle's on the same seeded inputs."""
import numpy as np
import pytest

from test_gpu_parity import same_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,B,target,np_", [(3000, 12, 18, True), (3000, 12, 30, False), (3000, 40, 55, True),
                                            (400, 30, 45, True)])
def test_split_communities_identical(gpu, oracle, n, B, target, np_):
    """Clusters of every size: below 0.001 N they are not split; a one-vertex cluster of a
    small graph is 'split' into itself and an empty block, as the reference does."""
    src, dst, planted = gpu.dcsbm.generate(n, 10 * n, 6, seed=400 + B)
    rng = np.random.default_rng(B)
    a = rng.integers(0, B - 2, n).astype(np.int32)
    a[:B - 2] = np.arange(B - 2)
    a[n - 1] = B - 1   # a singleton cluster
    a[n - 2] = B - 2
    a[n - 3] = B - 2   # a two-vertex cluster
    G, O = gpu.Graph(n, src, dst), oracle.Graph(n, src, dst)
    gb, ob = gpu.Blockmodel(B, G, 0.5, a), oracle.Blockmodel(O, B, a)
    args = gpu.Args(seed=7, nonparametric=np_)
    gpu.divisive.split_communities(gb, G, target, args, step=3)
    ob.split_communities(oracle.make_config(nonparametric=np_), 7, 3, target)
    assert gb.num_blocks() == ob.num_blocks
    same_state(gb, ob)


@pytest.mark.parametrize("np_,mix", [(True, False), (False, False), (False, True), (True, True)])
def test_top_down_identical_c1(gpu, oracle, np_, mix):
    src, dst, planted = gpu.dcsbm.generate_config("C1", seed=0)
    G, O = gpu.Graph(1000, src, dst), oracle.Graph(1000, src, dst)
    a_g, B_g, mdl_g, st = gpu.divisive.run(G, gpu.Args(algorithm="hybrid_mcmc", seed=1, nonparametric=np_, mix=mix))
    a_o, B_o, mdl_o, ost = oracle.top_down(O, oracle.make_config("hybrid_mcmc", nonparametric=np_), 1, mix)
    assert B_g == B_o
    assert np.array_equal(a_g, a_o)
    assert abs(mdl_g - mdl_o) <= 1e-12 * abs(mdl_o)
    assert st["outer_steps"] == ost.outer_steps


@pytest.mark.parametrize("split", ["snowball", "single-snowball", "connectivity-snowball"])
@pytest.mark.parametrize("init", ["random", "degree-weighted", "high-degree"])
def test_snowball_splits_identical(gpu, oracle, split, init):
    """The snowball splits (top_down_sbp.cpp:262-426): host frontier processes per cluster,
    counted and applied on the device, against the oracle."""
    n, B = 2500, 8
    src, dst, planted = gpu.dcsbm.generate(n, 10 * n, 6, seed=450)
    a = (np.arange(n) % B).astype(np.int32)
    G, O = gpu.Graph(n, src, dst), oracle.Graph(n, src, dst)
    gb, ob = gpu.Blockmodel(B, G, 0.5, a), oracle.Blockmodel(O, B, a)
    args = gpu.Args(seed=5, nonparametric=True, split=split, splitinit=init)
    gpu.divisive.split_communities(gb, G, 13, args, step=2)
    ob.split_communities(oracle.make_config(nonparametric=True, split=split, splitinit=init), 5, 2, 13)
    assert gb.num_blocks() == ob.num_blocks == 13
    same_state(gb, ob)

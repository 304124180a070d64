"""The sequential Metropolis-Hastings chain evaluated in wide windows on a thread-block
cluster (one CTA per SM, 16 window entries each) against the oracle's one-vertex-at-a-time
chain (finetune::propose_move / move_vertex, reference src/finetune.cpp:822-869): the
applied move count and the whole integer state after the chain are bit-exact.  Cells
dense in global memory or hashed (a zero dense budget); greedy, Hastings-corrected and
nonparametric acceptance; block counts from a few hundred, where conflicts end most
windows early, to 100,000, where windows are taken whole."""
import numpy as np
import pytest

from test_gpu_parity import make_pair, same_state

pytestmark = pytest.mark.gpu


@pytest.fixture
def cluster_ctx(gpu):
    ctx = gpu.core.default_context()
    ctx.set_cluster_blocks(0)
    yield ctx
    ctx.set_cluster_blocks(8192)
    ctx.set_cells_budget(16 << 30)


def _chain(gpu, oracle, n, B, m, mode, seed):
    G, O, gb, ob, a, _ = make_pair(gpu, oracle, n, 12 * n, 9, B, seed=seed)
    order = np.random.default_rng(seed).permutation(n)[:m].astype(np.int32)
    args = gpu.Args(algorithm="hybrid_mcmc", greedy=mode == "greedy", nonparametric=mode == "np")
    cfg = oracle.make_config("hybrid_mcmc", greedy=mode == "greedy", nonparametric=mode == "np")
    for it in range(2):
        applied = gpu.finetune.mh_chain(gb, order, seed=8, iteration=it, step=3, args=args)
        want = ob.mh_chain(order, 8, it, 3, cfg)
        assert applied == want, (it, applied, want)
        same_state(gb, ob)


@pytest.mark.parametrize("cells", ["dense", "hash"])
@pytest.mark.parametrize("mode", ["greedy", "hastings", "np"])
@pytest.mark.parametrize("n,B", [(2500, 300), (9000, 5000)])
def test_cluster_chain_identical(gpu, oracle, cluster_ctx, n, B, cells, mode):
    cluster_ctx.set_cells_budget(0 if cells == "hash" else 16 << 30)
    _chain(gpu, oracle, n, B, 3000, mode, seed=70 + B)


@pytest.mark.parametrize("mode", ["greedy", "hastings"])
def test_cluster_chain_hashed_100k_blocks(gpu, oracle, cluster_ctx, mode):
    """Hashed cells at 100,000 blocks (the large-graph regime: 1.5 vertices per block)."""
    cluster_ctx.set_cells_budget(0)
    _chain(gpu, oracle, 150000, 100000, 20000, mode, seed=91)

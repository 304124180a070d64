"""The sequential phases on a thread-block cluster against the oracle's one-at-a-time forms.

The Metropolis-Hastings chain, evaluated in wide windows (one CTA per SM, 16 window entries
each), against finetune::propose_move / move_vertex (reference src/finetune.cpp:822-869):
the applied move count and the whole integer state after the chain are bit-exact.  Cells
dense in global memory or hashed (a zero dense budget); greedy, Hastings-corrected and
nonparametric acceptance; block counts from a few hundred, where conflicts end most
windows early, to 100,000, where windows are taken whole.  The merge carry-out follows
below."""
import numpy as np
import pytest

from test_gpu_parity import make_pair, same_state

pytestmark = pytest.mark.gpu


@pytest.fixture
def cluster_ctx(gpu):
    ctx = gpu.core.default_context()
    ctx.set_cluster_blocks(0)
    yield ctx
    ctx.set_cluster_blocks(65536)
    ctx.set_chain_cluster_blocks(129)
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


# ---- the exact merge carry-out on a cluster (block_merge::carry_out_best_merges_advanced,
# reference src/block_merge.cpp:40-117): up to 256 queue entries re-scored per round, the
# pop / put-back / merge rule replayed on one thread, exact conflict masks from per-block
# reader lists.  The merges, every put-back and the state after the pass are bit-exact.

def _merge(gpu, oracle, n, e, B, nmerge, seed, np_mode=False, identity=False):
    G, O, gb, ob, a, _ = make_pair(gpu, oracle, n, e, 9, B, seed=seed,
                                   assignment=np.arange(n) if identity else None)
    args = gpu.Args(seed=21, nonparametric=np_mode)
    gpu.block_merge.merge_blocks(gb, G, args=args, step=5, num_blocks_to_merge=nmerge)
    ob.merge_blocks(oracle.make_config(nonparametric=np_mode), seed=21, step=5, num_to_merge=nmerge)
    assert gb.num_blocks() == B - nmerge == ob.num_blocks
    same_state(gb, ob)


@pytest.mark.parametrize("cells", ["dense", "hash"])
@pytest.mark.parametrize("np_mode", [False, True])
@pytest.mark.parametrize("B,frac", [(3000, 0.5), (400, 0.5), (60, 0.5), (9000, 0.9)])
def test_cluster_carry_identical(gpu, oracle, cluster_ctx, B, frac, cells, np_mode):
    cluster_ctx.set_cells_budget(0 if cells == "hash" else 16 << 30)
    n = max(B, 3000)
    _merge(gpu, oracle, n, 12 * n, B, int(B * frac), seed=80 + B, np_mode=np_mode, identity=B == n)


def test_cluster_carry_hashed_200k_blocks(gpu, oracle, cluster_ctx):
    """The first merge pass of a 200,000-vertex graph: singleton blocks, hashed cells,
    100,000 merges."""
    cluster_ctx.set_cells_budget(0)
    _merge(gpu, oracle, 200000, 2400000, 200000, 100000, seed=93, identity=True)

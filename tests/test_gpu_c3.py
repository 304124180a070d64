"""The large high-overlap configuration (1,000,000 vertices, about 20M edges, 100 planted
blocks of Dirichlet(0.5) sizes, degrees 2.1 in [5, 500], within:between 1.5): the first
golden-section step of sbp::stochastic_block_partition (reference src/sbp.cpp:23-35) on the
device against the oracle, bit-exact.

The step starts from the 1,000,000-block identity partition.  The merge pass to 500,000
blocks runs the proposal kernel, then the exact carry-out on a thread-block cluster with
hashed cells (a dense 10^12-cell matrix is out of reach); the hybrid MCMC that follows runs
its high-degree chain on a cluster with hashed cells and its Gibbs batches on the whole
device.  After each phase the whole integer state (assignment, block degrees, sizes,
blockmatrix) must equal the oracle's, and the MDL its canonical value within 1e-12.  The
oracle needs about two minutes of the host's cores for the step."""
import numpy as np
import pytest

from test_gpu_parity import MDL_REL_TOL_CANONICAL, same_state

pytestmark = pytest.mark.gpu


def test_c3_first_golden_section_step(gpu, oracle):
    src, dst, _ = gpu.dcsbm.generate_config("C3", seed=0)
    n = gpu.dcsbm.CONFIGS["C3"]["num_vertices"]
    ident = np.arange(n, dtype=np.int32)
    G = gpu.Graph(n, src, dst)
    O = oracle.Graph(n, src, dst)
    gb = gpu.Blockmodel(n, G, 0.5, ident)
    ob = oracle.Blockmodel(O, n, ident)
    args = gpu.Args(algorithm="hybrid_mcmc", seed=1)
    cfg = oracle.make_config("hybrid_mcmc")
    _, st = gpu.block_merge.merge_blocks(gb, G, args=args, step=0, num_blocks_to_merge=n // 2)
    ob.merge_blocks(cfg, seed=1, step=0, num_to_merge=n // 2)
    assert st["merges"] == n // 2
    assert gb.num_blocks() == n - n // 2 == ob.num_blocks
    same_state(gb, ob)
    _, st = gpu.finetune.mcmc(0, G, gb, True, args)
    ost = ob.mcmc(cfg, seed=1, step=0, golden_ratio_not_reached=True)
    assert st["mcmc_iterations"] == ost.mcmc_iterations
    assert st["proposals"] == ost.proposals
    same_state(gb, ob)
    can = ob.mdl()[1]
    assert abs(gb.getOverall_entropy() - can) <= MDL_REL_TOL_CANONICAL * abs(can)

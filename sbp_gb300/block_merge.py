"""block_merge:: namespace of the reference (include/block_merge.hpp:32-56) on the device."""
import ctypes

import numpy as np

from ._lib import Stats, i32p, f64p
from .core import Args

NUM_AGG_PROPOSALS_PER_BLOCK = 10  # include/block_merge.hpp:23


def _p(a, t):
    return a.ctypes.data_as(t)


def merge_blocks(blockmodel, graph=None, num_edges=None, args=None, step=0, num_blocks_to_merge=None):
    """block_merge::merge_blocks (src/block_merge.cpp:178-228): merges
    blockmodel.num_blocks_to_merge blocks and rebuilds the blockmodel.
    Returns (blockmodel, stats dict)."""
    a = args or Args()
    cfg = a.config()
    n = blockmodel.num_blocks_to_merge if num_blocks_to_merge is None else int(num_blocks_to_merge)
    st = Stats()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_merge_blocks(blockmodel.h, ctypes.byref(cfg), int(a.seed),
                                                                int(step), n, ctypes.byref(st)))
    blockmodel.num_blocks_to_merge = int(blockmodel.num_blocks() * blockmodel.block_reduction_rate)
    return blockmodel, st.as_dict()


def merge_proposals(blockmodel, seed, step):
    """The per-block best proposals of block_merge::merge_blocks (src/block_merge.cpp:189-217)."""
    B = blockmodel.num_blocks()
    best = np.zeros(B, np.int32)
    dS = np.zeros(B, np.float64)
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_merge_proposals(blockmodel.h, int(seed), int(step),
                                                                   _p(best, i32p), _p(dS, f64p)))
    return best, dS

"""divisive:: namespace of the reference (include/top_down_sbp.hpp, src/top_down_sbp.cpp):
top-down partitioning by cluster splits, on the device."""
import ctypes

import numpy as np

from ._lib import Stats, i32p
from .core import Args


def split_communities(blockmodel, graph=None, target_num_communities=None, args=None, step=0):
    """divisive::split_communities (src/top_down_sbp.cpp:472-530) with --split random."""
    a = args or Args()
    cfg = a.config()
    if target_num_communities is None:
        raise ValueError("target_num_communities is required")
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_split_communities(blockmodel.h, ctypes.byref(cfg), int(a.seed),
                                                                     int(step), int(target_num_communities)))
    return blockmodel


def run(graph, args=None):
    """divisive::run (src/top_down_sbp.cpp:435-470); args.mix continues agglomeratively
    once the bracket forms (continue_agglomerative, :67-98).

    Returns (assignment, num_blocks, mdl, stats dict)."""
    a = args or Args()
    cfg = a.config()
    out = np.zeros(graph.num_vertices(), np.int32)
    B = ctypes.c_int64()
    mdl = ctypes.c_double()
    st = Stats()
    graph.ctx.check(graph.ctx.lib.sbpgpu_sbp_top_down(graph.h, ctypes.byref(cfg), int(a.seed), int(bool(a.mix)),
                                                      out.ctypes.data_as(i32p), ctypes.byref(B), ctypes.byref(mdl),
                                                      ctypes.byref(st)))
    return out, int(B.value), float(mdl.value), st.as_dict()

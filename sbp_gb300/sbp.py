"""sbp:: namespace of the reference (include/sbp.hpp:18-21) on the device."""
import ctypes

import numpy as np

from ._lib import Stats, i32p
from .core import Args


def stochastic_block_partition(graph, args=None, divide_and_conquer=False):
    """sbp::stochastic_block_partition (src/sbp.cpp:16-72): agglomerative golden-section
    search with block merges and MCMC finetuning, all on the device.

    Returns (assignment, num_blocks, mdl, stats dict)."""
    if divide_and_conquer:
        raise NotImplementedError("divide-and-conquer SBP is outside the device hot path")
    a = args or Args()
    cfg = a.config()
    out = np.zeros(graph.num_vertices(), np.int32)
    B = ctypes.c_int64()
    mdl = ctypes.c_double()
    st = Stats()
    graph.ctx.check(graph.ctx.lib.sbpgpu_sbp(graph.h, ctypes.byref(cfg), int(a.seed), out.ctypes.data_as(i32p),
                                             ctypes.byref(B), ctypes.byref(mdl), ctypes.byref(st)))
    return out, int(B.value), float(mdl.value), st.as_dict()

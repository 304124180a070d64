"""entropy:: namespace of the reference (include/entropy.hpp:33-81) on the device."""
import ctypes

import numpy as np

from ._lib import i32p, f64p


def _p(a, t):
    return a.ctypes.data_as(t)


def mdl(blockmodel, graph=None):
    """entropy::mdl (src/entropy.cpp:597-604)."""
    out = ctypes.c_double()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_mdl(blockmodel.h, ctypes.byref(out)))
    return out.value


def delta_mdl(blockmodel, vertices, proposals):
    """entropy::delta_mdl(Blockmodel, Delta, proposal) (src/entropy.cpp:298-403) for the moves
    vertices[i] -> proposals[i]; returns a float64 array."""
    v = np.ascontiguousarray(np.atleast_1d(vertices), dtype=np.int32)
    s = np.ascontiguousarray(np.atleast_1d(proposals), dtype=np.int32)
    if v.shape != s.shape:
        raise ValueError("vertices and proposals must have the same length")
    out = np.zeros(v.size, np.float64)
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_delta_mdl_batch(blockmodel.h, v.size, _p(v, i32p), _p(s, i32p),
                                                                   _p(out, f64p)))
    return out


def block_merge_delta_mdl(blockmodel, blocks, proposals):
    """entropy::block_merge_delta_mdl (src/entropy.cpp:129-182) for merges blocks[i] -> proposals[i]."""
    r = np.ascontiguousarray(np.atleast_1d(blocks), dtype=np.int32)
    s = np.ascontiguousarray(np.atleast_1d(proposals), dtype=np.int32)
    if r.shape != s.shape:
        raise ValueError("blocks and proposals must have the same length")
    out = np.zeros(r.size, np.float64)
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_merge_delta_mdl_batch(blockmodel.h, r.size, _p(r, i32p),
                                                                         _p(s, i32p), _p(out, f64p)))
    return out


class nonparametric:
    """entropy::nonparametric (src/entropy.cpp:617-1225, include/entropy.hpp:101-190) on the
    device, for a directed graph without degree correction."""

    @staticmethod
    def mdl(blockmodel, graph=None):
        """nonparametric::mdl (src/entropy.cpp:751-779)."""
        out = ctypes.c_double()
        blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_np_mdl(blockmodel.h, ctypes.byref(out)))
        return out.value

    @staticmethod
    def delta_mdl(blockmodel, vertices, proposals):
        """nonparametric::delta_mdl (src/entropy.cpp:1146-1178) for vertices[i] -> proposals[i]."""
        v = np.ascontiguousarray(np.atleast_1d(vertices), dtype=np.int32)
        s = np.ascontiguousarray(np.atleast_1d(proposals), dtype=np.int32)
        if v.shape != s.shape:
            raise ValueError("vertices and proposals must have the same length")
        out = np.zeros(v.size, np.float64)
        blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_np_delta_mdl_batch(blockmodel.h, v.size, _p(v, i32p),
                                                                          _p(s, i32p), _p(out, f64p)))
        return out

    @staticmethod
    def block_merge_delta_mdl(blockmodel, blocks, proposals):
        """nonparametric::block_merge_delta_mdl (src/entropy.cpp:1198-1223)."""
        r = np.ascontiguousarray(np.atleast_1d(blocks), dtype=np.int32)
        s = np.ascontiguousarray(np.atleast_1d(proposals), dtype=np.int32)
        if r.shape != s.shape:
            raise ValueError("blocks and proposals must have the same length")
        out = np.zeros(r.size, np.float64)
        blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_np_merge_delta_mdl_batch(blockmodel.h, r.size, _p(r, i32p),
                                                                                _p(s, i32p), _p(out, f64p)))
        return out


def null_mdl_v1(num_edges):
    """entropy::null_mdl_v1 (src/entropy.cpp:571-585) for the parametric entropy."""
    E = float(num_edges)
    log_posterior_p = E * np.log(1.0 / E)
    x = 1.0 / E
    h = ((1 + x) * np.log(1 + x)) - (x * np.log(x))
    return (E * h) - log_posterior_p


def normalize_mdl_v1(mdl_value, graph):
    """entropy::normalize_mdl_v1 (src/entropy.cpp:563-565)."""
    return mdl_value / null_mdl_v1(graph.num_edges())

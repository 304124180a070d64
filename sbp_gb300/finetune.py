"""finetune:: namespace of the reference (include/finetune.hpp:36-157) on the device."""
import ctypes

import numpy as np

from ._lib import Stats, i32p, i64p
from .core import Args

DOM_GIBBS, DOM_MH, DOM_MERGE = 1, 2, 3


def _p(a, t):
    return a.ctypes.data_as(t)


def _cfg(args):
    return (args or Args()).config()


def mcmc(iteration, graph, blockmodel, golden_ratio_not_reached=True, args=None):
    """finetune::mcmc (src/finetune.cpp:754-771); mutates and returns blockmodel.
    Returns (blockmodel, stats dict)."""
    a = args or Args()
    cfg = a.config()
    st = Stats()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_mcmc(blockmodel.h, ctypes.byref(cfg), int(a.seed), int(iteration),
                                                        int(bool(golden_ratio_not_reached)), ctypes.byref(st)))
    return blockmodel, st.as_dict()


def asynchronous_gibbs(blockmodel, graph, golden_ratio_not_reached=True, args=None, iteration=0):
    """finetune::asynchronous_gibbs (src/finetune.cpp:34-107)."""
    a = Args(**{**(args or Args()).__dict__, "algorithm": "async_gibbs"})
    return mcmc(iteration, graph, blockmodel, golden_ratio_not_reached, a)


def hybrid_mcmc(blockmodel, graph, golden_ratio_not_reached=True, args=None, iteration=0):
    """finetune::hybrid_mcmc (src/finetune.cpp:563-646)."""
    a = Args(**{**(args or Args()).__dict__, "algorithm": "hybrid_mcmc"})
    return mcmc(iteration, graph, blockmodel, golden_ratio_not_reached, a)


def metropolis_hastings(blockmodel, graph, golden_ratio_not_reached=True, args=None, iteration=0):
    """finetune::metropolis_hastings (src/finetune.cpp:773-820)."""
    a = Args(**{**(args or Args()).__dict__, "algorithm": "metropolis_hastings"})
    return mcmc(iteration, graph, blockmodel, golden_ratio_not_reached, a)


def propose_new_blocks(blockmodel, vertices, seed, c1, c2, c3=DOM_GIBBS):
    """common::propose_new_block for each vertex under the canonical stream counter
    (vertex, c1, c2, c3) (src/common.cpp:138-198)."""
    v = np.ascontiguousarray(np.atleast_1d(vertices), dtype=np.int32)
    out = np.zeros(v.size, np.int32)
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_propose_batch(blockmodel.h, v.size, _p(v, i32p), int(seed),
                                                                 int(c1), int(c2), int(c3), _p(out, i32p)))
    return out


def gibbs_batch(blockmodel, vertices, seed, iteration, step, args=None):
    """One asynchronous-Gibbs batch: propose_gibbs_move_v3 for every vertex against one
    snapshot, then Blockmodel::move_vertex(VertexMove_v3) in vertex-id order.
    Returns (accepted proposals per vertex or -1, number of applied moves)."""
    cfg = _cfg(args)
    v = np.ascontiguousarray(np.atleast_1d(vertices), dtype=np.int32)
    moves = np.zeros(v.size, np.int32)
    applied = ctypes.c_int64()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_gibbs_batch(blockmodel.h, ctypes.byref(cfg), v.size, _p(v, i32p),
                                                               int(seed), int(iteration), int(step), _p(moves, i32p),
                                                               ctypes.byref(applied)))
    return moves, applied.value


def propose_gibbs_moves(blockmodel, vertices, seed, iteration, step, args=None):
    """finetune::propose_gibbs_move_v3 (src/finetune.cpp:871-901) for every vertex against
    the current state, nothing applied: the accepted proposal of each, or -1."""
    cfg = _cfg(args)
    v = np.ascontiguousarray(np.atleast_1d(vertices), dtype=np.int32)
    moves = np.zeros(v.size, np.int32)
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_gibbs_propose(blockmodel.h, ctypes.byref(cfg), v.size,
                                                                 _p(v, i32p), int(seed), int(iteration), int(step),
                                                                 _p(moves, i32p)))
    return moves


def mh_chain(blockmodel, vertices, seed, iteration, step, args=None):
    """finetune::propose_move over vertices in order, each accepted move applied at once
    (src/finetune.cpp:842-869).  Returns the number of applied moves."""
    cfg = _cfg(args)
    v = np.ascontiguousarray(np.atleast_1d(vertices), dtype=np.int32)
    applied = ctypes.c_int64()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_mh_chain(blockmodel.h, ctypes.byref(cfg), v.size, _p(v, i32p),
                                                            int(seed), int(iteration), int(step),
                                                            ctypes.byref(applied)))
    return applied.value


def propose_move(blockmodel, vertex, graph=None, args=None, iteration=0, step=0):
    """finetune::propose_move (src/finetune.cpp:842-869): the canonical MH proposal for one
    vertex, scored and accepted as the chain does, applied when accepted.  Returns the
    reference's VertexMove as (delta_entropy, did_move, vertex, proposed_block); vertex and
    block are -1 when nothing was proposed."""
    a = args or Args()
    cfg = a.config()
    prop = ctypes.c_int32()
    dS = ctypes.c_double()
    moved = ctypes.c_int32()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_propose_move(blockmodel.h, ctypes.byref(cfg), int(vertex),
                                                                int(a.seed), int(iteration), int(step),
                                                                ctypes.byref(prop), ctypes.byref(dS),
                                                                ctypes.byref(moved)))
    p = prop.value
    return dS.value, bool(moved.value), (int(vertex) if p >= 0 else -1), p


def move_vertex(vertex, proposal, blockmodel, graph=None, args=None, iteration=0, step=0):
    """finetune::move_vertex (src/finetune.cpp:822-840) for a given proposal.  Returns
    (delta_entropy, did_move, vertex, proposed_block)."""
    a = args or Args()
    cfg = a.config()
    dS = ctypes.c_double()
    moved = ctypes.c_int32()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_move_vertex(blockmodel.h, ctypes.byref(cfg), int(vertex),
                                                               int(proposal), int(a.seed), int(iteration), int(step),
                                                               ctypes.byref(dS), ctypes.byref(moved)))
    return dS.value, bool(moved.value), int(vertex), int(proposal)


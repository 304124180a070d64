"""sample:: namespace of the reference (include/sample.hpp, src/sample.cpp) and the sampled
partition of src/main.cpp:98-140, on the device."""
import ctypes
import dataclasses

import numpy as np

from . import _lib
from ._lib import Stats, i32p, i64p
from .core import Args, Blockmodel, Graph

ALGORITHMS = {"max_degree": 0, "random": 1, "degree_product": 2, "detach": 3, "expansion_snowball": 4,
              "degree_product_snowball": 5}


@dataclasses.dataclass
class Sample:
    """sample::Sample: the sampled graph and mapping[v] = the vertex's id in it, or -1."""
    graph: Graph
    mapping: np.ndarray


def _alg(name):
    if name not in ALGORITHMS:
        raise ValueError("sampling algorithm must be one of %s" % sorted(ALGORITHMS))
    return ALGORITHMS[name]


def sample_mapping(graph, algorithm="random", sample_size=0.5, seed=0):
    """The vertex mapping of sample::sample with args.samplingalg = algorithm."""
    m = np.zeros(graph.num_vertices(), np.int32)
    n = ctypes.c_int64()
    graph.ctx.check(graph.ctx.lib.sbpgpu_sample(graph.h, _alg(algorithm), float(sample_size), int(seed),
                                                m.ctypes.data_as(i32p), ctypes.byref(n)))
    return m, int(n.value)


def from_vertices(graph, mapping):
    """sample::from_vertices (src/sample.cpp:240-253)."""
    m = np.ascontiguousarray(mapping, dtype=np.int32)
    n = int((m >= 0).sum())
    h = ctypes.c_void_p()
    graph.ctx.check(graph.ctx.lib.sbpgpu_graph_subgraph(graph.h, m.ctypes.data_as(i32p), n, ctypes.byref(h)))
    return Graph._adopt(h, graph.ctx)


def sample(graph, algorithm="random", sample_size=0.5, seed=0):
    """sample::sample (src/sample.cpp:328-341): the sample and its graph."""
    m, _ = sample_mapping(graph, algorithm, sample_size, seed)
    return Sample(from_vertices(graph, m), m)


def detach(graph):
    """sample::detach (src/sample.cpp:12-26): the vertices of degree above 1."""
    return sample(graph, "detach", 1.0)


def extend(graph, sample_assignment, num_blocks, smp, seed=0):
    """sample::extend (src/sample.cpp:159-199): the full graph's assignment."""
    a = np.ascontiguousarray(sample_assignment, dtype=np.int32)
    m = np.ascontiguousarray(smp.mapping, dtype=np.int32)
    out = np.zeros(graph.num_vertices(), np.int32)
    graph.ctx.check(graph.ctx.lib.sbpgpu_extend(graph.h, a.ctypes.data_as(i32p), a.size, int(num_blocks),
                                                m.ctypes.data_as(i32p), int(seed), out.ctypes.data_as(i32p)))
    return out


def reattach(graph, sample_assignment, num_blocks, smp, seed=0):
    """sample::reattach (src/sample.cpp:365-405): the full graph's assignment after a detach."""
    a = np.ascontiguousarray(sample_assignment, dtype=np.int32)
    m = np.ascontiguousarray(smp.mapping, dtype=np.int32)
    out = np.zeros(graph.num_vertices(), np.int32)
    graph.ctx.check(graph.ctx.lib.sbpgpu_reattach(graph.h, a.ctypes.data_as(i32p), a.size, int(num_blocks),
                                                  m.ctypes.data_as(i32p), int(seed), out.ctypes.data_as(i32p)))
    return out


def finetune_assignment(blockmodel, graph=None, args=None):
    """finetune::finetune_assignment (src/finetune.cpp:903-932); returns the stats dict."""
    a = args or Args()
    cfg = a.config()
    st = Stats()
    blockmodel.ctx.check(blockmodel.ctx.lib.sbpgpu_finetune_assignment(blockmodel.h, ctypes.byref(cfg), int(a.seed),
                                                                       ctypes.byref(st)))
    return st.as_dict()


def partition(graph, args=None):
    """main.cpp:82-150: with args.detach, vertices of degree 0 or 1 are set aside first and
    reattached at the end; the rest is partitioned whole (args.samplesize >= 1) or through
    a sample, extended and finetuned.

    Returns (assignment, num_blocks, mdl, stats dict)."""
    a = args or Args()
    if not a.samplesize > 0:
        raise ValueError("samplesize must be > 0")
    if a.detach:
        det = detach(graph)
        inner = dataclasses.replace(a, detach=False)
        sub_asg, B, _, st = partition(det.graph, inner)
        asg = reattach(graph, sub_asg, B, det, a.seed)
        bm = Blockmodel(B, graph, 0.5, asg)
        from . import entropy
        mdl = entropy.nonparametric.mdl(bm) if a.nonparametric else entropy.mdl(bm)
        return asg, B, mdl, st
    if a.samplesize >= 1.0:
        from .sbp import stochastic_block_partition
        return stochastic_block_partition(graph, a)
    cfg = a.config()
    out = np.zeros(graph.num_vertices(), np.int32)
    B = ctypes.c_int64()
    mdl = ctypes.c_double()
    st = Stats()
    graph.ctx.check(graph.ctx.lib.sbpgpu_sbp_sampled(graph.h, ctypes.byref(cfg), int(a.seed), _alg(a.samplingalg),
                                                     float(a.samplesize), out.ctypes.data_as(i32p), ctypes.byref(B),
                                                     ctypes.byref(mdl), ctypes.byref(st)))
    return out, int(B.value), float(mdl.value), st.as_dict()

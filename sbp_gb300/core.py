"""Host-side mirror of the reference's hot-path types: Args, Graph, Blockmodel.

Names, argument meaning and error behaviour follow vtsynergy/SBP
(include/args.hpp, include/graph.hpp, include/blockmodel/blockmodel.hpp); the state
lives on the GPU behind the libsbpgpu C ABI.  Invalid arguments raise ValueError /
IndexError like the reference's std::invalid_argument / IndexOutOfBoundsException.
"""
import atexit
import ctypes
import os
import dataclasses
import weakref

import numpy as np

from . import _lib
from ._lib import Config, Stats, check, i32p, i64p, f64p

ALGORITHMS = {"async_gibbs": 0, "hybrid_mcmc": 1, "metropolis_hastings": 2}
SPLITS = {"random": 0, "snowball": 1, "single-snowball": 2, "connectivity-snowball": 3}
SPLIT_INITS = {"random": 0, "degree-weighted": 1, "high-degree": 2}


@dataclasses.dataclass
class Args:
    """The hot-path subset of the reference's Args (include/args.hpp:61-212)."""
    algorithm: str = "hybrid_mcmc"
    batches: int = 1
    mh_percent: float = 0.075
    greedy: bool = True
    ordered: bool = False
    approximate: bool = False
    asynciterations: int = 2**31 - 1
    threads: int = 1               # accepted for compatibility; the device uses all SMs
    nonparametric: bool = False    # entropy::nonparametric (directed, not degree-corrected)
    seed: int = 0                  # seeds the canonical proposal stream
    samplesize: float = 1.0        # --samplesize: below 1, partition a sample and extend it (main.cpp:98-140)
    samplingalg: str = "random"    # --samplingalg: random | max_degree | degree_product | *_snowball
    detach: bool = False           # --detach: set degree-0/1 vertices aside and reattach them
    mix: bool = False              # --mix: top-down, then agglomerative once the bracket forms
    split: str = "random"          # --split: random | snowball | single-snowball | connectivity-snowball
    splitinit: str = "random"      # --splitinit: random | degree-weighted | high-degree
    max_iterations: int = 100      # MAX_NUM_ITERATIONS (include/finetune.hpp:34)

    def config(self):
        if self.algorithm not in ALGORITHMS:
            raise ValueError("algorithm must be one of %s" % sorted(ALGORITHMS))
        if self.batches < 1:
            raise ValueError("batches must be >= 1")
        # --nonparametric sets greedy off (include/args.hpp:204-207)
        greedy = bool(self.greedy) and not self.nonparametric
        if self.split not in SPLITS or self.splitinit not in SPLIT_INITS:
            raise ValueError("split must be one of %s and splitinit one of %s" % (sorted(SPLITS), sorted(SPLIT_INITS)))
        return Config(ALGORITHMS[self.algorithm], int(self.batches), float(self.mh_percent), int(greedy),
                      int(bool(self.ordered)), int(bool(self.approximate)), int(self.asynciterations),
                      int(self.max_iterations), int(bool(self.nonparametric)), SPLITS[self.split],
                      SPLIT_INITS[self.splitinit])


class Context:
    """One CUDA device + stream; not thread-safe."""

    def __init__(self, device=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        st = self.lib.sbpgpu_ctx_create(int(device), ctypes.byref(h))
        if st != 0:
            raise _lib.SbpGpuError(st, "cannot create a CUDA context on device %d" % device)
        self.h = h
        self._graphs = weakref.WeakSet()

    def close(self):
        """Destroys the context after every graph (and blockmodel) created on it."""
        if getattr(self, "h", None):
            for g in list(self._graphs):
                g.close()
            self.lib.sbpgpu_ctx_destroy(self.h)
            self.h = None

    __del__ = close

    def check(self, status):
        check(status, self.h)

    def synchronize(self):
        self.check(self.lib.sbpgpu_ctx_synchronize(self.h))

    def set_timing(self, enabled):
        self.lib.sbpgpu_set_timing(self.h, int(bool(enabled)))

    def set_cells_budget(self, nbytes):
        """Device bytes the merge carry-out may use for dense cell counts (0: hashed store)."""
        self.check(self.lib.sbpgpu_ctx_set_cells_budget(self.h, int(nbytes)))

    def set_cluster_blocks(self, min_blocks):
        """Smallest block count at which the MH chain and the merge carry-out run on a
        thread-block cluster (defaults 129 and 65536; 0: always, the chain once there are
        more than 128 blocks); results do not depend on it."""
        self.check(self.lib.sbpgpu_ctx_set_cluster_blocks(self.h, int(min_blocks)))

    def set_chain_cluster_blocks(self, min_blocks):
        """The MH chain's threshold alone (default 129)."""
        self.check(self.lib.sbpgpu_ctx_set_chain_cluster_blocks(self.h, int(min_blocks)))

    def set_cancel(self, requested=True):
        """Requests (or withdraws) cancellation of the running partition on this context;
        it stops between golden-section steps with SBPGPU_ECANCELED.  Thread-safe."""
        self.check(self.lib.sbpgpu_ctx_set_cancel(self.h, int(bool(requested))))

    def inject_alloc_failure(self, after):
        """Test hook: device allocation number `after` + 1 from now fails as an out-of-memory
        allocation does; negative: none."""
        self.check(self.lib.sbpgpu_ctx_inject_alloc_failure(self.h, int(after)))

    def read_timing(self):
        t = _lib.KernelTiming()
        self.check(self.lib.sbpgpu_read_timing(self.h, ctypes.byref(t)))
        return t.as_dict()


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


@atexit.register
def _close_default_context():
    # Tear device state down while the CUDA runtime is still alive, children first.
    global _default_ctx
    if _default_ctx is not None:
        _default_ctx.close()
        _default_ctx = None


def load_partition(path, num_vertices):
    """The true partition of Graph::load (src/graph.cpp:54-69): "vertex block" per line,
    1-based; vertices without a line get -1."""
    a = np.full(int(num_vertices), -1, np.int32)
    with open(path) as f:
        for line in f:
            p = line.replace(",", " ").split()
            if len(p) >= 2 and not line.lstrip().startswith(("%", "#")):
                a[int(p[0]) - 1] = int(p[1]) - 1
    return a


def _p(a, t):
    return a.ctypes.data_as(t)


class Graph:
    """Directed multigraph in input edge order (Graph::add_edge, src/graph.cpp:10-18).

    num_edges: Graph::num_edges (include/graph.hpp:99), the count the description lengths
    use; the number of edges given by default.  Pass half of it for arrays that hold both
    directions of an undirected edge list, as the reference's loader counts them
    (src/graph.cpp:145-147).  undirected: args.undirected for the nonparametric entropy
    (include/sbpgpu.h, sbpgpu_graph_set_undirected).  degree_corrected: args.degreecorrected
    for the nonparametric description length and single-move deltas
    (sbpgpu_graph_set_degree_corrected)."""

    def __init__(self, num_vertices, src, dst, ctx=None, num_edges=None, undirected=False, degree_corrected=False):
        self.ctx = ctx or default_context()
        self.src = np.ascontiguousarray(src, dtype=np.int32)
        self.dst = np.ascontiguousarray(dst, dtype=np.int32)
        if self.src.shape != self.dst.shape or self.src.ndim != 1:
            raise ValueError("src and dst must be 1-D arrays of equal length")
        self._N = int(num_vertices)
        if self.src.size and (min(self.src.min(), self.dst.min()) < 0 or
                              max(self.src.max(), self.dst.max()) >= self._N):
            raise IndexError("edge endpoint out of range")
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sbpgpu_graph_create(self.ctx.h, self._N, int(self.src.size),
                                                        _p(self.src, i32p), _p(self.dst, i32p), ctypes.byref(h)))
        self.h = h
        self._bms = weakref.WeakSet()
        self.ctx._graphs.add(self)
        if num_edges is not None:
            self.ctx.check(self.ctx.lib.sbpgpu_graph_set_model_edges(self.h, int(num_edges)))
        if undirected:
            self.ctx.check(self.ctx.lib.sbpgpu_graph_set_undirected(self.h, 1))
        if degree_corrected:
            self.ctx.check(self.ctx.lib.sbpgpu_graph_set_degree_corrected(self.h, 1))

    @classmethod
    def _adopt(cls, handle, ctx):
        """A Graph object for a graph the library built (edge arrays not kept on the host)."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.h = handle
        self._N = int(ctx.lib.sbpgpu_graph_num_vertices(handle))
        self.src = self.dst = None
        self._E = int(ctx.lib.sbpgpu_graph_num_edges(handle))
        self._bms = weakref.WeakSet()
        ctx._graphs.add(self)
        return self

    @classmethod
    def load(cls, path, undirected=False, ctx=None):
        """Graph::load (src/graph.cpp:33-233): a TSV edge list or a Matrix Market file parsed
        on the device (include/sbpgpu.h, sbpgpu_graph_load).  The edge arrays are not kept
        on the host."""
        self = cls.__new__(cls)
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sbpgpu_graph_load(self.ctx.h, os.fsencode(path), int(bool(undirected)),
                                                      ctypes.byref(h)))
        self.h = h
        self._N = int(self.ctx.lib.sbpgpu_graph_num_vertices(h))
        self.src = self.dst = None
        self._E = int(self.ctx.lib.sbpgpu_graph_num_edges(h))
        self._bms = weakref.WeakSet()
        self.ctx._graphs.add(self)
        return self

    def close(self):
        """Destroys the graph after every blockmodel built on it (finalisers may run in any
        order when objects are collected together)."""
        if getattr(self, "h", None):
            for bm in list(self._bms):
                bm.close()
            self.ctx.lib.sbpgpu_graph_destroy(self.h)
            self.h = None

    __del__ = close

    def num_vertices(self):
        return self._N

    def num_edges(self):
        """Graph::num_edges: the count the description lengths use (half the stored edges
        for an undirected edge list)."""
        return int(self.ctx.lib.sbpgpu_graph_model_edges(self.h))

    def undirected(self):
        """args.undirected as the nonparametric entropy reads it."""
        return bool(self.ctx.lib.sbpgpu_graph_undirected(self.h))

    def degree_corrected(self):
        """args.degreecorrected as the nonparametric description length reads it."""
        return bool(self.ctx.lib.sbpgpu_graph_degree_corrected(self.h))

    def num_stored_edges(self):
        """The directed edges stored (the length of the edge arrays)."""
        return self._E if self.src is None else int(self.src.size)

    def out_neighbors(self, v):
        return self.dst[self.src == v]

    def in_neighbors(self, v):
        return self.src[self.dst == v]


class Blockmodel:
    """Blockmodel(num_blocks, graph, block_reduction_rate, assignment) (blockmodel.hpp:82-88)."""

    def __init__(self, num_blocks, graph, block_reduction_rate=0.5, assignment=None, _handle=None):
        self.graph = graph
        self.ctx = graph.ctx
        self.block_reduction_rate = block_reduction_rate
        self.num_blocks_to_merge = 0
        if _handle is not None:
            self.h = _handle
            graph._bms.add(self)
            return
        h = ctypes.c_void_p()
        if assignment is None:
            ptr = None
            if num_blocks != graph.num_vertices():
                raise ValueError("without an assignment num_blocks must equal the number of vertices")
        else:
            a = np.ascontiguousarray(assignment, dtype=np.int32)
            if a.shape != (graph.num_vertices(),):
                raise ValueError("assignment must hold one block per vertex")
            if a.size and (a.min() < 0 or a.max() >= num_blocks):
                raise IndexError("assignment value out of range")
            ptr = _p(a, i32p)
        self.ctx.check(self.ctx.lib.sbpgpu_bm_create(graph.h, int(num_blocks), ptr, ctypes.byref(h)))
        self.h = h
        graph._bms.add(self)
        self.num_blocks_to_merge = int(num_blocks * block_reduction_rate)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sbpgpu_bm_destroy(self.h)
            self.h = None

    __del__ = close

    def copy(self):
        """Blockmodel::copy (blockmodel.cpp:139-153): device-to-device."""
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sbpgpu_bm_copy(self.h, ctypes.byref(h)))
        return Blockmodel(0, self.graph, self.block_reduction_rate, _handle=h)

    def num_blocks(self):
        return int(self.ctx.lib.sbpgpu_bm_num_blocks(self.h))

    def nnz(self):
        return int(self.ctx.lib.sbpgpu_bm_nnz(self.h))

    def getOverall_entropy(self):
        return float(self.ctx.lib.sbpgpu_bm_entropy(self.h))

    def read(self):
        B, nnz, N = self.num_blocks(), self.nnz(), self.graph.num_vertices()
        a = np.zeros(N, np.int32)
        dout, din, dtot, sizes = (np.zeros(B, np.int64) for _ in range(4))
        rows, cols = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32)
        cnt = np.zeros(nnz, np.int64)
        self.ctx.check(self.ctx.lib.sbpgpu_bm_read(self.h, _p(a, i32p), _p(dout, i64p), _p(din, i64p),
                                                   _p(dtot, i64p), _p(sizes, i64p), _p(rows, i32p), _p(cols, i32p),
                                                   _p(cnt, i64p)))
        return dict(assignment=a, d_out=dout, d_in=din, d_tot=dtot, sizes=sizes, rows=rows, cols=cols, counts=cnt)

    # accessors named as in blockmodel.hpp
    def block_assignment(self):
        a = np.zeros(self.graph.num_vertices(), np.int32)
        self.ctx.check(self.ctx.lib.sbpgpu_bm_read(self.h, _p(a, i32p), None, None, None, None, None, None, None))
        return a

    def degrees_out(self):
        return self.read()["d_out"]

    def degrees_in(self):
        return self.read()["d_in"]

    def degrees(self):
        return self.read()["d_tot"]

    def block_sizes(self):
        return self.read()["sizes"]

    def blockmatrix(self):
        """Dense copy of the block-edge-count matrix (small B only)."""
        d = self.read()
        B = self.num_blocks()
        M = np.zeros((B, B), np.int64)
        M[d["rows"], d["cols"]] = d["counts"]
        return M

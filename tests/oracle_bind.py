"""ctypes binding of the CPU oracle (oracle/libsbp_oracle.so) for the test-suite.

The oracle is test infrastructure: only tests, ``__graft_entry__.smoke`` and the
CPU-baseline leg of ``bench.py`` load it, and only as the checker / baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "libsbp_oracle.so")

i32p = ctypes.POINTER(ctypes.c_int32)
i64p = ctypes.POINTER(ctypes.c_int64)
u32p = ctypes.POINTER(ctypes.c_uint32)
f64p = ctypes.POINTER(ctypes.c_double)


class OraConfig(ctypes.Structure):
    _fields_ = [
        ("algorithm", ctypes.c_int32),
        ("batches", ctypes.c_int32),
        ("mh_percent", ctypes.c_float),
        ("greedy", ctypes.c_int32),
        ("ordered", ctypes.c_int32),
        ("approximate", ctypes.c_int32),
        ("asynciterations", ctypes.c_int32),
        ("max_iterations", ctypes.c_int32),
        ("nonparametric", ctypes.c_int32),
        ("split", ctypes.c_int32),
        ("splitinit", ctypes.c_int32),
    ]


SPLITS = {"random": 0, "snowball": 1, "single-snowball": 2, "connectivity-snowball": 3}
SPLIT_INITS = {"random": 0, "degree-weighted": 1, "high-degree": 2}


class OraStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "proposals", "merge_proposals", "moves", "mcmc_iterations", "merges", "edges_swept", "outer_steps")]


ALGORITHMS = {"async_gibbs": 0, "hybrid_mcmc": 1, "metropolis_hastings": 2}


def make_config(algorithm="hybrid_mcmc", batches=1, mh_percent=0.075, greedy=True, ordered=False,
                approximate=False, asynciterations=2**31 - 1, max_iterations=100, nonparametric=False,
                split="random", splitinit="random"):
    return OraConfig(ALGORITHMS[algorithm], batches, mh_percent, int(greedy), int(ordered),
                     int(approximate), asynciterations, max_iterations, int(nonparametric), SPLITS[split],
                     SPLIT_INITS[splitinit])


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.ora_philox.argtypes = [u32p, u32p, u32p]
        L.ora_graph_create.restype = ctypes.c_void_p
        L.ora_graph_create.argtypes = [ctypes.c_int64, ctypes.c_int64, i32p, i32p]
        L.ora_graph_destroy.argtypes = [ctypes.c_void_p]
        L.ora_bm_create.restype = ctypes.c_void_p
        L.ora_bm_create.argtypes = [ctypes.c_void_p, ctypes.c_int64, i32p]
        L.ora_bm_copy.restype = ctypes.c_void_p
        L.ora_bm_copy.argtypes = [ctypes.c_void_p]
        L.ora_bm_destroy.argtypes = [ctypes.c_void_p]
        L.ora_bm_num_blocks.restype = ctypes.c_int64
        L.ora_bm_num_blocks.argtypes = [ctypes.c_void_p]
        L.ora_bm_nnz.restype = ctypes.c_int64
        L.ora_bm_nnz.argtypes = [ctypes.c_void_p]
        L.ora_bm_read.argtypes = [ctypes.c_void_p, i32p, i64p, i64p, i64p, i64p, i32p, i32p, i64p]
        L.ora_bm_get.restype = ctypes.c_int64
        L.ora_bm_get.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64]
        L.ora_mdl.argtypes = [ctypes.c_void_p, f64p, f64p]
        L.ora_delta_mdl.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, f64p, i64p]
        L.ora_merge_delta_mdl.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, f64p, i64p]
        for fn in (L.ora_vertex_delta, L.ora_merge_delta):
            fn.restype = ctypes.c_int64
            fn.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, i32p, i32p, i64p, ctypes.c_int64]
        L.ora_propose_vertex.restype = ctypes.c_int64
        L.ora_propose_vertex.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint32,
                                         ctypes.c_uint32, ctypes.c_uint32]
        L.ora_propose_merge.restype = ctypes.c_int64
        L.ora_propose_merge.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.c_int32]
        L.ora_gibbs_batch.restype = ctypes.c_int64
        L.ora_gibbs_batch.argtypes = [ctypes.c_void_p, i32p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint32,
                                      ctypes.c_uint32, ctypes.POINTER(OraConfig), i32p, f64p]
        L.ora_apply_moves.restype = ctypes.c_int64
        L.ora_apply_moves.argtypes = [ctypes.c_void_p, i32p]
        L.ora_step_sample.argtypes = [ctypes.c_void_p, i32p, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint8),
                                      ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(OraConfig), ctypes.c_int32,
                                      i64p]
        L.ora_merge_proposals.restype = ctypes.c_int64
        L.ora_merge_proposals.argtypes = [ctypes.c_void_p, i32p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_int32, i32p, f64p]
        L.ora_mh_chain.restype = ctypes.c_int64
        L.ora_mh_chain.argtypes = [ctypes.c_void_p, i32p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint32,
                                   ctypes.c_uint32, ctypes.POINTER(OraConfig)]
        L.ora_mcmc.restype = ctypes.c_int
        L.ora_mcmc.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraConfig), ctypes.c_uint64, ctypes.c_int32,
                               ctypes.c_int32, ctypes.POINTER(OraStats)]
        L.ora_merge_blocks.restype = ctypes.c_int
        L.ora_merge_blocks.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraConfig), ctypes.c_uint64,
                                       ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(OraStats)]
        L.ora_sbp.restype = ctypes.c_int64
        L.ora_sbp.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraConfig), ctypes.c_uint64, i32p, f64p,
                              ctypes.POINTER(OraStats)]
        L.ora_np_mdl.argtypes = [ctypes.c_void_p, f64p, f64p]
        L.ora_np_terms.argtypes = [ctypes.c_void_p, f64p]
        L.ora_np_delta_mdl.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, f64p, i64p]
        L.ora_np_merge_delta_mdl.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, f64p, i64p]
        L.ora_bm_nonempty.restype = ctypes.c_int64
        L.ora_bm_nonempty.argtypes = [ctypes.c_void_p]
        L.ora_sample.restype = ctypes.c_int64
        L.ora_sample.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_uint64, i32p]
        L.ora_subgraph.restype = ctypes.c_void_p
        L.ora_subgraph.argtypes = [ctypes.c_void_p, i32p, ctypes.c_int64]
        L.ora_graph_num_edges.restype = ctypes.c_int64
        L.ora_graph_num_edges.argtypes = [ctypes.c_void_p]
        L.ora_graph_model_edges.restype = ctypes.c_int64
        L.ora_graph_model_edges.argtypes = [ctypes.c_void_p]
        L.ora_graph_set_model_edges.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.ora_graph_set_undirected.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.ora_graph_set_degree_corrected.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.ora_log_q.restype = ctypes.c_double
        L.ora_log_q.argtypes = [ctypes.c_int64, ctypes.c_int64]
        L.ora_spence.restype = ctypes.c_double
        L.ora_spence.argtypes = [ctypes.c_double]
        L.ora_graph_edges.argtypes = [ctypes.c_void_p, i32p, i32p]
        L.ora_extend.argtypes = [ctypes.c_void_p, i32p, ctypes.c_int64, ctypes.c_int64, i32p, ctypes.c_uint64, i32p]
        L.ora_reattach.argtypes = [ctypes.c_void_p, i32p, ctypes.c_int64, ctypes.c_int64, i32p, ctypes.c_uint64, i32p]
        L.ora_finetune_assignment.restype = ctypes.c_int
        L.ora_finetune_assignment.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraConfig), ctypes.c_uint64,
                                              ctypes.POINTER(OraStats)]
        L.ora_sbp_sampled.restype = ctypes.c_int64
        L.ora_sbp_sampled.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraConfig), ctypes.c_uint64, ctypes.c_int32,
                                      ctypes.c_double, i32p, f64p, ctypes.POINTER(OraStats)]
        L.ora_split_communities.restype = ctypes.c_int
        L.ora_split_communities.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraConfig), ctypes.c_uint64,
                                            ctypes.c_uint32, ctypes.c_int64]
        L.ora_top_down.restype = ctypes.c_int64
        L.ora_top_down.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraConfig), ctypes.c_uint64, ctypes.c_int32, i32p,
                                   f64p, ctypes.POINTER(OraStats)]
        L.ora_null_mdl_v1.restype = ctypes.c_double
        L.ora_null_mdl_v1.argtypes = [ctypes.c_double]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().ora_philox(_p(c, u32p), _p(k, u32p), _p(out, u32p))
    return out


def log_q(n, k):
    return float(lib().ora_log_q(int(n), int(k)))


def spence(x):
    return float(lib().ora_spence(float(x)))


class Graph:
    """num_edges: the count the description lengths use (Graph::num_edges); the stored
    directed edges by default, half of them for an undirected edge list.  undirected:
    args.undirected for the nonparametric entropy.  degree_corrected: args.degreecorrected."""

    def __init__(self, num_vertices, src, dst, num_edges=None, undirected=False, degree_corrected=False):
        self.src = np.ascontiguousarray(src, dtype=np.int32)
        self.dst = np.ascontiguousarray(dst, dtype=np.int32)
        self.N = int(num_vertices)
        self.E = int(self.src.size)
        self.h = lib().ora_graph_create(self.N, self.E, _p(self.src, i32p), _p(self.dst, i32p))
        if num_edges is not None:
            lib().ora_graph_set_model_edges(self.h, int(num_edges))
        if undirected:
            lib().ora_graph_set_undirected(self.h, 1)
        if degree_corrected:
            lib().ora_graph_set_degree_corrected(self.h, 1)

    def model_edges(self):
        return int(lib().ora_graph_model_edges(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_graph_destroy(self.h)
            self.h = None


SAMPLERS = {"max_degree": 0, "random": 1, "degree_product": 2, "detach": 3, "expansion_snowball": 4,
            "degree_product_snowball": 5}


def sample(graph, algorithm, sample_size, seed):
    m = np.zeros(graph.N, np.int32)
    n = int(lib().ora_sample(graph.h, SAMPLERS[algorithm], float(sample_size), seed, _p(m, i32p)))
    return m, n


def subgraph_edges(graph, mapping):
    m = np.ascontiguousarray(mapping, dtype=np.int32)
    n = int((m >= 0).sum())
    h = lib().ora_subgraph(graph.h, _p(m, i32p), n)
    E = int(lib().ora_graph_num_edges(h))
    src, dst = np.zeros(E, np.int32), np.zeros(E, np.int32)
    lib().ora_graph_edges(h, _p(src, i32p), _p(dst, i32p))
    lib().ora_graph_destroy(h)
    return n, src, dst


def extend(graph, sample_assignment, num_blocks, mapping, seed):
    a = np.ascontiguousarray(sample_assignment, dtype=np.int32)
    m = np.ascontiguousarray(mapping, dtype=np.int32)
    out = np.zeros(graph.N, np.int32)
    lib().ora_extend(graph.h, _p(a, i32p), a.size, int(num_blocks), _p(m, i32p), seed, _p(out, i32p))
    return out


def reattach(graph, sample_assignment, num_blocks, mapping, seed):
    a = np.ascontiguousarray(sample_assignment, dtype=np.int32)
    m = np.ascontiguousarray(mapping, dtype=np.int32)
    out = np.zeros(graph.N, np.int32)
    lib().ora_reattach(graph.h, _p(a, i32p), a.size, int(num_blocks), _p(m, i32p), seed, _p(out, i32p))
    return out


def sbp_sampled(graph, cfg, seed, algorithm, sample_size):
    out = np.zeros(graph.N, np.int32)
    mdl = ctypes.c_double()
    st = OraStats()
    B = lib().ora_sbp_sampled(graph.h, ctypes.byref(cfg), seed, SAMPLERS[algorithm], float(sample_size),
                              _p(out, i32p), ctypes.byref(mdl), ctypes.byref(st))
    assert B > 0, B
    return out, int(B), mdl.value, st


def top_down(graph, cfg, seed, mix=False):
    out = np.zeros(graph.N, np.int32)
    mdl = ctypes.c_double()
    st = OraStats()
    B = lib().ora_top_down(graph.h, ctypes.byref(cfg), seed, int(mix), _p(out, i32p), ctypes.byref(mdl),
                           ctypes.byref(st))
    assert B > 0, B
    return out, int(B), mdl.value, st


class Blockmodel:
    def __init__(self, graph, num_blocks=None, assignment=None, _handle=None):
        self.graph = graph
        if _handle is not None:
            self.h = _handle
            return
        a = np.ascontiguousarray(assignment, dtype=np.int32)
        self.h = lib().ora_bm_create(graph.h, int(num_blocks), _p(a, i32p))

    def copy(self):
        return Blockmodel(self.graph, _handle=lib().ora_bm_copy(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_bm_destroy(self.h)
            self.h = None

    @property
    def num_blocks(self):
        return int(lib().ora_bm_num_blocks(self.h))

    def read(self):
        B = self.num_blocks
        nnz = int(lib().ora_bm_nnz(self.h))
        a = np.zeros(self.graph.N, np.int32)
        dout, din, dtot, sizes = (np.zeros(B, np.int64) for _ in range(4))
        rows, cols = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32)
        cnt = np.zeros(nnz, np.int64)
        lib().ora_bm_read(self.h, _p(a, i32p), _p(dout, i64p), _p(din, i64p), _p(dtot, i64p), _p(sizes, i64p),
                          _p(rows, i32p), _p(cols, i32p), _p(cnt, i64p))
        return dict(assignment=a, d_out=dout, d_in=din, d_tot=dtot, sizes=sizes, rows=rows, cols=cols, counts=cnt)

    def get(self, r, c):
        return int(lib().ora_bm_get(self.h, r, c))

    def mdl(self):
        lit, can = ctypes.c_double(), ctypes.c_double()
        lib().ora_mdl(self.h, ctypes.byref(lit), ctypes.byref(can))
        return lit.value, can.value

    def delta_mdl(self, vertex, proposal):
        lit, fx = ctypes.c_double(), ctypes.c_int64()
        lib().ora_delta_mdl(self.h, vertex, proposal, ctypes.byref(lit), ctypes.byref(fx))
        return lit.value, fx.value

    def merge_delta_mdl(self, block, proposal):
        lit, fx = ctypes.c_double(), ctypes.c_int64()
        lib().ora_merge_delta_mdl(self.h, block, proposal, ctypes.byref(lit), ctypes.byref(fx))
        return lit.value, fx.value

    def np_mdl(self):
        lit, can = ctypes.c_double(), ctypes.c_double()
        lib().ora_np_mdl(self.h, ctypes.byref(lit), ctypes.byref(can))
        return lit.value, can.value

    def np_terms(self):
        out = np.zeros(4, np.float64)
        lib().ora_np_terms(self.h, _p(out, f64p))
        return dict(sparse_entropy=out[0], partition_dl=out[1], degree_dl=out[2], edges_dl=out[3])

    def np_delta_mdl(self, vertex, proposal):
        lit, fx = ctypes.c_double(), ctypes.c_int64()
        lib().ora_np_delta_mdl(self.h, vertex, proposal, ctypes.byref(lit), ctypes.byref(fx))
        return lit.value, fx.value

    def np_merge_delta_mdl(self, block, proposal):
        lit, fx = ctypes.c_double(), ctypes.c_int64()
        lib().ora_np_merge_delta_mdl(self.h, block, proposal, ctypes.byref(lit), ctypes.byref(fx))
        return lit.value, fx.value

    def nonempty(self):
        return int(lib().ora_bm_nonempty(self.h))

    def _delta(self, fn, a, b):
        cap = 4096
        r, c, v = np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros(cap, np.int64)
        n = int(fn(self.h, a, b, _p(r, i32p), _p(c, i32p), _p(v, i64p), cap))
        return {(int(r[i]), int(c[i])): int(v[i]) for i in range(min(n, cap))}

    def vertex_delta(self, vertex, proposal):
        return self._delta(lib().ora_vertex_delta, vertex, proposal)

    def merge_delta(self, block, proposal):
        return self._delta(lib().ora_merge_delta, block, proposal)

    def propose_vertex(self, vertex, seed, c1, c2, c3):
        return int(lib().ora_propose_vertex(self.h, vertex, seed, c1, c2, c3))

    def propose_merge(self, block, seed, step, index):
        return int(lib().ora_propose_merge(self.h, block, seed, step, index))

    def gibbs_batch(self, vertices, seed, iteration, step, cfg):
        v = np.ascontiguousarray(vertices, dtype=np.int32)
        moves = np.zeros(v.size, np.int32)
        dS = np.zeros(v.size, np.float64)
        n = lib().ora_gibbs_batch(self.h, _p(v, i32p), v.size, seed, iteration, step, ctypes.byref(cfg),
                                  _p(moves, i32p), _p(dS, f64p))
        return int(n), moves, dS

    def merge_proposals(self, blocks, seed, step, nonparametric=False):
        """Best merge proposal and delta of each listed block (the merge pass's proposal
        loop); returns (best, dS, draws)."""
        b = np.ascontiguousarray(blocks, np.int32)
        best = np.zeros(b.size, np.int32)
        dS = np.zeros(b.size, np.float64)
        draws = lib().ora_merge_proposals(self.h, _p(b, i32p), b.size, int(seed), int(step), int(bool(nonparametric)),
                                          _p(best, i32p), _p(dS, f64p))
        return best, dS, int(draws)

    def step_sample(self, blocks, hub, seed, step, cfg, sweeps):
        """A bounded sample of a golden-section step (merge proposals of the listed blocks,
        their carry-out to half as many merges, hybrid sweeps over the merged blocks'
        vertices); returns (proposals drawn, merges, vertex proposals)."""
        b = np.ascontiguousarray(blocks, np.int32)
        h = np.ascontiguousarray(hub, np.uint8)
        c = np.zeros(3, np.int64)
        lib().ora_step_sample(self.h, _p(b, i32p), b.size, h.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                              int(seed), int(step), ctypes.byref(cfg), int(sweeps), _p(c, i64p))
        return int(c[0]), int(c[1]), int(c[2])

    def apply_moves(self, moves_per_vertex):
        m = np.ascontiguousarray(moves_per_vertex, dtype=np.int32)
        return int(lib().ora_apply_moves(self.h, _p(m, i32p)))

    def mh_chain(self, order, seed, iteration, step, cfg):
        o = np.ascontiguousarray(order, dtype=np.int32)
        return int(lib().ora_mh_chain(self.h, _p(o, i32p), o.size, seed, iteration, step, ctypes.byref(cfg)))

    def mcmc(self, cfg, seed, step, golden_ratio_not_reached=True):
        st = OraStats()
        rc = lib().ora_mcmc(self.h, ctypes.byref(cfg), seed, step, int(golden_ratio_not_reached),
                            ctypes.byref(st))
        assert rc == 0
        return st

    def finetune_assignment(self, cfg, seed):
        st = OraStats()
        assert lib().ora_finetune_assignment(self.h, ctypes.byref(cfg), seed, ctypes.byref(st)) == 0
        return st

    def split_communities(self, cfg, seed, step, target):
        assert lib().ora_split_communities(self.h, ctypes.byref(cfg), seed, step, target) == 0

    def merge_blocks(self, cfg, seed, step, num_to_merge):
        st = OraStats()
        rc = lib().ora_merge_blocks(self.h, ctypes.byref(cfg), seed, step, num_to_merge, ctypes.byref(st))
        assert rc == 0, rc
        return st


def sbp(graph, cfg, seed):
    out = np.zeros(graph.N, np.int32)
    mdl = ctypes.c_double()
    st = OraStats()
    B = lib().ora_sbp(graph.h, ctypes.byref(cfg), seed, _p(out, i32p), ctypes.byref(mdl), ctypes.byref(st))
    assert B > 0, B
    return out, int(B), mdl.value, st


def null_mdl_v1(num_edges):
    return float(lib().ora_null_mdl_v1(float(num_edges)))

"""ctypes binding of libsbpgpu.so (declarations in include/sbpgpu.h).

The library is built in-tree by ``sbp_gb300.build.build()``; loading fails loudly when
it is missing -- there is no CPU fallback.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsbpgpu.so")

i32p = ctypes.POINTER(ctypes.c_int32)
i64p = ctypes.POINTER(ctypes.c_int64)
f64p = ctypes.POINTER(ctypes.c_double)
vp = ctypes.c_void_p

SBPGPU_OK = 0
SBPGPU_ENOMEM = 2
STATUS_NAMES = {0: "SBPGPU_OK", 1: "SBPGPU_EINVAL", 2: "SBPGPU_ENOMEM", 3: "SBPGPU_ETIMEOUT",
                4: "SBPGPU_EDEVICE", 5: "SBPGPU_EUNSUPPORTED", 6: "SBPGPU_ECANCELED"}


class Config(ctypes.Structure):
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


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "proposals", "merge_proposals", "moves", "mcmc_iterations", "merges", "edges_swept", "outer_steps",
        "kernel_launches", "gibbs_proposals", "gibbs_edges", "chain_rounds", "carry_rounds", "carry_evaluations",
        "carry_keys")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class KernelTiming(ctypes.Structure):
    _fields_ = [
        ("gibbs_propose_ms", ctypes.c_double), ("gibbs_propose_launches", ctypes.c_int64),
        ("gibbs_propose_bytes", ctypes.c_int64),
        ("mh_chain_ms", ctypes.c_double), ("mh_chain_launches", ctypes.c_int64),
        ("merge_propose_ms", ctypes.c_double), ("merge_propose_launches", ctypes.c_int64),
        ("merge_propose_bytes", ctypes.c_int64),
        ("carry_out_ms", ctypes.c_double), ("carry_out_launches", ctypes.c_int64),
        ("rebuild_ms", ctypes.c_double), ("rebuild_launches", ctypes.c_int64), ("rebuild_bytes", ctypes.c_int64),
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


# name -> (restype, argtypes); every symbol declared in include/sbpgpu.h.
class Eval(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("nmi", "f1", "precision", "recall", "rand_index", "accuracy")] + \
        [("true_blocks", ctypes.c_int64), ("found_blocks", ctypes.c_int64)]

    def as_dict(self):
        return {n: (float if t is ctypes.c_double else int)(getattr(self, n)) for n, t in self._fields_}


class Job(ctypes.Structure):
    _fields_ = [
        ("num_vertices", ctypes.c_int64), ("num_edges", ctypes.c_int64),
        ("src", ctypes.POINTER(ctypes.c_int32)), ("dst", ctypes.POINTER(ctypes.c_int32)),
        ("config", Config), ("seed", ctypes.c_uint64), ("out_assignment", ctypes.POINTER(ctypes.c_int32)),
    ]


class JobResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int), ("num_blocks", ctypes.c_int64), ("mdl", ctypes.c_double),
        ("queued_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("stats", Stats),
        ("error", ctypes.c_char * 256),
    ]


SIGNATURES = {
    "sbpgpu_default_config": (None, [ctypes.POINTER(Config)]),
    "sbpgpu_ctx_create": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(vp)]),
    "sbpgpu_ctx_destroy": (None, [vp]),
    "sbpgpu_last_error": (ctypes.c_char_p, [vp]),
    "sbpgpu_ctx_synchronize": (ctypes.c_int, [vp]),
    "sbpgpu_ctx_stream": (vp, [vp]),
    "sbpgpu_ctx_set_cells_budget": (ctypes.c_int, [vp, ctypes.c_int64]),
    "sbpgpu_ctx_set_cluster_blocks": (ctypes.c_int, [vp, ctypes.c_int64]),
    "sbpgpu_ctx_set_chain_cluster_blocks": (ctypes.c_int, [vp, ctypes.c_int64]),
    "sbpgpu_ctx_set_cancel": (ctypes.c_int, [vp, ctypes.c_int32]),
    "sbpgpu_ctx_inject_alloc_failure": (ctypes.c_int, [vp, ctypes.c_int64]),
    "sbpgpu_graph_create": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.c_int64, i32p, i32p, ctypes.POINTER(vp)]),
    "sbpgpu_graph_create_device": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.c_int64, vp, vp, ctypes.POINTER(vp)]),
    "sbpgpu_graph_load": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(vp)]),
    "sbpgpu_graph_destroy": (None, [vp]),
    "sbpgpu_graph_num_vertices": (ctypes.c_int64, [vp]),
    "sbpgpu_graph_num_edges": (ctypes.c_int64, [vp]),
    "sbpgpu_graph_model_edges": (ctypes.c_int64, [vp]),
    "sbpgpu_graph_set_model_edges": (ctypes.c_int, [vp, ctypes.c_int64]),
    "sbpgpu_graph_undirected": (ctypes.c_int32, [vp]),
    "sbpgpu_graph_set_undirected": (ctypes.c_int, [vp, ctypes.c_int32]),
    "sbpgpu_graph_degree_corrected": (ctypes.c_int32, [vp]),
    "sbpgpu_graph_set_degree_corrected": (ctypes.c_int, [vp, ctypes.c_int32]),
    "sbpgpu_bm_create": (ctypes.c_int, [vp, ctypes.c_int64, i32p, ctypes.POINTER(vp)]),
    "sbpgpu_bm_copy": (ctypes.c_int, [vp, ctypes.POINTER(vp)]),
    "sbpgpu_bm_destroy": (None, [vp]),
    "sbpgpu_bm_num_blocks": (ctypes.c_int64, [vp]),
    "sbpgpu_bm_nnz": (ctypes.c_int64, [vp]),
    "sbpgpu_bm_read": (ctypes.c_int, [vp, i32p, i64p, i64p, i64p, i64p, i32p, i32p, i64p]),
    "sbpgpu_bm_entropy": (ctypes.c_double, [vp]),
    "sbpgpu_mdl": (ctypes.c_int, [vp, f64p]),
    "sbpgpu_delta_mdl_batch": (ctypes.c_int, [vp, ctypes.c_int64, i32p, i32p, f64p]),
    "sbpgpu_delta_mdl_batch_noalloc": (ctypes.c_int, [vp, ctypes.c_int64, i32p, i32p, f64p]),
    "sbpgpu_merge_delta_mdl_batch": (ctypes.c_int, [vp, ctypes.c_int64, i32p, i32p, f64p]),
    "sbpgpu_np_mdl": (ctypes.c_int, [vp, f64p]),
    "sbpgpu_np_delta_mdl_batch": (ctypes.c_int, [vp, ctypes.c_int64, i32p, i32p, f64p]),
    "sbpgpu_np_merge_delta_mdl_batch": (ctypes.c_int, [vp, ctypes.c_int64, i32p, i32p, f64p]),
    "sbpgpu_propose_batch": (ctypes.c_int, [vp, ctypes.c_int64, i32p, ctypes.c_uint64, ctypes.c_uint32,
                                            ctypes.c_uint32, ctypes.c_uint32, i32p]),
    "sbpgpu_gibbs_batch": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_int64, i32p, ctypes.c_uint64,
                                          ctypes.c_uint32, ctypes.c_uint32, i32p, i64p]),
    "sbpgpu_gibbs_propose": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_int64, i32p, ctypes.c_uint64,
                                            ctypes.c_uint32, ctypes.c_uint32, i32p]),
    "sbpgpu_mh_chain": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_int64, i32p, ctypes.c_uint64,
                                       ctypes.c_uint32, ctypes.c_uint32, i64p]),
    "sbpgpu_propose_move": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_int32, ctypes.c_uint64,
                                           ctypes.c_uint32, ctypes.c_uint32, i32p, f64p, i32p]),
    "sbpgpu_move_vertex": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, f64p, i32p]),
    "sbpgpu_mcmc": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.POINTER(Stats)]),
    "sbpgpu_merge_blocks": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_uint64, ctypes.c_int32,
                                           ctypes.c_int64, ctypes.POINTER(Stats)]),
    "sbpgpu_merge_proposals": (ctypes.c_int, [vp, ctypes.c_uint64, ctypes.c_int32, i32p, f64p]),
    "sbpgpu_sbp": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_uint64, i32p, i64p, f64p,
                                  ctypes.POINTER(Stats)]),
    "sbpgpu_evaluate": (ctypes.c_int, [vp, ctypes.c_int64, i32p, i32p, ctypes.POINTER(Eval)]),
    "sbpgpu_partition_scores": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, i64p,
                                               ctypes.POINTER(Eval)]),
    "sbpgpu_split_communities": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_uint64, ctypes.c_int32,
                                                ctypes.c_int64]),
    "sbpgpu_sbp_top_down": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_uint64, ctypes.c_int32, i32p, i64p,
                                           f64p, ctypes.POINTER(Stats)]),
    "sbpgpu_sample": (ctypes.c_int, [vp, ctypes.c_int32, ctypes.c_double, ctypes.c_uint64, i32p, i64p]),
    "sbpgpu_graph_subgraph": (ctypes.c_int, [vp, i32p, ctypes.c_int64, ctypes.POINTER(vp)]),
    "sbpgpu_extend": (ctypes.c_int, [vp, i32p, ctypes.c_int64, ctypes.c_int64, i32p, ctypes.c_uint64, i32p]),
    "sbpgpu_reattach": (ctypes.c_int, [vp, i32p, ctypes.c_int64, ctypes.c_int64, i32p, ctypes.c_uint64, i32p]),
    "sbpgpu_finetune_assignment": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_uint64, ctypes.POINTER(Stats)]),
    "sbpgpu_sbp_sampled": (ctypes.c_int, [vp, ctypes.POINTER(Config), ctypes.c_uint64, ctypes.c_int32, ctypes.c_double,
                                          i32p, i64p, f64p, ctypes.POINTER(Stats)]),
    "sbpgpu_job_footprint": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]),
    "sbpgpu_server_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64,
                                            ctypes.POINTER(vp)]),
    "sbpgpu_server_submit": (ctypes.c_int, [vp, ctypes.POINTER(Job), i64p]),
    "sbpgpu_server_wait": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.POINTER(JobResult)]),
    "sbpgpu_server_wait_for": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(JobResult)]),
    "sbpgpu_server_cancel": (ctypes.c_int, [vp, ctypes.c_int64]),
    "sbpgpu_server_pause": (ctypes.c_int, [vp, ctypes.c_int32]),
    "sbpgpu_server_inject_alloc_failure": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.c_int64]),
    "sbpgpu_server_destroy": (None, [vp]),
    "sbpgpu_sbp_batch": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.POINTER(Job), ctypes.POINTER(JobResult)]),
    "sbpgpu_set_timing": (None, [vp, ctypes.c_int32]),
    "sbpgpu_read_timing": (ctypes.c_int, [vp, ctypes.POINTER(KernelTiming)]),
}

_lib = None


class SbpGpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


def load(build_if_missing=True):
    """Loads libsbpgpu.so; builds it first if it is missing (nvcc required)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError("libsbpgpu.so is missing; run sbp_gb300.build.build()")
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return _lib


def check(status, ctx=None):
    if status != SBPGPU_OK:
        msg = load().sbpgpu_last_error(ctx).decode() if ctx else ""
        raise SbpGpuError(status, msg)

"""Partition quality against a true partition.

evaluate() is evaluate::evaluate_blockmodel (reference src/evaluate.cpp:9-180) through the
device (sbpgpu_evaluate): contingency table on the GPU; NMI, pair-counting F1 / precision /
recall / Rand index and the matched accuracy on the host.  nmi() is a host restatement of
calculate_nmi (evaluate.cpp:63-98) used where no context is wanted.
"""
import ctypes

import numpy as np


def evaluate(true_assignment, assignment, ctx=None):
    """Returns a dict with nmi, f1, precision, recall, rand_index, accuracy, true_blocks and
    found_blocks; true_assignment < 0 marks unlabelled vertices."""
    from . import _lib
    from .core import default_context
    c = ctx or default_context()
    t = np.ascontiguousarray(true_assignment, dtype=np.int32)
    a = np.ascontiguousarray(assignment, dtype=np.int32)
    if t.shape != a.shape:
        raise ValueError("assignments differ in length")
    out = _lib.Eval()
    c.check(c.lib.sbpgpu_evaluate(c.h, t.size, t.ctypes.data_as(_lib.i32p), a.ctypes.data_as(_lib.i32p),
                                  ctypes.byref(out)))
    return out.as_dict()


def partition_scores(num_vertices, contingency_table):
    """calculate_f1_score and calculate_nmi (reference src/evaluate.cpp:9-98) of a contingency
    table given as the reference passes it (a rows x columns matrix of counts): a dict with
    f1, precision, recall, rand_index and nmi.  Host arithmetic in the library; no device."""
    from . import _lib
    m = np.ascontiguousarray(contingency_table, dtype=np.int64)
    if m.ndim != 2 or m.size == 0:
        raise ValueError("the contingency table must be a non-empty matrix")
    out = _lib.Eval()
    st = _lib.load().sbpgpu_partition_scores(int(num_vertices), m.shape[0], m.shape[1], m.ctypes.data_as(_lib.i64p),
                                             ctypes.byref(out))
    if st != 0:
        raise ValueError("invalid contingency table or vertex count")
    d = out.as_dict()
    return {k: d[k] for k in ("f1", "precision", "recall", "rand_index", "nmi")}


def calculate_f1_score(num_vertices, contingency_table):
    """evaluate::calculate_f1_score (reference src/evaluate.cpp:9-61)."""
    return partition_scores(num_vertices, contingency_table)["f1"]


def nmi(true_assignment, assignment):
    t = np.asarray(true_assignment, dtype=np.int64)
    a = np.asarray(assignment, dtype=np.int64)
    if t.shape != a.shape:
        raise ValueError("assignments differ in length")
    n = t.size
    tb = np.unique(t, return_inverse=True)[1]
    ab = np.unique(a, return_inverse=True)[1]
    joint = np.zeros((tb.max() + 1, ab.max() + 1), np.float64)
    np.add.at(joint, (tb, ab), 1.0)
    pj = joint / n
    pt = joint.sum(axis=1) / n  # marginals from integer counts: exact for a single block
    pa = joint.sum(axis=0) / n
    nz = pj > 0
    mi = (pj[nz] * np.log(pj[nz] / np.outer(pt, pa)[nz])).sum()
    ht = -(pt[pt > 0] * np.log(pt[pt > 0])).sum()
    ha = -(pa[pa > 0] * np.log(pa[pa > 0])).sum()
    if ht * ha == 0:
        return 1.0 if ht == ha else 0.0
    return float(mi / np.sqrt(ht * ha))

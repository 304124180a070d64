"""Partition quality against a planted partition: normalised mutual information.

Follows evaluate::calculate_nmi (reference src/evaluate.cpp:63-98): contingency table
of (true block, found block), joint and marginal entropies in natural log,
NMI = I / sqrt(H_true * H_found).
"""
import numpy as np


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

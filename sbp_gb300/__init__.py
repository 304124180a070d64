"""GB300 (sm_103a) implementation of SBP's data-parallel hot path.

The MCMC vertex-move sweep (asynchronous Gibbs, hybrid MCMC, Metropolis-Hastings) and
the block-merge pass, scored by delta-MDL over a device-resident blockmodel, behind
the reference's API names: Graph, Blockmodel, Args and the entropy / finetune /
block_merge / sbp namespaces.  The compute path is libsbpgpu.so (hand-written CUDA,
include/sbpgpu.h); there is no CPU fallback.
"""
from . import block_merge, dcsbm, divisive, entropy, evaluate, finetune, sample, sbp, serve
from ._lib import SbpGpuError, load
from .core import Args, Blockmodel, Context, Graph, default_context

__all__ = ["Args", "Blockmodel", "Context", "Graph", "SbpGpuError", "block_merge", "dcsbm", "default_context",
           "entropy", "evaluate", "finetune", "load", "sbp", "serve"]

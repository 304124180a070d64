"""The C-ABI library builds for sm_103a, loads without a GPU and exports every symbol
that include/sbpgpu.h declares; the Python binding declares the same set.  No device
calls are made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    with open(os.path.join(ROOT, "include", "sbpgpu.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sbpgpu_[a-z_0-9]+)\s*\(", text)))


def test_library_builds_and_exports_header_symbols():
    from sbp_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    from sbp_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == header_functions()


def test_default_config_matches_reference_defaults():
    import sbp_gb300
    from sbp_gb300 import _lib
    L = sbp_gb300.load()
    c = _lib.Config()
    L.sbpgpu_default_config(ctypes.byref(c))
    # include/args.hpp: hybrid_mcmc, 1 batch, mh_percent 0.075, greedy, unordered, 100 iterations
    assert (c.algorithm, c.batches, c.greedy, c.ordered, c.approximate, c.max_iterations) == (1, 1, 1, 0, 0, 100)
    assert abs(c.mh_percent - 0.075) < 1e-7
    a = sbp_gb300.Args().config()
    assert (a.algorithm, a.batches, a.greedy, a.max_iterations) == (1, 1, 1, 100)


def test_args_validation():
    import sbp_gb300
    with pytest.raises(ValueError):
        sbp_gb300.Args(algorithm="nope").config()
    c = sbp_gb300.Args(nonparametric=True).config()
    assert (c.nonparametric, c.greedy) == (1, 0)  # --nonparametric sets greedy off (args.hpp:204-207)


def test_entry_points_reject_null_handles_without_device():
    import sbp_gb300
    L = sbp_gb300.load()
    assert L.sbpgpu_mdl(None, None) == 1
    assert L.sbpgpu_bm_num_blocks(None) == 0
    assert L.sbpgpu_graph_num_vertices(None) == 0

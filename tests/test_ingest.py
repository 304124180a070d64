"""Graph ingest (sbpgpu_graph_load): TSV and Matrix Market files parsed on the device give
the graph the reference's loaders build (src/graph.cpp:33-233) -- same vertex and edge
counts and the same edge order, checked through identical partitions."""
import numpy as np
import pytest

from sbp_gb300 import _lib
from sbp_gb300.core import load_partition


def _edges(undirected, src, dst):
    """The reference's insertion order: each edge, then its reverse when undirected."""
    s, d = [], []
    for u, v in zip(src.tolist(), dst.tolist()):
        s.append(u)
        d.append(v)
        if undirected and u != v:
            s.append(v)
            d.append(u)
    return np.array(s, np.int32), np.array(d, np.int32)


def _write_tsv(path, src, dst):
    with open(path, "w", newline="") as f:
        f.write("% a comment line\n# another\n\n")
        for i, (u, v) in enumerate(zip(src.tolist(), dst.tolist())):
            sep = ["\t", " ", ","][i % 3]
            end = "\r\n" if i % 5 == 0 else "\n"
            weight = "%s1" % sep if i % 2 else ""
            f.write("%d%s%d%s%s" % (u + 1, sep, v + 1, weight, end))


def _write_mtx(path, n, src, dst, symmetric):
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate pattern %s\n" % ("symmetric" if symmetric else "general"))
        f.write("% generated\n")
        f.write("%d %d %d\n" % (n, n, src.size))
        for u, v in zip(src.tolist(), dst.tolist()):
            f.write("%d %d\n" % (u + 1, v + 1))


def _same_partition(gpu, G1, G2):
    a1, B1, m1, _ = gpu.sbp.stochastic_block_partition(G1, gpu.Args(algorithm="hybrid_mcmc", seed=2))
    a2, B2, m2, _ = gpu.sbp.stochastic_block_partition(G2, gpu.Args(algorithm="hybrid_mcmc", seed=2))
    assert B1 == B2 and m1 == m2 and np.array_equal(a1, a2)


@pytest.mark.gpu
@pytest.mark.parametrize("undirected", [False, True])
def test_tsv_load_matches_reference_construction(gpu, tmp_path, undirected):
    src, dst, _ = gpu.dcsbm.generate(800, 6000, 8, seed=31)
    path = tmp_path / "g.tsv"
    _write_tsv(path, src, dst)
    G = gpu.Graph.load(str(path), undirected=undirected)
    s2, d2 = _edges(undirected, src, dst)
    n = int(max(src.max(), dst.max())) + 1
    # the reference's undirected Graph counts each stored pair once (graph.cpp:145-147)
    Em = s2.size // 2 if undirected else s2.size
    assert G.num_vertices() == n and G.num_stored_edges() == s2.size and G.num_edges() == Em
    _same_partition(gpu, G, gpu.Graph(n, s2, d2, num_edges=Em))


@pytest.mark.gpu
@pytest.mark.parametrize("symmetric", [False, True])
def test_matrix_market_load(gpu, tmp_path, symmetric):
    src, dst, _ = gpu.dcsbm.generate(700, 5000, 7, seed=32)
    path = tmp_path / "g.mtx"
    _write_mtx(path, 750, src, dst, symmetric)  # the size line may exceed the largest id
    G = gpu.Graph.load(str(path))
    s2, d2 = _edges(symmetric, src, dst)
    assert G.num_vertices() == 750 and G.num_edges() == s2.size == G.num_stored_edges()
    _same_partition(gpu, G, gpu.Graph(750, s2, d2))


@pytest.mark.gpu
def test_load_errors(gpu, tmp_path):
    with pytest.raises(_lib.SbpGpuError):
        gpu.Graph.load(str(tmp_path / "missing.tsv"))
    bad = tmp_path / "bad.tsv"
    bad.write_text("1 2\n3 x\n")
    with pytest.raises(_lib.SbpGpuError):
        gpu.Graph.load(str(bad))
    dense = tmp_path / "dense.mtx"
    dense.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(_lib.SbpGpuError):
        gpu.Graph.load(str(dense))


def test_truth_partition_file(tmp_path):
    p = tmp_path / "truth.tsv"
    p.write_text("% comment\n1\t2\n3\t1\n2\t3\n")
    assert load_partition(str(p), 4).tolist() == [1, 2, 0, -1]

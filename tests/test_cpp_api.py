"""The C++ host interface (include/sbp_gb300.hpp) through tests/cpp/test_api.cpp: known
answers on the reference's toy graph, delta-MDL against MDL differences, copies and error
behaviour, and a full partition of the C1 graph that must equal the Python path's result
for the same seed."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_api.cpp")
INC = os.path.join(ROOT, "include")


def test_cpp_interface_compiles():
    """The header, the test program and the integration guide's search loop compile without
    a GPU (no link)."""
    for src in (SRC, os.path.join(ROOT, "tests", "cpp", "example_search_loop.cpp")):
        r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", INC, src],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_host_types_without_library(tmp_path):
    """Delta, the BlockMatrix snapshot, edge_weights, early_stop and accept of the C++
    interface, built and run without the library (tests/cpp/test_host_types.cpp)."""
    exe = str(tmp_path / "test_host_types")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", INC,
                        os.path.join(ROOT, "tests", "cpp", "test_host_types.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr


def test_host_adjacency_build(tmp_path):
    """The threaded host adjacency build of graph upload (sbp_gb300/csrc/host_csr.h) equals
    one sequential pass over the edges, at 1 to 16 threads (tests/cpp/test_host_csr.cpp)."""
    exe = str(tmp_path / "test_host_csr")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-Wall", "-Wextra", "-Werror",
                        os.path.join(ROOT, "tests", "cpp", "test_host_csr.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr


def _write_toy(golden, path):
    with open(path, "w") as f:
        f.write("%d %d\n" % (golden["num_vertices"], len(golden["edges"])))
        for u, v in golden["edges"]:
            f.write("%d %d\n" % (u, v))
        f.write("%d\n" % golden["num_blocks"])
        f.write(" ".join(str(a) for a in golden["assignment"]) + "\n")
        f.write(repr(float(golden["mdl"])) + "\n")
        for k in ("block_degrees_out", "block_degrees_in", "block_degrees"):
            f.write(" ".join(str(x) for x in golden[k]) + "\n")
        f.write(repr(float(golden["nonparametric"]["mdl"])) + "\n")


@pytest.mark.gpu
def test_cpp_interface_on_gpu(gpu, golden, tmp_path):
    lib_dir = os.path.dirname(gpu._lib.LIB_PATH)
    exe = str(tmp_path / "test_api")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", INC, SRC, "-L", lib_dir, "-lsbpgpu",
                        "-Wl,-rpath," + lib_dir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    toy = tmp_path / "toy.txt"
    _write_toy(golden, toy)
    src, dst, _ = gpu.dcsbm.generate_config("C1", seed=0)
    graph = tmp_path / "graph.txt"
    with open(graph, "w") as f:
        f.write("%d %d\n" % (1000, src.size))
        for u, v in zip(src, dst):
            f.write("%d %d\n" % (u, v))
    out = tmp_path / "assignment.txt"
    seed = 5
    r = subprocess.run([exe, str(toy), str(graph), str(seed), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = open(out).read().split("\n")
    B_cpp, mdl_cpp = int(lines[0].split()[0]), float(lines[0].split()[1])
    a_cpp = np.array([int(x) for x in lines[1:] if x.strip()], np.int32)
    G = gpu.Graph(1000, src, dst)
    a_py, B_py, mdl_py, _ = gpu.sbp.stochastic_block_partition(G, gpu.Args(algorithm="hybrid_mcmc", seed=seed))
    assert B_cpp == B_py
    assert mdl_cpp == mdl_py
    assert np.array_equal(a_cpp, a_py)

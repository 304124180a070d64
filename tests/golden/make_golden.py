"""Extract the reference's known-answer fixtures into tests/golden/toy_example.json.

Run in a container that has the reference checkout (read-only) mounted:

    python tests/golden/make_golden.py /path/to/SBP

The script reads the reference's own gtest sources as text (it executes nothing
from them) and records:
  * the 11-vertex / 23-edge toy graph and its assignments
    (test/toy_example.hpp:43-73, 130-132, 163, 181-184),
  * the known answers the reference's tests assert
    (test/entropy_test.cpp, test/blockmodel_test.cpp, test/finetune_test.cpp,
     test/block_merge_test.cpp).
The JSON is committed; the tests never read the reference at run time.
"""
import json
import os
import re
import sys


def read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def ints(text):
    return [int(x) for x in re.findall(r"-?\d+", text)]


def main(root):
    toy = read(root, "test/toy_example.hpp")
    edges_block = re.search(r"std::vector<std::vector<long>> edges \{(.*?)\};", toy, re.S).group(1)
    edges = [ints(m) for m in re.findall(r"\{([^{}]*)\}", edges_block)]
    assignment = ints(re.search(r"\bassignment = \{([^}]*)\};", toy).group(1))
    entropy = float(re.search(r"const double ENTROPY = ([0-9.]+);", toy).group(1))
    merge_assignment = ints(re.search(r"assignment2 = \{([^}]*)\};", toy).group(1))
    complex_assignment = ints(re.search(r"ComplexToySetUp.*?assignment = \{([^}]*)\};", toy, re.S).group(1))
    # the block degrees after the vertex-7 move (test/toy_example.hpp: new_block_degrees,
    # asserted by test/common_test.cpp:17-36)
    # in ToySetUp (the vertex-7 move) and BlockMergeTest (block 0 into 1), in that order
    nbd = [{}, {}, {}]
    for k, v in re.findall(r"new_block_degrees\.block_degrees(_out|_in|) = \{([^}]*)\};", toy):
        next(d for d in nbd if k not in d)[k] = ints(v)
    # ComplexToySetUp: vertex 6 into block 0 of the six-block model (BlockDegreesAfterUpdates,
    # asserted by test/common_test.cpp:38-77)
    nbd[2] = {k: ints(v) for k, v in re.findall(r"BlockDegreesAfterUpdates\.block_degrees(_out|_in|) = \{([^}]*)\};",
                                                 toy)}

    bm_test = read(root, "test/blockmodel_test.cpp")
    deg = {}
    for kind, blk, val in re.findall(r"EXPECT_EQ\(B\.degrees(_out|_in|)\((\d)\), (\d+)\);", bm_test):
        deg.setdefault(kind or "_tot", {})[int(blk)] = int(val)

    ft = read(root, "test/finetune_test.cpp")
    body = re.search(r"TEST_F\(FinetuneTest, BlockmodelDeltasAreCorrect\)(.*?)\n}", ft, re.S).group(1)
    vdelta = {f"{a},{b}": int(c) for a, b, c in re.findall(r"delta\.get\((\d),(\d)\), (-?\d+)\)", body)}
    vdelta_size = int(re.search(r"entries\(\)\.size\(\), (\d+)\)", body).group(1))
    body = re.search(r"TEST_F\(FinetuneTest, SpecialCaseBlockmodelDeltasAreCorrect\)(.*?)\n}", ft, re.S).group(1)
    sdelta = {f"{a},{b}": int(c) for a, b, c in re.findall(r"delta\.get\((\d),(\d)\), (-?\d+)\)", body)}

    # the rows and columns of the two blocks after a move (finetune_test.cpp:44-83, :174-224):
    # vertex 7 to block 0, vertex 5 (a self-loop) to block 0, and vertex 6 of the six-block
    # model to block 0
    cells_after = []
    for name, which, vertex in (("SparseEdgeCountUpdatesAreCorrect", "toy", 7),
                                ("SparseEdgeCountUpdatesWithSelfEdgesAreCorrect", "toy", 5),
                                ("SpecialCaseGivesCorrectSparseEdgeCountUpdates", "complex", 6)):
        body = re.search(r"TEST_F\(FinetuneTest, %s\)(.*?)\n}" % name, ft, re.S).group(1)
        vals = [[k, int(i), int(v)] for k, i, v in
                re.findall(r"updates\.(block_row|block_col|proposal_row|proposal_col)\[(\d)\], (\d+)\)", body)]
        cells_after.append({"blockmodel": which, "vertex": vertex, "proposal": 0, "values": vals})

    # max-degree sampling of the toy graph (sample_test.cpp:8-51): its vertex and edge counts
    # and the edges the sampled graph must hold, in sample ids
    smt = read(root, "test/sample_test.cpp")
    sample_size = float(re.search(r"args\.samplesize = ([0-9.]+);", smt).group(1))
    sedges_block = re.search(r"sample_edges = \{(.*?)\};", smt, re.S).group(1)
    sample_edges = [ints(m) for m in re.findall(r"\{([^{}]*)\}", sedges_block)]
    sample_counts = ints(" ".join(re.findall(r"EXPECT_EQ\(s\.graph\.num_(?:vertices|edges)\(\), (\d+)\);", smt)))

    bmt = read(root, "test/block_merge_test.cpp")
    mdelta = {f"{a},{b}": int(c) for a, b, c in re.findall(r"delta\.get\((\d),(\d)\), (-?\d+)\)", bmt)}
    mdelta_size = int(re.search(r"entries\(\)\.size\(\), (\d+)\)", bmt).group(1))

    et = read(root, "test/entropy_test.cpp")
    null_mdl = float(re.search(r"hand_calculated_mdl = ([0-9.E+e]+);", et).group(1))
    big_E = float(re.search(r"const long E = ([0-9.E+e]+);", et).group(1))

    npt = read(root, "test/nonparametric_entropy_test.cpp")
    npc = {name: float(val) for name, val in re.findall(r"const double ([A-Z_0-9]+) = ([0-9.]+);", npt)}

    evt = read(root, "test/evaluate_test.cpp")

    def matrix(name):
        block = re.search(name + r" = \{(.*?)\};", evt, re.S).group(1)
        return [ints(row) for row in re.findall(r"\{([^{}]*)\}", block)]

    evc = {name: float(val) for name, val in re.findall(r"\b([A-Z][A-Za-z0-9]*) = ([0-9.]+);", evt)}

    out = {
        "source": "vtsynergy/SBP test/toy_example.hpp, test/*_test.cpp",
        "num_vertices": 11,
        "edges": edges,
        "assignment": assignment,
        "num_blocks": 3,
        "mdl": entropy,
        "mdl_tolerance": "EXPECT_FLOAT_EQ (4 float ULPs)",
        "block_degrees_out": [deg["_out"][i] for i in range(3)],
        "block_degrees_in": [deg["_in"][i] for i in range(3)],
        "block_degrees": [deg["_tot"][i] for i in range(3)],
        "vertex_move": {"vertex": 7, "proposal": 0, "delta": vdelta, "delta_entries": vdelta_size,
                        "after_assignment": [0, 0, 0, 0, 1, 1, 1, 0, 2, 2, 2],
                        "after_degrees_out": nbd[0]["_out"], "after_degrees_in": nbd[0]["_in"],
                        "after_degrees": nbd[0][""]},
        "special_case": {"num_blocks": 6, "assignment": complex_assignment, "vertex": 6, "proposal": 0,
                         "delta": sdelta, "after_degrees_out": nbd[2]["_out"], "after_degrees_in": nbd[2]["_in"],
                         "after_degrees": nbd[2][""]},
        "block_merge": {"block": 0, "proposal": 1, "delta": mdelta, "delta_entries": mdelta_size,
                        "after_assignment": merge_assignment, "after_degrees_out": nbd[1]["_out"],
                        "after_degrees_in": nbd[1]["_in"], "after_degrees": nbd[1][""]},
        "null_mdl_v1": {"num_edges": big_E, "value": null_mdl},
        # nonparametric_entropy_test.cpp:19-27 on the toy blockmodel above (not degree-corrected)
        "nonparametric": {"mdl": npc["SIMPLE_NONPARAMETRIC_ENTROPY"], "sparse_entropy": npc["SIMPLE_SPARSE_ENTROPY"],
                          "partition_dl": npc["PARTITION_DL"], "edges_dl": npc["EDGES_DL"],
                          "degree_corrected": {"mdl": npc["NONPARAMETRIC_ENTROPY"],
                                               "sparse_entropy": npc["SPARSE_ENTROPY"],
                                               "degree_dl": npc["DEGREE_DL"]}},
    }
    out["cells_after_move"] = cells_after
    out["sample_max_degree"] = {"sample_size": sample_size, "num_vertices": sample_counts[0],
                                "num_edges": sample_counts[1], "edges": sample_edges}
    # evaluate_test.cpp:17-44: calculate_f1_score on two contingency tables (EXPECT_FLOAT_EQ)
    out["evaluate"] = {"matrix": matrix("Matrix"), "num_vertices": int(evc["N"]), "f1": evc["F1"],
                       "rand_index": evc["RandIndex"], "recall": evc["Recall"], "precision": evc["Precision"],
                       "matrix2": matrix("Matrix2"), "num_vertices2": int(evc["N2"]), "f1_2": evc["F12"]}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "toy_example.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path to the reference checkout>")
    main(sys.argv[1])

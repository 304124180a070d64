"""Pins the CPU oracle to the reference's own known answers (test/toy_example.hpp and
test/*_test.cpp, extracted into tests/golden/toy_example.json) and checks its internal
identities.  CPU only."""
import math

import numpy as np
import pytest


def toy(oracle, golden, assignment=None, num_blocks=None):
    edges = np.array(golden["edges"], dtype=np.int32)
    g = oracle.Graph(golden["num_vertices"], edges[:, 0], edges[:, 1])
    a = golden["assignment"] if assignment is None else assignment
    B = golden["num_blocks"] if num_blocks is None else num_blocks
    return g, oracle.Blockmodel(g, B, a)


def float_eq(a, b, ulps=4):
    # gtest EXPECT_FLOAT_EQ: within 4 ULPs in single precision
    return abs(np.float32(a) - np.float32(b)) <= ulps * np.spacing(np.float32(max(abs(a), abs(b))))


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for Philox4x32-10.
    assert oracle.philox([0, 0, 0, 0], [0, 0]).tolist() == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert oracle.philox([0xffffffff] * 4, [0xffffffff] * 2).tolist() == [0x408f276d, 0x41c83b0e, 0xa20bc7c6,
                                                                          0x6d5451fd]
    assert oracle.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                         [0xa4093822, 0x299f31d0]).tolist() == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_toy_mdl(oracle, golden):
    # entropy_test.cpp:59-62
    _, B = toy(oracle, golden)
    lit, can = B.mdl()
    assert float_eq(lit, golden["mdl"])
    assert abs(lit - can) <= 1e-12 * abs(lit)


def test_toy_block_degrees(oracle, golden):
    # blockmodel_test.cpp:25-35
    _, B = toy(oracle, golden)
    d = B.read()
    assert d["d_out"].tolist() == golden["block_degrees_out"]
    assert d["d_in"].tolist() == golden["block_degrees_in"]
    assert d["d_tot"].tolist() == golden["block_degrees"]


def test_toy_vertex_delta(oracle, golden):
    # finetune_test.cpp:88-103: six entries, (0,1) and (2,1) absent
    _, B = toy(oracle, golden)
    mv = golden["vertex_move"]
    d = B.vertex_delta(mv["vertex"], mv["proposal"])
    assert len(d) == mv["delta_entries"]
    for key, val in mv["delta"].items():
        r, c = map(int, key.split(","))
        assert d.get((r, c), 0) == val


def test_toy_delta_sums_to_zero(oracle, golden):
    # finetune_test.cpp:106-127 (vertex 10 has a self edge)
    _, B = toy(oracle, golden)
    for v in (7, 10):
        assert sum(B.vertex_delta(v, 0).values()) == 0


def test_toy_delta_mdl_equals_mdl_difference(oracle, golden):
    # entropy_test.cpp:95-107
    g, B = toy(oracle, golden)
    mv = golden["vertex_move"]
    lit, fx = B.delta_mdl(mv["vertex"], mv["proposal"])
    assert lit == fx / 2**24
    after = oracle.Blockmodel(g, 3, mv["after_assignment"])
    assert float_eq(lit, after.mdl()[0] - B.mdl()[0])


def test_toy_special_case(oracle, golden):
    # finetune_test.cpp:226-239 and entropy_test.cpp:161-186
    sc = golden["special_case"]
    g, B3 = toy(oracle, golden, sc["assignment"], sc["num_blocks"])
    d = B3.vertex_delta(sc["vertex"], sc["proposal"])
    assert len(d) == 6
    for key, val in sc["delta"].items():
        r, c = map(int, key.split(","))
        assert d[(r, c)] == val
    lit, fx = B3.delta_mdl(sc["vertex"], sc["proposal"])
    a2 = list(sc["assignment"])
    a2[sc["vertex"]] = sc["proposal"]
    B5 = oracle.Blockmodel(g, sc["num_blocks"], a2)
    assert float_eq(lit, B5.mdl()[0] - B3.mdl()[0])


def test_toy_block_merge(oracle, golden):
    # block_merge_test.cpp:11-21 and entropy_test.cpp:250-263
    g, B = toy(oracle, golden)
    bm = golden["block_merge"]
    d = B.merge_delta(bm["block"], bm["proposal"])
    assert len(d) == bm["delta_entries"]
    for key, val in bm["delta"].items():
        r, c = map(int, key.split(","))
        assert d.get((r, c), 0) == val
    lit, fx = B.merge_delta_mdl(bm["block"], bm["proposal"])
    assert lit == fx / 2**24
    B2 = oracle.Blockmodel(g, 3, bm["after_assignment"])
    assert float_eq(lit, B2.mdl()[0] - B.mdl()[0])


def test_null_mdl(oracle, golden):
    # entropy_test.cpp:198-217
    nm = golden["null_mdl_v1"]
    assert float_eq(oracle.null_mdl_v1(nm["num_edges"]), nm["value"])


def test_literal_equals_fixed_on_random_moves(oracle):
    from sbp_gb300 import dcsbm
    src, dst, planted = dcsbm.generate(600, 6000, 8, seed=3)
    g = oracle.Graph(600, src, dst)
    rng = np.random.default_rng(0)
    B = oracle.Blockmodel(g, 30, rng.integers(0, 30, 600))
    for _ in range(300):
        v, s = int(rng.integers(600)), int(rng.integers(30))
        lit, fx = B.delta_mdl(v, s)
        assert lit == fx / 2**24  # exact: every term is a multiple of 2^-24
    for _ in range(100):
        r, s = rng.choice(30, 2, replace=False)
        lit, fx = B.merge_delta_mdl(int(r), int(s))
        assert lit == fx / 2**24


def test_delta_mdl_tracks_mdl(oracle):
    """dS from the table form matches the change of the full MDL (ratio-form logs) up to
    the float-log rounding the reference itself has (hazard H4)."""
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(400, 4000, 6, seed=4)
    g = oracle.Graph(400, src, dst)
    rng = np.random.default_rng(1)
    a = rng.integers(0, 12, 400)
    B = oracle.Blockmodel(g, 12, a)
    base = B.mdl()[0]
    for _ in range(40):
        v, s = int(rng.integers(400)), int(rng.integers(12))
        if s == a[v]:
            continue
        a2 = a.copy()
        a2[v] = s
        if np.bincount(a2, minlength=12).min() == 0:
            continue
        lit, _ = B.delta_mdl(v, s)
        after = oracle.Blockmodel(g, 12, a2).mdl()[0]
        assert abs(lit - (after - base)) <= 1e-4 * abs(base)


def test_sampler_matches_reference_distribution(oracle):
    """The canonical draw -> block mapping of propose_new_block gives the reference's
    distribution: P(s) = sum over neighbours u of 1/k * W_{b(u)}[s] / sum(W_{b(u)})."""
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(200, 2400, 5, seed=5)
    g = oracle.Graph(200, src, dst)
    rng = np.random.default_rng(2)
    a = rng.integers(0, 8, 200)
    B = oracle.Blockmodel(g, 8, a)
    M = np.zeros((8, 8))
    np.add.at(M, (a[src], a[dst]), 1)
    v = int(np.argmax(np.bincount(src, minlength=200) + np.bincount(dst, minlength=200)))
    nbrs = list(dst[src == v]) + [u for u in src[dst == v] if u != v]
    expect = np.zeros(8)
    for u in nbrs:
        nb = a[u]
        W = M[nb, :] + M[:, nb]
        W[nb] -= M[nb, nb]
        expect += W / W.sum() / len(nbrs)
    n = 20000
    got = np.bincount([B.propose_vertex(v, 7, i, 0, 1) for i in range(n)], minlength=8)
    chi2 = ((got - n * expect) ** 2 / np.maximum(n * expect, 1e-9))[expect > 0].sum()
    assert chi2 < 40  # 7 degrees of freedom; p ~ 1e-6
    assert got[expect == 0].sum() == 0


def test_gibbs_apply_equals_rebuild(oracle):
    """Applying accepted moves in vertex order (serial loop) leaves the blockmodel equal to
    a rebuild from the final assignment."""
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(500, 5000, 6, seed=6)
    g = oracle.Graph(500, src, dst)
    rng = np.random.default_rng(3)
    B = oracle.Blockmodel(g, 40, rng.integers(0, 40, 500))
    cfg = oracle.make_config("async_gibbs")
    n, moves, _ = B.gibbs_batch(np.arange(500), seed=11, iteration=0, step=0, cfg=cfg)
    d = B.read()
    R = oracle.Blockmodel(g, 40, d["assignment"]).read()
    for k in ("d_out", "d_in", "d_tot", "sizes", "rows", "cols", "counts"):
        assert np.array_equal(d[k], R[k]), k


def test_oracle_sbp_recovers_planted_blocks(oracle):
    from sbp_gb300 import dcsbm, evaluate
    src, dst, planted = dcsbm.generate_config("C1", seed=0)
    g = oracle.Graph(1000, src, dst)
    asg, B, mdl, st = oracle.sbp(g, oracle.make_config("hybrid_mcmc"), seed=1)
    assert B > 1
    assert evaluate.nmi(planted, asg) > 0.6
    assert mdl < oracle.Blockmodel(g, 1, np.zeros(1000, np.int32)).mdl()[0]


# ---- nonparametric entropy (entropy::nonparametric, entropy.cpp:617-1225)

def test_np_toy_terms(oracle, golden):
    # nonparametric_entropy_test.cpp:57-67, :81-85, :95-99, :111-115 on the toy blockmodel
    _, B = toy(oracle, golden)
    npg = golden["nonparametric"]
    t = B.np_terms()
    assert float_eq(t["sparse_entropy"], npg["sparse_entropy"])
    assert float_eq(t["partition_dl"], npg["partition_dl"])
    assert t["degree_dl"] == 0.0
    assert float_eq(t["edges_dl"], npg["edges_dl"])
    lit, can = B.np_mdl()
    assert float_eq(lit, npg["mdl"])
    assert abs(lit - can) <= 1e-6  # lgamma terms rounded to 2^-24 each


def test_np_toy_delta_mdl_equals_mdl_difference(oracle, golden):
    # nonparametric_entropy_test.cpp:118-133 (vertex 7 to block 0)
    g, B = toy(oracle, golden)
    mv = golden["vertex_move"]
    lit, fx = B.np_delta_mdl(mv["vertex"], mv["proposal"])
    after = oracle.Blockmodel(g, 3, mv["after_assignment"])
    assert float_eq(lit, after.np_mdl()[0] - B.np_mdl()[0])
    assert abs(lit - fx / 2**24) <= 1e-6


def test_np_delta_tracks_mdl_on_random_moves(oracle):
    """Vertex moves and merges, including moves that empty or occupy a block: the canonical
    delta equals the change of the canonical MDL exactly, and the reference's double
    arithmetic to within its rounding.  For a vertex with a self-loop the reference's vterm
    moves the in-degree by its in-edges without the loop (entropy.cpp:826-827, :861-875)
    while the blockmodel moves it by one more, so there only delta and literal agree."""
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(300, 3000, 6, seed=9)
    loops = set(src[src == dst].tolist())
    g = oracle.Graph(300, src, dst)
    rng = np.random.default_rng(4)
    a = rng.integers(0, 20, 300)
    a[a == 19] = 18  # block 19 starts empty
    a[a == 17] = 16
    a[7] = 17        # block 17 holds one vertex
    B = oracle.Blockmodel(g, 20, a)
    assert B.nonempty() == 19
    base_lit, base_can = B.np_mdl()
    cases = [(7, 3), (int(np.flatnonzero(a == 2)[0]), 19)] + [
        (int(rng.integers(300)), int(rng.integers(20))) for _ in range(80)]
    checked = 0
    for v, s in cases:
        if s == a[v]:
            continue
        lit, fx = B.np_delta_mdl(v, s)
        assert abs(lit - fx / 2**24) <= 1e-6
        if v in loops:
            continue
        a2 = a.copy()
        a2[v] = s
        after_lit, after_can = oracle.Blockmodel(g, 20, a2).np_mdl()
        assert fx == round((after_can - base_can) * 2**24), (v, s)
        assert abs(lit - (after_lit - base_lit)) <= 1e-7 * abs(base_lit)
        checked += 1
    assert checked > 40
    sizes = np.bincount(a, minlength=20)
    for _ in range(40):
        r, s = (int(x) for x in rng.choice(20, 2, replace=False))
        lit, fx = B.np_merge_delta_mdl(r, s)
        assert abs(lit - fx / 2**24) <= 1e-6
        if sizes[r] == 0 or sizes[s] == 0:
            assert fx == 0 and lit == 0.0  # block_merge_delta_mdl returns 0 (entropy.cpp:1203-1204)
            continue
        after_can = oracle.Blockmodel(g, 20, np.where(a == r, s, a)).np_mdl()[1]
        assert fx == round((after_can - base_can) * 2**24), (r, s)


def test_np_sbp_recovers_planted_blocks(oracle):
    from sbp_gb300 import dcsbm, evaluate
    src, dst, planted = dcsbm.generate(1000, 8000, 11, seed=2)
    g = oracle.Graph(1000, src, dst)
    asg, B, mdl, st = oracle.sbp(g, oracle.make_config("hybrid_mcmc", nonparametric=True), seed=1)
    assert B > 1
    assert evaluate.nmi(planted, asg) > 0.6


# ---- sampling (sample.cpp) and the sampled partition (main.cpp:98-140)

def test_oracle_samplers(oracle):
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(500, 4000, 5, seed=11)
    g = oracle.Graph(500, src, dst)
    deg = np.bincount(src, minlength=500) + np.bincount(dst, minlength=500)
    deg -= np.bincount(src[src == dst], minlength=500) > 0
    for alg in ("max_degree", "random", "degree_product"):
        m, n = oracle.sample(g, alg, 0.3, 5)
        assert sorted(m[m >= 0].tolist()) == list(range(n))
        assert n >= 150 if alg == "degree_product" else n == 150
    m, n = oracle.sample(g, "max_degree", 0.3, 5)
    order = np.argsort(-deg, kind="stable")  # utils::argsort: stable, descending
    assert np.array_equal(np.flatnonzero(m >= 0), np.sort(order[:150]))
    assert all(m[order[i]] == i for i in range(150))
    m, n = oracle.sample(g, "detach", 1.0, 0)
    assert np.array_equal(m >= 0, deg > 1)
    # from_vertices keeps the edges between sampled vertices, each source's out-neighbours
    # in their original order (the sample graph lists them by sample id)
    m, n = oracle.sample(g, "random", 0.5, 3)
    n2, s2, d2 = oracle.subgraph_edges(g, m)
    keep = np.flatnonzero((m[src] >= 0) & (m[dst] >= 0))
    keep = keep[np.argsort(m[src[keep]], kind="stable")]
    want = [(int(m[src[i]]), int(m[dst[i]])) for i in keep]
    assert n2 == n and list(zip(s2.tolist(), d2.tolist())) == want


def test_oracle_extend_rules(oracle):
    # vertex 2 has neighbours in blocks 1, 1, 0: it takes block 1; vertex 4 then follows
    # vertex 2 (already assigned, id order); vertex 5 has no neighbours: a drawn block
    src = np.array([0, 1, 3, 2, 4, 2], np.int32)
    dst = np.array([2, 2, 2, 4, 0, 0], np.int32)
    g = oracle.Graph(6, src, dst)
    mapping = np.array([0, 1, -1, 2, -1, -1], np.int32)
    asg = oracle.extend(g, [1, 1, 0], 3, mapping, 9)
    assert asg[:5].tolist() == [1, 1, 1, 0, 1]
    assert 0 <= asg[5] < 3


def test_oracle_sampled_partition(oracle):
    from sbp_gb300 import dcsbm, evaluate
    src, dst, planted = dcsbm.generate_config("C1", seed=0)
    g = oracle.Graph(1000, src, dst)
    asg, B, mdl, st = oracle.sbp_sampled(g, oracle.make_config("hybrid_mcmc"), 1, "max_degree", 0.5)
    assert B > 1 and asg.max() < B
    assert evaluate.nmi(planted, asg) > 0.6


def test_oracle_snowball_samplers_and_reattach(oracle):
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(800, 6000, 5, seed=12)
    src = np.concatenate([src, [800, 802, 803]]).astype(np.int32)   # 800 -> 801 pendant pair,
    dst = np.concatenate([dst, [801, 802, 5]]).astype(np.int32)     # 802 self-loop, 803 -> 5
    g = oracle.Graph(805, src, dst)                                  # 804 isolated
    for alg in ("expansion_snowball", "degree_product_snowball"):
        m, n = oracle.sample(g, alg, 0.25, 4)
        assert n >= 201 and sorted(m[m >= 0].tolist()) == list(range(n))
    m, n = oracle.sample(g, "detach", 1.0, 0)
    assert all(m[v] == -1 for v in (800, 801, 802, 803, 804))
    sa = np.arange(n, dtype=np.int32) % 7
    asg = oracle.reattach(g, sa, 7, m, 3)
    assert asg[803] == sa[m[5]]              # takes its sampled neighbour's block
    assert asg[800] == asg[801]              # a detached pair shares one draw
    assert asg.min() >= 0 and asg.max() < 7


@pytest.mark.parametrize("split", ["snowball", "single-snowball", "connectivity-snowball"])
@pytest.mark.parametrize("init", ["random", "degree-weighted", "high-degree"])
def test_oracle_snowball_splits(oracle, split, init):
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(1500, 15000, 6, seed=21)
    g = oracle.Graph(1500, src, dst)
    a = (np.arange(1500) % 5).astype(np.int32)
    b = oracle.Blockmodel(g, 5, a)
    b.split_communities(oracle.make_config(nonparametric=True, split=split, splitinit=init), 3, 0, 9)
    d = b.read()
    assert b.num_blocks == 9 and np.bincount(d["assignment"], minlength=9).min() > 0
    # every vertex keeps its cluster or moves to one of the new blocks
    assert all(x == y or x >= 5 for x, y in zip(d["assignment"].tolist(), a.tolist()))


# ---- degree-corrected nonparametric entropy (args.degreecorrected: entropy.hpp:117-133,
# entropy.cpp:617-764, :994-1110)

def _toy_dc(oracle, golden):
    edges = np.array(golden["edges"], dtype=np.int32)
    g = oracle.Graph(golden["num_vertices"], edges[:, 0], edges[:, 1], degree_corrected=True)
    return g, oracle.Blockmodel(g, golden["num_blocks"], golden["assignment"])


def _li2(z):
    if z > 0.5:
        return math.pi ** 2 / 6 - math.log(z) * math.log1p(-z) - _li2(1 - z)
    s, p, k = 0.0, z, 1
    while p / (k * k) > 1e-18 * max(s, 1e-300):
        s += p / (k * k)
        p *= z
        k += 1
    return s


def _log_q(n, k):
    """log_q (entropy.cpp:688-707) in plain Python, independently of the oracle."""
    if n <= 0 or k < 1:
        return 0.0
    k = min(k, n)
    if k < n ** 0.25:
        lb = 0.0 if n - 1 == 0 or k - 1 == 0 else math.lgamma(n) - math.lgamma(k) - math.lgamma(n - k + 1)
        return lb - math.lgamma(k + 1)
    u = k / math.sqrt(n)
    v, d = u, 1.0
    while d > 1e-8:
        nv = u * math.sqrt(_li2(-math.expm1(-v)))
        d, v = abs(nv - v), nv
    lf = math.log(v) - math.log1p(-math.exp(-v) * (1 + u * u / 2)) / 2 - math.log(2) * 1.5 - math.log(u) - math.log(math.pi)
    return lf - math.log(n) + math.sqrt(n) * (2 * v / u - u * math.log1p(-math.exp(-v)))


def _toy_degree_dl(golden):
    """get_deg_dl_dist (entropy.cpp:709-743) on the toy blockmodel, from its edge list."""
    from collections import Counter
    n, a = golden["num_vertices"], golden["assignment"]
    kout, kin = Counter(), Counter()
    for u, v in golden["edges"]:
        kout[u] += 1
        kin[v] += 1
    S = 0.0
    for b in range(golden["num_blocks"]):
        vs = [v for v in range(n) if a[v] == b]
        S += _log_q(sum(kout[v] for v in vs), len(vs)) + _log_q(sum(kin[v] for v in vs), len(vs))
        S -= sum(math.lgamma(c + 1) for c in Counter(kin[v] for v in vs).values())
        S -= sum(math.lgamma(c + 1) for c in Counter(kout[v] for v in vs).values())
        S += 2 * math.lgamma(len(vs) + 1)
    return S


def test_dc_toy_terms(oracle, golden):
    """SPARSE_ENTROPY (nonparametric_entropy_test.cpp:22, :77-83) is the reference's known
    answer.  Its DEGREE_DL (:26, :101-107) and the MDL built from it (:20) are not what
    get_deg_dl_dist computes as written: restated independently above it gives 27.8710,
    not 18.7445 (the reference's own MDL test compares with yet another constant, :70-71),
    so the degree term is checked against that restatement instead."""
    _, B = _toy_dc(oracle, golden)
    npg, dc = golden["nonparametric"], golden["nonparametric"]["degree_corrected"]
    t = B.np_terms()
    assert float_eq(t["sparse_entropy"], dc["sparse_entropy"])
    assert float_eq(t["partition_dl"], npg["partition_dl"])
    assert float_eq(t["edges_dl"], npg["edges_dl"])
    assert t["degree_dl"] == pytest.approx(_toy_degree_dl(golden), rel=1e-12)
    lit, can = B.np_mdl()
    assert lit == pytest.approx(t["sparse_entropy"] + t["partition_dl"] + t["degree_dl"] + t["edges_dl"], rel=1e-15)
    assert abs(lit - can) <= 1e-6


def test_dc_log_q_approaches_partition_counts(oracle):
    """log_q is an approximation of the log of q(n, k), the number of partitions of n into
    at most k parts: against exact counts it is within 4% at n = 8 and closes in as n grows."""
    nmax, kmax = 2000, 400
    q = np.zeros((nmax + 1, kmax + 1), dtype=object)
    q[0, :] = 1
    for n in range(1, nmax + 1):
        for k in range(1, kmax + 1):
            q[n, k] = q[n, k - 1] + (q[n - k, k] if n >= k else 0)
    for n, k, tol in [(8, 4, 0.05), (50, 10, 0.01), (200, 20, 2e-3), (300, 300, 2e-3), (1000, 5, 3e-3),
                      (1000, 30, 5e-4), (2000, 50, 2e-4), (2000, 400, 2e-4)]:
        exact = math.log(q[n, min(k, n)])
        assert abs(oracle.log_q(n, k) / exact - 1) < tol, (n, k)
        assert oracle.log_q(n, k) == pytest.approx(_log_q(n, k), rel=1e-12)
    assert oracle.log_q(0, 3) == 0.0 and oracle.log_q(5, 0) == 0.0


def test_dc_spence_identities(oracle):
    # spence(x) = Li2(1 - x): Li2(0) = 0, Li2(1) = pi^2/6, Li2(1/2) = pi^2/12 - log^2(2)/2,
    # Li2(-1) = -pi^2/12
    assert oracle.spence(1.0) == 0.0
    assert oracle.spence(0.0) == pytest.approx(math.pi ** 2 / 6, rel=1e-15)
    assert oracle.spence(0.5) == pytest.approx(math.pi ** 2 / 12 - math.log(2) ** 2 / 2, rel=1e-14)
    assert oracle.spence(2.0) == pytest.approx(-math.pi ** 2 / 12, rel=1e-14)


def test_dc_delta_tracks_mdl_on_random_moves(oracle):
    """Degree-corrected vertex moves: the canonical delta equals the change of the
    canonical MDL exactly (every log_q term is rounded once, the same way on both sides),
    and the literal delta the reference's double arithmetic to within its rounding.  The
    reference's vterm quirk for vertices with a self-loop applies here too."""
    from sbp_gb300 import dcsbm
    src, dst, _ = dcsbm.generate(300, 3000, 6, seed=19)
    loops = set(src[src == dst].tolist())
    g = oracle.Graph(300, src, dst, degree_corrected=True)
    rng = np.random.default_rng(8)
    a = rng.integers(0, 20, 300)
    a[a == 19] = 18  # block 19 starts empty
    B = oracle.Blockmodel(g, 20, a)
    base_lit, base_can = B.np_mdl()
    checked = 0
    for _ in range(80):
        v, s = int(rng.integers(300)), int(rng.integers(20))
        if s == a[v]:
            continue
        lit, fx = B.np_delta_mdl(v, s)
        assert abs(lit - fx / 2**24) <= 1e-5
        if v in loops:
            continue
        a2 = a.copy()
        a2[v] = s
        after_lit, after_can = oracle.Blockmodel(g, 20, a2).np_mdl()
        assert fx == round((after_can - base_can) * 2**24), (v, s)
        assert abs(lit - (after_lit - base_lit)) <= 1e-7 * abs(base_lit)
        checked += 1
    assert checked > 40


def test_block_neighbours_known_answers(oracle, golden):
    # dict_transpose_matrix_test.cpp:16-34: the neighbours of block 1 (keys of its row and
    # column) are {0, 1, 2} on the toy blockmodel and {0, 3, 4, 5} on the six-block one
    edges = np.array(golden["edges"], dtype=np.int32)
    g = oracle.Graph(golden["num_vertices"], edges[:, 0], edges[:, 1])
    for B, a, want in ((3, golden["assignment"], {0, 1, 2}), (6, [0, 0, 0, 1, 2, 3, 3, 4, 5, 1, 5], {0, 3, 4, 5})):
        d = oracle.Blockmodel(g, B, np.array(a, np.int32)).read()
        rows, cols = np.asarray(d["rows"]), np.asarray(d["cols"])
        assert set(cols[rows == 1].tolist()) | set(rows[cols == 1].tolist()) == want


def test_block_degrees_after_changes(oracle, golden):
    # toy_example.hpp's degrees after the vertex-7 move, after merging block 0 into 1, and
    # after moving vertex 6 of the six-block model into block 0 (common_test.cpp:17-77)
    edges = np.array(golden["edges"], dtype=np.int32)
    g = oracle.Graph(golden["num_vertices"], edges[:, 0], edges[:, 1])
    sc = golden["special_case"]
    moved = list(sc["assignment"])
    moved[sc["vertex"]] = sc["proposal"]
    for case, B, a in ((golden["vertex_move"], 3, golden["vertex_move"]["after_assignment"]),
                       (golden["block_merge"], 3, golden["block_merge"]["after_assignment"]),
                       (sc, 6, moved)):
        d = oracle.Blockmodel(g, B, np.array(a, np.int32)).read()
        assert d["d_out"].tolist() == case["after_degrees_out"]
        assert d["d_in"].tolist() == case["after_degrees_in"]
        assert d["d_tot"].tolist() == case["after_degrees"]


def _cells_after_move_check(read_after, golden):
    """The rows (block_row / proposal_row) and columns of the current and the proposed block
    after each move of finetune_test.cpp's edge-count-update tests."""
    for case in golden["cells_after_move"]:
        toy = case["blockmodel"] == "toy"
        a = list(golden["assignment"] if toy else golden["special_case"]["assignment"])
        B = golden["num_blocks"] if toy else golden["special_case"]["num_blocks"]
        cur, s = a[case["vertex"]], case["proposal"]
        a[case["vertex"]] = s
        M = read_after(B, a)
        for kind, i, v in case["values"]:
            got = {"block_row": M[cur][i], "block_col": M[i][cur], "proposal_row": M[s][i], "proposal_col": M[i][s]}[kind]
            assert got == v, (case["vertex"], kind, i)


def test_cells_after_move_known_answers(oracle, golden):
    edges = np.array(golden["edges"], dtype=np.int32)
    g = oracle.Graph(golden["num_vertices"], edges[:, 0], edges[:, 1])

    def read_after(B, a):
        d = oracle.Blockmodel(g, B, np.array(a, np.int32)).read()
        M = np.zeros((B, B), np.int64)
        M[np.asarray(d["rows"]), np.asarray(d["cols"])] = np.asarray(d["counts"])
        return M

    _cells_after_move_check(read_after, golden)


def test_max_degree_sample_known_answer(oracle, golden):
    # sample_test.cpp:26-51: 40% of the toy graph by degree is 4 vertices and 5 edges,
    # among them the listed ones (sample ids)
    edges = np.array(golden["edges"], dtype=np.int32)
    g = oracle.Graph(golden["num_vertices"], edges[:, 0], edges[:, 1])
    want = golden["sample_max_degree"]
    m, n = oracle.sample(g, "max_degree", want["sample_size"], 0)
    assert n == want["num_vertices"]
    ns, src, dst = oracle.subgraph_edges(g, m)
    assert ns == want["num_vertices"] and src.size == want["num_edges"]
    got = set(zip(src.tolist(), dst.tolist()))
    assert all(tuple(e) in got for e in want["edges"])

"""Batched and served partitioning: every job's result in the mix equals the same
partition run alone (same graph, arguments and seed), with the kernels of many jobs
sharing the device."""
import numpy as np
import pytest

from sbp_gb300 import _lib


def test_server_host_logic_without_gpu(tmp_path):
    """The server's queue, admission, pause, bounded waits, cancellation and failure paths,
    with server.cu compiled as plain C++ against stand-ins for the library calls it makes
    (tests/cpp/test_server_host.cpp)."""
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "test_server_host")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(root, "include"), "-x", "c++",
                        os.path.join(root, "sbp_gb300", "csrc", "server.cu"), "-x", "none",
                        os.path.join(root, "tests", "cpp", "test_server_host.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for _ in range(3):
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr


def test_footprint_grows_with_the_graph():
    from sbp_gb300 import serve
    a = serve.footprint(1000, 20000, 0)
    b = serve.footprint(2000, 40000, 0)
    assert 0 < a < b
    assert serve.footprint(1000, 20000, 1 << 20) == a + (1 << 20)


def _graphs(gpu, count, seed0):
    out = []
    rng = np.random.default_rng(seed0)
    for i in range(count):
        n = int(rng.integers(300, 2500))
        src, dst, planted = gpu.dcsbm.generate(n, 15 * n, int(np.sqrt(n) / 4) + 2, dmin=5, dmax=60,
                                               ratio=float(rng.uniform(1.5, 3.0)), seed=seed0 + i)
        out.append((n, src, dst, planted))
    return out


@pytest.mark.gpu
def test_server_results_equal_alone(gpu):
    graphs = _graphs(gpu, 12, 400)
    args = gpu.Args(algorithm="hybrid_mcmc")
    alone = []
    for i, (n, src, dst, _) in enumerate(graphs):
        G = gpu.Graph(n, src, dst)
        a, B, mdl, _ = gpu.sbp.stochastic_block_partition(G, gpu.Args(algorithm="hybrid_mcmc", seed=i))
        alone.append((a, B, mdl))
        G.close()
    # a small HBM budget forces queueing behind admission; 6 workers run jobs concurrently
    budget = 3 * gpu.serve.footprint(2500, 37500, 64 << 20)
    with gpu.serve.Server(workers=6, hbm_budget=budget, cells_budget=64 << 20) as srv:
        tickets = [srv.submit(n, src, dst, args, seed=i) for i, (n, src, dst, _) in enumerate(graphs)]
        mixed = [srv.wait(t) for t in tickets]
    for (a, B, mdl), (a2, B2, mdl2, info) in zip(alone, mixed):
        assert B == B2
        assert np.array_equal(a, a2)
        assert mdl == mdl2
        assert info["run_ms"] > 0


@pytest.mark.gpu
def test_batch_matches_server_and_reports_errors(gpu):
    graphs = _graphs(gpu, 5, 700)
    res = gpu.serve.partition_batch([(n, s, d) for n, s, d, _ in graphs], gpu.Args(algorithm="async_gibbs"),
                                    seeds=list(range(5)), workers=3)
    for i, (n, src, dst, _) in enumerate(graphs):
        G = gpu.Graph(n, src, dst)
        a, B, mdl, _ = gpu.sbp.stochastic_block_partition(G, gpu.Args(algorithm="async_gibbs", seed=i))
        assert np.array_equal(a, res[i][0]) and B == res[i][1]
        G.close()
    # a job whose edges leave the vertex range fails alone; the server keeps serving
    with gpu.serve.Server(workers=2, hbm_budget=1 << 34) as srv:
        bad = srv.submit(10, np.array([0, 50], np.int32), np.array([1, 2], np.int32))
        good = srv.submit(graphs[0][0], graphs[0][1], graphs[0][2], gpu.Args(algorithm="async_gibbs"), seed=0)
        with pytest.raises(_lib.SbpGpuError):
            srv.wait(bad)
        assert np.array_equal(srv.wait(good)[0], res[0][0])


# ---- failure handling, made on the host: an injected allocation failure, a cancelled
# request, a wait that runs out, a job refused over the budget.  Nothing faults the GPU.

@pytest.mark.gpu
def test_context_survives_allocation_failure_and_cancel(gpu):
    n, src, dst, _ = _graphs(gpu, 1, 950)[0]
    G = gpu.Graph(n, src, dst)
    args = gpu.Args(algorithm="hybrid_mcmc", seed=2)
    want = gpu.sbp.stochastic_block_partition(G, args)
    ctx = G.ctx
    ctx.inject_alloc_failure(2)
    with pytest.raises(_lib.SbpGpuError) as e:
        gpu.sbp.stochastic_block_partition(G, args)
    assert e.value.status == 2
    ctx.inject_alloc_failure(-1)
    ctx.set_cancel(True)  # requested before the call: it stops at its first step
    with pytest.raises(_lib.SbpGpuError) as e:
        gpu.sbp.stochastic_block_partition(G, args)
    assert e.value.status == 6
    got = gpu.sbp.stochastic_block_partition(G, args)  # the request was consumed
    assert got[1] == want[1] and np.array_equal(got[0], want[0]) and got[2] == want[2]
    G.close()


@pytest.mark.gpu
def test_server_failures_leave_it_serving(gpu):
    graphs = _graphs(gpu, 2, 960)
    args = gpu.Args(algorithm="async_gibbs")
    alone = []
    for i, (n, src, dst, _) in enumerate(graphs):
        G = gpu.Graph(n, src, dst)
        alone.append(gpu.sbp.stochastic_block_partition(G, gpu.Args(algorithm="async_gibbs", seed=i))[0])
        G.close()
    big_src, big_dst, _ = gpu.dcsbm.generate_config("C2", seed=3)
    budget = gpu.serve.footprint(60000, big_src.size, 64 << 20)
    with gpu.serve.Server(workers=2, hbm_budget=budget, cells_budget=64 << 20) as srv:
        # a job that could never fit the budget is refused at submission
        with pytest.raises(_lib.SbpGpuError) as e:
            srv.submit(3_000_000, big_src, big_dst, args)
        assert e.value.status == 2
        srv.pause()
        (n0, s0, d0, _), (n1, s1, d1, _) = graphs
        t_fail = srv.submit(n0, s0, d0, args, seed=0)
        srv.inject_alloc_failure(t_fail, 3)
        t_cancel = srv.submit(n1, s1, d1, args, seed=1)
        t_ok = srv.submit(n1, s1, d1, args, seed=1)
        srv.cancel(t_cancel)
        with pytest.raises(_lib.SbpGpuError) as e:  # paused: nothing runs
            srv.wait(t_ok, timeout=0.2)
        assert e.value.status == 3
        srv.pause(False)
        with pytest.raises(_lib.SbpGpuError) as e:
            srv.wait(t_fail)
        assert e.value.status == 2
        with pytest.raises(_lib.SbpGpuError) as e:
            srv.wait(t_cancel)
        assert e.value.status == 6
        assert np.array_equal(srv.wait(t_ok)[0], alone[1])
        # a running job stops at its next golden-section step
        t_run = srv.submit(50000, big_src, big_dst, gpu.Args(algorithm="hybrid_mcmc"), seed=0)
        with pytest.raises(_lib.SbpGpuError) as e:
            srv.wait(t_run, timeout=0.5)
        assert e.value.status == 3
        srv.cancel(t_run)
        with pytest.raises(_lib.SbpGpuError) as e:
            srv.wait(t_run)
        assert e.value.status == 6
        # and the server goes on serving
        t_after = srv.submit(n0, s0, d0, args, seed=0)
        assert np.array_equal(srv.wait(t_after)[0], alone[0])

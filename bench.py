"""Benchmark: the first golden-section step of SBP on the 1M-vertex, 20M-edge directed DCSBM
graph (the large high-overlap configuration), on one GB300 per rank.

The step is what sbp::stochastic_block_partition does first (src/sbp.cpp:23-35): from the
N-block identity partition, the block-merge pass to N/2 blocks (10 merge proposals per
block, the sequential carry-out) and then the hybrid-MCMC finetune until its early stop.
Metric: proposals/s, counting the merge proposals drawn (10 per block, repeats included, as
the reference's loop does) plus the vertex proposals visited.

Default (N=1): one JSON line with `value` (the step timed on the device with the graph
resident), the end-to-end number through the C ABI with host buffers (graph upload, the
step, the assignment read back), the roofline of the dominant kernel, the whole SBP's wall
time, NMI and block count as extra keys, and a CPU baseline: the CPU oracle on a bounded
sample of the same step.

--impl reference: the reference's CPU path for the same step and metric on all host
cores.  The reference cannot be built here (it needs MPI, tsl::robin_map, abseil, pcg and
nlohmann/json, none of which ship with it), so its line-cited port in oracle/ runs, one
bounded sample of the step per bench step (see cpu_sample).

Multi-GPU: replicas only -- each rank runs the step on its own copy of the graph; value is
the proposals of all ranks over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIG = "C3"  # --config
SEED = 1
METRIC = "proposals/s"
SAMPLE_DIV = 4         # the CPU sample: 1/4 of the first step's blocks
SAMPLE_SWEEPS = 4      # hybrid-MCMC sweeps of the CPU sample (the first step's count on C3)


def workload_desc():
    from sbp_gb300 import dcsbm
    c = dcsbm.CONFIGS[CONFIG]
    return {"workload": "first golden-section step of SBP (merge pass N -> N/2 blocks, then hybrid MCMC until its "
                        "early stop) on the directed DCSBM graph N=%d E~%d, %d planted blocks, Dirichlet(%g) sizes, "
                        "power-law degrees 2.1 in [%d,%d], within:between %g" %
                        (c["num_vertices"], c["num_edges"], c["num_blocks"], c["alpha"], c["dmin"], c["dmax"],
                         c["ratio"]),
            "num_vertices": c["num_vertices"], "num_edges_target": c["num_edges"], "algorithm": "hybrid_mcmc",
            "graph_seed": 0, "proposal_seed": SEED, "ids": "int32",
            "counts": "int32 block-edge counts (exact: every count is at most E < 2^31)",
            "proposals": "merge proposals drawn (10 per block) + vertex proposals visited",
            "l2": "flushed between steps (256 MiB write)"}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def combine_ranks(device_s, proposals, device):
    """Replicas: the slowest rank's time and the proposals of all ranks (max / sum over the
    process group when one is initialised)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(device_s)], dtype=torch.float64, device=device)
    p = torch.tensor([float(proposals)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return t.item(), p.item()


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kind):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(kind)
    except Exception:
        return None


# Algorithmic bytes of each kernel category over the timed steps.  A vertex proposal
# reads its CSR offsets (8 B) and, per neighbour, the neighbour id and its block (8 B)
# and the cell count and block degree it needs (12 B); the sampler and the special
# cells add 64 B.  The sequential chain does the same work per visited vertex.
def algorithmic_bytes(kind, stats):
    if kind == "gibbs_propose":
        return 72 * stats["gibbs_proposals"] + 20 * stats["gibbs_edges"]
    if kind == "mh_chain":
        return 72 * (stats["proposals"] - stats["gibbs_proposals"]) + 20 * (stats["edges_swept"] - stats["gibbs_edges"])
    if kind == "carry_out":
        # per recomputed merge delta: the 4 special cells, degrees and the block map (64 B);
        # per walked key: the key, its two cells and its block degree (16 B)
        return 64 * stats["carry_evaluations"] + 16 * stats["carry_keys"]
    return None


def hub_mask(n, src, dst, mh_percent=0.075):
    """Graph::sort_vertices (src/graph.cpp:235-268): the top mh_percent of the vertices by
    degree (out + in - has a self-loop), stable in vertex order, are the high-degree
    vertices the hybrid MCMC walks as a sequential chain."""
    deg = np.bincount(src, minlength=n) + np.bincount(dst, minlength=n)
    deg -= np.bincount(src[src == dst], minlength=n) > 0
    order = np.argsort(-deg, kind="stable")
    mask = np.zeros(n, bool)
    limit = np.float32(mh_percent) * np.float32(n)  # float arithmetic as graph.cpp:252
    mask[order[:int(np.count_nonzero(np.arange(n, dtype=np.float32) < limit))]] = True
    return mask


def split_planted(planted, n, target_blocks, seed=3):
    """The planted partition with every planted block split at random into sub-blocks,
    about target_blocks blocks in all, numbered densely."""
    rng = np.random.default_rng(seed)
    k = max(1, -(-target_blocks // (int(planted.max()) + 1)))
    _, a = np.unique(planted.astype(np.int64) * k + rng.integers(0, k, n), return_inverse=True)
    return a.astype(np.int32)


class CpuSample:
    """The oracle (the reference's hot path restated, OpenMP over all host cores) on a bounded
    sample of the bench step (ora_step_sample): the merge pass's proposal loop
    (block_merge.cpp:188-217) over a random 1/SAMPLE_DIV of the blocks of the N-block
    identity partition, the carry-out of their queue to half as many merges
    (block_merge.cpp:40-117), then SAMPLE_SWEEPS hybrid-MCMC sweeps (finetune.cpp:563-646)
    over the vertices of the merged blocks, their high-degree vertices as the sequential
    chain.  Measured against the complete step on the same cores, such a sample runs about
    2.4 times faster per proposal (its carry-out has fewer put-backs and smaller blocks), so
    it favours the CPU."""

    def __init__(self, src, dst, n):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_bind as ob
        ob.build()
        self.ob = ob
        self.cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(self.cores))
        self.n = n
        self.g = ob.Graph(n, src, dst)
        self.hub = hub_mask(n, src, dst)
        self.cfg = ob.make_config("hybrid_mcmc")

    def run(self, index=0):
        bm = self.ob.Blockmodel(self.g, self.n, np.arange(self.n, dtype=np.int32))
        rng = np.random.default_rng(1000 + index)
        m = max(2, self.n // SAMPLE_DIV)
        blocks = np.sort(rng.choice(self.n, m, replace=False)).astype(np.int32)
        t0 = time.perf_counter()
        draws, merges, vprops = bm.step_sample(blocks, self.hub, SEED, 0, self.cfg, SAMPLE_SWEEPS)
        dt = time.perf_counter() - t0
        return {"value": (draws + vprops) / dt, "unit": METRIC, "cores": int(os.environ["OMP_NUM_THREADS"]),
                "kind": "port",
                "sample": "first golden-section step on a random 1/%d of the blocks: %d merge proposals drawn, "
                          "%d merges carried out, %d hybrid-MCMC vertex proposals (%d sweeps) in %.2f s"
                          % (SAMPLE_DIV, draws, merges, vprops, SAMPLE_SWEEPS, dt)}


def reference_arm(args):
    """The complete bench step on the CPU, once: the oracle's merge_blocks from the N-block
    identity partition to N/2 blocks and its hybrid MCMC with the pre-bracket early stop,
    all host cores -- the same work the device arm times per step, so no sampling enters
    the ratio.  One step takes about two minutes of host time, so --steps / --warmup do not
    repeat it."""
    ws, rank, local = dist_info()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    from sbp_gb300 import dcsbm
    ob.build()
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    src, dst, planted = dcsbm.generate_config(CONFIG, seed=0)
    n = dcsbm.CONFIGS[CONFIG]["num_vertices"]
    g = ob.Graph(n, src, dst)
    bm = ob.Blockmodel(g, n, np.arange(n, dtype=np.int32))
    cfg = ob.make_config("hybrid_mcmc")
    t0 = time.perf_counter()
    s1 = bm.merge_blocks(cfg, seed=SEED, step=0, num_to_merge=n // 2)
    s2 = bm.mcmc(cfg, seed=SEED, step=0, golden_ratio_not_reached=True)
    dt = time.perf_counter() - t0
    props = 10 * n + s2.proposals
    value = props / dt
    cores = int(os.environ["OMP_NUM_THREADS"])
    sample = ("the complete step once: merge pass %d -> %d blocks (%d merges) and hybrid MCMC (%d sweeps, %d vertex "
              "proposals), %d proposals in %.1f s" % (n, n - n // 2, s1.merges, s2.mcmc_iterations, s2.proposals,
                                                       props, dt))
    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": 1, "warmup": 0,
           "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "int64+f64", "data": "synthetic (seeded DCSBM)", "config": workload_desc(), "impl": "reference",
           "note": "one complete step (about two minutes of host time) instead of --steps %d --warmup %d samples"
                   % (args.steps, args.warmup),
           "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def profile_phase(args):
    """One phase of the same workload at a fixed block count, for profilers: the planted
    partition with every planted block split at random into sub-blocks (about --blocks
    blocks in all; the identity partition when --blocks is at least N), then either the
    merge pass to half as many blocks or --iterations hybrid-MCMC iterations.  Prints a
    short JSON summary with the per-kernel CUDA-event times, not a bench line."""
    import torch
    import sbp_gb300 as sb
    from sbp_gb300 import build as _b
    _b.build()
    src, dst, planted = sb.dcsbm.generate_config(CONFIG, seed=0)
    n = sb.dcsbm.CONFIGS[CONFIG]["num_vertices"]
    a = np.arange(n, dtype=np.int32) if args.blocks >= n else split_planted(planted, n, args.blocks)
    B = int(a.max()) + 1
    ctx = sb.Context(0)
    if args.cells_budget is not None:
        ctx.set_cells_budget(args.cells_budget)
    ctx.set_timing(True)
    G = sb.Graph(n, src, dst, ctx=ctx)
    bm = sb.Blockmodel(B, G, 0.5, a)
    sargs = sb.Args(algorithm="hybrid_mcmc", seed=SEED, max_iterations=args.iterations)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if args.phase == "merge":
        _, st = sb.block_merge.merge_blocks(bm, G, args=sargs, step=0, num_blocks_to_merge=B // 2)
    else:
        _, st = sb.finetune.mcmc(0, G, bm, True, sargs)
    ctx.synchronize()
    print(json.dumps({"phase": args.phase, "config": CONFIG, "blocks_before": B, "blocks_after": bm.num_blocks(),
                      "seconds": time.perf_counter() - t0, "stats": st, "kernel_timing": ctx.read_timing()}))


def _mixed_graph(n, seed):
    from sbp_gb300 import dcsbm
    r = np.random.default_rng(seed)
    src, dst, planted = dcsbm.generate(int(n), 20 * int(n), int(np.sqrt(n) / 4) + 2, dmin=5, dmax=100,
                                       ratio=float(r.uniform(1.5, 3.0)), seed=seed)
    return int(n), src, dst, planted


def mixed_graphs(count, n_lo, n_hi, seed_base=0):
    """Independent directed DCSBM graphs: N log-uniform in [n_lo, n_hi], about 20 N edges,
    floor(sqrt(N) / 4) + 2 planted blocks, within:between ratio uniform in [1.5, 3.0], degree
    propensities power-law 2.1 in [5, 100]; graph i uses seed seed_base + i.  Many graphs
    are generated by a pool of spawned processes (before this process starts CUDA)."""
    rng = np.random.default_rng(20240 + seed_base)
    sizes = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), count)).astype(np.int64)
    seeds = [seed_base + i for i in range(count)]
    if count * float(np.mean(sizes)) < 2e6:
        return [_mixed_graph(n, sd) for n, sd in zip(sizes, seeds)]
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_mixed_graph, sizes, seeds, chunksize=4))


def plain_one_at_a_time(graphs, sargs, only=None):
    """The plain path: each graph uploaded, partitioned and read back in turn on one context
    (graph i with seed i); `only`: the indices to run, others get None."""
    import torch
    import sbp_gb300 as sb
    ctx = sb.Context(0)
    ctx.set_cells_budget(256 << 20)
    results, service = [], []
    for i, (n, src, dst, _) in enumerate(graphs):
        if only is not None and i not in only:
            results.append(None)
            service.append(None)
            continue
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        G = sb.Graph(n, src, dst, ctx=ctx)
        a, B, mdl, _ = sb.sbp.stochastic_block_partition(G, sb.Args(algorithm=sargs.algorithm, seed=i))
        G.close()
        service.append(time.perf_counter() - t0)
        results.append((a, B, mdl))
    ctx.close()
    return results, service


def many_streams():
    """Concurrent jobs run on many streams; without this the process maps all streams onto
    8 hardware queues and kernels of unrelated jobs wait behind one another.  Must be set
    before CUDA starts in this process."""
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")


def batched_workload(args):
    """Many mixed-size graphs partitioned concurrently on one GPU (the batched
    configuration) against the same graphs partitioned one at a time; both produce the
    same partitions, so NMI is equal by construction (checked)."""
    many_streams()
    import sbp_gb300 as sb
    from sbp_gb300 import build as _b
    _b.build()
    graphs = mixed_graphs(args.jobs, 500, 20000)
    sargs = sb.Args(algorithm="hybrid_mcmc")
    plain, service = plain_one_at_a_time(graphs, sargs)
    t0 = time.perf_counter()
    res = sb.serve.partition_batch([(n, s, d) for n, s, d, _ in graphs], sargs, seeds=list(range(len(graphs))),
                                   workers=args.workers, hbm_budget=args.hbm_budget, cells_budget=256 << 20)
    t_batch = time.perf_counter() - t0
    same = all(np.array_equal(p[0], r[0]) and p[1] == r[1] for p, r in zip(plain, res))
    nmis = [sb.evaluate.nmi(g[3], r[0]) for g, r in zip(graphs, res)]
    t_plain = float(np.sum(service))
    print(json.dumps({"workload": "batched", "metric": "jobs/s", "value": len(graphs) / t_batch, "unit": "jobs/s",
                      "jobs": len(graphs), "workers": args.workers,
                      "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"), "batched_s": t_batch, "plain_s": t_plain,
                      "plain_jobs_per_s": len(graphs) / t_plain, "speedup_vs_plain": t_plain / t_batch,
                      "identical_to_plain": bool(same), "mean_nmi": float(np.mean(nmis)),
                      "total_vertices": int(sum(g[0] for g in graphs)),
                      "total_edges": int(sum(g[1].size for g in graphs)),
                      "config": {"workload": "%d directed DCSBM graphs, N log-uniform in [500, 20000], ~20 N edges, "
                                             "floor(sqrt(N)/4)+2 planted blocks, ratio U[1.5, 3], degrees 2.1 in "
                                             "[5, 100], seeds 0..%d, hybrid MCMC" % (len(graphs), len(graphs) - 1),
                                 "data": "synthetic (seeded DCSBM)"}}))


def served_workload(args):
    """A Poisson stream of partition requests served concurrently, against the same stream
    served one request at a time on the plain path (its latencies follow from each
    request's measured plain service time: a single FIFO server)."""
    import concurrent.futures as cf
    many_streams()
    import sbp_gb300 as sb
    from sbp_gb300 import build as _b
    _b.build()
    graphs = mixed_graphs(args.jobs, 1000, args.max_vertices, seed_base=10000)
    sargs = sb.Args(algorithm="hybrid_mcmc")
    k = args.plain_sample if 0 < args.plain_sample < len(graphs) else len(graphs)
    sample = set(np.random.default_rng(5).choice(len(graphs), k, replace=False).tolist())
    plain, service = plain_one_at_a_time(graphs, sargs, only=sample)
    fit = None
    if k < len(graphs):
        # service time of the requests not run on the plain path: a least-squares line in
        # the edge count through the measured ones
        xs = np.array([graphs[i][1].size for i in sorted(sample)], float)
        ys = np.array([service[i] for i in sorted(sample)], float)
        b, a = np.polyfit(xs, ys, 1)
        r2 = 1.0 - float(np.sum((ys - (a + b * xs)) ** 2) / np.sum((ys - ys.mean()) ** 2))
        fit = {"measured": k, "seconds_per_edge": b, "seconds_fixed": a, "r2": r2}
        service = [service[i] if i in sample else a + b * graphs[i][1].size for i in range(len(graphs))]
    plain_rate = len(graphs) / float(np.sum(service))
    rate = args.rate if args.rate else args.rate_factor * plain_rate
    arrivals = np.cumsum(np.random.default_rng(77).exponential(1.0 / rate, len(graphs)))
    finish_plain, t_free = [], 0.0
    for a_t, s_t in zip(arrivals, service):
        t_free = max(a_t, t_free) + s_t
        finish_plain.append(t_free)
    lat_plain = np.array(finish_plain) - arrivals
    done = [None] * len(graphs)
    with sb.serve.Server(workers=args.workers, hbm_budget=args.hbm_budget, cells_budget=256 << 20) as srv, \
            cf.ThreadPoolExecutor(max_workers=64) as pool:
        t0 = time.perf_counter()
        futures = []
        for i, (n, src, dst, _) in enumerate(graphs):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tk = srv.submit(n, src, dst, sargs, seed=i)

            def finish(tk=tk, i=i):
                out = srv.wait(tk)
                done[i] = (time.perf_counter() - t0, out)
            futures.append(pool.submit(finish))
        for f in futures:
            f.result()
        makespan = time.perf_counter() - t0
    lat = np.array([done[i][0] - arrivals[i] for i in range(len(graphs))])
    differ = [i for i in sorted(sample) if not np.array_equal(plain[i][0], done[i][1][0])]
    same = not differ
    print(json.dumps({"workload": "served", "metric": "jobs/s", "value": len(graphs) / makespan, "unit": "jobs/s",
                      "requests": len(graphs), "offered_rate_per_s": rate, "workers": args.workers,
                      "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                      "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                      "plain_p50_ms": 1e3 * float(np.percentile(lat_plain, 50)),
                      "plain_p99_ms": 1e3 * float(np.percentile(lat_plain, 99)),
                      "plain_jobs_per_s": plain_rate, "identical_to_plain": bool(same),
                      "differing_requests": [{"request": i, "num_vertices": graphs[i][0], "blocks": [plain[i][1], done[i][1][1]],
                                              "mdl": [plain[i][2], done[i][1][2]]} for i in differ],
                      "plain_service": "measured for every request" if fit is None else
                      dict(fit, note="measured for a seeded sample (their partitions compared), the rest "
                                     "predicted by the fit"),
                      "served_s": makespan,
                      "mean_nmi": float(np.mean([sb.evaluate.nmi(graphs[i][3], done[i][1][0])
                                                 for i in range(len(graphs))])),
                      "config": {"workload": "%d requests, Poisson arrivals at %.2f/s, N log-uniform in [1000, %d], "
                                             "~20 N edges, floor(sqrt(N)/4)+2 planted blocks, ratio U[1.5, 3], "
                                             "hybrid MCMC" % (len(graphs), rate, args.max_vertices),
                                 "data": "synthetic (seeded DCSBM)"}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end C ABI run (profiling)")
    ap.add_argument("--no-full-sbp", action="store_true", help="skip the whole-SBP run after the timed steps")
    ap.add_argument("--config", default=CONFIG, choices=["C1", "C2", "C3", "C3S"])
    ap.add_argument("--cells-budget", type=int, default=None,
                    help="device bytes for the carry-out's dense cell counts (library default if unset)")
    ap.add_argument("--phase", default="sbp", choices=["sbp", "merge", "mcmc"],
                    help="merge / mcmc: one phase at --blocks blocks for profilers (no bench line)")
    ap.add_argument("--blocks", type=int, default=1500)
    ap.add_argument("--iterations", type=int, default=2)
    ap.add_argument("--workload", default="sbp", choices=["sbp", "batched", "served"],
                    help="batched / served: many graphs through the partition server (own JSON line)")
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--hbm-budget", type=int, default=64 << 30)
    ap.add_argument("--rate", type=float, default=0.0, help="served: offered requests/s (0: derived)")
    ap.add_argument("--max-vertices", type=int, default=50000)
    ap.add_argument("--plain-sample", type=int, default=0,
                    help="served: run only this many requests on the plain path (0: all)")
    ap.add_argument("--rate-factor", type=float, default=0.8,
                    help="served: offered rate as a multiple of the plain path's throughput")
    args = ap.parse_args()
    globals()["CONFIG"] = args.config
    if args.impl == "reference":
        return reference_arm(args)
    if args.phase != "sbp":
        return profile_phase(args)
    if args.workload == "batched":
        return batched_workload(args)
    if args.workload == "served":
        return served_workload(args)

    import torch
    import sbp_gb300 as sb
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from sbp_gb300 import build as _b
    _b.build()
    src, dst, planted = sb.dcsbm.generate_config(CONFIG, seed=0)
    n = sb.dcsbm.CONFIGS[CONFIG]["num_vertices"]
    ident = np.arange(n, dtype=np.int32)
    ctx = sb.Context(local)
    if args.cells_budget is not None:
        ctx.set_cells_budget(args.cells_budget)
    G = sb.Graph(n, src, dst, ctx=ctx)  # resident in HBM before the timed region
    sargs = sb.Args(algorithm="hybrid_mcmc", seed=SEED)
    stream = torch.cuda.ExternalStream(ctx.lib.sbpgpu_ctx_stream(ctx.h), device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=local)

    def first_step(graph):
        """Blockmodel(N, graph, 0.5) on the identity partition (sbp.cpp:23), built before
        the caller's timing starts."""
        return sb.Blockmodel(n, graph, 0.5, ident)

    def run_step(bm):
        """The golden-section step (sbp.cpp:27-35): merge_blocks to N/2 blocks, then the
        hybrid-MCMC finetune with the pre-bracket early stop.  Returns (proposals drawn,
        merge stats, mcmc stats)."""
        _, s1 = sb.block_merge.merge_blocks(bm, bm.graph, args=sargs, step=0, num_blocks_to_merge=n // 2)
        _, s2 = sb.finetune.mcmc(0, bm.graph, bm, True, sargs)
        return 10 * n + s2["proposals"], s1, s2

    for _ in range(args.warmup):
        bm = first_step(G)
        run_step(bm)
        bm.close()
    torch.cuda.synchronize()

    ctx.set_timing(True)
    ctx.read_timing()  # reset accumulators
    clocks = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    step_ms, totals, proposals, iters = [], {}, 0, []
    t_all0 = time.perf_counter()
    for _ in range(args.steps):
        bm = first_step(G)
        flush.fill_(1)
        ctx.synchronize()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        p, s1, s2 = run_step(bm)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        proposals += p
        iters.append(s2["mcmc_iterations"])
        for st in (s1, s2):
            for k, v in st.items():
                totals[k] = totals.get(k, 0) + v
        last_bm = bm
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - t_all0
    clk = clocks.stop()
    timing = ctx.read_timing()
    ctx.set_timing(False)
    step_blocks = last_bm.num_blocks()
    step_mdl = last_bm.getOverall_entropy()
    last_bm.close()
    device_s = sum(step_ms) / 1e3
    slowest_s, all_props = combine_ranks(device_s, proposals, local)
    value = all_props / slowest_s

    # end to end through the C ABI with host buffers: graph upload, the step, the
    # assignment read back
    e2e_s, e2e_props = 0.0, 0
    for _ in range(0 if args.no_e2e else max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Gh = sb.Graph(n, src, dst, ctx=ctx)
        bm = first_step(Gh)
        p, _, _ = run_step(bm)
        asg_h = bm.block_assignment()
        bm.close()
        Gh.close()
        torch.cuda.synchronize()
        e2e_s += time.perf_counter() - t0
        e2e_props += p
    E = int(src.size)
    loops = int(np.sum(src == dst))
    h2d = 4 * ((n + 1) * 2 + E + (E - loops) + n + E + (E + 2) + n) + 4 * n
    d2h = 4 * n

    # the whole SBP once, for the full-SBP wall time and quality beside the step rate
    full = {}
    if not args.no_full_sbp:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        asg, B, mdl, st = sb.sbp.stochastic_block_partition(G, sargs)
        torch.cuda.synchronize()
        full = {"full_sbp_s": time.perf_counter() - t0, "full_sbp_blocks": int(B), "full_sbp_mdl": mdl,
                "full_sbp_nmi": sb.evaluate.nmi(planted, asg), "full_sbp_outer_steps": st["outer_steps"],
                "full_sbp_proposals": st["proposals"] + st["merge_proposals"]}

    # roofline of the dominant kernel category
    cats = {k[:-3]: v for k, v in timing.items() if k.endswith("_ms")}
    dom = max(cats, key=lambda k: cats[k])
    launches = timing.get(dom + "_launches", 0) or 1
    peak, peak_kind = measured_peak_hbm()
    alg_bytes = algorithmic_bytes(dom, totals)
    roof = {"kernel": dom, "bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": peak_kind,
            "launches": launches, "avg_launch_ms": cats[dom] / launches,
            "time_share": cats[dom] / max(1e-9, sum(step_ms)),
            "traffic": ncu_traffic(dom)}
    if alg_bytes:
        achieved = alg_bytes / launches / (cats[dom] / launches / 1e3) / 1e9
        roof.update({"achieved": achieved, "frac": achieved / peak})
    else:
        roof.update({"achieved": None, "frac": None,
                     "note": "latency-bound sequential phase; no bandwidth roofline applies"})
    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic (seeded DCSBM)",
           "config": dict(workload_desc(), parallelism="replicas" if ws > 1 else "single GPU"),
           "wall_s": wall, "step_blocks": int(step_blocks), "step_mdl": step_mdl,
           "step_mcmc_iterations": iters[-1] if iters else None,
           "proposals_per_step": proposals / args.steps,
           "merge_proposals_drawn_per_step": 10.0 * n,
           "vertex_proposals_per_step": totals.get("proposals", 0) / args.steps,
           "merges_per_step": totals.get("merges", 0) / args.steps,
           "edges_swept_per_s": totals.get("edges_swept", 0) / device_s,
           "kernel_ms": cats, "gpu_launches": int(totals.get("kernel_launches", 0)),
           "e2e": {"value": e2e_props / e2e_s if e2e_s > 0 else None, "unit": METRIC,
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "roofline": roof, "clocks": clk}
    out.update(full)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = CpuSample(src, dst, n).run(0)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

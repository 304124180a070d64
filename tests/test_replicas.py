"""Multi-GPU is replicas only: every rank partitions its own copy of the graph and the
bench reports all ranks' proposals over the slowest rank's time.  The cross-rank logic
runs here on CPU with two gloo ranks; no GPU is involved."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_info()
        slowest, props = bench.combine_ranks(1.5 + rank, 1000 * (rank + 1), "cpu")
        # the reference arm prints only on rank 0; other ranks return without work
        buf = io.StringIO()
        if rank != 0:
            with redirect_stdout(buf):
                bench.reference_arm(type("A", (), {"warmup": 0, "steps": 1, "gpus": world})())
        dist.barrier()
        results[rank] = (ws, r, slowest, props, buf.getvalue())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replicas_combine_over_gloo(world):
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, results)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        ws, rank, slowest, props, out = results[r]
        assert (ws, rank) == (world, r)
        assert slowest == 1.5 + (world - 1)                       # max over ranks
        assert props == sum(1000 * (k + 1) for k in range(world))  # all ranks' work
        if r != 0:
            assert out == ""


def test_single_process_combine_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(2.5, 77, "cpu") == (2.5, 77.0)

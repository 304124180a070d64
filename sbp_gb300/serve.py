"""Batched and served partitioning (sbpgpu_server_* in include/sbpgpu.h).

A Server partitions many independent graphs concurrently on one GPU: worker threads in the
library, each with its own context and stream, admit jobs in submission order while the
estimated device footprint of the jobs in flight fits the HBM budget.  Every job's result
equals stochastic_block_partition of the same graph, arguments and seed run alone.

Set CUDA_DEVICE_MAX_CONNECTIONS=32 in the environment before CUDA starts in the process:
with the default of 8 hardware queues the workers' streams share queues and their kernels
wait behind one another (about 3x lower throughput measured with 16 workers).
"""
import ctypes

import numpy as np

from . import _lib
from .core import Args

_i32p = ctypes.POINTER(ctypes.c_int32)


def footprint(num_vertices, num_edges, cells_budget):
    """Estimated device bytes of one job."""
    return int(_lib.load().sbpgpu_job_footprint(int(num_vertices), int(num_edges), int(cells_budget)))


class Server:
    """Partition server on one device.  submit() returns a ticket; wait(ticket) returns
    (assignment, num_blocks, mdl, info) with info holding queued_ms, run_ms and the stats."""

    def __init__(self, device=0, workers=16, hbm_budget=64 << 30, cells_budget=256 << 20):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        st = self.lib.sbpgpu_server_create(int(device), int(workers), int(hbm_budget), int(cells_budget),
                                           ctypes.byref(h))
        if st != 0:
            raise _lib.SbpGpuError(st, "cannot create a partition server")
        self.h = h
        self._keep = {}

    def submit(self, num_vertices, src, dst, args=None, seed=None):
        a = args or Args()
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        out = np.zeros(int(num_vertices), np.int32)
        job = _lib.Job(int(num_vertices), src.size, src.ctypes.data_as(_i32p), dst.ctypes.data_as(_i32p), a.config(),
                       int(a.seed if seed is None else seed), out.ctypes.data_as(_i32p))
        t = ctypes.c_int64()
        st = self.lib.sbpgpu_server_submit(self.h, ctypes.byref(job), ctypes.byref(t))
        if st != 0:
            raise _lib.SbpGpuError(st, "job rejected")
        self._keep[t.value] = (src, dst, out, job)
        return t.value

    def wait(self, ticket, timeout=None):
        """The job's result; with `timeout` (seconds) raises SbpGpuError(SBPGPU_ETIMEOUT)
        when it is not done by then, and the ticket stays valid."""
        r = _lib.JobResult()
        if timeout is None:
            st = self.lib.sbpgpu_server_wait(self.h, int(ticket), ctypes.byref(r))
        else:
            st = self.lib.sbpgpu_server_wait_for(self.h, int(ticket), int(timeout * 1000), ctypes.byref(r))
        if st == 3:
            raise _lib.SbpGpuError(st, "job not done within %s s" % timeout)
        if st != 0:
            raise _lib.SbpGpuError(st, "unknown ticket")
        src, dst, out, job = self._keep.pop(ticket)
        if r.status != 0:
            raise _lib.SbpGpuError(r.status, r.error.decode(errors="replace"))
        info = {"queued_ms": r.queued_ms, "run_ms": r.run_ms, "stats": r.stats.as_dict()}
        return out, int(r.num_blocks), float(r.mdl), info

    def cancel(self, ticket):
        """Cancels a queued job at once or a running one at its next golden-section step;
        its wait() then raises SbpGpuError(SBPGPU_ECANCELED) unless it finished first."""
        st = self.lib.sbpgpu_server_cancel(self.h, int(ticket))
        if st != 0:
            raise _lib.SbpGpuError(st, "unknown ticket")

    def pause(self, paused=True):
        """Stops (or resumes) the start of queued jobs; running jobs go on."""
        self.lib.sbpgpu_server_pause(self.h, int(bool(paused)))

    def inject_alloc_failure(self, ticket, after):
        """Test hook: the queued job fails its device allocation number `after` + 1."""
        st = self.lib.sbpgpu_server_inject_alloc_failure(self.h, int(ticket), int(after))
        if st != 0:
            raise _lib.SbpGpuError(st, "job unknown or already started")

    def close(self):
        if getattr(self, "h", None):
            self.lib.sbpgpu_server_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def partition_batch(graphs, args=None, seeds=None, workers=16, hbm_budget=64 << 30, cells_budget=256 << 20,
                    device=0):
    """The batched form: graphs is a list of (num_vertices, src, dst); returns one
    (assignment, num_blocks, mdl, info) per graph, in order."""
    with Server(device, workers, hbm_budget, cells_budget) as s:
        tickets = [s.submit(n, src, dst, args, None if seeds is None else seeds[i])
                   for i, (n, src, dst) in enumerate(graphs)]
        return [s.wait(t) for t in tickets]

"""The allocation-free delta-MDL batch (sbpgpu_delta_mdl_batch_noalloc) against the
allocating entry point (sbpgpu_delta_mdl_batch), both called through the C ABI.

Both run the same scoring kernel, so the values must agree to the delta-MDL tolerance
(they are in fact identical).  Two calls in a row check that the staging array carries
nothing from one call into the next; entries whose proposal is the vertex's own block
take the zero-delta path.  That the call allocates nothing is checked through the
context's allocation-failure injection: with the next device allocation set to fail, the
allocation-free call still succeeds while the allocating one reports SBPGPU_ENOMEM.  This
file is collected last so the check also runs after every other GPU test in the same
process."""
import numpy as np
import pytest

from sbp_gb300 import _lib

pytestmark = pytest.mark.gpu

DELTA_REL_TOL = 1e-10
MAX_BATCH = 65536


def _call(lib, name, bm, v, s):
    out = np.full(v.size, np.nan, np.float64)
    st = getattr(lib, name)(bm.h, v.size, v.ctypes.data_as(_lib.i32p), s.ctypes.data_as(_lib.i32p),
                            out.ctypes.data_as(_lib.f64p))
    return st, out


def test_noalloc_delta_matches_allocating_entry_point(gpu):
    n, B = 3000, 40
    src, dst, _ = gpu.dcsbm.generate(n, 36000, 9, seed=123)
    ctx = gpu.Context(0)
    try:
        G = gpu.Graph(n, src, dst, ctx=ctx)
        rng = np.random.default_rng(9)
        a = rng.integers(0, B, n).astype(np.int32)
        a[:B] = np.arange(B)
        bm = gpu.Blockmodel(B, G, 0.5, a)
        lib = ctx.lib
        for size in (MAX_BATCH, 5000):  # the largest accepted batch, then a smaller one
            v = rng.integers(0, n, size).astype(np.int32)
            s = rng.integers(0, B, size).astype(np.int32)
            s = np.where(s == a[v], (s + 1) % B, s).astype(np.int32)
            own = rng.random(size) < 0.1  # these propose the vertex's own block
            s[own] = a[v[own]]
            st, want = _call(lib, "sbpgpu_delta_mdl_batch", bm, v, s)
            assert st == _lib.SBPGPU_OK, lib.sbpgpu_last_error(ctx.h)
            assert np.all(want[own] == 0.0)
            for _ in range(2):
                ctx.inject_alloc_failure(0)  # the next device allocation through ctx fails
                st, got = _call(lib, "sbpgpu_delta_mdl_batch_noalloc", bm, v, s)
                ctx.inject_alloc_failure(-1)
                assert st == _lib.SBPGPU_OK, lib.sbpgpu_last_error(ctx.h)
                assert np.all(np.abs(got - want) <= DELTA_REL_TOL * np.maximum(1.0, np.abs(want)))
                assert np.all(got[own] == 0.0)
        ctx.inject_alloc_failure(0)  # control: the allocating entry point does allocate
        st, _ = _call(lib, "sbpgpu_delta_mdl_batch", bm, v, s)
        ctx.inject_alloc_failure(-1)
        assert st == _lib.SBPGPU_ENOMEM
    finally:
        ctx.close()


def test_noalloc_rejects_batches_beyond_its_limit(gpu):
    n, B = 500, 6
    src, dst, _ = gpu.dcsbm.generate(n, 4000, 3, seed=5)
    ctx = gpu.Context(0)
    try:
        G = gpu.Graph(n, src, dst, ctx=ctx)
        a = (np.arange(n) % B).astype(np.int32)
        bm = gpu.Blockmodel(B, G, 0.5, a)
        v = (np.arange(MAX_BATCH + 1) % n).astype(np.int32)
        s = ((a[v] + 1) % B).astype(np.int32)
        st, _ = _call(ctx.lib, "sbpgpu_delta_mdl_batch_noalloc", bm, v, s)
        assert st == 1  # SBPGPU_EINVAL
        assert b"65536" in ctx.lib.sbpgpu_last_error(ctx.h)
    finally:
        ctx.close()

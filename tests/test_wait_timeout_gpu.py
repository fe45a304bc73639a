"""Failure detection of the split GEMMs' bounded waits, without a GPU fault.

zest_gpu_selftest_wait_timeout runs one kernel whose mbarrier wait nothing
ever completes: the wait gives up after its limit and sets the error flag,
a second wait in the same kernel (with the GEMMs' own 2 s limit) gives up as
soon as it sees the flag, the flag reaches the host through the same mapped
host word as a GEMM timeout, and the call returns ZEST_GPU_ERR_TIMEOUT.
Afterwards the flag is clear and the context still transforms correctly."""
import time

import numpy as np
import pytest

from oracle import zt_grid_shape

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


def test_expired_wait_is_reported_and_the_context_stays_usable(ctx):
    import zest_gb300 as zg
    rng = np.random.default_rng(3)
    L, batch = 20, 2
    g = rng.normal(size=int(np.prod(zt_grid_shape(L))) * batch)
    ctx.set_precision(zg.PRECISION_SPLIT, 6)
    try:
        before = ctx.zt_forward(g, L, batch=batch)
        for _ in range(2):  # the flag is cleared after each report
            t0 = time.perf_counter()
            rc = ctx.lib.zest_gpu_selftest_wait_timeout(ctx._h, 0.05)
            dt = time.perf_counter() - t0
            assert rc == zg.ERR_TIMEOUT
            assert b"bounded wait expired" in ctx.lib.zest_gpu_last_error()
            assert dt < 1.5  # the second wait did not sit out its own 2 s limit
            after = ctx.zt_forward(g, L, batch=batch)
            np.testing.assert_array_equal(after, before)
    finally:
        ctx.set_precision(zg.PRECISION_FP64)


def test_wait_limit_is_checked(ctx):
    import zest_gb300 as zg
    for bad in (0.0, 1e-4, 3.0, float("nan")):
        assert ctx.lib.zest_gpu_selftest_wait_timeout(ctx._h, bad) == zg.ERR_INVALID

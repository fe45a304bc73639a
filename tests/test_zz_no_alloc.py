"""Zernike rotation that allocates no device memory
(zest_gpu_zt_rotate_noalloc), called through the C-ABI on caller-owned device
buffers and compared with zest_gpu_zt_rotate on the same inputs, on two calls
in a row: the first sets up the scratch array, the second reuses it.
Tolerance 1e-13 relative max-norm (both run the same FP64 kernels)."""
import ctypes

import numpy as np
import pytest

from oracle import zidx, zt_coeff_size

pytestmark = pytest.mark.gpu

TOL = 1e-13


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rand_zt(rng, L, batch):
    c = np.zeros((batch, zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[:, zidx(n, l, m)] = rng.normal(size=(batch, 2)) * (n + 1) ** -1.5
                if m == 0:
                    c[:, zidx(n, l, m), 1] = 0.0
    return c


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    import zest_gb300
    from zest_gb300 import build
    build.build()
    torch.cuda.set_device(0)
    ctx = zest_gb300.Context(0)
    yield torch, zest_gb300, ctx
    ctx.close()


def _noalloc(zg, stream, L, batch, coeffs, euler, rtype, wig, wig_order):
    lib = zg.library()
    return lib.zest_gpu_zt_rotate_noalloc(ctypes.c_void_p(stream), L, batch, ctypes.c_void_p(coeffs),
                                          ctypes.c_void_p(euler), rtype, ctypes.c_void_p(wig), wig_order)


# One module load (the library's kernels and its fixed scratch array) is the
# only device memory the set-up call may bring in; later calls bring in none.
MODULE_LOAD_TOLERANCE = 64 << 20


def _torch_counters(torch):
    st = torch.cuda.memory_stats(0)
    return {k: st.get(k, 0) for k in ("allocation.all.allocated", "segment.all.allocated",
                                      "allocated_bytes.all.allocated", "reserved_bytes.all.allocated")}


def _free_bytes_after(torch, fn):
    """Device free bytes before and after fn(), measured on a synchronized
    device.  The free figure covers the whole device, which other processes
    may share, so a mismatch is measured once more before it counts."""
    for attempt in range(2):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        out = fn()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info(0)[0]
        if attempt == 1 or free1 == free0:
            return free0, free1, out
    raise AssertionError("unreachable")


def test_zt_rotate_noalloc_matches_context_path(env):
    torch, zg, ctx = env
    L, batch = 40, 5
    # the caller's Wigner table, made once at set-up (order above L is allowed)
    wig = torch.from_numpy(ctx.wignerd_table(L + 3)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for call, rtype in enumerate([zg.ROTATION_OBJECT, zg.ROTATION_COORDINATE]):
        rng = np.random.default_rng(call)
        c = rand_zt(rng, L, batch).ravel()
        euler = rng.uniform(-np.pi, np.pi, size=3 * batch)
        ref = ctx.zt_rotate(c.copy(), L, euler.copy(), batch=batch, rotation_type=rtype)
        dc = torch.from_numpy(c).cuda()
        de = torch.from_numpy(euler).cuda()
        dc_start = dc.clone()
        counters0 = _torch_counters(torch)

        def run():
            dc.copy_(dc_start)
            return _noalloc(zg, stream, L, batch, dc.data_ptr(), de.data_ptr(), rtype, wig.data_ptr(), L + 3)

        free0, free1, rc = _free_bytes_after(torch, run)
        assert rc == 0, zg.library().zest_gpu_last_error()
        assert relmax(dc.cpu().numpy(), ref) < TOL
        # no allocation through torch's allocator
        assert _torch_counters(torch) == counters0
        if call == 0:  # the set-up call: at most one module load
            assert free0 - free1 <= MODULE_LOAD_TOLERANCE
        else:  # past the set-up call, device memory use does not move
            assert free1 == free0


def test_zt_rotate_noalloc_rejects_oversize_and_short_table(env):
    torch, zg, ctx = env
    lib = zg.library()
    wig = torch.from_numpy(ctx.wignerd_table(8)).cuda()
    # every call below returns before any launch, so a small buffer stands in
    c = torch.zeros(64, dtype=torch.float64, device="cuda")
    e = torch.zeros(3, dtype=torch.float64, device="cuda")
    before = c.clone()
    # order 1436 at batch 1: the vector list and one item's phases exceed the fixed scratch
    rc = _noalloc(zg, 0, 1436, 1, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_UNSUPPORTED
    assert b"scratch" in lib.zest_gpu_last_error()
    # order 1435 at batch 1 fits: the size check passes and the short Wigner table is what fails
    rc = _noalloc(zg, 0, 1435, 1, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_INVALID
    assert b"Wigner" in lib.zest_gpu_last_error()
    # order 200 fits up to batch 428
    rc = _noalloc(zg, 0, 200, 429, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_UNSUPPORTED
    rc = _noalloc(zg, 0, 200, 428, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_INVALID
    # a Wigner table smaller than the expansion order
    rc = _noalloc(zg, 0, 12, 1, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_INVALID
    torch.cuda.synchronize()
    assert torch.equal(c, before)

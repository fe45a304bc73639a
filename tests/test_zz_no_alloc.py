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
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        rc = _noalloc(zg, stream, L, batch, dc.data_ptr(), de.data_ptr(), rtype, wig.data_ptr(), L + 3)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info(0)[0]
        assert rc == 0, zg.library().zest_gpu_last_error()
        assert relmax(dc.cpu().numpy(), ref) < TOL
        if call > 0:  # past the set-up call, device memory use does not move
            assert free1 == free0


def test_zt_rotate_noalloc_rejects_oversize_and_short_table(env):
    torch, zg, ctx = env
    lib = zg.library()
    wig = torch.from_numpy(ctx.wignerd_table(8)).cuda()
    c = torch.zeros(2 * zt_coeff_size(1448), dtype=torch.float64, device="cuda")
    e = torch.zeros(3, dtype=torch.float64, device="cuda")
    before = c.clone()
    # order 1448: the vector list alone is above the fixed scratch size
    rc = _noalloc(zg, 0, 1448, 1, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_UNSUPPORTED
    assert b"scratch" in lib.zest_gpu_last_error()
    # order 200 fits up to batch 428
    rc = _noalloc(zg, 0, 200, 429, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_UNSUPPORTED
    # a Wigner table smaller than the expansion order
    rc = _noalloc(zg, 0, 12, 1, c.data_ptr(), e.data_ptr(), 0, wig.data_ptr(), 8)
    assert rc == zg.ERR_INVALID
    torch.cuda.synchronize()
    assert torch.equal(c, before)

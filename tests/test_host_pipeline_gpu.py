"""Host-memory Zernike transforms cut into chunks whose uploads, transforms
and downloads overlap (zest_gpu_set_host_chunk_bytes).

Chunking must not change any result: the pipelined call gives bit for bit
what one unchunked call gives, for batches that do not divide evenly into
chunks, for chunks of one item, for expansions above and below the grid order
(the forward transform writes only the orders the grid resolves and leaves the
rest of the host buffer as it was), in FP64 and split precision."""
import numpy as np
import pytest

from oracle import zidx, zt_coeff_size, zt_grid_shape

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


def rand_zt(rng, L, batch):
    c = np.zeros((batch, zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[:, zidx(n, l, m)] = rng.normal(size=(batch, 2)) / (n + 1)
                if m == 0:
                    c[:, zidx(n, l, m), 1] = 0.0
    return c.ravel()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("Lg,Le,batch,items_per_chunk", [(24, 24, 7, 3), (24, 30, 5, 1), (30, 20, 6, 4)])
def test_chunked_host_transforms_are_bitwise_unchunked(ctx, precision, Lg, Le, batch, items_per_chunk):
    rng = np.random.default_rng(100 + Lg + Le + batch)
    gsz = int(np.prod(zt_grid_shape(Lg)))
    csz = 2 * zt_coeff_size(Le)
    item = 8 * max(gsz, csz)
    grids = rng.normal(size=gsz * batch)
    coeffs = rand_zt(rng, Le, batch)
    ctx.set_precision(precision)
    try:
        ctx.set_host_chunk_bytes(0)
        f_ref = ctx.zt_forward(grids, Lg, Le, batch=batch, out=np.full(csz * batch, np.nan))
        b_ref = ctx.zt_backward(coeffs, Le, Lg, batch=batch)
        ctx.set_host_chunk_bytes(items_per_chunk * item)
        f = ctx.zt_forward(grids, Lg, Le, batch=batch, out=np.full(csz * batch, np.nan))
        b = ctx.zt_backward(coeffs, Le, Lg, batch=batch)
    finally:
        ctx.set_host_chunk_bytes(512 << 20)
        ctx.set_precision(0)
    # orders above the grid's stay NaN in both
    np.testing.assert_array_equal(np.isnan(f), np.isnan(f_ref))
    if Le > Lg:
        assert np.isnan(f).any()
    np.testing.assert_array_equal(f[~np.isnan(f)], f_ref[~np.isnan(f_ref)])
    np.testing.assert_array_equal(b, b_ref)


def test_chunked_pinned_round_trip(ctx):
    # pinned host buffers (the copies overlap), order 64 x 24 in chunks of 5
    torch = pytest.importorskip("torch")
    L, batch = 64, 24
    rng = np.random.default_rng(7)
    gsz = int(np.prod(zt_grid_shape(L)))
    c = torch.from_numpy(rand_zt(rng, L, batch)).pin_memory()
    g = torch.empty(gsz * batch, dtype=torch.float64).pin_memory()
    c2 = torch.empty_like(c).pin_memory()
    ctx.set_host_chunk_bytes(5 * 8 * gsz)
    try:
        ctx.zt_backward(c, L, batch=batch, out=g)
        ctx.zt_forward(g, L, batch=batch, out=c2)
    finally:
        ctx.set_host_chunk_bytes(512 << 20)
    err = float((c2 - c).abs().max() / c.abs().max())
    assert err < 1e-12


def test_registered_host_buffers_match_device_path(ctx):
    """Host arrays pinned with zest_gpu_host_register go through the chunked
    pipeline and give bit for bit the device-memory results; unregistering
    them afterwards succeeds."""
    torch = pytest.importorskip("torch")
    import zest_gb300 as zg
    rng = np.random.default_rng(9)
    L, batch = 28, 6
    coeffs = rand_zt(rng, L, batch)
    ctx.set_host_chunk_bytes(2 * int(np.prod(zt_grid_shape(L))) * 8)
    grids = np.zeros(batch * int(np.prod(zt_grid_shape(L))))
    back = np.zeros_like(coeffs)
    for h in (coeffs, grids, back):
        zg.host_register(h)
    try:
        ctx.zt_backward(coeffs, L, batch=batch, out=grids)
        ctx.zt_forward(grids, L, batch=batch, out=back)
    finally:
        for h in (coeffs, grids, back):
            zg.host_unregister(h)
        ctx.set_host_chunk_bytes(512 << 20)
    g_dev = ctx.zt_backward(torch.from_numpy(coeffs).cuda(), L, batch=batch)
    c_dev = ctx.zt_forward(g_dev, L, batch=batch)
    assert np.array_equal(grids, g_dev.cpu().numpy())
    assert np.array_equal(back, c_dev.cpu().numpy())

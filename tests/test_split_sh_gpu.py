"""SH transforms in split precision (the Legendre sums on the tensor cores,
6 digit slices) against the FP64 form on the same inputs.  LonLat grids of
order 2 and above take the longitude DFT on the tensor cores too (the
Zernike DFT stages with one radial node); LatLon grids keep the FP64 FFT.

Tolerance: 1e-11 relative max-norm per item, the bound the split form is
built to.  Covered: both layouts (including an odd LatLon grid, whose middle
latitude the reference counts twice), the smallest orders of the DFT path
(2, 3), all four conventions, truncation in both directions, single sums (up
to 256 terms) and K-chunked ones (order 600: folded node counts and DFT
lengths above 256), narrow column tiles (2 x batch <= 16 and <= 32) and wide
ones (batch 30), and the round trip at order 1024 (the C2 configuration's order) against the input coefficients."""
import numpy as np
import pytest

from oracle import st_grid_shape, tri_idx, tri_size

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


def relmax_items(a, b, batch):
    a = np.asarray(a).reshape(batch, -1)
    b = np.asarray(b).reshape(batch, -1)
    return max(float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300)) for x, y in zip(a, b))


def rand_st(rng, L, batch):
    c = rng.normal(size=(batch, tri_size(L), 2))
    for l in range(L):
        c[:, tri_idx(l, 0), 1] = 0.0
        c[:, tri_idx(l, 0):tri_idx(l, 0) + l + 1] /= (l + 1)
    return c.ravel()


def both(ctx, fn):
    import zest_gb300 as zg
    ctx.set_precision(zg.PRECISION_FP64)
    want = fn()
    ctx.set_precision(zg.PRECISION_SPLIT, 6)
    try:
        got = fn()
    finally:
        ctx.set_precision(zg.PRECISION_FP64)
    return got, want


@pytest.mark.parametrize("L,layout,batch", [(2, 0, 1), (3, 0, 2), (8, 0, 1), (33, 0, 3), (33, 1, 3), (64, 1, 2),
                                            (64, 0, 12), (100, 0, 30), (101, 1, 5), (600, 0, 2)])
def test_split_sh_matches_fp64(ctx, L, layout, batch):
    rng = np.random.default_rng(L * 10 + layout)
    c = rand_st(rng, L, batch)
    for conv in [(0, 0), (1, 1), (0, 1), (1, 0)] if L <= 101 else [(0, 0)]:
        g_split, g64 = both(ctx, lambda: ctx.st_backward(c, L, batch=batch, conv=conv, layout=layout))
        assert relmax_items(g_split, g64, batch) < 1e-11, ("backward", conv)
        f_split, f64 = both(ctx, lambda: ctx.st_forward(g64, L, batch=batch, conv=conv, layout=layout))
        assert relmax_items(f_split, f64, batch) < 1e-11, ("forward", conv)


def test_split_sh_truncation(ctx):
    rng = np.random.default_rng(5)
    batch = 2
    for Lg, Le in [(40, 25), (25, 40)]:
        c = rand_st(rng, Le, batch)
        g_split, g64 = both(ctx, lambda: ctx.st_backward(c, Le, Lg, batch=batch))
        assert relmax_items(g_split, g64, batch) < 1e-11
        g = rng.normal(size=int(np.prod(st_grid_shape(Lg))) * batch)
        out0 = np.full(2 * tri_size(Le) * batch, 7.0)
        f_split, f64 = both(ctx, lambda: ctx.st_forward(g, Lg, Le, batch=batch, out=out0.copy()))
        assert relmax_items(f_split, f64, batch) < 1e-11


def test_split_sh_round_trip_order1024(ctx):
    import zest_gb300 as zg
    rng = np.random.default_rng(1024)
    L, batch = 1024, 2
    c = rand_st(rng, L, batch)
    ctx.set_precision(zg.PRECISION_SPLIT, 6)
    try:
        g = ctx.st_backward(c, L, batch=batch)
        back = ctx.st_forward(g, L, batch=batch)
    finally:
        ctx.set_precision(zg.PRECISION_FP64)
    assert relmax_items(back, c, batch) < 1e-11

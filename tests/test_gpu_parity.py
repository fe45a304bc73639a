"""Parity of the CUDA path (through the C-ABI) with the reference.

Small cases compare against the golden vectors produced by the compiled
reference (tests/golden/); larger ones against the CPU oracle on the same
seeded inputs; full sizes through size-independent properties (band-limited
round trips).  Tolerance of the plain (FP64) form: 1e-12 relative max-norm,
max|x - x_ref| / max|x_ref| (the bar the reference parity is quoted at)."""
import numpy as np
import pytest

from kats import ST_KATS, ZT_KATS, ball_points, sphere_points
from oracle import tri_idx, tri_size, zidx, zt_coeff_size

pytestmark = pytest.mark.gpu

TOL = 1e-12
CONVS_ZT = [(1, 0, 0), (0, 0, 0), (1, 1, 0), (0, 1, 0), (1, 1, 1), (0, 1, 1), (1, 0, 1), (0, 0, 1)]
CONVS_ST = [(0, 0), (1, 0), (0, 1), (1, 1)]


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


def rand_zt(rng, L, power=1.5, batch=1):
    c = np.zeros((batch, zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[:, zidx(n, l, m)] = rng.normal(size=(batch, 2)) * (n + 1) ** -power
                if m == 0:
                    c[:, zidx(n, l, m), 1] = 0.0
    return c


def rand_st(rng, L, batch=1):
    c = np.zeros((batch, tri_size(L), 2))
    for l in range(L):
        for m in range(l + 1):
            c[:, tri_idx(l, m)] = rng.normal(size=(batch, 2)) / (l + 1)
            if m == 0:
                c[:, tri_idx(l, m), 1] = 0.0
    return c


# ---- tables: bit-identical to the reference ----
def test_tables_bitwise(ctx, golden):
    t = golden("tables")
    for sn, sp in CONVS_ST:
        np.testing.assert_array_equal(ctx.plm_table(20, sn, sp, t["z"]), t[f"plm_{sn}_{sp}"])
    for zn in (0, 1):
        np.testing.assert_array_equal(ctx.radial_table(20, zn, t["r"]), t[f"rz_{zn}"])
    np.testing.assert_array_equal(ctx.wignerd_table(16), t["wignerd_16"])


def test_tables_large_vs_oracle(ctx, oracle):
    z = np.cos(np.linspace(1e-3, np.pi - 1e-3, 257))
    for sn, sp in [(0, 0), (1, 1)]:
        np.testing.assert_array_equal(ctx.plm_table(300, sn, sp, z), oracle.plm_real(300, sn, sp, z))
    r = np.linspace(0.0, 1.0, 101)
    np.testing.assert_array_equal(ctx.radial_table(150, 0, r), oracle.radial_zernike(150, 0, r))
    np.testing.assert_array_equal(ctx.wignerd_table(90), oracle.wignerd(90))


# ---- Zernike ----
def test_zt_config1(ctx, golden):
    g = golden("zt_config1")
    c = ctx.zt_forward(np.ascontiguousarray(g["grid"]).ravel(), 20)
    assert relmax(c, g["coeffs"]) < TOL
    rt = ctx.zt_backward(np.ascontiguousarray(g["coeffs"]).ravel(), 20)
    assert relmax(rt, g["roundtrip"]) < TOL


@pytest.mark.parametrize("L", [1, 2, 3, 6, 11, 16])
@pytest.mark.parametrize("conv", CONVS_ZT)
def test_zt_golden(ctx, golden, L, conv):
    z = golden("zt_random")
    key = f"{L}_{conv[0]}{conv[1]}{conv[2]}"
    if "c_" + key not in z:
        pytest.skip("fixture holds this order for one convention only")
    g = ctx.zt_backward(z["c_" + key].ravel(), L, conv=conv)
    assert relmax(g, z["g_" + key]) < TOL
    f = ctx.zt_forward(np.ascontiguousarray(z["g_" + key]).ravel(), L, conv=conv)
    assert relmax(f, z["f_" + key]) < TOL


def test_zt_order_mismatch(ctx, golden):
    z = golden("zt_random")
    assert relmax(ctx.zt_backward(z["trunc_c"].ravel(), 9, 6), z["trunc_g96"]) < TOL
    g99 = np.ascontiguousarray(z["trunc_g99"]).ravel()
    assert relmax(ctx.zt_forward(g99, 9, 6), z["trunc_f96"]) < TOL
    assert relmax(ctx.zt_forward(g99, 9, 12), z["trunc_f9_12"]) < TOL
    assert relmax(ctx.zt_backward(z["trunc_c6"].ravel(), 6, 9), z["trunc_g69"]) < TOL


def test_forward_leaves_orders_above_the_grid_untouched(ctx):
    # zernike_glq_transformer.hpp:640-655 / sh_glq_transformer.hpp:632-647 write
    # only the coefficients below min(expansion order, grid order)
    from zest_gb300 import zt_coeff_size, st_coeff_size, zt_grid_shape, st_grid_shape
    rng = np.random.default_rng(11)
    g = rng.normal(size=int(np.prod(zt_grid_shape(6))))
    out = np.full(2 * zt_coeff_size(9), 7.5)
    ctx.zt_forward(g, 6, 9, out=out)
    assert np.all(out[2 * zt_coeff_size(6):] == 7.5)
    assert np.array_equal(out[:2 * zt_coeff_size(6)], ctx.zt_forward(g, 6, 6))
    gs = rng.normal(size=int(np.prod(st_grid_shape(6))))
    outs = np.full(2 * st_coeff_size(9), -2.0)
    ctx.st_forward(gs, 6, 9, out=outs)
    assert np.all(outs[2 * st_coeff_size(6):] == -2.0)
    assert np.array_equal(outs[:2 * st_coeff_size(6)], ctx.st_forward(gs, 6, 6))


@pytest.mark.parametrize("L,batch", [(33, 3), (64, 2)])
def test_zt_vs_oracle_batched(ctx, oracle, L, batch):
    rng = np.random.default_rng(L)
    c = rand_zt(rng, L, batch=batch)
    g = ctx.zt_backward(c.ravel(), L, batch=batch).reshape(batch, -1)
    f = ctx.zt_forward(g.ravel(), L, batch=batch).reshape(batch, -1)
    for b in range(batch):
        assert relmax(g[b], oracle.zt_backward(c[b], L)) < TOL
        assert relmax(f[b], oracle.zt_forward(g[b], L)) < TOL


def test_zt_roundtrip_full_size(ctx):
    # band-limited coefficients survive backward -> forward at the order-200 grid
    rng = np.random.default_rng(200)
    L, batch = 200, 2
    c = rand_zt(rng, L, power=1.5, batch=batch)
    g = ctx.zt_backward(c.ravel(), L, batch=batch)
    f = ctx.zt_forward(g, L, batch=batch).reshape(batch, -1, 2)
    assert relmax(f, c) < TOL


def test_zt_device_pointers(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    L, batch = 24, 4
    c = rand_zt(rng, L, batch=batch).ravel()
    host = ctx.zt_backward(c, L, batch=batch)
    dev_c = torch.from_numpy(c).cuda()
    dev_g = ctx.zt_backward(dev_c, L, batch=batch)
    ctx.synchronize()
    np.testing.assert_array_equal(dev_g.cpu().numpy(), host)
    dev_f = ctx.zt_forward(dev_g, L, batch=batch)
    ctx.synchronize()
    np.testing.assert_array_equal(dev_f.cpu().numpy(), ctx.zt_forward(host, L, batch=batch))


def test_zt_kat_z000(ctx):
    # tests/test_zernike_glq_transformer.cpp:57-136
    from zest_gb300 import zt_grid_shape
    for zn, sn, sp in CONVS_ZT:
        L = 6
        znorm = np.sqrt(3.0) if zn == 0 else 1.0
        shnorm = 0.5 / np.sqrt(np.pi) if sn == 1 else 1.0
        grid = np.full(int(np.prod(zt_grid_shape(L))), znorm * shnorm)
        c = ctx.zt_forward(grid, L, conv=(zn, sn, sp)).reshape(-1, 2)
        ref = np.zeros_like(c)
        ref[0, 0] = 1.0
        assert np.max(np.abs(c - ref)) < 1e-10


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("kat", range(len(ZT_KATS)))
def test_zt_kats(ctx, oracle, kat, precision):
    # tests/test_zernike_glq_transformer.cpp:136-870 (the cases in tests/kats.py):
    # single Zernike functions expand to their one coefficient and evaluate
    # back, in all conventions, in the FP64 and the split-precision form
    import zest_gb300
    (n, l, m), f, normed, want = ZT_KATS[kat]
    L = 6
    lon, z, r = ball_points(oracle, L)
    LON, Z, R = np.meshgrid(lon, z, r, indexing="ij")
    if precision:
        ctx.set_precision(zest_gb300.PRECISION_SPLIT, 6)
    try:
        for zn, sn, sp in CONVS_ZT:
            znorm = normed if zn == 0 else 1.0
            shnorm = 0.5 / np.sqrt(np.pi) if sn == 1 else 1.0
            phase = -1.0 if sp == 0 else 1.0
            grid = np.ascontiguousarray(znorm * shnorm * f(LON, Z, R, phase))
            c = np.asarray(ctx.zt_forward(grid.ravel(), L, conv=(zn, sn, sp))).reshape(-1, 2)
            ref = np.zeros_like(c)
            ref[zidx(n, l, m)] = want
            assert np.max(np.abs(c - ref)) < 1e-10, (zn, sn, sp)
            back = ctx.zt_backward(np.ascontiguousarray(c).ravel(), L, conv=(zn, sn, sp))
            assert np.max(np.abs(np.ravel(back) - grid.ravel())) < 1e-10, (zn, sn, sp)
    finally:
        ctx.set_precision(zest_gb300.PRECISION_FP64)


# ---- SH ----
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("latlon", [0, 1])
@pytest.mark.parametrize("kat", range(len(ST_KATS)))
def test_st_kats(ctx, oracle, kat, latlon, precision):
    # tests/test_sh_glq_transformer.cpp:53-777 (the cases in tests/kats.py),
    # both layouts, all conventions, the FP64 and the split-precision form
    import zest_gb300
    f, want = ST_KATS[kat]
    L = 6
    lon, z = sphere_points(oracle, L, latlon)
    if latlon:
        Z, LON = np.meshgrid(z, lon, indexing="ij")
    else:
        LON, Z = np.meshgrid(lon, z, indexing="ij")
    if precision:
        ctx.set_precision(zest_gb300.PRECISION_SPLIT, 6)
    try:
        for sn, sp in CONVS_ST:
            shnorm = 0.5 / np.sqrt(np.pi) if sn == 1 else 1.0
            phase = -1.0 if sp == 0 else 1.0
            grid = np.ascontiguousarray(shnorm * f(LON, Z, phase))
            c = np.asarray(ctx.st_forward(grid.ravel(), L, conv=(sn, sp), layout=latlon)).reshape(-1, 2)
            ref = np.zeros_like(c)
            for (l, m), v in want.items():
                ref[tri_idx(l, m)] = v
            assert np.max(np.abs(c - ref)) < 1e-10, (sn, sp)
            back = ctx.st_backward(np.ascontiguousarray(c).ravel(), L, conv=(sn, sp), layout=latlon)
            assert np.max(np.abs(np.ravel(back) - grid.ravel())) < 1e-10, (sn, sp)
    finally:
        ctx.set_precision(zest_gb300.PRECISION_FP64)


@pytest.mark.parametrize("L", [1, 2, 5, 8, 16, 24])
@pytest.mark.parametrize("latlon", [0, 1])
@pytest.mark.parametrize("conv", CONVS_ST)
def test_st_golden(ctx, golden, L, latlon, conv):
    s = golden("st_random")
    key = f"{L}_{latlon}_{conv[0]}{conv[1]}"
    if "c_" + key not in s:
        pytest.skip("fixture holds this order for one convention only")
    g = ctx.st_backward(s["c_" + key].ravel(), L, conv=conv, layout=latlon)
    assert relmax(g, s["g_" + key]) < TOL
    f = ctx.st_forward(np.ascontiguousarray(s["g_" + key]).ravel(), L, conv=conv, layout=latlon)
    assert relmax(f, s["f_" + key]) < TOL


@pytest.mark.parametrize("L,latlon", [(65, 0), (128, 0), (77, 1)])
def test_st_vs_oracle(ctx, oracle, L, latlon):
    rng = np.random.default_rng(L)
    batch = 2
    c = rand_st(rng, L, batch=batch)
    g = ctx.st_backward(c.ravel(), L, batch=batch, layout=latlon).reshape(batch, -1)
    f = ctx.st_forward(g.ravel(), L, batch=batch, layout=latlon).reshape(batch, -1)
    for b in range(batch):
        assert relmax(g[b], oracle.st_backward(c[b], L, latlon=bool(latlon))) < TOL
        assert relmax(f[b], oracle.st_forward(g[b], L, latlon=bool(latlon))) < TOL


def test_st_roundtrip_full_size(ctx):
    rng = np.random.default_rng(1024)
    L, batch = 1024, 2
    c = rand_st(rng, L, batch=batch)
    g = ctx.st_backward(c.ravel(), L, batch=batch)
    f = ctx.st_forward(g, L, batch=batch).reshape(batch, -1, 2)
    assert relmax(f, c) < TOL


# ---- rotations ----
@pytest.mark.parametrize("L", [2, 5, 10, 17])
def test_rotations_golden(ctx, golden, L):
    r = golden("rotation")
    for rtype, key in [(0, "zobj"), (1, "zcoord")]:
        c = r[f"zc_{L}"].ravel().copy()
        ctx.zt_rotate(c, L, r[f"ze_{L}"].copy(), rotation_type=rtype)
        assert relmax(c, r[f"{key}_{L}"]) < TOL
    c = r[f"zc_{L}"].ravel().copy()
    ctx.zt_polar_rotate(c, L, np.array([r[f"ze_{L}"][0]]))
    assert relmax(c, r[f"zpolar_{L}"]) < TOL
    import zest_gb300
    c = r[f"zc_{L}"].ravel().copy()
    ctx.zt_rotate(c, L, zest_gb300.euler_from_matrix(r[f"zmat_{L}"]))
    assert relmax(c, r[f"zmatobj_{L}"]) < TOL
    for rtype, key in [(0, "sobj"), (1, "scoord")]:
        s = r[f"sc_{L}"].ravel().copy()
        ctx.st_rotate(s, L + 3, r[f"ze_{L}"].copy(), rotation_type=rtype)
        assert relmax(s, r[f"{key}_{L}"]) < TOL
    s = r[f"sc_{L}"].ravel().copy()
    ctx.st_polar_rotate(s, L + 3, np.array([r[f"ze_{L}"][1]]), rotation_type=1)
    assert relmax(s, r[f"spolar_{L}"]) < TOL


def test_rotation_batch_vs_oracle(ctx, oracle):
    rng = np.random.default_rng(11)
    L, batch = 64, 16
    c = rand_zt(rng, L, power=1.0, batch=batch)
    e = np.stack([rng.uniform(0, 2 * np.pi, batch), np.arccos(rng.uniform(-1, 1, batch)),
                  rng.uniform(0, 2 * np.pi, batch)], axis=1)
    out = c.ravel().copy()
    ctx.zt_rotate(out, L, np.ascontiguousarray(e).ravel(), batch=batch)
    out = out.reshape(batch, -1, 2)
    for b in range(batch):
        assert relmax(out[b], oracle.zt_rotate(c[b], L, e[b])) < TOL


def test_rotation_group_law(ctx):
    # rotating by R and then by R^-1 (ZYZ: (a,b,g)^-1 = (-g,-b,-a)) is the identity
    rng = np.random.default_rng(5)
    L = 40
    c = rand_zt(rng, L, power=1.0)
    e = np.array([0.7, 1.9, -2.3])
    x = c.ravel().copy()
    ctx.zt_rotate(x, L, e)
    ctx.zt_rotate(x, L, np.array([-e[2], -e[1], -e[0]]))
    assert relmax(x, c) < TOL


def test_invalid_arguments_return_codes(ctx):
    import zest_gb300
    lib = zest_gb300.library()
    assert lib.zest_gpu_zt_forward(ctx._h, 2, 0, 0, 4, 4, 1, None, None, 1) == 1   # bad convention
    assert lib.zest_gpu_zt_forward(ctx._h, 1, 0, 0, 4, 4, 1, None, None, 1) == 1   # null data
    assert lib.zest_gpu_zt_forward(ctx._h, 1, 0, 0, 99999, 4, 1, None, None, 1) == 1  # order too large
    assert lib.zest_gpu_st_forward(ctx._h, 0, 0, 7, 4, 4, 1, None, None, 1) == 1   # bad layout
    assert lib.zest_gpu_set_precision(ctx._h, 9, 0) == 1
    # zero-sized work is a no-op
    assert lib.zest_gpu_zt_forward(ctx._h, 1, 0, 0, 4, 4, 0, None, None, 1) == 0

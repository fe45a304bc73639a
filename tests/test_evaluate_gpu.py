"""Evaluation at arbitrary points (zt/st GridEvaluator) and power spectra on
the GPU, through the C-ABI.

Parity: against the reference's outputs (tests/golden/evaluate.npz,
spectra.npz) and against the oracle at larger sizes, 1e-12 relative max-norm
for the evaluations (FP64; the GEMM sums in another order than the
reference's loops) and 1e-14 for the spectra (summed in the reference's
order).  Properties: the evaluator at the quadrature points is the backward
transform; host and device memory give identical results; the entries the
reference leaves unwritten stay as they were."""
import numpy as np
import pytest

from oracle import rad_size, tri_idx, tri_size, zidx, zt_coeff_size, zt_grid_shape

pytestmark = pytest.mark.gpu

CONVS_ZT = [(1, 0, 0), (0, 0, 0), (1, 1, 0), (0, 1, 0), (1, 1, 1), (0, 1, 1), (1, 0, 1), (0, 0, 1)]
CONVS_ST = [(0, 0), (1, 0), (0, 1), (1, 1)]


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rand_zt(rng, L, batch=1):
    c = np.zeros((batch, zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[:, zidx(n, l, m)] = rng.normal(size=(batch, 2)) / (n + 1)
                if m == 0:
                    c[:, zidx(n, l, m), 1] = 0.0
    return c


def rand_st(rng, L, batch=1):
    c = rng.normal(size=(batch, tri_size(L), 2))
    for l in range(L):
        c[:, tri_idx(l, 0), 1] = 0.0
    return c


@pytest.mark.parametrize("L", [1, 6, 13, 24])
def test_zt_evaluate_matches_reference(ctx, golden, L):
    e = golden("evaluate")
    lon, colat, rad = e[f"lon_{L}"], e[f"colat_{L}"], e[f"rad_{L}"]
    for conv in CONVS_ZT:
        key = "".join(map(str, conv))
        got = ctx.zt_evaluate(e[f"zc_{L}"].ravel(), L, lon, colat, rad, conv=conv)
        assert relmax(got, e[f"zv_{L}_{key}"]) < 1e-12, conv


@pytest.mark.parametrize("L", [1, 6, 13, 24])
def test_st_evaluate_matches_reference(ctx, golden, L):
    e = golden("evaluate")
    for conv in CONVS_ST:
        key = "".join(map(str, conv))
        got = ctx.st_evaluate(e[f"sc_{L}"].ravel(), L + 2, e[f"lon_{L}"], e[f"colat_{L}"], conv=conv)
        assert relmax(got, e[f"sv_{L}_{key}"]) < 1e-12, conv


def test_zt_evaluate_batch_order64_vs_oracle(ctx, oracle):
    rng = np.random.default_rng(21)
    L, batch = 64, 3
    lon = rng.uniform(0, 2 * np.pi, 40)
    colat = rng.uniform(0, np.pi, 30)
    rad = rng.uniform(0, 1, 20)
    c = rand_zt(rng, L, batch)
    got = ctx.zt_evaluate(c.ravel(), L, lon, colat, rad, batch=batch, conv=(0, 1, 1)).reshape(batch, -1)
    for b in range(batch):
        want = oracle.zt_evaluate(c[b], L, lon, colat, rad, 0, 1, 1)
        assert relmax(got[b], want) < 1e-12, b


def test_st_evaluate_batch_order200_vs_oracle(ctx, oracle):
    rng = np.random.default_rng(22)
    L, batch = 200, 2
    lon = rng.uniform(-np.pi, np.pi, 50)
    colat = rng.uniform(0, np.pi, 70)
    c = rand_st(rng, L, batch)
    got = ctx.st_evaluate(c.ravel(), L, lon, colat, batch=batch).reshape(batch, -1)
    for b in range(batch):
        assert relmax(got[b], oracle.st_evaluate(c[b], L, lon, colat)) < 1e-12, b


def test_evaluate_at_quadrature_points_is_the_backward_transform(ctx, oracle):
    rng = np.random.default_rng(23)
    L, batch = 40, 2
    nlon, nlat, nrad = zt_grid_shape(L)
    lon = 2 * np.pi * np.arange(nlon) / nlon
    colat = np.arccos(np.asarray(oracle.gl_nodes_weights(nlat)[0]))
    rad = 0.5 * (1 + np.asarray(oracle.gl_nodes_weights(nrad)[0]))
    c = rand_zt(rng, L, batch).ravel()
    for conv in [(1, 0, 0), (0, 1, 1)]:
        ev = ctx.zt_evaluate(c, L, lon, colat, rad, batch=batch, conv=conv)
        bw = ctx.zt_backward(c, L, batch=batch, conv=conv)
        assert relmax(ev, bw) < 1e-12


def test_device_and_host_memory_agree(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(24)
    L, batch = 20, 4
    lon = rng.uniform(0, 2 * np.pi, 9)
    colat = rng.uniform(0, np.pi, 8)
    rad = rng.uniform(0, 1, 7)
    c = rand_zt(rng, L, batch).ravel()
    host = ctx.zt_evaluate(c, L, lon, colat, rad, batch=batch)
    dev = ctx.zt_evaluate(torch.from_numpy(c).cuda(), L, torch.from_numpy(lon).cuda(), colat, rad, batch=batch)
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    s = rand_st(rng, L, batch).ravel()
    host = ctx.st_evaluate(s, L, lon, colat, batch=batch)
    dev = ctx.st_evaluate(torch.from_numpy(s).cuda(), L, lon, colat, batch=batch)
    np.testing.assert_array_equal(dev.cpu().numpy(), host)


def test_evaluate_edge_cases(ctx):
    rng = np.random.default_rng(25)
    c = rand_zt(rng, 5).ravel()
    assert ctx.zt_evaluate(c, 5, np.zeros(0), np.ones(3), np.ones(2)).size == 0
    # order 0: no terms, zero values
    v = ctx.zt_evaluate(np.zeros(0), 0, np.ones(3), np.ones(2), np.ones(2), out=np.full(12, 5.0))
    np.testing.assert_array_equal(v, 0.0)
    v = ctx.st_evaluate(np.zeros(0), 0, np.ones(3), np.ones(2), out=np.full(6, 5.0))
    np.testing.assert_array_equal(v, 0.0)
    # one point, order 1: the constant term
    one = ctx.zt_evaluate(rand_zt(rng, 1).ravel() + 1.0, 1, [0.3], [0.2], [0.5])
    assert one.shape == (1,) and np.isfinite(one).all()


@pytest.mark.parametrize("L", [1, 2, 7, 16, 31])
def test_zt_power_spectrum_matches_reference(ctx, golden, L):
    p = golden("spectra")
    for sn in (0, 1):
        got = ctx.zt_power_spectrum(p[f"zc_{L}"].ravel(), L, sh_norm=sn)
        np.testing.assert_allclose(got, p[f"zp_{L}_{sn}"], rtol=1e-14, atol=0)


def test_zt_power_spectrum_leaves_l_equal_n_alone(ctx, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(26)
    L, batch = 30, 3
    c = rand_zt(rng, L, batch)
    out = np.full(batch * rad_size(L), np.nan)
    got = ctx.zt_power_spectrum(c.ravel(), L, batch=batch, out=out).reshape(batch, -1)
    dev = ctx.zt_power_spectrum(torch.from_numpy(c.ravel()).cuda(), L, batch=batch,
                                out=torch.full((batch * rad_size(L),), float("nan"), dtype=torch.float64,
                                               device="cuda")).cpu().numpy().reshape(batch, -1)
    for b in range(batch):
        want = oracle.zt_power_spectrum(c[b], L, 0, out=np.full(rad_size(L), np.nan))
        np.testing.assert_array_equal(np.isnan(got[b]), np.isnan(want))
        np.testing.assert_allclose(got[b][~np.isnan(want)], want[~np.isnan(want)], rtol=1e-14)
        np.testing.assert_array_equal(np.isnan(dev[b]), np.isnan(want))
    # the untouched entries are exactly l = n (and n = 0)
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            idx = ((n + 1) * (n + 1)) // 4 + l // 2
            assert np.isnan(got[0][idx]) == (l == n)


def test_st_power_spectra_vs_oracle(ctx, oracle):
    rng = np.random.default_rng(27)
    L, batch = 100, 3
    a = rand_st(rng, L, batch)
    b = rand_st(rng, L, batch)
    for sn in (0, 1):
        ps = ctx.st_power_spectrum(a.ravel(), L, batch=batch, sh_norm=sn).reshape(batch, -1)
        for k in range(batch):
            np.testing.assert_allclose(ps[k], oracle.st_power_spectrum(a[k], L, sn), rtol=1e-14)
        for out_len in (L, L + 1, 7):
            x = ctx.st_cross_power_spectrum(a.ravel(), b.ravel(), L, batch=batch, sh_norm=sn, out_len=out_len,
                                            out=np.full(batch * out_len, -3.0)).reshape(batch, -1)
            for k in range(batch):
                want = oracle.st_cross_power_spectrum(a[k], b[k], L, sn, out_len=out_len, out=np.full(out_len, -3.0))
                np.testing.assert_allclose(x[k], want, rtol=1e-14)

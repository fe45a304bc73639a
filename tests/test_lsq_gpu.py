"""Least-squares fits of expansions to scattered data (st/zt LSQTransformer) on
the GPU.

The reference solves these with LAPACK's dgels, and LAPACK is absent on both
machines, so the reference's own fit cannot run here (parity unpinned against
it).  Checked instead:
  * recovery: data generated from a known expansion at scattered points (the
    basis from the oracle's tables: P_lm at sin(latitude) for SH, as the
    reference's RealSHGenerator, and R_nl(r) P_lm(cos colatitude) for
    Zernike) is fitted back to that expansion to 1e-10;
  * with noise added, the fit equals numpy's least-squares solution of the
    same design matrix to 1e-9;
  * batches fit each data vector on its own; too few points are refused."""
import numpy as np
import pytest

from oracle import rad_size, tri_idx, tri_size, zidx, zt_coeff_size

pytestmark = pytest.mark.gpu


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


def st_design(oracle, L, lat, lon, sn, sp):
    P = oracle.plm_real(L, sn, sp, np.sin(lat))  # [tri(l,m)][i]
    cols, keys = [], []
    for l in range(L):
        for m in range(l + 1):
            p = P[tri_idx(l, m)]
            cols.append(p * np.cos(m * lon))
            keys.append((tri_idx(l, m), 0))
            if m:
                cols.append(p * np.sin(m * lon))
                keys.append((tri_idx(l, m), 1))
    return np.stack(cols, axis=1), keys


def zt_design(oracle, L, r, lon, colat, zn, sn, sp):
    P = oracle.plm_real(L, sn, sp, np.cos(colat))
    R = oracle.radial_zernike(L, zn, r)  # [rad_idx(n,l)][i]
    cols, keys = [], []
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            rr = R[((n + 1) * (n + 1)) // 4 + l // 2]
            for m in range(l + 1):
                p = rr * P[tri_idx(l, m)]
                cols.append(p * np.cos(m * lon))
                keys.append((zidx(n, l, m), 0))
                if m:
                    cols.append(p * np.sin(m * lon))
                    keys.append((zidx(n, l, m), 1))
    return np.stack(cols, axis=1), keys


def to_pairs(x, keys, npairs):
    c = np.zeros((npairs, 2))
    for v, (k, j) in zip(x, keys):
        c[k, j] = v
    return c


@pytest.mark.parametrize("conv", [(0, 0), (1, 1)])
def test_st_lsq_recovers_expansion(ctx, oracle, conv):
    rng = np.random.default_rng(31)
    L, N, batch = 16, 1500, 3
    lat = np.arcsin(rng.uniform(-1, 1, N))
    lon = rng.uniform(0, 2 * np.pi, N)
    A, keys = st_design(oracle, L, lat, lon, *conv)
    x = rng.normal(size=(batch, A.shape[1]))
    data = x @ A.T
    got = ctx.st_lsq(data.ravel(), L, lat, lon, batch=batch, conv=conv).reshape(batch, -1, 2)
    for b in range(batch):
        assert relmax(got[b], to_pairs(x[b], keys, tri_size(L))) < 1e-10
    # noisy data: numpy's least-squares solution of the same design matrix
    noisy = data[0] + rng.normal(scale=0.1, size=N)
    want = to_pairs(np.linalg.lstsq(A, noisy, rcond=None)[0], keys, tri_size(L))
    got = ctx.st_lsq(noisy, L, lat, lon, conv=conv).reshape(-1, 2)
    assert relmax(got, want) < 1e-9


@pytest.mark.parametrize("conv", [(1, 0, 0), (0, 1, 1)])
def test_zt_lsq_recovers_expansion(ctx, oracle, conv):
    rng = np.random.default_rng(32)
    L, N, batch = 8, 900, 2
    r = rng.uniform(0, 1, N) ** (1 / 3)
    lon = rng.uniform(0, 2 * np.pi, N)
    colat = np.arccos(rng.uniform(-1, 1, N))
    A, keys = zt_design(oracle, L, r, lon, colat, *conv)
    x = rng.normal(size=(batch, A.shape[1]))
    data = x @ A.T
    got = ctx.zt_lsq(data.ravel(), L, r, lon, colat, batch=batch, conv=conv).reshape(batch, -1, 2)
    for b in range(batch):
        assert relmax(got[b], to_pairs(x[b], keys, zt_coeff_size(L))) < 1e-10
    noisy = data[1] + rng.normal(scale=0.05, size=N)
    want = to_pairs(np.linalg.lstsq(A, noisy, rcond=None)[0], keys, zt_coeff_size(L))
    got = ctx.zt_lsq(noisy, L, r, lon, colat, conv=conv).reshape(-1, 2)
    assert relmax(got, want) < 1e-9


def test_lsq_device_memory_and_refusal(ctx, oracle):
    torch = pytest.importorskip("torch")
    import zest_gb300 as zg
    rng = np.random.default_rng(33)
    L, N = 10, 400
    lat = np.arcsin(rng.uniform(-1, 1, N))
    lon = rng.uniform(0, 2 * np.pi, N)
    A, _ = st_design(oracle, L, lat, lon, 0, 0)
    data = rng.normal(size=A.shape[1]) @ A.T
    host = ctx.st_lsq(data, L, lat, lon)
    dev = ctx.st_lsq(torch.from_numpy(data).cuda(), L, lat, lon)
    np.testing.assert_allclose(dev.cpu().numpy(), host, rtol=0, atol=1e-12 * np.max(np.abs(host)))
    with pytest.raises(zg.ZestGPUError) as ex:
        ctx.st_lsq(data[:50], L, lat[:50], lon[:50])  # 50 points, 100 unknowns
    assert ex.value.code == zg.ERR_UNSUPPORTED


def test_st_lsq_many_panels_vs_numpy(ctx, oracle):
    """Order 32 (1,024 unknowns: 32 panels of the blocked QR) on 2,500 points
    with 5 noisy data vectors, against numpy's least-squares solution."""
    rng = np.random.default_rng(34)
    L, N, batch = 32, 2500, 5
    lat = np.arcsin(rng.uniform(-1, 1, N))
    lon = rng.uniform(0, 2 * np.pi, N)
    A, keys = st_design(oracle, L, lat, lon, 0, 0)
    data = rng.normal(size=(batch, A.shape[1])) @ A.T + rng.normal(scale=0.1, size=(batch, N))
    want = np.linalg.lstsq(A, data.T, rcond=None)[0].T
    got = ctx.st_lsq(data.ravel(), L, lat, lon, batch=batch).reshape(batch, -1, 2)
    for b in range(batch):
        assert relmax(got[b], to_pairs(want[b], keys, tri_size(L))) < 1e-9

"""Adjoints (vector-Jacobian products) of the transforms and of the rotation.

Checked three ways:
  * the transpose identity <F g, c> = <g, F^T c> (and the same for B), which
    for the GLQ forward transform F = G^+ B^T W is the quadrature-weighted
    transpose identity; checked also against that explicit formula, with W
    and G built here from the oracle's GL nodes;
  * FP64 central finite differences, h = 1e-6, of a loss through the map;
  * for the rotation, the gradient of the alignment loss
    ||rotate(f, a) - g||^2 with respect to the Euler angles a (order 64,
    batch 256) against central differences: agreement to 1e-7 relative.
Tolerances: 1e-12 relative for the identities (FP64 rounding of the
transforms), 1e-7 for the finite differences."""
import numpy as np
import pytest

from oracle import zidx, zt_coeff_size, st_grid_shape, zt_grid_shape

pytestmark = pytest.mark.gpu

ZT_CONVS = [(1, 0, 0), (0, 0, 0), (1, 1, 1), (0, 1, 0)]


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


def rand_zt(rng, L, batch=1, power=1.0):
    c = np.zeros((batch, zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[:, zidx(n, l, m)] = rng.normal(size=(batch, 2)) * (n + 1) ** -power
                if m == 0:
                    c[:, zidx(n, l, m), 1] = 0.0
    return c


def rand_st(rng, L, batch=1):
    c = rng.normal(size=(batch, L * (L + 1) // 2, 2))
    for l in range(L):
        c[:, l * (l + 1) // 2, 1] = 0.0
    return c


def rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("conv", ZT_CONVS)
def test_zt_transpose_identities(ctx, conv):
    rng = np.random.default_rng(1)
    L, batch = 17, 3
    g = rng.normal(size=int(np.prod(zt_grid_shape(L))) * batch)
    c = rand_zt(rng, L, batch).ravel()
    Fg = ctx.zt_forward(g, L, batch=batch, conv=conv)
    Ftc = ctx.zt_forward_vjp(c, L, batch=batch, conv=conv)
    assert rel(np.dot(Fg, c), np.dot(g, Ftc)) < 1e-12
    Bc = ctx.zt_backward(c, L, batch=batch, conv=conv)
    Btg = ctx.zt_backward_vjp(g, L, batch=batch, conv=conv)
    assert rel(np.dot(Bc, g), np.dot(c, Btg)) < 1e-12


def test_zt_forward_vjp_is_quadrature_weighted_backward(ctx, oracle):
    # F^T c = W B(G^+ c) with W = (2 pi / nlon) w_lat w_rad r^2 / 2 and
    # G = S (1 or 1/(2n+3)), S = 4 pi (geo) / 1 (qm)
    rng = np.random.default_rng(2)
    L = 12
    nlon, nlat, nrad = zt_grid_shape(L)
    _, wl = oracle.gl_nodes_weights(nlat)
    xr, wr = oracle.gl_nodes_weights(nrad)
    r = (1 + np.asarray(xr)) / 2
    W = (2 * np.pi / nlon) * np.asarray(wl)[None, :, None] * (np.asarray(wr) * r * r / 2)[None, None, :]
    for zn, sn, sp in ZT_CONVS:
        c = rand_zt(rng, L)[0]
        Ginv = np.zeros_like(c)
        for n in range(L):
            for l in range(n & 1, n + 1, 2):
                for m in range(l + 1):
                    g = (4 * np.pi if sn == 0 else 1.0) * (1.0 if zn == 0 else 1.0 / (2 * n + 3))
                    Ginv[zidx(n, l, m)] = [1 / g, 1 / g if m else 0.0]
        want = W * oracle.zt_backward(c * Ginv, L, zn=zn, sn=sn, sp=sp).reshape(nlon, nlat, nrad)
        got = ctx.zt_forward_vjp(c.ravel(), L, conv=(zn, sn, sp)).reshape(nlon, nlat, nrad)
        assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))


def test_zt_vjp_truncation(ctx):
    # expansion order above / below the grid order
    rng = np.random.default_rng(3)
    for Lg, Le in [(9, 12), (12, 9)]:
        g = rng.normal(size=int(np.prod(zt_grid_shape(Lg))))
        c = rand_zt(rng, Le).ravel()
        assert rel(np.dot(ctx.zt_forward(g, Lg, Le), c), np.dot(g, ctx.zt_forward_vjp(c, Lg, Le))) < 1e-12
        assert rel(np.dot(ctx.zt_backward(c, Le, Lg), g), np.dot(c, ctx.zt_backward_vjp(g, Le, Lg))) < 1e-12


@pytest.mark.parametrize("layout,L", [(0, 16), (0, 9), (1, 16), (1, 9)])
def test_st_transpose_identities(ctx, layout, L):
    # includes the odd LatLon grid, whose middle latitude the reference counts twice
    rng = np.random.default_rng(4)
    batch = 2
    for conv in [(0, 0), (1, 1)]:
        g = rng.normal(size=int(np.prod(st_grid_shape(L, layout))) * batch)
        c = rand_st(rng, L, batch).ravel()
        Fg = ctx.st_forward(g, L, batch=batch, conv=conv, layout=layout)
        Ftc = ctx.st_forward_vjp(c, L, batch=batch, conv=conv, layout=layout)
        assert rel(np.dot(Fg, c), np.dot(g, Ftc)) < 1e-12
        Bc = ctx.st_backward(c, L, batch=batch, conv=conv, layout=layout)
        Btg = ctx.st_backward_vjp(g, L, batch=batch, conv=conv, layout=layout)
        assert rel(np.dot(Bc, g), np.dot(c, Btg)) < 1e-12


def test_zt_forward_vjp_vs_finite_differences_order100(ctx):
    # forward-transform vjp at order 100, batch 32: loss(g) = <w, F g> +
    # |F g|^2 / 2, central differences with h = 1e-6 along random directions.
    # (A loss like |F g - t|^2 / 2 with a large constant |t|^2 would bury the
    # difference quotient in rounding: eps |loss| / h.)
    rng = np.random.default_rng(5)
    L, batch = 100, 32
    gsz = int(np.prod(zt_grid_shape(L)))
    g = rng.normal(size=gsz * batch)
    f = ctx.zt_forward(g, L, batch=batch)
    w = rng.normal(size=f.size) * np.abs(f)

    def loss(x):
        fx = ctx.zt_forward(x, L, batch=batch)
        return np.dot(w, fx) + 0.5 * np.dot(fx, fx)

    grad = ctx.zt_forward_vjp(w + f, L, batch=batch)
    h = 1e-6
    # directions with a large projection on the gradient: along a random
    # direction the derivative is ~sqrt(N) smaller than the loss and the
    # quotient would measure the transform's rounding, not the adjoint
    # (scaled to |g|, so that h d is a relative step of h and not far below it)
    u = grad / np.linalg.norm(grad)
    for _ in range(3):
        r = rng.normal(size=g.size)
        d = (u + 0.5 * r / np.linalg.norm(r)) * np.linalg.norm(g)
        fd = (loss(g + h * d) - loss(g - h * d)) / (2 * h)
        assert rel(fd, np.dot(grad, d)) < 1e-7


def test_rotation_vjp_coefficients(ctx):
    rng = np.random.default_rng(6)
    L, batch = 33, 4
    x = rand_zt(rng, L, batch).ravel()
    y = rand_zt(rng, L, batch).ravel()
    e = rng.uniform(-np.pi, np.pi, size=3 * batch)
    for rtype in (0, 1):
        Dx = ctx.zt_rotate(x.copy(), L, e.copy(), batch=batch, rotation_type=rtype)
        xb, _ = ctx.zt_rotate_vjp(x, L, e, y, batch=batch, rotation_type=rtype, want_euler=False)
        assert rel(np.dot(Dx, y), np.dot(x, xb)) < 1e-12


@pytest.mark.parametrize("rtype", [0, 1])
def test_alignment_gradient_vs_finite_differences(ctx, rtype):
    # rotational alignment at order 64, batch 256: L(a) = ||rotate(f, a) - g||^2,
    # g = rotate(f, a_true) + N(0, 1e-3); dL/da by the adjoint vs central
    # differences (h = 1e-6), per item and angle
    rng = np.random.default_rng(7 + rtype)
    L, batch = 64, 256
    f = rand_zt(rng, L, batch).ravel()
    a_true = np.stack([rng.uniform(0, 2 * np.pi, batch), np.arccos(rng.uniform(-1, 1, batch)),
                       rng.uniform(0, 2 * np.pi, batch)], axis=1).ravel()
    g = ctx.zt_rotate(f.copy(), L, a_true.copy(), batch=batch, rotation_type=rtype)
    g = g + rng.normal(scale=1e-3, size=g.size)
    a = a_true + rng.normal(scale=0.3, size=a_true.size)

    def losses(angles):
        r = ctx.zt_rotate(f.copy(), L, angles.copy(), batch=batch, rotation_type=rtype) - g
        return np.sum(r.reshape(batch, -1) ** 2, axis=1)

    r = ctx.zt_rotate(f.copy(), L, a.copy(), batch=batch, rotation_type=rtype) - g
    _, ga = ctx.zt_rotate_vjp(f, L, a, 2 * r, batch=batch, rotation_type=rtype, want_coeffs=False)
    ga = ga.reshape(batch, 3)
    h = 1e-6
    for k in range(3):
        dp = a.copy().reshape(batch, 3)
        dm = a.copy().reshape(batch, 3)
        dp[:, k] += h
        dm[:, k] -= h
        fd = (losses(dp.ravel()) - losses(dm.ravel())) / (2 * h)
        scale = np.maximum(np.abs(fd), np.max(np.abs(fd)) * 1e-3)
        assert np.max(np.abs(ga[:, k] - fd) / scale) < 1e-7, k


def test_sh_rotation_gradient_vs_finite_differences(ctx):
    rng = np.random.default_rng(9)
    L, batch = 24, 8
    f = rand_st(rng, L, batch).ravel()
    g = rand_st(rng, L, batch).ravel()
    a = rng.uniform(-np.pi, np.pi, size=3 * batch)

    def losses(angles):
        r = ctx.st_rotate(f.copy(), L, angles.copy(), batch=batch) - g
        return np.sum(r.reshape(batch, -1) ** 2, axis=1)

    r = ctx.st_rotate(f.copy(), L, a.copy(), batch=batch) - g
    xb, ga = ctx.st_rotate_vjp(f, L, a, 2 * r, batch=batch)
    ga = ga.reshape(batch, 3)
    h = 1e-6
    for k in range(3):
        dp = a.copy().reshape(batch, 3)
        dm = a.copy().reshape(batch, 3)
        dp[:, k] += h
        dm[:, k] -= h
        fd = (losses(dp.ravel()) - losses(dm.ravel())) / (2 * h)
        scale = np.maximum(np.abs(fd), np.max(np.abs(fd)) * 1e-3)
        assert np.max(np.abs(ga[:, k] - fd) / scale) < 1e-7
    # coefficient cotangent: D^T (2 r) against the identity <D f, y> = <f, D^T y>
    y = rand_st(rng, L, batch).ravel()
    xb, _ = ctx.st_rotate_vjp(f, L, a, y, batch=batch, want_euler=False)
    Df = ctx.st_rotate(f.copy(), L, a.copy(), batch=batch)
    assert rel(np.dot(Df, y), np.dot(f, xb)) < 1e-12

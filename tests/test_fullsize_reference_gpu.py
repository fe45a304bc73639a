"""Full-size configurations against the compiled reference itself.

The reference library (oracle/_ref, built from the reference's own sources by
oracle/build_ref.py) transforms the same seeded inputs on the host, and the
CUDA path, through the C-ABI, must agree with it:

  * Zernike order 200 (the headline size), one function with coefficients
    N(0, (n+1)^-3), GLQTransformerGeo: backward grid and forward coefficients
    (zernike_glq_transformer.hpp:640-707);
  * spherical harmonics lmax 1023 (order 1024), LonLat grid, one item with
    coefficients N(0, (l+1)^-2) (sh_glq_transformer.hpp:632-668);
  * a ragged batch whose orders span 8..128, each item rotated by Haar Euler
    angles (Rotor::rotate, rotor.hpp:210-243) and backward-transformed.

Tolerances, relative max-norm max|x - x_ref| / max|x_ref| per item: 1e-12
for the FP64 form, 1e-11 for the split-precision (tcgen05) form."""
import numpy as np
import pytest

from oracle import tri_idx, tri_size, zt_coeff_size, zt_grid_shape

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_SPLIT = 1e-11
FORMS = [(0, TOL_FP64), (1, TOL_SPLIT)]


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def zt_coeffs(rng, L, power):
    """c_nlm ~ N(0, (n+1)^(-2 power)) for valid (n, l, m), Im(m=0) = 0."""
    T = zt_coeff_size(L)
    sd = np.zeros(T)
    m0 = np.zeros(T, dtype=bool)
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            base = (n + 1) * (n + 3) * (2 * n + 1) // 24 + (l * l) // 4
            sd[base:base + l + 1] = (n + 1.0) ** -power
            m0[base] = True
    c = rng.standard_normal((T, 2)) * sd[:, None]
    c[m0, 1] = 0.0
    return c


def st_coeffs(rng, L):
    """a_lm, b_lm ~ N(0, (l+1)^-2), b_l0 = 0."""
    l_of = np.repeat(np.arange(L), np.arange(1, L + 1))
    c = rng.standard_normal((tri_size(L), 2)) / (l_of[:, None] + 1.0)
    c[[tri_idx(l, 0) for l in range(L)], 1] = 0.0
    return c


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def reference():
    from oracle import Reference
    try:
        return Reference()
    except (FileNotFoundError, OSError) as exc:
        pytest.skip(f"compiled reference unavailable: {exc}")


@pytest.fixture(scope="module")
def zt200(reference):
    """Order-200 coefficients, the reference's backward grid of them and the
    reference's forward transform of that grid."""
    L = 200
    c = zt_coeffs(np.random.default_rng(1), L, 1.5)
    g_ref = reference.zt_backward(c, L)
    f_ref = reference.zt_forward(g_ref, L)
    return L, c, g_ref, f_ref


@pytest.mark.parametrize("precision,tol", FORMS)
def test_zt_order200_vs_reference(ctx, zt200, precision, tol):
    L, c, g_ref, f_ref = zt200
    ctx.set_precision(precision)
    try:
        g = ctx.zt_backward(c.ravel(), L)
        f = ctx.zt_forward(np.ascontiguousarray(g_ref).ravel(), L)
    finally:
        ctx.set_precision(0)
    err_g, err_f = relmax(g, g_ref), relmax(f, f_ref)
    assert err_g < tol, f"backward grid {err_g:.3e}"
    assert err_f < tol, f"forward coefficients {err_f:.3e}"


@pytest.fixture(scope="module")
def st1024(reference):
    L = 1024
    c = st_coeffs(np.random.default_rng(1024), L)
    g_ref = reference.st_backward(c, L)
    f_ref = reference.st_forward(g_ref, L)
    return L, c, g_ref, f_ref


@pytest.mark.parametrize("precision,tol", FORMS)
def test_st_lmax1023_vs_reference(ctx, st1024, precision, tol):
    L, c, g_ref, f_ref = st1024
    ctx.set_precision(precision)
    try:
        g = ctx.st_backward(c.ravel(), L)
        f = ctx.st_forward(np.ascontiguousarray(g_ref).ravel(), L)
    finally:
        ctx.set_precision(0)
    err_g, err_f = relmax(g, g_ref), relmax(f, f_ref)
    assert err_g < tol, f"backward grid {err_g:.3e}"
    assert err_f < tol, f"forward coefficients {err_f:.3e}"


@pytest.fixture(scope="module")
def ragged(reference):
    """48 items, orders spanning 8..128 (127 and 128 included), coefficients
    N(0, (n+1)^-2), Haar-uniform Euler angles; the reference's rotate +
    backward grids of every item."""
    rng = np.random.default_rng(4096)
    orders = np.sort(np.concatenate([[8, 127, 128], rng.integers(8, 129, size=45)])).astype(np.int32)
    cs = [zt_coeffs(rng, int(L), 1.0).ravel() for L in orders]
    e = np.stack([rng.uniform(0, 2 * np.pi, orders.size), np.arccos(rng.uniform(-1, 1, orders.size)),
                  rng.uniform(0, 2 * np.pi, orders.size)], axis=1)
    flat = np.concatenate(cs)
    _, want = reference.zt_rotate_backward_ragged(orders, flat.copy(), e, 8, want_grids=True)
    return orders, flat, e, want


@pytest.mark.parametrize("precision,tol", FORMS)
def test_ragged_rotate_backward_vs_reference(ctx, ragged, precision, tol):
    torch = pytest.importorskip("torch")
    orders, flat, e, want = ragged
    gsz = [int(np.prod(zt_grid_shape(int(L)))) for L in orders]
    coeffs = torch.from_numpy(flat.copy()).cuda()
    euler = torch.from_numpy(np.ascontiguousarray(e).ravel()).cuda()
    grids = torch.zeros(sum(gsz), dtype=torch.float64, device="cuda")
    ctx.set_precision(precision)
    try:
        ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)
        ctx.synchronize()
    finally:
        ctx.set_precision(0)
    got = grids.cpu().numpy()
    off, worst = 0, {}
    for L, gs in zip(orders, gsz):
        err = relmax(got[off:off + gs], want[off:off + gs])
        worst[int(L)] = max(worst.get(int(L), 0.0), err)
        off += gs
    bad = {L: v for L, v in worst.items() if not v < tol}
    assert not bad, f"orders above tolerance: {bad}"
    assert 127 in worst and 128 in worst

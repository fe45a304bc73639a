"""Coefficient layouts beside the transforms, through the C-ABI, against the
compiled reference:

  * to_complex_expansion / to_real_expansion of Zernike, SH and per-n
    Zernike SH (row-skipping) expansions, with changes of every convention
    (zernike_expansion.hpp:484-775, real_sh_expansion.hpp:345-436):
    bit-identical, since every factor is computed as the reference does;
  * Rotor::rotate of a per-n Zernike SH span (rotor.hpp:165-193): 1e-13
    relative max-norm against the reference, and bit-identical to the row n
    of the whole-expansion rotation (the same kernel);
  * the SH backward transform of a row-skipping expansion
    (sh_glq_transformer.hpp:680-754), its truncation included: 1e-12."""
import numpy as np
import pytest

from oracle import zidx, zt_coeff_size

pytestmark = pytest.mark.gpu

CONVS = [(zn, sn, sp) for zn in (0, 1) for sn in (0, 1) for sp in (0, 1)]


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


@pytest.fixture(scope="module")
def reference():
    from oracle import Reference
    try:
        return Reference()
    except (FileNotFoundError, OSError) as exc:
        pytest.skip(f"compiled reference unavailable: {exc}")


def pairs(kind, L):
    import zest_gb300 as zg
    return {0: zg.zt_coeff_size, 1: zg.st_coeff_size, 2: zg.rows_coeff_size}[kind](L)


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("L", [1, 2, 5, 13, 40])
def test_convert_bitwise_vs_reference(ctx, reference, kind, L):
    rng = np.random.default_rng(100 * kind + L)
    for src in CONVS:
        for dst in CONVS:
            if kind != 0 and src[0] != dst[0]:
                continue  # only a whole Zernike expansion changes its Zernike normalisation
            c = rng.normal(size=(pairs(kind, L), 2))
            for to_complex in (1, 0):
                want = reference.convert(c, kind, L, src, dst, to_complex)
                got = ctx.convert_expansion(c.ravel().copy(), kind, L, src, dst, to_complex)
                np.testing.assert_array_equal(got.reshape(want.shape), want)


def test_convert_round_trip_and_batch(ctx):
    import zest_gb300 as zg
    rng = np.random.default_rng(7)
    L, batch = 9, 3
    c = rng.normal(size=(batch, zg.zt_coeff_size(L), 2))
    x = ctx.convert_expansion(c.ravel().copy(), zg.EXPANSION_ZERNIKE, L, (0, 0, 0), (1, 1, 1), True, batch=batch)
    y = ctx.convert_expansion(x.copy(), zg.EXPANSION_ZERNIKE, L, (1, 1, 1), (0, 0, 0), False, batch=batch)
    assert relmax(y, c) < 1e-15
    one = ctx.convert_expansion(c[1].ravel().copy(), zg.EXPANSION_ZERNIKE, L, (0, 0, 0), (1, 1, 1), True)
    np.testing.assert_array_equal(x.reshape(batch, -1)[1], one)
    sh = rng.normal(size=(zg.st_coeff_size(L), 2)).ravel()
    with pytest.raises(zg.ZestGPUError):  # a Zernike normalisation change needs a Zernike expansion
        ctx.convert_expansion(sh, zg.EXPANSION_SH, L, (0, 0, 0), (1, 0, 0), True)


@pytest.mark.parametrize("L", [1, 2, 7, 12, 33])
@pytest.mark.parametrize("rtype", [0, 1])
def test_rows_rotate_vs_reference(ctx, reference, L, rtype):
    import zest_gb300 as zg
    rng = np.random.default_rng(L + 50 * rtype)
    n = L - 1
    c = rng.normal(size=(zg.rows_coeff_size(L), 2))
    e = rng.uniform(-np.pi, np.pi, 3)
    want = reference.rows_rotate(c, L, e, rtype)
    got = ctx.rows_rotate(c.ravel().copy(), L, e.copy(), rotation_type=rtype)
    assert relmax(got, want) < 1e-13
    if n == 0:
        return  # a whole expansion leaves n = 0 unrotated (rotor.hpp:232 starts at n = 1); the row span does not
    # the same vectors as row n of a whole Zernike expansion of order L
    full = np.zeros((zt_coeff_size(L), 2))
    base = zidx(n, 0, 0)
    full[base:base + c.shape[0]] = c
    rot = ctx.zt_rotate(full.ravel().copy(), L, e.copy(), rotation_type=rtype).reshape(-1, 2)
    np.testing.assert_array_equal(got.reshape(-1, 2), rot[base:base + c.shape[0]])


@pytest.mark.parametrize("Le,Lg", [(7, 7), (6, 9), (9, 6), (8, 5), (20, 20)])
@pytest.mark.parametrize("latlon", [0, 1])
def test_st_backward_rows_vs_reference(ctx, reference, Le, Lg, latlon):
    import zest_gb300 as zg
    rng = np.random.default_rng(Le * 31 + Lg + latlon)
    for sn, sp in [(0, 0), (1, 1)]:
        c = rng.normal(size=(zg.rows_coeff_size(Le), 2))
        want = reference.st_backward_rows(c, Le, Lg, sn, sp, bool(latlon))
        got = ctx.st_backward_rows(c.ravel().copy(), Le, Lg, conv=(sn, sp), layout=latlon)
        assert relmax(got, want) < 1e-12

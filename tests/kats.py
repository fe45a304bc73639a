"""Known-answer cases of the reference's transform tests, shared by the
oracle tests (tests/test_oracle_golden.py) and the device tests
(tests/test_gpu_parity.py), with the reference's quadrature points."""
import numpy as np

from oracle import st_grid_shape, zt_grid_shape


def ball_points(oracle, L):
    """BallGLQGridPoints (zernike_glq_transformer.hpp:336-501): longitudes
    2 pi i / nlon, z = cos(colatitude) at the GL nodes, r = (1 + x) / 2 at the
    GL nodes; the same as the reference's points in points.npz to 1e-15."""
    nlon, nlat, nrad = zt_grid_shape(L)
    z, _ = oracle.gl_nodes_weights(nlat)
    x, _ = oracle.gl_nodes_weights(nrad)
    return 2.0 * np.pi * np.arange(nlon) / nlon, z, 0.5 * (1.0 + x)


def sphere_points(oracle, L, latlon):
    """SphereGLQGridPoints (sh_glq_transformer.hpp:385-504): longitudes over
    the layout's longitude count, z at the GL nodes of its latitude count."""
    shape = st_grid_shape(L, bool(latlon))
    nlon, nlat = (shape[1], shape[0]) if latlon else shape
    z, _ = oracle.gl_nodes_weights(nlat)
    return 2.0 * np.pi * np.arange(nlon) / nlon, z


# tests/test_zernike_glq_transformer.cpp:136-519: functions that are a single
# Zernike function (times its normalisation, and the phase where m is odd)
# expand to that one coefficient; :521-870: their backward transforms give the
# sampled function back.  Entries: (n, l, m), function of (lon, z = cos colat,
# r, phase), the normed factor, the expected {cos, sin} coefficient.
ZT_KATS = [
    ((2, 0, 0), lambda lon, z, r, ph: 2.5 * r * r - 1.5, np.sqrt(7.0), (1.0, 0.0)),
    ((1, 1, 0), lambda lon, z, r, ph: r * np.sqrt(3.0) * z, np.sqrt(5.0), (1.0, 0.0)),
    ((2, 2, 1), lambda lon, z, r, ph: ph * r * r * np.sqrt(15.0) * np.sqrt(1.0 - z * z) * z * np.cos(lon),
     np.sqrt(7.0), (1.0, 0.0)),
    ((3, 3, 2), lambda lon, z, r, ph: r ** 3 * np.sqrt(105.0 / 4.0) * (1.0 - z * z) * z * np.sin(2.0 * lon),
     3.0, (0.0, 1.0)),
    ((5, 3, 1), lambda lon, z, r, ph: ph * (5.5 * r * r - 4.5) * r ** 3 * np.sqrt(21.0 / 8.0)
     * np.sqrt(1.0 - z * z) * (5.0 * z * z - 1.0) * np.cos(lon), np.sqrt(13.0), (1.0, 0.0)),
]


# tests/test_sh_glq_transformer.cpp:53-777: single spherical harmonics (and a
# sum of two) expand to their coefficients and evaluate back, in both grid
# layouts.  Entries: function of (lon, z = cos colat, phase), {(l, m): {cos, sin}}.
ST_KATS = [
    (lambda lon, z, ph: np.ones_like(z), {(0, 0): (1.0, 0.0)}),
    (lambda lon, z, ph: np.sqrt(3.0) * z, {(1, 0): (1.0, 0.0)}),
    (lambda lon, z, ph: ph * np.sqrt(15.0) * np.sqrt(1.0 - z * z) * z * np.cos(lon), {(2, 1): (1.0, 0.0)}),
    (lambda lon, z, ph: ph * np.sqrt(21.0 / 8.0) * np.sqrt(1.0 - z * z) * (5.0 * z * z - 1.0) * np.cos(lon),
     {(3, 1): (1.0, 0.0)}),
    (lambda lon, z, ph: ph * np.sqrt(315.0 / 8.0) * np.sqrt(1.0 - z * z) * (1.0 - z * z) * z * np.sin(3.0 * lon),
     {(4, 3): (0.0, 1.0)}),
    (lambda lon, z, ph: ph * (np.sqrt(21.0 / 8.0) * np.sqrt(1.0 - z * z) * (5.0 * z * z - 1.0) * np.cos(lon)
                              + np.sqrt(315.0 / 8.0) * np.sqrt(1.0 - z * z) * (1.0 - z * z) * z * np.sin(3.0 * lon)),
     {(3, 1): (1.0, 0.0), (4, 3): (0.0, 1.0)}),
]

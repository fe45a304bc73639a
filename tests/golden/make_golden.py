"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout where the reference sources are available (the reference
library is compiled from them by oracle/build_ref.py into oracle/_ref/):

    python tests/golden/make_golden.py

Every array stored here is an output of the compiled reference library
(sebsassi/zest) on seeded synthetic inputs; the inputs are stored beside the
outputs.  The fixtures are small (orders <= 24) so that the CPU tests stay fast.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from oracle import (Reference, tri_idx, tri_size, zidx, zt_coeff_size,  # noqa: E402
                    zt_grid_shape, zt_sample_config1)

CONVS_ZT = [(1, 0, 0), (0, 0, 0), (1, 1, 0), (0, 1, 0), (1, 1, 1), (0, 1, 1), (1, 0, 1), (0, 0, 1)]
CONVS_ST = [(0, 0), (1, 0), (0, 1), (1, 1)]


def rand_zt(rng, L, power=1.5):
    c = np.zeros((zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[zidx(n, l, m)] = rng.normal(size=2) * (n + 1) ** -power
                if m == 0:
                    c[zidx(n, l, m), 1] = 0.0
    return c


def rand_st(rng, L):
    c = np.zeros((tri_size(L), 2))
    for l in range(L):
        for m in range(l + 1):
            c[tri_idx(l, m)] = rng.normal(size=2) / (l + 1)
            if m == 0:
                c[tri_idx(l, m), 1] = 0.0
    return c


def main():
    ref = Reference()
    out = {}

    # Gauss-Legendre nodes and weights, both layouts (cos style).
    gl = {}
    for n in [1, 2, 3, 4, 5, 8, 21, 24, 69, 70, 71, 101, 104, 201, 208, 512, 1024]:
        for packed in (0, 1):
            x, w = ref.gl_nodes_weights(n, bool(packed))
            gl[f"x_{n}_{packed}"] = x
            gl[f"w_{n}_{packed}"] = w
    np.savez_compressed(os.path.join(HERE, "gl.npz"), **gl)

    # P_lm tables (all SH conventions) and radial Zernike tables (both norms)
    # at the order-20 ball-grid nodes.
    L = 20
    _, nt, nr = zt_grid_shape(L)
    z, _ = ref.gl_nodes_weights(nt)
    x, _ = ref.gl_nodes_weights(nr)
    r = 0.5 * (1.0 + x)
    tab = {"z": z, "r": r}
    for sn, sp in CONVS_ST:
        tab[f"plm_{sn}_{sp}"] = ref.plm_real(L, sn, sp, z)
    for zn in (0, 1):
        tab[f"rz_{zn}"] = ref.radial_zernike(L, zn, r)
    tab["wignerd_16"] = ref.wignerd(16)
    np.savez_compressed(os.path.join(HERE, "tables.npz"), **tab)

    # Config 1: order 20, f = r exp(-(sin colat cos lon)^2), GLQTransformerGeo.
    lon, colat, rad = ref.zt_grid_points(L)
    f = zt_sample_config1(lon, colat, rad)
    c = ref.zt_forward(f, L, L, 1, 0, 0)
    g = ref.zt_backward(c, L, L, 1, 0, 0)
    np.savez_compressed(os.path.join(HERE, "zt_config1.npz"), lon=lon, colat=colat, rad=rad,
                        grid=f, coeffs=c, roundtrip=g)

    # Random band-limited Zernike expansions, every convention, small orders,
    # plus order-mismatch (truncation / zero padding) cases.
    rng = np.random.default_rng(20240501)
    zt = {}
    for L in [1, 2, 3, 6, 11, 16]:
        for conv in (CONVS_ZT if L < 16 else CONVS_ZT[:1]):
            key = f"{L}_{conv[0]}{conv[1]}{conv[2]}"
            c = rand_zt(rng, L)
            g = ref.zt_backward(c, L, L, *conv)
            zt["c_" + key] = c
            zt["g_" + key] = g
            zt["f_" + key] = ref.zt_forward(g, L, L, *conv)
    c = rand_zt(rng, 9)
    zt["trunc_c"] = c
    zt["trunc_g96"] = ref.zt_backward(c, 9, 6, 1, 0, 0)
    g = ref.zt_backward(c, 9, 9, 1, 0, 0)
    zt["trunc_g99"] = g
    zt["trunc_f96"] = ref.zt_forward(g, 9, 6, 1, 0, 0)
    zt["trunc_f9_12"] = ref.zt_forward(g, 9, 12, 1, 0, 0)
    c6 = c[: zt_coeff_size(6)].copy()
    zt["trunc_c6"] = c6
    zt["trunc_g69"] = ref.zt_backward(c6, 6, 9, 1, 0, 0)
    np.savez_compressed(os.path.join(HERE, "zt_random.npz"), **zt)

    # Random SH expansions, both grid layouts, every convention.
    st = {}
    for L in [1, 2, 5, 8, 16, 24]:
        for latlon in (0, 1):
            for conv in (CONVS_ST if L < 16 else CONVS_ST[:1]):
                key = f"{L}_{latlon}_{conv[0]}{conv[1]}"
                c = rand_st(rng, L)
                g = ref.st_backward(c, L, L, *conv, bool(latlon))
                st["c_" + key] = c
                st["g_" + key] = g
                st["f_" + key] = ref.st_forward(g, L, L, *conv, bool(latlon))
    np.savez_compressed(os.path.join(HERE, "st_random.npz"), **st)

    # Rotations: Euler angles (object and coordinate), rotation matrices,
    # polar rotations; Zernike and SH.
    rot = {}
    for L in [2, 5, 10, 17]:
        c = rand_zt(rng, L)
        e = rng.uniform(0.0, 2.0 * np.pi, 3)
        rot[f"zc_{L}"] = c
        rot[f"ze_{L}"] = e
        rot[f"zobj_{L}"] = ref.zt_rotate(c, L, e, 0)
        rot[f"zcoord_{L}"] = ref.zt_rotate(c, L, e, 1)
        rot[f"zpolar_{L}"] = ref.zt_polar_rotate(c, L, e[0], 0)
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(q) < 0:
            q[:, 0] *= -1
        rot[f"zmat_{L}"] = q
        rot[f"zmatobj_{L}"] = ref.zt_rotate_matrix(c, L, q, 0)
        s = rand_st(rng, L + 3)
        rot[f"sc_{L}"] = s
        rot[f"sobj_{L}"] = ref.st_rotate(s, L + 3, e, 0)
        rot[f"scoord_{L}"] = ref.st_rotate(s, L + 3, e, 1)
        rot[f"spolar_{L}"] = ref.st_polar_rotate(s, L + 3, e[1], 1)
    np.savez_compressed(os.path.join(HERE, "rotation.npz"), **rot)

    # Evaluation at arbitrary points (zt/st GridEvaluator) and the Zernike power
    # spectrum.  The reference's SH spectra do not compile against its SH spans
    # (they read ExpansionType::sh_norm), so they have no fixture.
    rng2 = np.random.default_rng(20240611)
    ev = {}
    for L, nlon, nlat, nrad in [(1, 3, 2, 2), (6, 7, 5, 4), (13, 11, 9, 6), (24, 5, 17, 3)]:
        lon = rng2.uniform(-np.pi, 3 * np.pi, nlon)
        colat = rng2.uniform(0.0, np.pi, nlat)
        rad = rng2.uniform(0.0, 1.0, nrad)
        ev[f"lon_{L}"], ev[f"colat_{L}"], ev[f"rad_{L}"] = lon, colat, rad
        c = rand_zt(rng2, L, power=1.0)
        ev[f"zc_{L}"] = c
        for conv in CONVS_ZT:
            key = "".join(map(str, conv))
            ev[f"zv_{L}_{key}"] = ref.zt_evaluate(c, L, lon, colat, rad, *conv)
        s = rand_st(rng2, L + 2)
        ev[f"sc_{L}"] = s
        for conv in CONVS_ST:
            key = "".join(map(str, conv))
            ev[f"sv_{L}_{key}"] = ref.st_evaluate(s, L + 2, lon, colat, *conv)
    np.savez_compressed(os.path.join(HERE, "evaluate.npz"), **ev)

    ps = {}
    for L in [1, 2, 7, 16, 31]:
        c = rand_zt(rng2, L, power=1.0)
        ps[f"zc_{L}"] = c
        for sn in (0, 1):
            ps[f"zp_{L}_{sn}"] = ref.zt_power_spectrum(c, L, sn)
    np.savez_compressed(os.path.join(HERE, "spectra.npz"), **ps)

    # Points of the quadrature grids (BallGLQGridPoints, SphereGLQGridPoints).
    pts = {}
    for L in [1, 2, 5, 20, 64, 201]:
        pts[f"zlon_{L}"], pts[f"zcolat_{L}"], pts[f"zrad_{L}"] = ref.zt_grid_points(L)
    for L in [1, 3, 8, 12, 100]:
        for latlon in (0, 1):
            pts[f"slon_{L}_{latlon}"], pts[f"scolat_{L}_{latlon}"] = ref.st_grid_points(L, latlon)
    np.savez_compressed(os.path.join(HERE, "points.npz"), **pts)

    for name in sorted(os.listdir(HERE)):
        if name.endswith(".npz"):
            print(name, os.path.getsize(os.path.join(HERE, name)))


if __name__ == "__main__":
    main()

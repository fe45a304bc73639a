"""Parity oracle for the zest GLQ transform + rotation path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by the cpu_baseline leg of bench.py, always as the
checker.  The product package (zest_gb300) never imports this module.

Two CPU implementations are exposed with the same call signatures:
  * ``Oracle``  -- zest_oracle.c, the C restatement written for this project
  * ``Reference`` -- oracle/_ref/libzest_ref.so, the reference library itself
    compiled from its sources (only where its sources are available).
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")

_c_sz = ctypes.c_size_t
_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_p_dbl = ctypes.POINTER(ctypes.c_double)


def _is_native(path: str) -> bool:
    try:
        with open(path, "rb") as f:
            hdr = f.read(20)
    except OSError:
        return False
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine(), -1)
    return hdr[:4] == b"\x7fELF" and int.from_bytes(hdr[18:20], "little") == want


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "zest_oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(ORACLE_SO) and _is_native(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    tmp = ORACLE_SO + ".tmp"
    subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared",
                    src, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_p_dbl)


def pad8(n: int) -> int:
    return (n + 7) & ~7


# ---- shapes (restated from the reference layouts) ----
def zt_grid_shape(L: int):
    """(lon, lat, rad) of the ball grid, include/zernike_glq_transformer.hpp:50-131."""
    return (2 * L - 1 if L else 0, L + 1, pad8(L + 1))


def zt_coeff_size(L: int) -> int:
    return (L + 1) * (L + 3) * (2 * L + 1) // 24


def zidx(n: int, l: int, m: int) -> int:
    return (n + 1) * (n + 3) * (2 * n + 1) // 24 + (l * l) // 4 + m


def tri_size(L: int) -> int:
    return L * (L + 1) // 2


def tri_idx(l: int, m: int) -> int:
    return l * (l + 1) // 2 + m


def rad_idx(n: int, l: int) -> int:
    return ((n + 1) * (n + 1)) // 4 + l // 2


def rad_size(L: int) -> int:
    return ((L + 1) * (L + 1)) // 4


def st_grid_shape(L: int, latlon: bool = False):
    """LonLat [lon][lat] = (2L-1, pad8(L)); LatLon [lat][lon] = (L, pad8(2L-1)),
    include/sh_glq_transformer.hpp:48-197."""
    if latlon:
        return (L, pad8(2 * L - 1 if L else 0))
    return (2 * L - 1 if L else 0, pad8(L))


def wignerd_size(L: int) -> int:
    return L * (L + 1) * (2 * L + 1) // 6


class _Lib:
    prefix = ""

    def __init__(self, path: str):
        self.lib = ctypes.CDLL(path)
        self.path = path

    def _f(self, name, argtypes, restype=_c_int):
        fn = getattr(self.lib, self.prefix + name)
        fn.argtypes = argtypes
        fn.restype = restype
        return fn

    # -- tables --
    def gl_nodes_weights(self, n: int, packed: bool = False):
        sz = (n + 1) // 2 if packed else n
        x = np.zeros(sz)
        w = np.zeros(sz)
        self._gl(n, packed, x, w)
        return x, w

    def plm_real(self, L: int, sh_norm: int, sh_phase: int, z: np.ndarray):
        z = np.ascontiguousarray(z, dtype=np.float64)
        out = np.zeros((tri_size(L), z.size))
        self._f("plm_real", [_c_sz, _c_int, _c_int, _c_sz, _p_dbl, _p_dbl])(L, sh_norm, sh_phase, z.size, _ptr(z), _ptr(out))
        return out

    def radial_zernike(self, L: int, znorm: int, r: np.ndarray):
        r = np.ascontiguousarray(r, dtype=np.float64)
        out = np.zeros((rad_size(L), r.size))
        self._f("radial_zernike", [_c_sz, _c_int, _c_sz, _p_dbl, _p_dbl])(L, znorm, r.size, _ptr(r), _ptr(out))
        return out

    def wignerd(self, L: int):
        out = np.zeros(wignerd_size(L))
        self._f("wignerd", [_c_sz, _p_dbl])(L, _ptr(out))
        return out

    # -- transforms --
    def zt_forward(self, grid: np.ndarray, Lg: int, Le: int | None = None, zn: int = 1, sn: int = 0, sp: int = 0):
        Le = Lg if Le is None else Le
        grid = np.ascontiguousarray(grid, dtype=np.float64)
        assert grid.size == np.prod(zt_grid_shape(Lg))
        out = np.zeros((zt_coeff_size(Le), 2))
        self._zt_fwd(zn, sn, sp, Lg, Le, grid, out)
        return out

    def zt_backward(self, coeffs: np.ndarray, Le: int, Lg: int | None = None, zn: int = 1, sn: int = 0, sp: int = 0):
        Lg = Le if Lg is None else Lg
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        assert coeffs.size == 2 * zt_coeff_size(Le)
        out = np.zeros(zt_grid_shape(Lg))
        self._zt_bwd(zn, sn, sp, Le, Lg, coeffs, out)
        return out

    def st_forward(self, grid, Lg, Le=None, sn=0, sp=0, latlon=False):
        Le = Lg if Le is None else Le
        grid = np.ascontiguousarray(grid, dtype=np.float64)
        out = np.zeros((tri_size(Le), 2))
        self._st_fwd(sn, sp, int(latlon), Lg, Le, grid, out)
        return out

    def st_backward(self, coeffs, Le, Lg=None, sn=0, sp=0, latlon=False):
        Lg = Le if Lg is None else Lg
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.zeros(st_grid_shape(Lg, latlon))
        self._st_bwd(sn, sp, int(latlon), Le, Lg, coeffs, out)
        return out

    def zt_rotate(self, coeffs, L, euler, rtype=0, zn=1, sn=0, sp=0):
        c = np.array(coeffs, dtype=np.float64, copy=True, order="C")
        e = np.ascontiguousarray(euler, dtype=np.float64)
        self._zt_rot(zn, sn, sp, L, c, e, rtype)
        return c

    def st_rotate(self, coeffs, L, euler, rtype=0, sn=0, sp=0):
        c = np.array(coeffs, dtype=np.float64, copy=True, order="C")
        e = np.ascontiguousarray(euler, dtype=np.float64)
        self._st_rot(sn, sp, L, c, e, rtype)
        return c

    def zt_polar_rotate(self, coeffs, L, angle, rtype=0, zn=1, sn=0, sp=0):
        c = np.array(coeffs, dtype=np.float64, copy=True, order="C")
        self._zt_polar(zn, sn, sp, L, c, angle, rtype)
        return c

    def st_polar_rotate(self, coeffs, L, angle, rtype=0, sn=0, sp=0):
        c = np.array(coeffs, dtype=np.float64, copy=True, order="C")
        self._st_polar(sn, sp, L, c, angle, rtype)
        return c

    # -- evaluation at arbitrary points, power spectra --
    def zt_evaluate(self, coeffs, L, lon, colat, rad, zn=1, sn=0, sp=0):
        lon = np.ascontiguousarray(lon, dtype=np.float64)
        colat = np.ascontiguousarray(colat, dtype=np.float64)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.zeros((lon.size, colat.size, rad.size))
        self._zt_eval(zn, sn, sp, L, c, lon, colat, rad, out)
        return out

    def st_evaluate(self, coeffs, L, lon, colat, sn=0, sp=0):
        lon = np.ascontiguousarray(lon, dtype=np.float64)
        colat = np.ascontiguousarray(colat, dtype=np.float64)
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.zeros((lon.size, colat.size))
        self._st_eval(sn, sp, L, c, lon, colat, out)
        return out

    def zt_power_spectrum(self, coeffs, L, sn=0, out=None):
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.zeros(rad_size(L)) if out is None else np.array(out, dtype=np.float64, copy=True)
        self._zt_ps(sn, L, c, out)
        return out


class Oracle(_Lib):
    """The C restatement (oracle/zest_oracle.c)."""
    prefix = "oracle_"

    def __init__(self):
        super().__init__(build_oracle())

    def _gl(self, n, packed, x, w):
        self._f("gl_nodes_weights", [_c_sz, _c_int, _p_dbl, _p_dbl], None)(n, int(packed), _ptr(x), _ptr(w))

    def _zt_fwd(self, zn, sn, sp, Lg, Le, grid, out):
        self._f("zt_forward", [_c_sz, _c_sz, _c_int, _c_int, _c_int, _p_dbl, _p_dbl], None)(Lg, Le, zn, sn, sp, _ptr(grid), _ptr(out))

    def _zt_bwd(self, zn, sn, sp, Le, Lg, coeffs, out):
        self._f("zt_backward", [_c_sz, _c_sz, _c_int, _c_int, _c_int, _p_dbl, _p_dbl], None)(Le, Lg, zn, sn, sp, _ptr(coeffs), _ptr(out))

    def _st_fwd(self, sn, sp, latlon, Lg, Le, grid, out):
        self._f("st_forward", [_c_sz, _c_sz, _c_int, _c_int, _c_int, _p_dbl, _p_dbl], None)(Lg, Le, sn, sp, latlon, _ptr(grid), _ptr(out))

    def _st_bwd(self, sn, sp, latlon, Le, Lg, coeffs, out):
        self._f("st_backward", [_c_sz, _c_sz, _c_int, _c_int, _c_int, _p_dbl, _p_dbl], None)(Le, Lg, sn, sp, latlon, _ptr(coeffs), _ptr(out))

    def plm_real(self, L, sh_norm, sh_phase, z):
        z = np.ascontiguousarray(z, dtype=np.float64)
        out = np.zeros((tri_size(L), z.size))
        self._f("plm_real", [_c_sz, _c_int, _c_int, _c_sz, _p_dbl, _p_dbl], None)(L, sh_norm, sh_phase, z.size, _ptr(z), _ptr(out))
        return out

    def radial_zernike(self, L, znorm, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        out = np.zeros((rad_size(L), r.size))
        self._f("radial_zernike", [_c_sz, _c_int, _c_sz, _p_dbl, _p_dbl], None)(L, znorm, r.size, _ptr(r), _ptr(out))
        return out

    def wignerd(self, L):
        out = np.zeros(wignerd_size(L))
        self._f("wignerd", [_c_sz, _p_dbl], None)(L, _ptr(out))
        return out

    def _zt_rot(self, zn, sn, sp, L, c, e, rtype):
        # the rotation acts on the complex form; conventions only enter through
        # same-convention conversions, which are independent of (zn, sn, sp)
        self._f("zt_rotate", [_c_sz, _p_dbl, _p_dbl, _c_int], None)(L, _ptr(c), _ptr(e), rtype)

    def _st_rot(self, sn, sp, L, c, e, rtype):
        self._f("st_rotate", [_c_sz, _p_dbl, _p_dbl, _c_int], None)(L, _ptr(c), _ptr(e), rtype)

    def _zt_polar(self, zn, sn, sp, L, c, angle, rtype):
        self._f("zt_polar_rotate", [_c_sz, _p_dbl, _c_dbl, _c_int], None)(L, _ptr(c), angle, rtype)

    def _st_polar(self, sn, sp, L, c, angle, rtype):
        self._f("st_polar_rotate", [_c_sz, _p_dbl, _c_dbl, _c_int], None)(L, _ptr(c), angle, rtype)

    def _zt_eval(self, zn, sn, sp, L, c, lon, colat, rad, out):
        self._f("zt_evaluate", [_c_sz, _c_int, _c_int, _c_int, _p_dbl, _c_sz, _p_dbl, _c_sz, _p_dbl, _c_sz, _p_dbl,
                                _p_dbl], None)(L, zn, sn, sp, _ptr(c), lon.size, _ptr(lon), colat.size, _ptr(colat),
                                               rad.size, _ptr(rad), _ptr(out))

    def _st_eval(self, sn, sp, L, c, lon, colat, out):
        self._f("st_evaluate", [_c_sz, _c_int, _c_int, _p_dbl, _c_sz, _p_dbl, _c_sz, _p_dbl, _p_dbl], None)(
            L, sn, sp, _ptr(c), lon.size, _ptr(lon), colat.size, _ptr(colat), _ptr(out))

    def _zt_ps(self, sn, L, c, out):
        self._f("zt_power_spectrum", [_c_sz, _c_int, _p_dbl, _p_dbl], None)(L, sn, _ptr(c), _ptr(out))

    def st_power_spectrum(self, coeffs, L, sn=0):
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.zeros(L)
        self._f("st_power_spectrum", [_c_sz, _c_int, _p_dbl, _p_dbl], None)(L, sn, _ptr(c), _ptr(out))
        return out

    def st_cross_power_spectrum(self, a, b, L, sn=0, out_len=None, out=None):
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        out_len = L if out_len is None else out_len
        out = np.zeros(out_len) if out is None else np.array(out, dtype=np.float64, copy=True)
        self._f("st_cross_power_spectrum", [_c_sz, _c_int, _p_dbl, _p_dbl, _c_sz, _p_dbl], None)(
            L, sn, _ptr(a), _ptr(b), out_len, _ptr(out))
        return out

    def euler_from_matrix(self, mat):
        m = np.ascontiguousarray(mat, dtype=np.float64).reshape(9)
        e = np.zeros(3)
        self._f("euler_from_matrix", [_p_dbl, _p_dbl], None)(_ptr(m), _ptr(e))
        return e


class Reference(_Lib):
    """The reference library compiled from its sources (oracle/_ref)."""
    prefix = "ref_"

    def __init__(self, path: str | None = None):
        if path is None:
            from oracle import build_ref
            path = build_ref.build()
            if path is None:
                raise FileNotFoundError("reference sources are not available on this machine")
        super().__init__(path)

    def _gl(self, n, packed, x, w):
        self._f("gl_nodes_weights", [_c_sz, _c_int, _c_int, _p_dbl, _p_dbl])(n, int(packed), 0, _ptr(x), _ptr(w))

    def _zt_fwd(self, zn, sn, sp, Lg, Le, grid, out):
        self._f("zt_forward", [_c_int, _c_int, _c_int, _c_sz, _c_sz, _p_dbl, _p_dbl])(zn, sn, sp, Lg, Le, _ptr(grid), _ptr(out))

    def _zt_bwd(self, zn, sn, sp, Le, Lg, coeffs, out):
        self._f("zt_backward", [_c_int, _c_int, _c_int, _c_sz, _c_sz, _p_dbl, _p_dbl])(zn, sn, sp, Le, Lg, _ptr(coeffs), _ptr(out))

    def _st_fwd(self, sn, sp, latlon, Lg, Le, grid, out):
        self._f("st_forward", [_c_int, _c_int, _c_int, _c_sz, _c_sz, _p_dbl, _p_dbl])(sn, sp, latlon, Lg, Le, _ptr(grid), _ptr(out))

    def _st_bwd(self, sn, sp, latlon, Le, Lg, coeffs, out):
        self._f("st_backward", [_c_int, _c_int, _c_int, _c_sz, _c_sz, _p_dbl, _p_dbl])(sn, sp, latlon, Le, Lg, _ptr(coeffs), _ptr(out))

    def _zt_rot(self, zn, sn, sp, L, c, e, rtype):
        self._f("zt_rotate", [_c_int, _c_int, _c_int, _c_sz, _p_dbl, _p_dbl, _c_int])(zn, sn, sp, L, _ptr(c), _ptr(e), rtype)

    def _st_rot(self, sn, sp, L, c, e, rtype):
        self._f("st_rotate", [_c_int, _c_int, _c_sz, _p_dbl, _p_dbl, _c_int])(sn, sp, L, _ptr(c), _ptr(e), rtype)

    def _zt_polar(self, zn, sn, sp, L, c, angle, rtype):
        self._f("zt_polar_rotate", [_c_int, _c_int, _c_int, _c_sz, _p_dbl, _c_dbl, _c_int])(zn, sn, sp, L, _ptr(c), angle, rtype)

    def _st_polar(self, sn, sp, L, c, angle, rtype):
        self._f("st_polar_rotate", [_c_int, _c_int, _c_sz, _p_dbl, _c_dbl, _c_int])(sn, sp, L, _ptr(c), angle, rtype)

    def rows_rotate(self, coeffs, L, euler, rtype=0, sn=0, sp=0):
        c = np.array(coeffs, dtype=np.float64, copy=True, order="C")
        e = np.ascontiguousarray(euler, dtype=np.float64)
        self._f("rows_rotate", [_c_int, _c_int, _c_sz, _p_dbl, _p_dbl, _c_int])(sn, sp, L, _ptr(c), _ptr(e), rtype)
        return c

    def st_backward_rows(self, coeffs, Le, Lg=None, sn=0, sp=0, latlon=False):
        Lg = Le if Lg is None else Lg
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.zeros(st_grid_shape(Lg, latlon))
        self._f("st_backward_rows", [_c_int, _c_int, _c_int, _c_sz, _c_sz, _p_dbl, _p_dbl])(
            sn, sp, int(latlon), Le, Lg, _ptr(c), _ptr(out))
        return out

    def convert(self, coeffs, kind, L, src, dst, to_complex):
        c = np.array(coeffs, dtype=np.float64, copy=True, order="C")
        self._f("convert", [_c_int, _c_sz, _p_dbl] + [_c_int] * 7)(kind, L, _ptr(c), *src, *dst, int(to_complex))
        return c

    def zt_grid_points(self, L: int):
        lon = np.zeros(zt_grid_shape(L)[0])
        colat = np.zeros(zt_grid_shape(L)[1])
        r = np.zeros(zt_grid_shape(L)[2])
        self._f("zt_grid_points", [_c_sz, _p_dbl, _p_dbl, _p_dbl])(L, _ptr(lon), _ptr(colat), _ptr(r))
        return lon, colat, r

    def st_grid_points(self, L: int, latlon: int = 0):
        nlon, nlat = st_grid_shape(L, bool(latlon))
        if latlon:
            nlon, nlat = nlat, nlon
        lon = np.zeros(nlon)
        colat = np.zeros(nlat)
        self._f("st_grid_points", [_c_sz, _c_int, _p_dbl, _p_dbl])(L, int(latlon), _ptr(lon), _ptr(colat))
        return lon, colat

    def zt_rotate_matrix(self, coeffs, L, mat, rtype=0, zn=1, sn=0, sp=0):
        c = np.array(coeffs, dtype=np.float64, copy=True, order="C")
        m = np.ascontiguousarray(mat, dtype=np.float64).reshape(9)
        self._f("zt_rotate_matrix", [_c_int, _c_int, _c_int, _c_sz, _p_dbl, _p_dbl, _c_int])(zn, sn, sp, L, _ptr(c), _ptr(m), rtype)
        return c

    def _zt_eval(self, zn, sn, sp, L, c, lon, colat, rad, out):
        self._f("zt_evaluate", [_c_int, _c_int, _c_int, _c_sz, _p_dbl, _c_sz, _p_dbl, _c_sz, _p_dbl, _c_sz, _p_dbl, _p_dbl])(
            zn, sn, sp, L, _ptr(c), lon.size, _ptr(lon), colat.size, _ptr(colat), rad.size, _ptr(rad), _ptr(out))

    def _st_eval(self, sn, sp, L, c, lon, colat, out):
        self._f("st_evaluate", [_c_int, _c_int, _c_sz, _p_dbl, _c_sz, _p_dbl, _c_sz, _p_dbl, _p_dbl])(
            sn, sp, L, _ptr(c), lon.size, _ptr(lon), colat.size, _ptr(colat), _ptr(out))

    def _zt_ps(self, sn, L, c, out):
        self._f("zt_power_spectrum", [_c_int, _c_sz, _p_dbl, _p_dbl])(sn, L, _ptr(c), _ptr(out))

    def zt_fwd_bwd_steps(self, grids, L, nthreads, nsteps=1, zn=1, sn=0, sp=0):
        """`nsteps` timed steps of forward + backward of every grid on
        `nthreads` threads; each thread builds its transformer once, before
        the timing.  Returns (seconds per step, coefficients, grids)."""
        grids = np.ascontiguousarray(grids, dtype=np.float64)
        batch = grids.shape[0]
        coeffs = np.zeros((batch, zt_coeff_size(L), 2))
        out = np.zeros_like(grids)
        secs = np.zeros(nsteps)
        fn = self._f("zt_fwd_bwd_steps", [_c_int, _c_int, _c_int, _c_sz, _c_sz, _p_dbl, _p_dbl, _p_dbl, _c_int,
                                          _c_int, _p_dbl])
        fn(zn, sn, sp, L, batch, _ptr(grids), _ptr(coeffs), _ptr(out), nthreads, nsteps, _ptr(secs))
        return secs, coeffs, out

    def st_bwd_fwd_steps(self, coeffs, L, nthreads, nsteps=1, sn=0, sp=0):
        """`nsteps` timed steps of backward + forward of every SH expansion
        (LonLat grids) on `nthreads` threads; each thread builds its
        transformer once, before the timing.  Returns (seconds per step,
        grids, coefficients)."""
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        batch = coeffs.shape[0]
        grids = np.zeros((batch,) + tuple(st_grid_shape(L)))
        out = np.zeros_like(coeffs)
        secs = np.zeros(nsteps)
        fn = self._f("st_bwd_fwd_steps", [_c_int, _c_int, _c_sz, _c_sz, _p_dbl, _p_dbl, _p_dbl, _c_int, _c_int,
                                          _p_dbl])
        fn(sn, sp, L, batch, _ptr(coeffs), _ptr(grids), _ptr(out), nthreads, nsteps, _ptr(secs))
        return secs, grids, out

    def zt_rotate_backward_ragged(self, orders, coeffs, euler, nthreads, rtype=0, zn=1, sn=0, sp=0,
                                  want_grids=False):
        """Rotor::rotate then backward_transform of items of sorted, uneven
        orders on `nthreads` threads (set-up untimed).  `coeffs` (the items'
        coefficients back to back) is rotated in place.  Returns (seconds,
        grids back to back or None)."""
        orders = np.ascontiguousarray(orders, dtype=np.int32)
        e = np.ascontiguousarray(euler, dtype=np.float64).ravel()
        assert coeffs.dtype == np.float64 and coeffs.flags["C_CONTIGUOUS"]
        grids = None
        if want_grids:
            grids = np.zeros(sum(int(np.prod(zt_grid_shape(int(L)))) for L in orders))
        fn = self._f("zt_rotate_backward_ragged", [_c_int, _c_int, _c_int, _c_sz, ctypes.POINTER(_c_int), _p_dbl,
                                                   _p_dbl, _c_int, _p_dbl, _c_int], _c_dbl)
        secs = fn(zn, sn, sp, orders.size, orders.ctypes.data_as(ctypes.POINTER(_c_int)), _ptr(coeffs), _ptr(e),
                  rtype, _ptr(grids) if grids is not None else None, nthreads)
        return secs, grids


def zt_sample_config1(lon: np.ndarray, colat: np.ndarray, r: np.ndarray) -> np.ndarray:
    """f(lon, colat, r) = r * exp(-x^2), x = sin(colat) cos(lon) -- the sampled
    function of examples/zernike_example.cpp:30 with the argument order of
    BallGLQGridPoints::generate_values (include/zernike_glq_transformer.hpp:406)."""
    x = np.sin(colat)[None, :, None] * np.cos(lon)[:, None, None]
    return r[None, None, :] * np.exp(-x * x)

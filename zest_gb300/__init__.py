"""zest_gb300 -- GB300-native (sm_103a) Gauss-Legendre-quadrature transforms
and rotations of zest (sebsassi/zest), bound through the C-ABI of
include/zest_gpu.h.

This module is a thin ctypes binding: every call goes to libzest_gb300.so,
which must be built (``python -m zest_gb300.build``).  There is no CPU
fallback: without the library, or without a GB300, calls raise.

Arrays: numpy arrays are host memory (staged by the library); torch CUDA
tensors are device memory (used in place, on the context's stream).  All data
is float64 in the reference's layouts (see include/zest_gpu.h).
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libzest_gb300.so")

# conventions (zest::zt::ZernikeNorm, zest::st::SHNorm, zest::st::SHPhase)
ZERNIKE_NORMED, ZERNIKE_UNNORMED = 0, 1
SH_GEO, SH_QM = 0, 1
SH_PHASE_NONE, SH_PHASE_CS = 0, 1
ROTATION_OBJECT, ROTATION_COORDINATE = 0, 1
EXPANSION_ZERNIKE, EXPANSION_SH, EXPANSION_ZERNIKE_ROW = 0, 1, 2
LAYOUT_LONLAT, LAYOUT_LATLON = 0, 1
PRECISION_FP64, PRECISION_SPLIT = 0, 1
MEM_DEVICE, MEM_HOST = 0, 1
# status codes of the C-ABI (ZEST_GPU_ERR_*)
OK, ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED = 0, 1, 2, 3, 4, 5

# the reference's transformer aliases (zernike_glq_transformer.hpp:967-1025)
ZT_ACOUSTICS = (ZERNIKE_UNNORMED, SH_QM, SH_PHASE_NONE)
ZT_NORMAL_ACOUSTICS = (ZERNIKE_NORMED, SH_QM, SH_PHASE_NONE)
ZT_QM = (ZERNIKE_UNNORMED, SH_QM, SH_PHASE_CS)
ZT_NORMAL_QM = (ZERNIKE_NORMED, SH_QM, SH_PHASE_CS)
ZT_GEO = (ZERNIKE_UNNORMED, SH_GEO, SH_PHASE_NONE)
ZT_NORMAL_GEO = (ZERNIKE_NORMED, SH_GEO, SH_PHASE_NONE)
# sh_glq_transformer.hpp:1215-1240
ST_ACOUSTICS = (SH_QM, SH_PHASE_NONE)
ST_QM = (SH_QM, SH_PHASE_CS)
ST_GEO = (SH_GEO, SH_PHASE_NONE)


class ZestGPUError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"zest_gpu error {code}: {msg}")
        self.code = code


_lib = None


def library() -> ctypes.CDLL:
    """Loads libzest_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ZestGPUError(-1, f"{LIB_PATH} is missing: build it with `python -m zest_gb300.build`")
        lib = ctypes.CDLL(LIB_PATH)
        _declare(lib)
        _lib = lib
    return _lib


_sz = ctypes.c_size_t
_i = ctypes.c_int
_vp = ctypes.c_void_p

_SIGNATURES = {
    "zest_gpu_ctx_create": [ctypes.POINTER(_vp), _i, _vp],
    "zest_gpu_ctx_destroy": [_vp],
    "zest_gpu_set_precision": [_vp, _i, _i],
    "zest_gpu_synchronize": [_vp],
    "zest_gpu_trim": [_vp],
    "zest_gpu_zt_forward": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_zt_backward": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_st_forward": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_st_backward": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_zt_rotate": [_vp, _sz, _sz, _vp, _vp, _i, _i],
    "zest_gpu_st_rotate": [_vp, _sz, _sz, _vp, _vp, _i, _i],
    "zest_gpu_zt_polar_rotate": [_vp, _sz, _sz, _vp, _vp, _i, _i],
    "zest_gpu_st_polar_rotate": [_vp, _sz, _sz, _vp, _vp, _i, _i],
    "zest_gpu_euler_from_matrix": [_vp, _vp],
    "zest_gpu_gl_nodes_weights": [_sz, _i, _vp, _vp],
    "zest_gpu_plm_table": [_vp, _sz, _i, _i, _sz, _vp, _vp, _i],
    "zest_gpu_radial_table": [_vp, _sz, _i, _sz, _vp, _vp, _i],
    "zest_gpu_wignerd_table": [_vp, _sz, _vp, _i],
    "zest_gpu_profile_enable": [_vp, _i],
    "zest_gpu_profile_read": [_vp, _i, _vp, _vp, _i],
    "zest_gpu_profile_stage_count": [],
    "zest_gpu_split_gemm": [_vp, _sz, _sz, _sz, _vp, _vp, _vp, _i],
    "zest_gpu_profile_flops": [_vp, _i, _vp, _vp],
    "zest_gpu_zt_rotate_noalloc": [_vp, _sz, _sz, _vp, _vp, _i, _vp, _sz],
    "zest_gpu_zt_forward_vjp": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_zt_backward_vjp": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_st_forward_vjp": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_st_backward_vjp": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_zt_rotate_vjp": [_vp, _sz, _sz, _vp, _vp, _i, _vp, _vp, _vp, _i],
    "zest_gpu_st_rotate_vjp": [_vp, _sz, _sz, _vp, _vp, _i, _vp, _vp, _vp, _i],
    "zest_gpu_zt_rotate_backward_ragged": [_vp, _i, _i, _i, _sz, _vp, _vp, _vp, _i, _vp],
    "zest_gpu_set_autotune": [_vp, _i],
    "zest_gpu_set_host_chunk_bytes": [_vp, _sz],
    "zest_gpu_host_register": [_vp, _sz],
    "zest_gpu_host_unregister": [_vp],
    "zest_gpu_selftest_wait_timeout": [_vp, ctypes.c_double],
    "zest_gpu_zt_grid_points": [_sz, _vp, _vp, _vp],
    "zest_gpu_st_grid_points": [_sz, _i, _vp, _vp],
    "zest_gpu_zt_evaluate": [_vp, _i, _i, _i, _sz, _sz, _vp, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _i],
    "zest_gpu_st_evaluate": [_vp, _i, _i, _sz, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _i],
    "zest_gpu_st_lsq": [_vp, _i, _i, _sz, _sz, _sz, _vp, _vp, _vp, _vp, _i],
    "zest_gpu_zt_lsq": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _vp, _vp, _vp, _i],
    "zest_gpu_st_power_spectrum": [_vp, _i, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_st_cross_power_spectrum": [_vp, _i, _sz, _sz, _vp, _vp, _sz, _vp, _i],
    "zest_gpu_zt_power_spectrum": [_vp, _i, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_rows_rotate": [_vp, _sz, _sz, _vp, _vp, _i, _i],
    "zest_gpu_st_backward_rows": [_vp, _i, _i, _i, _sz, _sz, _sz, _vp, _vp, _i],
    "zest_gpu_convert_expansion": [_vp, _i, _sz, _sz, _vp, _i, _i, _i, _i, _i, _i, _i, _i],
    "zest_gpu_plm_complex_table": [_vp, _sz, _i, _i, _sz, _vp, _vp, _i],
}
_SIZE_FUNCS = {
    "zest_gpu_zt_grid_size": [_sz],
    "zest_gpu_zt_coeff_size": [_sz],
    "zest_gpu_st_grid_size": [_sz, _i],
    "zest_gpu_st_coeff_size": [_sz],
}


def _declare(lib):
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _i
    for name, args in _SIZE_FUNCS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _sz
    lib.zest_gpu_last_error.argtypes = []
    lib.zest_gpu_last_error.restype = ctypes.c_char_p
    lib.zest_gpu_profile_stage_name.argtypes = [_i]
    lib.zest_gpu_profile_stage_name.restype = ctypes.c_char_p
    lib.zest_gpu_launch_count.argtypes = []
    lib.zest_gpu_launch_count.restype = ctypes.c_ulonglong


def exported_symbols() -> list[str]:
    return sorted(list(_SIGNATURES) + list(_SIZE_FUNCS)
                  + ["zest_gpu_last_error", "zest_gpu_profile_stage_name", "zest_gpu_launch_count"])


def host_register(array: np.ndarray) -> None:
    """Pins a C-contiguous numpy array's memory (cudaHostRegister) so that
    host-buffer transforms of it copy asynchronously; host_unregister undoes
    it and must come before the array is freed."""
    if not array.flags["C_CONTIGUOUS"]:
        raise ValueError("host_register needs a C-contiguous array")
    _check(library().zest_gpu_host_register(_vp(array.ctypes.data), int(array.nbytes)))


def host_unregister(array: np.ndarray) -> None:
    _check(library().zest_gpu_host_unregister(_vp(array.ctypes.data)))


def launch_count() -> int:
    """Kernels launched by the library so far in this process."""
    return int(library().zest_gpu_launch_count())


def _check(code: int):
    if code != 0:
        msg = library().zest_gpu_last_error().decode(errors="replace")
        raise ZestGPUError(code, msg)


# ---- shapes ----
def pad8(n: int) -> int:
    return (n + 7) & ~7


def zt_grid_shape(order: int):
    return (2 * order - 1 if order else 0, order + 1, pad8(order + 1))


def zt_coeff_size(order: int) -> int:
    return (order + 1) * (order + 3) * (2 * order + 1) // 24


def st_grid_shape(order: int, layout: int = LAYOUT_LONLAT):
    if layout == LAYOUT_LATLON:
        return (order, pad8(2 * order - 1 if order else 0))
    return (2 * order - 1 if order else 0, pad8(order))


def rows_coeff_size(order: int) -> int:
    """Pairs of a row-skipping SH expansion of `order` (zt::ZernikeSHSpan)."""
    return ((order + 1) * (order + 1)) // 4


def st_coeff_size(order: int) -> int:
    return order * (order + 1) // 2


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(x, want_size: int):
    """(pointer, mem kind) of a float64 numpy array (host) or torch CUDA tensor."""
    if _is_torch(x):
        import torch
        if x.dtype != torch.float64 or not x.is_contiguous():
            raise ValueError("torch tensors must be contiguous float64")
        if x.numel() != want_size:
            raise ValueError(f"expected {want_size} elements, got {x.numel()}")
        return ctypes.c_void_p(x.data_ptr()), (MEM_DEVICE if x.is_cuda else MEM_HOST)
    if not isinstance(x, np.ndarray) or x.dtype != np.float64 or not x.flags["C_CONTIGUOUS"]:
        raise ValueError("numpy arrays must be C-contiguous float64")
    if x.size != want_size:
        raise ValueError(f"expected {want_size} elements, got {x.size}")
    return ctypes.c_void_p(x.ctypes.data), MEM_HOST


class Context:
    """A device + stream with cached tables and scratch (zest_gpu_context)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        lib = library()
        h = _vp()
        _check(lib.zest_gpu_ctx_create(ctypes.byref(h), device, _vp(stream or 0)))
        self._h = h
        self.lib = lib

    def close(self):
        if getattr(self, "_h", None):
            self.lib.zest_gpu_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_precision(self, precision: int, slices: int = 0):
        _check(self.lib.zest_gpu_set_precision(self._h, precision, slices))

    def synchronize(self):
        _check(self.lib.zest_gpu_synchronize(self._h))

    def trim(self):
        _check(self.lib.zest_gpu_trim(self._h))

    def profile(self, enable: bool = True):
        _check(self.lib.zest_gpu_profile_enable(self._h, int(enable)))

    def profile_flops(self, reset: bool = True):
        """(useful, issued) BF16 tensor flops of the split products since the last reset."""
        u = ctypes.c_double(0.0)
        i = ctypes.c_double(0.0)
        _check(self.lib.zest_gpu_profile_flops(self._h, int(reset), ctypes.byref(u), ctypes.byref(i)))
        return u.value, i.value

    def profile_read(self, reset: bool = True) -> dict:
        """{stage: (milliseconds, count)} accumulated since the last reset."""
        n = int(self.lib.zest_gpu_profile_stage_count())
        ms = np.zeros(n)
        cnt = np.zeros(n, dtype=np.int64)
        _check(self.lib.zest_gpu_profile_read(self._h, int(reset), _vp(ms.ctypes.data), _vp(cnt.ctypes.data), n))
        out = {}
        for i in range(n):
            if cnt[i]:
                out[self.lib.zest_gpu_profile_stage_name(i).decode()] = (float(ms[i]), int(cnt[i]))
        return out

    # ---- Zernike ----
    def zt_forward(self, grids, grid_order: int, exp_order: Optional[int] = None, batch: int = 1,
                   conv=ZT_GEO, out=None):
        exp_order = grid_order if exp_order is None else exp_order
        gsz = int(np.prod(zt_grid_shape(grid_order))) * batch
        csz = 2 * zt_coeff_size(exp_order) * batch
        gp, gm = _ptr(grids, gsz)
        if out is None:
            out = self._alloc_like(grids, csz)
        cp, cm = _ptr(out, csz)
        if gm != cm:
            raise ValueError("input and output must both be host or both be device memory")
        _check(self.lib.zest_gpu_zt_forward(self._h, *conv, grid_order, exp_order, batch, gp, cp, gm))
        return out

    def zt_backward(self, coeffs, exp_order: int, grid_order: Optional[int] = None, batch: int = 1,
                    conv=ZT_GEO, out=None):
        grid_order = exp_order if grid_order is None else grid_order
        gsz = int(np.prod(zt_grid_shape(grid_order))) * batch
        csz = 2 * zt_coeff_size(exp_order) * batch
        cp, cm = _ptr(coeffs, csz)
        if out is None:
            out = self._alloc_like(coeffs, gsz)
        gp, gm = _ptr(out, gsz)
        if gm != cm:
            raise ValueError("input and output must both be host or both be device memory")
        _check(self.lib.zest_gpu_zt_backward(self._h, *conv, exp_order, grid_order, batch, cp, gp, cm))
        return out

    # ---- SH ----
    def st_forward(self, grids, grid_order: int, exp_order: Optional[int] = None, batch: int = 1,
                   conv=ST_GEO, layout: int = LAYOUT_LONLAT, out=None):
        exp_order = grid_order if exp_order is None else exp_order
        gsz = int(np.prod(st_grid_shape(grid_order, layout))) * batch
        csz = 2 * st_coeff_size(exp_order) * batch
        gp, gm = _ptr(grids, gsz)
        if out is None:
            out = self._alloc_like(grids, csz)
        cp, cm = _ptr(out, csz)
        _check(self.lib.zest_gpu_st_forward(self._h, *conv, layout, grid_order, exp_order, batch, gp, cp, gm))
        return out

    def st_backward(self, coeffs, exp_order: int, grid_order: Optional[int] = None, batch: int = 1,
                    conv=ST_GEO, layout: int = LAYOUT_LONLAT, out=None):
        grid_order = exp_order if grid_order is None else grid_order
        gsz = int(np.prod(st_grid_shape(grid_order, layout))) * batch
        csz = 2 * st_coeff_size(exp_order) * batch
        cp, cm = _ptr(coeffs, csz)
        if out is None:
            out = self._alloc_like(coeffs, gsz)
        gp, gm = _ptr(out, gsz)
        _check(self.lib.zest_gpu_st_backward(self._h, *conv, layout, exp_order, grid_order, batch, cp, gp, cm))
        return out

    # ---- rotations (in place) ----
    def zt_rotate(self, coeffs, order: int, euler, batch: int = 1, rotation_type: int = ROTATION_OBJECT):
        cp, cm = _ptr(coeffs, 2 * zt_coeff_size(order) * batch)
        ep, em = _ptr(euler, 3 * batch)
        _check(self.lib.zest_gpu_zt_rotate(self._h, order, batch, cp, ep, rotation_type, cm))
        return coeffs

    def st_rotate(self, coeffs, order: int, euler, batch: int = 1, rotation_type: int = ROTATION_OBJECT):
        cp, cm = _ptr(coeffs, 2 * st_coeff_size(order) * batch)
        ep, em = _ptr(euler, 3 * batch)
        _check(self.lib.zest_gpu_st_rotate(self._h, order, batch, cp, ep, rotation_type, cm))
        return coeffs

    def zt_polar_rotate(self, coeffs, order: int, angles, batch: int = 1, rotation_type: int = ROTATION_OBJECT):
        cp, cm = _ptr(coeffs, 2 * zt_coeff_size(order) * batch)
        ap, am = _ptr(angles, batch)
        _check(self.lib.zest_gpu_zt_polar_rotate(self._h, order, batch, cp, ap, rotation_type, cm))
        return coeffs

    def st_polar_rotate(self, coeffs, order: int, angles, batch: int = 1, rotation_type: int = ROTATION_OBJECT):
        cp, cm = _ptr(coeffs, 2 * st_coeff_size(order) * batch)
        ap, am = _ptr(angles, batch)
        _check(self.lib.zest_gpu_st_polar_rotate(self._h, order, batch, cp, ap, rotation_type, cm))
        return coeffs

    def rows_rotate(self, coeffs, order: int, euler, batch: int = 1, rotation_type: int = ROTATION_OBJECT):
        """Rotor::rotate of row-skipping (single-parity) SH expansions of
        `order`: the coefficients of radial index n = order - 1 of a Zernike
        expansion (zt::ZernikeSHSpan)."""
        cp, cm = _ptr(coeffs, 2 * rows_coeff_size(order) * batch)
        ep, em = _ptr(euler, 3 * batch)
        _check(self.lib.zest_gpu_rows_rotate(self._h, order, batch, cp, ep, rotation_type, cm))
        return coeffs

    def st_backward_rows(self, coeffs, exp_order: int, grid_order: Optional[int] = None, batch: int = 1,
                         conv=ST_GEO, layout: int = LAYOUT_LONLAT, out=None):
        """SH backward transform of row-skipping (single-parity) expansions."""
        grid_order = exp_order if grid_order is None else grid_order
        gsz = int(np.prod(st_grid_shape(grid_order, layout))) * batch
        cp, cm = _ptr(coeffs, 2 * rows_coeff_size(exp_order) * batch)
        if out is None:
            out = self._alloc_like(coeffs, gsz)
        gp, gm = _ptr(out, gsz)
        _check(self.lib.zest_gpu_st_backward_rows(self._h, *conv, layout, exp_order, grid_order, batch, cp, gp, cm))
        return out

    def convert_expansion(self, coeffs, kind: int, order: int, src, dst, to_complex: bool, batch: int = 1):
        """to_complex_expansion / to_real_expansion in place: `src` and `dst`
        are (zernike_norm, sh_norm, sh_phase) triples."""
        n = {EXPANSION_ZERNIKE: zt_coeff_size, EXPANSION_SH: st_coeff_size,
             EXPANSION_ZERNIKE_ROW: rows_coeff_size}[kind](order)
        cp, cm = _ptr(coeffs, 2 * n * batch)
        _check(self.lib.zest_gpu_convert_expansion(self._h, kind, order, batch, cp, *src, *dst, int(to_complex), cm))
        return coeffs

    def set_autotune(self, enable: bool = True):
        _check(self.lib.zest_gpu_set_autotune(self._h, int(enable)))

    def set_host_chunk_bytes(self, nbytes: int):
        """Chunk size of the copy/compute pipeline of host-memory Zernike
        transforms (default 256 MiB; 0 turns it off)."""
        _check(self.lib.zest_gpu_set_host_chunk_bytes(self._h, int(nbytes)))

    def zt_rotate_backward_ragged(self, orders, coeffs, euler, grids, conv=ZT_GEO,
                                  rotation_type: int = ROTATION_OBJECT):
        """Rotate each expansion (in place) and backward-transform it to its own
        grid; orders non-decreasing, coeffs/euler/grids torch CUDA float64
        tensors packed in item order."""
        if not (_is_torch(coeffs) and _is_torch(euler) and _is_torch(grids)) or not coeffs.is_cuda:
            raise ValueError("coeffs, euler and grids must be CUDA tensors")
        o = np.ascontiguousarray(orders, dtype=np.int32)
        csz = int(sum(2 * zt_coeff_size(int(L)) for L in o))
        gsz = int(sum(int(np.prod(zt_grid_shape(int(L)))) for L in o))
        cp, _ = _ptr(coeffs, csz)
        ep, _ = _ptr(euler, 3 * o.size)
        gp, _ = _ptr(grids, gsz)
        _check(self.lib.zest_gpu_zt_rotate_backward_ragged(self._h, *conv, o.size, _vp(o.ctypes.data), cp, ep,
                                                           rotation_type, gp))
        return grids

    # ---- adjoints (vector-Jacobian products) ----
    def zt_forward_vjp(self, coeffs_cot, grid_order: int, exp_order: Optional[int] = None, batch: int = 1,
                       conv=ZT_GEO, out=None):
        """Grid cotangent of zt_forward(grids, grid_order, exp_order)."""
        exp_order = grid_order if exp_order is None else exp_order
        gsz = int(np.prod(zt_grid_shape(grid_order))) * batch
        csz = 2 * zt_coeff_size(exp_order) * batch
        cp, cm = _ptr(coeffs_cot, csz)
        if out is None:
            out = self._alloc_like(coeffs_cot, gsz)
        gp, gm = _ptr(out, gsz)
        _check(self.lib.zest_gpu_zt_forward_vjp(self._h, *conv, grid_order, exp_order, batch, cp, gp, cm))
        return out

    def zt_backward_vjp(self, grids_cot, exp_order: int, grid_order: Optional[int] = None, batch: int = 1,
                        conv=ZT_GEO, out=None):
        """Coefficient cotangent of zt_backward(coeffs, exp_order, grid_order)."""
        grid_order = exp_order if grid_order is None else grid_order
        gsz = int(np.prod(zt_grid_shape(grid_order))) * batch
        csz = 2 * zt_coeff_size(exp_order) * batch
        gp, gm = _ptr(grids_cot, gsz)
        if out is None:
            out = self._alloc_like(grids_cot, csz)
        cp, cm = _ptr(out, csz)
        _check(self.lib.zest_gpu_zt_backward_vjp(self._h, *conv, exp_order, grid_order, batch, gp, cp, gm))
        return out

    def st_forward_vjp(self, coeffs_cot, grid_order: int, exp_order: Optional[int] = None, batch: int = 1,
                       conv=ST_GEO, layout: int = LAYOUT_LONLAT, out=None):
        exp_order = grid_order if exp_order is None else exp_order
        gsz = int(np.prod(st_grid_shape(grid_order, layout))) * batch
        csz = 2 * st_coeff_size(exp_order) * batch
        cp, cm = _ptr(coeffs_cot, csz)
        if out is None:
            out = self._alloc_like(coeffs_cot, gsz)
        gp, gm = _ptr(out, gsz)
        _check(self.lib.zest_gpu_st_forward_vjp(self._h, *conv, layout, grid_order, exp_order, batch, cp, gp, cm))
        return out

    def st_backward_vjp(self, grids_cot, exp_order: int, grid_order: Optional[int] = None, batch: int = 1,
                        conv=ST_GEO, layout: int = LAYOUT_LONLAT, out=None):
        grid_order = exp_order if grid_order is None else grid_order
        gsz = int(np.prod(st_grid_shape(grid_order, layout))) * batch
        csz = 2 * st_coeff_size(exp_order) * batch
        gp, gm = _ptr(grids_cot, gsz)
        if out is None:
            out = self._alloc_like(grids_cot, csz)
        cp, cm = _ptr(out, csz)
        _check(self.lib.zest_gpu_st_backward_vjp(self._h, *conv, layout, exp_order, grid_order, batch, gp, cp, gm))
        return out

    def _rotate_vjp(self, fn, csize, coeffs, order, euler, out_cot, batch, rotation_type, want_coeffs, want_euler):
        cp, cm = _ptr(coeffs, csize * batch)
        ep, em = _ptr(euler, 3 * batch)
        yp, ym = _ptr(out_cot, csize * batch)
        xb = self._alloc_like(out_cot, csize * batch) if want_coeffs else None
        eb = self._alloc_like(out_cot, 3 * batch) if want_euler else None
        xbp = _ptr(xb, csize * batch)[0] if xb is not None else _vp(0)
        ebp = _ptr(eb, 3 * batch)[0] if eb is not None else _vp(0)
        _check(fn(self._h, order, batch, cp, ep, rotation_type, yp, xbp, ebp, ym))
        return xb, eb

    def zt_rotate_vjp(self, coeffs, order: int, euler, out_cot, batch: int = 1,
                      rotation_type: int = ROTATION_OBJECT, want_coeffs: bool = True, want_euler: bool = True):
        """(coeffs cotangent, euler cotangent) of y = zt_rotate(coeffs, order, euler)."""
        return self._rotate_vjp(self.lib.zest_gpu_zt_rotate_vjp, 2 * zt_coeff_size(order), coeffs, order, euler,
                                out_cot, batch, rotation_type, want_coeffs, want_euler)

    def st_rotate_vjp(self, coeffs, order: int, euler, out_cot, batch: int = 1,
                      rotation_type: int = ROTATION_OBJECT, want_coeffs: bool = True, want_euler: bool = True):
        return self._rotate_vjp(self.lib.zest_gpu_st_rotate_vjp, 2 * st_coeff_size(order), coeffs, order, euler,
                                out_cot, batch, rotation_type, want_coeffs, want_euler)

    def split_gemm(self, A: np.ndarray, B: np.ndarray) -> np.ndarray:
        """C = A B^T through the split-precision tensor-core path (host arrays)."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        M, K = A.shape
        N, K2 = B.shape
        if K != K2:
            raise ValueError("inner dimensions differ")
        C = np.zeros((M, N))
        _check(self.lib.zest_gpu_split_gemm(self._h, M, N, K, _vp(A.ctypes.data), _vp(B.ctypes.data),
                                            _vp(C.ctypes.data), MEM_HOST))
        return C

    # ---- tables ----
    def plm_table(self, order: int, sh_norm: int, sh_phase: int, z: np.ndarray, complex_basis: bool = False
                  ) -> np.ndarray:
        z = np.ascontiguousarray(z, dtype=np.float64)
        out = np.zeros((order * (order + 1) // 2, z.size))
        fn = self.lib.zest_gpu_plm_complex_table if complex_basis else self.lib.zest_gpu_plm_table
        _check(fn(self._h, order, sh_norm, sh_phase, z.size, _vp(z.ctypes.data), _vp(out.ctypes.data), MEM_HOST))
        return out

    def radial_table(self, order: int, zernike_norm: int, r: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(r, dtype=np.float64)
        out = np.zeros((((order + 1) * (order + 1)) // 4, r.size))
        _check(self.lib.zest_gpu_radial_table(self._h, order, zernike_norm, r.size,
                                              _vp(r.ctypes.data), _vp(out.ctypes.data), MEM_HOST))
        return out

    def wignerd_table(self, order: int) -> np.ndarray:
        out = np.zeros(order * (order + 1) * (2 * order + 1) // 6)
        _check(self.lib.zest_gpu_wignerd_table(self._h, order, _vp(out.ctypes.data), MEM_HOST))
        return out

    # ---- evaluation at arbitrary points (zt/st GridEvaluator) ----
    def _points(self, x, like):
        """A point array in the memory kind of `like` (numpy for host data,
        a CUDA float64 tensor for device data)."""
        if _is_torch(like):
            import torch
            if _is_torch(x):
                return x.to(dtype=torch.float64, device=like.device).contiguous()
            return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=like.device)
        if _is_torch(x):
            return x.detach().cpu().numpy().astype(np.float64)
        return np.ascontiguousarray(x, dtype=np.float64)

    def zt_evaluate(self, coeffs, order: int, lon, colat, rad, batch: int = 1, conv=ZT_GEO, out=None):
        """Values [batch][lon][lat][rad] of Zernike expansions on the product
        grid of the given longitudes, colatitudes and radii."""
        lon, colat, rad = (self._points(v, coeffs) for v in (lon, colat, rad))
        nlon, nlat, nrad = (int(v.numel() if _is_torch(v) else v.size) for v in (lon, colat, rad))
        cp, cm = _ptr(coeffs, 2 * zt_coeff_size(order) * batch)
        n = batch * nlon * nlat * nrad
        if out is None:
            out = self._alloc_like(coeffs, n)
        vp, vm = _ptr(out, n)
        if vm != cm:
            raise ValueError("coefficients and values must both be host or both be device memory")
        lp, _ = _ptr(lon, nlon)
        tp, _ = _ptr(colat, nlat)
        rp, _ = _ptr(rad, nrad)
        _check(self.lib.zest_gpu_zt_evaluate(self._h, *conv, order, batch, cp, nlon, lp, nlat, tp, nrad, rp, vp, cm))
        return out

    def st_evaluate(self, coeffs, order: int, lon, colat, batch: int = 1, conv=ST_GEO, out=None):
        """Values [batch][lon][lat] of SH expansions on the product grid."""
        lon, colat = (self._points(v, coeffs) for v in (lon, colat))
        nlon, nlat = (int(v.numel() if _is_torch(v) else v.size) for v in (lon, colat))
        cp, cm = _ptr(coeffs, 2 * st_coeff_size(order) * batch)
        n = batch * nlon * nlat
        if out is None:
            out = self._alloc_like(coeffs, n)
        vp, vm = _ptr(out, n)
        if vm != cm:
            raise ValueError("coefficients and values must both be host or both be device memory")
        lp, _ = _ptr(lon, nlon)
        tp, _ = _ptr(colat, nlat)
        _check(self.lib.zest_gpu_st_evaluate(self._h, *conv, order, batch, cp, nlon, lp, nlat, tp, vp, cm))
        return out

    # ---- least-squares fits (LSQTransformer) ----
    def st_lsq(self, data, order: int, lat, lon, batch: int = 1, conv=ST_GEO, out=None):
        """SH expansions of order `order` fitted to `batch` data vectors at
        (latitude, longitude) points (st::LSQTransformer::transform)."""
        lat, lon = (self._points(v, data) for v in (lat, lon))
        npts = int(lat.numel() if _is_torch(lat) else lat.size)
        dp, dm = _ptr(data, npts * batch)
        n = 2 * st_coeff_size(order) * batch
        if out is None:
            out = self._alloc_like(data, n)
        cp, cm = _ptr(out, n)
        if cm != dm:
            raise ValueError("data and coefficients must both be host or both be device memory")
        la, _ = _ptr(lat, npts)
        lo, _ = _ptr(lon, npts)
        _check(self.lib.zest_gpu_st_lsq(self._h, *conv, order, npts, batch, dp, la, lo, cp, dm))
        return out

    def zt_lsq(self, data, order: int, r, lon, colat, batch: int = 1, conv=ZT_GEO, out=None):
        """Zernike expansions fitted to data at (r, longitude, colatitude)
        points (zt::LSQTransformer::transform)."""
        r, lon, colat = (self._points(v, data) for v in (r, lon, colat))
        npts = int(r.numel() if _is_torch(r) else r.size)
        dp, dm = _ptr(data, npts * batch)
        n = 2 * zt_coeff_size(order) * batch
        if out is None:
            out = self._alloc_like(data, n)
        cp, cm = _ptr(out, n)
        if cm != dm:
            raise ValueError("data and coefficients must both be host or both be device memory")
        rp, _ = _ptr(r, npts)
        lo, _ = _ptr(lon, npts)
        co, _ = _ptr(colat, npts)
        _check(self.lib.zest_gpu_zt_lsq(self._h, *conv, order, npts, batch, dp, rp, lo, co, cp, dm))
        return out

    # ---- power spectra ----
    def st_power_spectrum(self, coeffs, order: int, batch: int = 1, sh_norm: int = 0, out=None):
        cp, cm = _ptr(coeffs, 2 * st_coeff_size(order) * batch)
        if out is None:
            out = self._alloc_like(coeffs, batch * order)
        op, om = _ptr(out, batch * order)
        if om != cm:
            raise ValueError("coefficients and spectrum must both be host or both be device memory")
        _check(self.lib.zest_gpu_st_power_spectrum(self._h, sh_norm, order, batch, cp, op, cm))
        return out

    def st_cross_power_spectrum(self, a, b, order: int, batch: int = 1, sh_norm: int = 0, out_len=None, out=None):
        out_len = order if out_len is None else out_len
        ap, am = _ptr(a, 2 * st_coeff_size(order) * batch)
        bp, bm = _ptr(b, 2 * st_coeff_size(order) * batch)
        if out is None:
            out = self._alloc_like(a, batch * out_len)
        op, om = _ptr(out, batch * out_len)
        if not (am == bm == om):
            raise ValueError("inputs and spectrum must all be host or all be device memory")
        _check(self.lib.zest_gpu_st_cross_power_spectrum(self._h, sh_norm, order, batch, ap, bp, out_len, op, am))
        return out

    def zt_power_spectrum(self, coeffs, order: int, batch: int = 1, sh_norm: int = 0, out=None):
        n = batch * (((order + 1) * (order + 1)) >> 2)
        cp, cm = _ptr(coeffs, 2 * zt_coeff_size(order) * batch)
        if out is None:
            out = self._alloc_like(coeffs, n)
        op, om = _ptr(out, n)
        if om != cm:
            raise ValueError("coefficients and spectrum must both be host or both be device memory")
        _check(self.lib.zest_gpu_zt_power_spectrum(self._h, sh_norm, order, batch, cp, op, cm))
        return out

    @staticmethod
    def _alloc_like(x, n):
        # zero-filled like the reference's containers: a forward transform to a
        # higher expansion order leaves the orders above the grid's untouched
        if _is_torch(x):
            import torch
            return torch.zeros(n, dtype=torch.float64, device=x.device)
        return np.zeros(n, dtype=np.float64)


def zt_grid_points(order: int):
    """(lon, colat, rad) of the Zernike GLQ grid, as BallGLQGridPoints."""
    nlon, nlat, nrad = zt_grid_shape(order)
    lon, colat, rad = np.zeros(nlon), np.zeros(nlat), np.zeros(nrad)
    _check(library().zest_gpu_zt_grid_points(order, _vp(lon.ctypes.data), _vp(colat.ctypes.data),
                                             _vp(rad.ctypes.data)))
    return lon, colat, rad


def st_grid_points(order: int, layout: int = 0):
    """(lon, colat) of the SH GLQ grid of a layout, as SphereGLQGridPoints
    (counts from the layout's shape, padding included)."""
    shape = st_grid_shape(order, layout)
    nlon, nlat = (shape[1], shape[0]) if layout else shape
    lon, colat = np.zeros(nlon), np.zeros(nlat)
    _check(library().zest_gpu_st_grid_points(order, layout, _vp(lon.ctypes.data), _vp(colat.ctypes.data)))
    return lon, colat


def gl_nodes_weights(n: int, packed: bool = False):
    sz = (n + 1) // 2 if packed else n
    x = np.zeros(sz)
    w = np.zeros(sz)
    _check(library().zest_gpu_gl_nodes_weights(n, int(packed), _vp(x.ctypes.data), _vp(w.ctypes.data)))
    return x, w


def euler_from_matrix(mat) -> np.ndarray:
    m = np.ascontiguousarray(mat, dtype=np.float64).reshape(9)
    e = np.zeros(3)
    _check(library().zest_gpu_euler_from_matrix(_vp(m.ctypes.data), _vp(e.ctypes.data)))
    return e

"""CPU-only checks of the product library: it builds, loads, exports every
symbol declared in include/zest_gpu.h, validates arguments without touching a
GPU, and its host-side Gauss-Legendre solve matches the reference."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture(scope="session")
def zlib():
    from zest_gb300 import build
    build.build()
    import zest_gb300
    return zest_gb300


def declared_symbols():
    names = set()
    for fname in os.listdir(os.path.join(ROOT, "include")):
        if fname.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fname)).read()
            names |= set(re.findall(r"\b(zest_gpu_\w+)\s*\(", txt))
    return sorted(names)


def test_exports_every_declared_symbol(zlib):
    lib = zlib.library()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding declares a signature for each of them
    assert set(declared_symbols()) <= set(zlib.exported_symbols())


def test_sizes(zlib):
    lib = zlib.library()
    for L in [0, 1, 2, 20, 200]:
        assert lib.zest_gpu_zt_grid_size(L) == int(np.prod(zlib.zt_grid_shape(L)))
        assert lib.zest_gpu_zt_coeff_size(L) == zlib.zt_coeff_size(L)
        assert lib.zest_gpu_st_coeff_size(L) == L * (L + 1) // 2
        for layout in (0, 1):
            assert lib.zest_gpu_st_grid_size(L, layout) == int(np.prod(zlib.st_grid_shape(L, layout)))
    assert zlib.zt_grid_shape(200) == (399, 201, 208)
    assert zlib.st_grid_shape(1024) == (2047, 1024)


def test_host_register_rejects_null_without_gpu(zlib):
    lib = zlib.library()
    assert lib.zest_gpu_host_register(None, 0) == 1  # ZEST_GPU_ERR_INVALID, before any CUDA call
    assert lib.zest_gpu_host_unregister(None) == 1


def test_null_context_is_rejected_without_gpu(zlib):
    lib = zlib.library()
    rc = lib.zest_gpu_zt_forward(None, 1, 0, 0, 4, 4, 1, None, None, 1)
    assert rc == 1  # ZEST_GPU_ERR_INVALID
    assert b"context" in lib.zest_gpu_last_error()
    assert lib.zest_gpu_ctx_create(None, 0, None) == 1


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 21, 24, 69, 70, 71, 101, 104, 201, 208, 512, 1024])
@pytest.mark.parametrize("packed", [0, 1])
def test_gl_solver_matches_reference(zlib, golden, n, packed):
    g = golden("gl")
    x, w = zlib.gl_nodes_weights(n, bool(packed))
    assert np.max(np.abs(x - g[f"x_{n}_{packed}"])) < 1e-15
    assert np.max(np.abs(w - g[f"w_{n}_{packed}"]) / g[f"w_{n}_{packed}"]) < 2e-15


def test_euler_from_matrix(zlib, oracle, golden):
    r = golden("rotation")
    for L in [2, 5, 10, 17]:
        m = r[f"zmat_{L}"]
        np.testing.assert_array_equal(zlib.euler_from_matrix(m), oracle.euler_from_matrix(m))


def test_no_cpu_fallback_path(zlib):
    # the product package must not reference the oracle
    pkg = os.path.join(ROOT, "zest_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp", ".hpp")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in txt and "from oracle" not in txt and "zest_oracle" not in txt, f


def test_grid_points_match_reference(zlib, golden):
    # BallGLQGridPoints / SphereGLQGridPoints of the reference (points.npz):
    # longitudes bit for bit; colatitudes and radii within 2 ulp (the
    # reference's nodes come from Bogaert's asymptotic formulas, these from a
    # double-double Newton solve)
    p = golden("points")
    for L in [1, 2, 5, 20, 64, 201]:
        lon, colat, rad = zlib.zt_grid_points(L)
        np.testing.assert_array_equal(lon, p[f"zlon_{L}"])
        np.testing.assert_allclose(colat, p[f"zcolat_{L}"], rtol=0, atol=5e-16)
        np.testing.assert_allclose(rad, p[f"zrad_{L}"], rtol=0, atol=2.5e-16)
    for L in [1, 3, 8, 12, 100]:
        for layout in (0, 1):
            lon, colat = zlib.st_grid_points(L, layout)
            np.testing.assert_array_equal(lon, p[f"slon_{L}_{layout}"])
            np.testing.assert_allclose(colat, p[f"scolat_{L}_{layout}"], rtol=0, atol=5e-16)

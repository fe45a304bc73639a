"""Sampling front-ends: BallGLQGridPoints / SphereGLQGridPoints::generate_values,
ZernikeTransformer / SHTransformer (host callables, include/zest/zest_gpu.hpp)
and their device-functor counterparts DeviceZernikeTransformer /
DeviceSHTransformer (include/zest/zest_gpu_sampling.cuh), compiled with nvcc
into tests/cpp/test_sampling.cu.

Checked against the reference's transform of the sampled configuration-C1
function f = r exp(-(sin colat cos lon)^2) at order 20 (golden zt_config1:
the reference sampled and transformed it), to 1e-12 relative max-norm (the
device's exp/sin/cos and the host's differ in the last bits); the Cartesian
form on a ball of radius 2 gives twice those coefficients; a batch of
f_b = (b + 1) f scales exactly; the SH samplers agree with the SH forward
transform of the same function sampled here on the library's points."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_sampling.cu")
BUILD = os.path.join(ROOT, "tests", "cpp", "_build")

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def binary():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    from zest_gb300 import build
    build.build()
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "test_sampling")
    lib_dir = os.path.join(ROOT, "zest_gb300")
    cmd = [nvcc, "-std=c++20", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-diag-suppress", "554",
           "-I", os.path.join(ROOT, "include"), SRC, "-L", lib_dir, "-lzest_gb300", "-Xlinker", "-rpath",
           "-Xlinker", lib_dir, "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


@pytest.fixture(scope="module")
def outputs(binary, tmp_path_factory):
    d = str(tmp_path_factory.mktemp("sampling"))
    res = subprocess.run([binary, d], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr

    def load(name):
        return np.fromfile(os.path.join(d, name))

    return load


def test_device_functor_matches_reference_transform(outputs, golden):
    want = golden("zt_config1")["coeffs"]
    assert relmax(outputs("zt_device.bin"), want) < 1e-12


def test_host_callable_matches_reference_transform(outputs, golden):
    want = golden("zt_config1")["coeffs"]
    assert relmax(outputs("zt_host.bin"), want) < 1e-12


def test_cartesian_form_on_radius_two(outputs, golden):
    want = golden("zt_config1")["coeffs"]
    assert relmax(outputs("zt_cart.bin"), 2.0 * np.asarray(want)) < 1e-12


def test_batched_device_sampling(outputs):
    one = outputs("zt_device.bin")
    batch = outputs("zt_batch.bin").reshape(3, -1)
    for b in range(3):
        assert relmax(batch[b], (b + 1) * one) < 1e-14


def test_points_match_reference(outputs, golden):
    c1 = golden("zt_config1")
    p = outputs("points.bin")
    n0, n1 = c1["lon"].size, c1["colat"].size
    np.testing.assert_array_equal(p[:n0], c1["lon"])
    np.testing.assert_allclose(p[n0:n0 + n1], c1["colat"], rtol=0, atol=5e-16)
    np.testing.assert_allclose(p[n0 + n1:], c1["rad"], rtol=0, atol=2.5e-16)


@pytest.mark.parametrize("layout,name", [(0, "st_device.bin"), (0, "st_host.bin"), (1, "st_latlon.bin")])
def test_sh_samplers_match_forward_of_sampled_grid(outputs, layout, name):
    import zest_gb300 as zg
    L = 12
    lon, colat = zg.st_grid_points(L, layout)
    x = np.sin(colat)[None, :] * np.cos(lon)[:, None]   # [lon][lat]
    g = np.exp(-x * x)
    if layout:
        g = g.T
    ctx = zg.Context(0)
    try:
        want = ctx.st_forward(np.ascontiguousarray(g).ravel(), L, layout=layout)
    finally:
        ctx.close()
    assert relmax(outputs(name), want) < 1e-12

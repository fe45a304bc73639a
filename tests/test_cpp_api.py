"""The C++20 interface (include/zest/*.hpp): the reference's classes and
signatures over the C-ABI.

tests/cpp/test_cpp_api.cpp is compiled with g++ against the headers and the
library.  Its compile-time checks (type enforcement of the conventions, grid
shapes) run on every machine; on a GPU it runs transforms and rotations of the
golden fixtures through the C++ classes (GLQTransformer, Rotor,
WignerdPiHalfCollection), which must agree with the reference's outputs to
1e-12 relative max-norm, as the C-ABI does."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_cpp_api.cpp")
BUILD = os.path.join(ROOT, "tests", "cpp", "_build")
TOL = 1e-12


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def binary():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    from zest_gb300 import build
    build.build()
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "test_cpp_api")
    lib_dir = os.path.join(ROOT, "zest_gb300")
    cmd = [gxx, "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", lib_dir, "-lzest_gb300", f"-Wl,-rpath,{lib_dir}", "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_cpp_interface_compiles_and_enforces_conventions(binary):
    res = subprocess.run([binary], capture_output=True, text=True)
    assert res.returncode == 0 and "compile-time checks passed" in res.stdout


def _write(d, name, x):
    np.ascontiguousarray(x, dtype=np.float64).tofile(os.path.join(d, name))
    return name


@pytest.mark.gpu
def test_cpp_interface_matches_golden(binary, golden, tmp_path):
    d = str(tmp_path)
    jobs, checks = [], []

    def job(op, conv, order, x, want, extra=None):
        i = len(jobs)
        inp = _write(d, f"in{i}.bin", x)
        ex = _write(d, f"ex{i}.bin", extra) if extra is not None else ""
        jobs.append(f"{op} {conv} {order} {inp} out{i}.bin {ex}".strip())
        checks.append((f"out{i}.bin", np.asarray(want), f"{op} {conv} {order}"))

    c1 = golden("zt_config1")
    job("zt_fwd", "100", 20, c1["grid"], c1["coeffs"])
    job("zt_bwd", "100", 20, c1["coeffs"], c1["roundtrip"])
    z = golden("zt_random")
    for conv in ["000", "100", "010", "110", "001", "101", "011", "111"]:
        for L in (6, 11):
            job("zt_bwd", conv, L, z[f"c_{L}_{conv}"], z[f"g_{L}_{conv}"])
            job("zt_fwd", conv, L, z[f"g_{L}_{conv}"], z[f"f_{L}_{conv}"])
    s = golden("st_random")
    for layout in (0, 1):
        for conv in ["00", "10", "01", "11"]:
            L = 8
            key = f"{L}_{layout}_{conv}"
            job("st_bwd", f"{layout}{conv}", L, s[f"c_{key}"], s[f"g_{key}"])
            job("st_fwd", f"{layout}{conv}", L, s[f"g_{key}"], s[f"f_{key}"])
    r = golden("rotation")
    for L in (5, 10):
        job("zt_rot", "0", L, r[f"zc_{L}"], r[f"zobj_{L}"], r[f"ze_{L}"])
        job("zt_rot", "1", L, r[f"zc_{L}"], r[f"zcoord_{L}"], r[f"ze_{L}"])
        job("zt_polar", "0", L, r[f"zc_{L}"], r[f"zpolar_{L}"], r[f"ze_{L}"][:1])
        job("zt_rot_matrix", "0", L, r[f"zc_{L}"], r[f"zmatobj_{L}"], r[f"zmat_{L}"])
        job("st_rot", "0", L + 3, r[f"sc_{L}"], r[f"sobj_{L}"], r[f"ze_{L}"])
        job("st_rot", "1", L + 3, r[f"sc_{L}"], r[f"scoord_{L}"], r[f"ze_{L}"])
        job("st_polar", "1", L + 3, r[f"sc_{L}"], r[f"spolar_{L}"], r[f"ze_{L}"][1:2])
    # GridEvaluator and power spectra (extra file: [nlon, nlat, nrad, lon, colat, rad])
    e = golden("evaluate")
    for L in (6, 13):
        pts = np.concatenate([[e[f"lon_{L}"].size, e[f"colat_{L}"].size, e[f"rad_{L}"].size],
                              e[f"lon_{L}"], e[f"colat_{L}"], e[f"rad_{L}"]])
        for conv in ["100", "011"]:
            job("zt_eval", conv, L, e[f"zc_{L}"], e[f"zv_{L}_{conv}"], pts)
        for conv in ["00", "11"]:
            job("st_eval", conv, L + 2, e[f"sc_{L}"], e[f"sv_{L}_{conv}"], pts)
    p = golden("spectra")
    for L in (7, 16):
        for sn in (0, 1):
            job("zt_ps", str(sn), L, p[f"zc_{L}"], p[f"zp_{L}_{sn}"], np.zeros(3))
    # transpose identities and the angle gradient through the C++ adjoints
    _write(d, "unused.bin", np.zeros(1))
    jobs.append(f"vjp_checks 0 0 unused.bin out{len(jobs)}.bin")
    vjp_out = f"out{len(jobs) - 1}.bin"
    with open(os.path.join(d, "jobs.txt"), "w") as f:
        f.write("\n".join(jobs) + "\n")
    res = subprocess.run([binary, d], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    for name, want, what in checks:
        got = np.fromfile(os.path.join(d, name))
        assert got.size == want.size, what
        assert relmax(got, want) < TOL, what
    r = np.fromfile(os.path.join(d, vjp_out))
    assert np.all(r[:3] < 1e-12), r
    assert r[3] < 1e-7, r

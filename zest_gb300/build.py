"""In-tree build of libzest_gb300.so (CUDA kernels + C-ABI) for sm_103a.

    python -m zest_gb300.build          # or zest_gb300.build.build()

Every translation unit under zest_gb300/csrc is compiled by nvcc in parallel
(one -gencode, sm_103a only) and linked into zest_gb300/libzest_gb300.so with
the CUDA runtime linked statically.  Objects live in zest_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libzest_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
              "-diag-suppress", "177"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _machine_of(path: str) -> int:
    try:
        with open(path, "rb") as f:
            hdr = f.read(20)
    except OSError:
        return -1
    if hdr[:4] != b"\x7fELF":
        return -1
    return int.from_bytes(hdr[18:20], "little")


def _native(path: str) -> bool:
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine(), -2)
    return _machine_of(path) == want


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in headers()])
    if os.path.exists(obj) and _native(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + ARCH + ["-I", INCLUDE, "-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if (os.path.exists(LIB) and _native(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs)):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB + ".tmp"] + objs
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))

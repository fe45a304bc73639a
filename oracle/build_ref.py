"""Build recipe for oracle/_ref/libzest_ref.so: the reference zest library
compiled from its own sources, wrapped by oracle/ref_shim.cpp.

Test infrastructure only (golden fixtures, CPU baseline arm of bench.py).

The reference checkout is named by `--reference DIR` or the environment
variable ZEST_REFERENCE_DIR; without either, a checkout in a directory named
`reference` beside this repository's root is used if present.  Where one is
found, its
headers and the few translation units the transform/rotation path needs are
staged into oracle/_ref/src/ and compiled with g++ directly -- the reference's
own CMake build is not used.  Without one, the sources staged earlier are
compiled.  oracle/_ref/ is git-ignored (it never enters the
repository history) but it is shipped with the working tree to the GPU host;
there, where the checkout is absent and the x86 objects have been removed,
the staged sources are compiled again for the host CPU.

The compiled reference keeps its defaults: -O3, C++20, no OpenMP, single
threaded pocketfft (include/pocketfft_spec.hpp:26-28).
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(REF_OUT, "src")


def reference_checkout(path: str | None = None) -> str | None:
    """The reference checkout: `path`, else ZEST_REFERENCE_DIR, else a
    directory named `reference` beside this repository's root where one with
    the reference's include/ and src/ exists, else None."""
    given = path or os.environ.get("ZEST_REFERENCE_DIR")
    if given:
        return given
    sibling = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    if os.path.isdir(os.path.join(sibling, "include")) and os.path.isdir(os.path.join(sibling, "src")):
        return sibling
    return None


# Translation units of the reference needed by ref_shim.cpp.
REF_SOURCES = [
    "plm_recursion.cpp",
    "radial_zernike_recursion.cpp",
    "wignerd_collection.cpp",
    "rotor.cpp",
    "grid_evaluator.cpp",
]

# The reference's own test programs for the transform and rotation path.
# They are staged beside the sources (never committed) and compiled, unchanged,
# against this project's drop-in headers by tests/test_reference_tests.py.
REF_TESTS = [
    "test_zernike_glq_transformer.cpp",
    "test_sh_glq_transformer.cpp",
    "test_rotor.cpp",
    "test_plm_recursion.cpp",
    "test_radial_zernike_recursion.cpp",
    "test_gauss_legendre.cpp",
]
TEST_STAGE = os.path.join(REF_OUT, "tests")

LIB = os.path.join(REF_OUT, "libzest_ref.so")


def _stage(checkout: str | None) -> str | None:
    """Copy reference headers + needed sources into oracle/_ref/src."""
    if not checkout:
        return None
    inc = os.path.join(checkout, "include")
    src = os.path.join(checkout, "src")
    if not os.path.isdir(inc):
        return None
    os.makedirs(os.path.join(STAGE, "include"), exist_ok=True)
    for name in os.listdir(inc):
        if name.endswith(".hpp"):
            shutil.copy2(os.path.join(inc, name), os.path.join(STAGE, "include", name))
    for name in REF_SOURCES:
        shutil.copy2(os.path.join(src, name), os.path.join(STAGE, name))
    tests = os.path.join(checkout, "tests")
    os.makedirs(TEST_STAGE, exist_ok=True)
    for name in REF_TESTS:
        if os.path.exists(os.path.join(tests, name)):
            shutil.copy2(os.path.join(tests, name), os.path.join(TEST_STAGE, name))
    return STAGE


def _is_elf_for_this_machine(path: str) -> bool:
    try:
        with open(path, "rb") as f:
            hdr = f.read(20)
    except OSError:
        return False
    if hdr[:4] != b"\x7fELF":
        return False
    machine = int.from_bytes(hdr[18:20], "little")
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine(), -1)
    return machine == want


def build(force: bool = False, verbose: bool = False, reference: str | None = None) -> str | None:
    """Build libzest_ref.so; returns its path or None when no sources exist."""
    staged = _stage(reference_checkout(reference))
    if staged is None and not os.path.isdir(STAGE):
        return None
    shim = os.path.join(HERE, "ref_shim.cpp")
    deps = [shim] + [os.path.join(STAGE, s) for s in REF_SOURCES]
    if (not force and os.path.exists(LIB) and _is_elf_for_this_machine(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)):
        return LIB
    flags = ["-std=c++20", "-O3", "-fPIC", "-shared", "-pthread", "-w"]
    if platform.machine() in ("aarch64", "arm64"):
        flags.append("-mcpu=native")
    cmd = (["g++"] + flags + ["-I", os.path.join(STAGE, "include")] + deps + ["-o", LIB + ".tmp"])
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--reference", help="reference checkout to stage the sources from")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    path = build(force=a.force, verbose=True, reference=a.reference)
    print(path if path else "reference sources unavailable")

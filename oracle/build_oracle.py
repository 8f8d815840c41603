"""Build recipe for the oracle's reference binaries (TEST INFRASTRUCTURE ONLY).

Compiles the reference's own sparse sign embedding generators, src/algebra/sparse_sign.c and
src/algebra/sparsestack.c of ITensorCPD.jl, from the reference checkout where it lies, into
oracle/_ref/libsparse_sign.so, with the reference's own compile line (deps/build.jl:15-17:
gcc -O3 -fPIC -shared).  Only the tests load it, to pin the structural rules the device
generator follows.  Without the checkout (as on a GPU machine) nothing is built.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

REF_SRC = Path("/root/reference/src/algebra")
OUT_DIR = Path(__file__).resolve().parent / "_ref"
SOURCES = ("sparse_sign.c", "sparsestack.c")


def build() -> Path | None:
    srcs = [REF_SRC / f for f in SOURCES]
    if not all(p.exists() for p in srcs) or shutil.which("gcc") is None:
        return None
    OUT_DIR.mkdir(exist_ok=True)
    lib = OUT_DIR / "libsparse_sign.so"
    if lib.exists() and all(lib.stat().st_mtime >= p.stat().st_mtime for p in srcs):
        return lib
    subprocess.run(["gcc", "-O3", "-fPIC", "-shared", "-o", str(lib), *map(str, srcs), "-lm"], check=True)
    return lib


if __name__ == "__main__":
    print(build())

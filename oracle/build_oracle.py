"""Build recipe for the oracle's compiled parts (TEST INFRASTRUCTURE ONLY).

``build_cpu`` compiles cpals_cpu.cpp, the C++/OpenMP GEMM-form ALS that the bench times as a
CPU baseline, into oracle/_build/libcpals_cpu.so.

Compiles the reference's own sparse sign embedding generators, src/algebra/sparse_sign.c and
src/algebra/sparsestack.c of ITensorCPD.jl, from the reference checkout where it lies, into
oracle/_ref/libsparse_sign.so, with the reference's own compile line (deps/build.jl:15-17:
gcc -O3 -fPIC -shared).  Only the tests load it, to pin the structural rules the device
generator follows.

The checkout is the directory named by the environment variable ITENSORCPD_REFERENCE (or the
``--reference DIR`` argument), else a checkout called ``reference`` beside this repository.
Without a checkout nothing is built.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

OUT_DIR = Path(__file__).resolve().parent / "_ref"
SOURCES = ("sparse_sign.c", "sparsestack.c")


def reference_dir(explicit: str | None = None) -> Path:
    """The reference checkout: the argument, else $ITENSORCPD_REFERENCE, else ../reference."""
    if explicit:
        return Path(explicit)
    env = os.environ.get("ITENSORCPD_REFERENCE")
    if env:
        return Path(env)
    return Path(__file__).resolve().parent.parent.parent / "reference"


CPU_SRC = Path(__file__).resolve().parent / "cpals_cpu.cpp"
CPU_LIB = Path(__file__).resolve().parent / "_build" / "libcpals_cpu.so"


def build_cpu() -> Path | None:
    """The C++/OpenMP GEMM-form ALS (cpals_cpu.cpp), the compiled CPU baseline."""
    if shutil.which("g++") is None:
        return None
    if CPU_LIB.exists() and CPU_LIB.stat().st_mtime >= CPU_SRC.stat().st_mtime:
        return CPU_LIB
    CPU_LIB.parent.mkdir(exist_ok=True)
    tmp = CPU_LIB.with_suffix(".so.tmp")
    subprocess.run(["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17", "-o", str(tmp), str(CPU_SRC)],
                   check=True)
    os.replace(tmp, CPU_LIB)
    return CPU_LIB


def build(reference: str | None = None) -> Path | None:
    build_cpu()
    src_dir = reference_dir(reference) / "src" / "algebra"
    srcs = [src_dir / f for f in SOURCES]
    if not all(p.exists() for p in srcs) or shutil.which("gcc") is None:
        return None
    OUT_DIR.mkdir(exist_ok=True)
    lib = OUT_DIR / "libsparse_sign.so"
    if lib.exists() and all(lib.stat().st_mtime >= p.stat().st_mtime for p in srcs):
        return lib
    subprocess.run(["gcc", "-O3", "-fPIC", "-shared", "-o", str(lib), *map(str, srcs), "-lm"], check=True)
    return lib


if __name__ == "__main__":
    import sys

    ref = sys.argv[sys.argv.index("--reference") + 1] if "--reference" in sys.argv else None
    print(build(ref))

"""The C ABI library: builds for sm_103a, loads, and exports every declared entry point (CPU only)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(cpals_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg.load()


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    for name in syms:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_ctypes_signatures_cover_the_header(pkg):
    from itensorcpd_gb300 import _lib as L

    assert set(L.SIGNATURES) == set(declared_symbols())


def test_version_and_status_strings(lib):
    assert lib.cpals_version() >= 100
    assert b"Error NAN" in lib.cpals_status_string(-3)
    assert lib.cpals_status_string(0) == b"ok"


def test_create_rejects_bad_arguments_before_touching_a_device(lib):
    # argument validation happens before any CUDA call, so it runs without a GPU
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 3)(4, 5, 6)
    assert lib.cpals_create(ctypes.byref(h), 0, 1, dims, 3, 0, 0, 0) == -1  # order 1
    assert lib.cpals_create(ctypes.byref(h), 0, 3, dims, 0, 0, 0, 0) == -1  # rank 0
    assert lib.cpals_create(ctypes.byref(h), 0, 3, dims, 4, 7, 0, 0) == -1  # dtype
    assert lib.cpals_create(ctypes.byref(h), 0, 3, dims, 4, 0, 9, 0) == -1  # mttkrp mode
    bad = (ctypes.c_int64 * 3)(4, 0, 6)
    assert lib.cpals_create(ctypes.byref(h), 0, 3, bad, 4, 0, 0, 0) == -1  # zero extent
    assert lib.cpals_create(None, 0, 3, dims, 4, 0, 0, 0) == -1
    assert lib.cpals_destroy(None) == 0


def test_null_handle_calls_fail_cleanly(lib):
    assert lib.cpals_set_tensor(None, None) == -1
    assert lib.cpals_mttkrp(None, 0, None) == -1
    assert lib.cpals_optimize(None, None, None, 0) == -1

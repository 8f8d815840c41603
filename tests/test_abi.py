"""The C ABI library: builds for sm_103a, loads, and exports every declared entry point (CPU only)."""
import ctypes
import re
from pathlib import Path

import numpy as np
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
    assert lib.cpals_create(ctypes.byref(h), 0, 3, dims, 4, 0, 0, 4) == -1  # low-memory tiles on FP64
    assert lib.cpals_create(ctypes.byref(h), 0, 3, dims, 4, 0, 1, 4 | 2) == -1  # ... or on the dimension tree
    assert lib.cpals_destroy(None) == 0


def test_null_handle_calls_fail_cleanly(lib):
    assert lib.cpals_set_tensor(None, None) == -1
    assert lib.cpals_mttkrp(None, 0, None) == -1
    assert lib.cpals_optimize(None, None, None, 0) == -1
    assert lib.cpals_mode_update(None, 0, None) == -1
    assert lib.cpals_tensor_norm(None, None, None) == -1
    assert lib.cpals_check_converge(None, None, None, None) == -1
    assert lib.cpals_batch_set_norms(None, None) == -1
    assert lib.cpals_batch_set_sweeps_per_launch(None, 0) == -1
    assert lib.cpals_mlp_forward(None, None, 1, None) == -1


def test_create_rejects_more_than_2_40_elements_without_overflow(lib):
    # 2^21 * 2^20 * 2^21 would overflow a 64-bit product checked after multiplying
    h = ctypes.c_void_p()
    big = (ctypes.c_int64 * 3)(1 << 21, 1 << 20, 1 << 21)
    assert lib.cpals_create(ctypes.byref(h), 0, 3, big, 4, 0, 0, 0) == -1
    big4 = (ctypes.c_int64 * 4)(1 << 31, 1 << 31, 1 << 31, 1 << 31)
    assert lib.cpals_create(ctypes.byref(h), 0, 4, big4, 4, 0, 0, 0) == -1


def test_check_struct_mirrors_the_header(pkg):
    # the ctypes mirror of cpals_check has the header's fields, in order, and its size
    import re

    from itensorcpd_gb300 import _lib as L

    text = (ROOT / "include" / "cpals.h").read_text()
    body = re.search(r"typedef struct cpals_check \{(.*?)\} cpals_check;", text, re.S).group(1)
    names = re.findall(r"^\s*(?:int32_t|double)\s+(\w+);", body, re.M)
    assert names == [f[0] for f in L.CpalsCheck._fields_]
    assert ctypes.sizeof(L.CpalsCheck) == 72


def test_diff_and_angle_checks_marshal_to_the_device_struct(pkg):
    from itensorcpd_gb300 import CPAngleCheck, CPD, CPDiffCheck
    from itensorcpd_gb300 import _lib as L
    from itensorcpd_gb300.api import _to_device_check

    d = CPDiffCheck(1e-5, 40)
    c = _to_device_check(d)
    assert (c.kind, c.max_counter, c.tolerance, c.lastfit, c.has_prev) == (L.CHECK_DIFF, 40, 1e-5, 1.0, 0)
    a = CPAngleCheck(1e-4, 7, iter=2, counter=1, norm_prev_iter=3.5, lastangle=0.25,
                     PrevCP=CPD([np.ones((2, 1))], np.ones(1)))
    c = _to_device_check(a)
    assert (c.kind, c.iter, c.counter, c.norm_prev, c.lastfit, c.has_prev) == (L.CHECK_ANGLE, 2, 1, 3.5, 0.25, 1)


def test_pivot_and_sketch_entries_reject_bad_arguments_before_touching_a_device(lib):
    """Argument checks of the QRCP / SE-QRCS / sketch entries run before any CUDA call."""
    A = np.zeros(6)
    perm = np.zeros(3, dtype=np.int64)
    rd = np.zeros(3)
    k = np.zeros(1, dtype=np.int64)
    def P(a):  # a typed pointer, as the loaded signatures expect
        ct = {np.dtype(np.float64): ctypes.c_double, np.dtype(np.int64): ctypes.c_int64,
              np.dtype(np.int32): ctypes.c_int32}[a.dtype]
        return a.ctypes.data_as(ctypes.POINTER(ct))

    assert lib.cpals_qrcp(0, 0, 3, P(A), 0, 0, -1.0, P(perm), P(rd), P(k), None, None) == -1  # m = 0
    assert lib.cpals_qrcp(0, 2, 0, P(A), 0, 0, -1.0, P(perm), P(rd), P(k), None, None) == -1  # n = 0
    assert lib.cpals_qrcp(0, 2, 3, None, 0, 0, -1.0, P(perm), P(rd), P(k), None, None) == -1  # no matrix
    assert lib.cpals_qrcp(0, 2, 3, P(A), 0, 0, -1.0, None, P(rd), P(k), None, None) == -1  # no perm
    for fn in (lib.cpals_unfolding_qrcp, lib.cpals_krp_qrcp):
        assert fn(None, 0, 0, None, 0, 0, -1.0, P(perm), P(rd), P(k), None, None) == -1
    rows = np.zeros(4, dtype=np.int32)
    vals = np.zeros(4)
    ns = np.zeros(1, dtype=np.int64)
    assert lib.cpals_seqrcs(None, 0, 0, 4, 1, P(rows), P(vals), 2, 0, 0, -1.0, P(perm), P(rd), P(k), P(ns),
                            None, None) == -1
    assert lib.cpals_omega_hadamard(None, 0, 4, 1, P(rows), P(vals), P(A)) == -1
    assert lib.cpals_sketched_matricization(None, 0, 4, 1, P(rows), P(vals), P(A)) == -1
    cs = np.zeros(5, dtype=np.int32)
    assert lib.cpals_sparse_sign(0, 0, 4, 1, 0, 1, P(rows), P(vals), P(cs)) == -1  # l = 0
    assert lib.cpals_sparse_sign(0, 4, -1, 1, 0, 1, P(rows), P(vals), P(cs)) == -1  # n < 0
    assert lib.cpals_sparse_sign(0, 4, 4, 0, 0, 1, P(rows), P(vals), P(cs)) == -1  # zeta = 0
    # n = 0 is a valid empty embedding: colstarts = [0], no device work
    assert lib.cpals_sparse_sign(0, 4, 0, 2, 0, 1, P(rows), P(vals), P(cs)) == 0 and cs[0] == 0


def test_seqrcs_subset_matches_the_oracle(lib, oracle):
    """cpals_seqrcs_subset (host code, no device) selects the oracle's SE-QRCS subset in both
    orders (SEQRCS.jl:109-111, 158-159, 205-207), including repeated and empty pivot rows."""
    rng = np.random.default_rng(9)

    def P(a, ct):
        return a.ctypes.data_as(ctypes.POINTER(ct))

    for (l, n, s, t) in [(20, 50, 3, 5), (7, 40, 2, 7), (30, 10, 1, 12), (9, 1, 4, 3)]:
        rows1 = np.concatenate([rng.choice(l, size=s, replace=False) for _ in range(n)]).astype(np.int32) + 1
        psk = rng.choice(l, size=t, replace=False).astype(np.int64) + 1
        rows0 = (rows1 - 1).astype(np.int32)
        for sorted_subset in (0, 1):
            out = np.zeros(n, dtype=np.int64)
            cnt = np.zeros(1, dtype=np.int64)
            assert lib.cpals_seqrcs_subset(l, n, s, P(rows0, ctypes.c_int32), t, P(psk, ctypes.c_int64), sorted_subset,
                                           P(out, ctypes.c_int64), P(cnt, ctypes.c_int64)) == 0
            ref = oracle.seqrcs_subset(l, n, s, rows1, psk, bool(sorted_subset))
            np.testing.assert_array_equal(out[: cnt[0]], ref)
    bad = np.array([5], dtype=np.int64)  # a pivot row beyond l
    rows0 = np.zeros(3, dtype=np.int32)
    out = np.zeros(3, dtype=np.int64)
    cnt = np.zeros(1, dtype=np.int64)
    assert lib.cpals_seqrcs_subset(4, 3, 1, P(rows0, ctypes.c_int32), 1, P(bad, ctypes.c_int64), 0,
                                   P(out, ctypes.c_int64), P(cnt, ctypes.c_int64)) == -1

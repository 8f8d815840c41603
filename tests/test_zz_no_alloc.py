"""cpals_mttkrp_fp64_noalloc: the MTTKRP for callers that cannot allocate GPU memory.

Some callers hold device buffers and a stream but may not call cudaMalloc when they
need the MTTKRP (a caching allocator's lock, a fixed memory budget, a host that owns
all allocations).  This entry point takes device pointers only and keeps its split-K
partial sums in a fixed device array.  It must give the same result as the handle-based
cpals_mttkrp (tolerance 1e-12 relative Frobenius, as every FP64 MTTKRP parity test), on
two calls in a row: the second call starts with the array holding the first call's data.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def lib(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg.load()


def _noalloc(lib, torch, T, F, mode, R):
    from itensorcpd_gb300 import _lib as L

    dt = L.DTYPE_F64 if T.dtype == np.float64 else L.DTYPE_F32
    t_d = torch.from_numpy(np.ascontiguousarray(T.reshape(-1, order="F"))).cuda()
    f_d = [torch.from_numpy(np.ascontiguousarray(np.asarray(f, dtype=np.float64).reshape(-1, order="F"))).cuda()
           for f in F]
    out = torch.empty(T.shape[mode] * R, dtype=torch.float64, device="cuda")
    ptrs = (L._DP * len(F))(*[C.cast(C.c_void_p(x.data_ptr()), L._DP) for x in f_d])
    dims = np.asarray(T.shape, dtype=np.int64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.cpals_mttkrp_fp64_noalloc(T.ndim, L.i64ptr(dims), R, mode, dt, C.c_void_p(t_d.data_ptr()), ptrs,
                                       C.cast(C.c_void_p(out.data_ptr()), L._DP), stream)
    assert st == 0, L.status_string(st)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(T.shape[mode], R, order="F")


# (40000, 6, 5) at rank 52: mode 0 needs I_0 * R = 2,080,000 of the array's 2,097,152 doubles,
# so one split's partial sums nearly fill it.  (The entry point also lowers the split count
# when several splits would not fit; with GB300's 152 SMs its split rule never asks for more
# than fit, so that branch only runs on GPUs with far more SMs.)
CASES = [((37, 45, 29), 20, np.float64), ((64, 70, 33, 5), 48, np.float32), ((100, 100, 100), 50, np.float64),
         ((40000, 6, 5), 52, np.float64)]


@pytest.mark.parametrize("dims,R,dt", CASES)
def test_noalloc_matches_handle_mttkrp_on_two_calls(pkg, lib, oracle, dims, R, dt):
    torch = pytest.importorskip("torch")
    T = np.asfortranarray(det_normal(5 + R, dims).astype(dt))
    F, lam = det_factors(dims, R, seed=R)
    with pkg.Engine(dims, R, dtype=dt, precision="fp64") as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        ref = [eng.mttkrp(n) for n in range(len(dims))]
    for call in range(2):
        for n in range(len(dims)):
            got = _noalloc(lib, torch, T, F, n, R)
            assert rel(got, ref[n]) <= TOL, (call, n, rel(got, ref[n]))
            # and directly against the oracle's explicit Khatri-Rao GEMM
            want = oracle.mttkrp_krp(T.astype(np.float64), F, n)
            assert rel(got, want) <= TOL, (call, n, rel(got, want))


def test_noalloc_rejects_sizes_beyond_the_array(lib):
    from itensorcpd_gb300 import _lib as L

    dims = np.asarray((40000, 3, 3), dtype=np.int64)  # I_0 * R = 2.56e6 > 2^21
    ptrs = (L._DP * 3)()
    one = C.c_double(0.0)
    p = C.cast(C.pointer(one), L._DP)
    ptrs[1] = p
    ptrs[2] = p
    st = lib.cpals_mttkrp_fp64_noalloc(3, L.i64ptr(dims), 64, 0, L.DTYPE_F64, C.c_void_p(1), ptrs, p, None)
    assert st == L.CPALS_E_ARG
    # a rank so large that I_0 * rank would overflow 64 bits is rejected as well
    st = lib.cpals_mttkrp_fp64_noalloc(3, L.i64ptr(dims), 1 << 62, 0, L.DTYPE_F64, C.c_void_p(1), ptrs, p, None)
    assert st == L.CPALS_E_ARG
    # as is a tensor of more than 2^40 elements
    big = np.asarray((1 << 21, 1 << 20, 2), dtype=np.int64)
    st = lib.cpals_mttkrp_fp64_noalloc(3, L.i64ptr(big), 1, 2, L.DTYPE_F64, C.c_void_p(1), ptrs, p, None)
    assert st == L.CPALS_E_ARG

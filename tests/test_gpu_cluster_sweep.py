"""The FP64 factorisation of the normal equations over a cluster of CTAs against the single-CTA
factorisation: the same pivots, the same operations per entry, so bit-identical factors,
lambdas, fits, leverage scores and sampled updates, at full rank and when the pivoted
Cholesky stops early (the QR fallback then runs on one CTA either way)."""
import contextlib

import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


@contextlib.contextmanager
def cluster_min_rank(r):
    from itensorcpd_gb300 import _lib as L

    lib = L.load()
    prev = lib.cpals_set_cluster_sweep_min_rank(int(r))
    try:
        yield
    finally:
        lib.cpals_set_cluster_sweep_min_rank(prev)


def run_all(pkg, dims, R, seed):
    from itensorcpd_gb300 import _lib as L

    T = np.asfortranarray(det_normal(seed, dims))
    F0, lam0 = det_factors(dims, R, seed=seed)
    out = {}
    with pkg.Engine(dims, R, precision="fp64") as e:
        e.set_tensor(T)
        e.set_factors(F0, lam0)
        out["lev"] = [e.leverage_scores(n) for n in range(len(dims))]
        rng = np.random.default_rng(seed)
        piv = np.stack([rng.integers(1, d + 1, size=3 * R) for d in dims[1:]], axis=1)
        e.sampled_update(0, piv)
        out["sampled"] = e.get_factors()
        e.set_factors(F0, lam0)
        l0 = e.launch_count()
        c = L.CpalsCheck()
        c.kind = L.CHECK_FIT
        c.tolerance = 1e-12
        c.max_counter = 2
        c.ref_norm = float(np.linalg.norm(T))
        c.lastfit = 1.0
        out["fits"] = e.optimize(c)
        out["launches"] = e.launch_count() - l0
        out["factors"] = e.get_factors()
    return out


def same(a, b):
    if isinstance(a, (list, tuple)):
        return len(a) == len(b) and all(same(x, y) for x, y in zip(a, b))
    return np.array_equal(np.asarray(a), np.asarray(b))


# R = 240 on 16 CTAs puts all fifteen diagonal entries of a CTA's rows in one thread
@pytest.mark.parametrize("dims,R", [((60, 50, 45), 40), ((80, 70, 66), 64), ((130, 120, 9), 100), ((140, 131, 130), 128),
                                    ((210, 205, 8, 3), 200), ((250, 245, 6, 4), 240), ((260, 257, 7, 5), 256)])
def test_cluster_sweep_is_bit_identical(built, dims, R):
    with cluster_min_rank(1):
        a = run_all(built, dims, R, seed=R)
    with cluster_min_rank(10**6):
        b = run_all(built, dims, R, seed=R)
    for key in ("lev", "sampled", "fits", "factors"):
        assert same(a[key], b[key]), key
    # the cluster sweep is one more launch per mode
    assert a["launches"] > b["launches"]


def test_cluster_sweep_rank_deficient_falls_back(built, oracle):
    # I_0 = 40 < R = 70: the Gram of F_0 has rank 40, the pivoted Cholesky stops there and the
    # leverage scores come from the rank-40 factor; the fp64 sweeps of modes 1 and 2 meet the
    # rank-deficient Hadamard product of two Grams only if their ranks drop, so check both
    dims, R = (40, 90, 80), 70
    with cluster_min_rank(1):
        a = run_all(built, dims, R, seed=5)
    with cluster_min_rank(10**6):
        b = run_all(built, dims, R, seed=5)
    for key in ("lev", "sampled", "fits", "factors"):
        assert same(a[key], b[key]), key
    F, _ = det_factors(dims, R, seed=5)
    ref = oracle.leverage_score_probabilities(F[0])
    assert np.linalg.norm(a["lev"][0] - ref) / np.linalg.norm(ref) < 1e-10

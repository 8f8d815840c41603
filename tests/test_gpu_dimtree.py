"""Order-4 dimension-tree MTTKRP (CPALS_FLAG_DIMTREE) against the oracle.

The tree computes every M_n from two partial contractions per sweep (modes {2,3} then
{0,1} contracted away), so its per-call MTTKRP must match the oracle's direct MTTKRP:
  * FP64 path: relative Frobenius error <= 1e-12 (the contraction order differs only by
    FP64 rounding);
  * split-BF16 path: <= 1e-4 against the FP64 oracle (the same bound as the direct
    tensor-core MTTKRP);
and a whole FitCheck run must follow the oracle's FP64 trajectory within 1e-8.
"""
import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


DT_SHAPES = [
    ((7, 9, 5, 6), 5),
    ((20, 16, 12, 10), 8),
    ((33, 3, 17, 64), 24),  # ragged, R not a multiple of 16
    ((16, 16, 16, 16), 70),  # R > 64: several rank tiles on the FP64 path
]


@pytest.mark.parametrize("dims,R", DT_SHAPES)
def test_dimtree_mttkrp_fp64_parity(built, oracle, dims, R):
    T = np.asfortranarray(det_normal(sum(dims) + 1, dims))
    F, lam = det_factors(dims, R, seed=R + 1)
    with built.Engine(dims, R, dtype=np.float64, precision="fp64", dimtree=True) as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        for n in range(4):
            ref = oracle.mttkrp_krp(T, F, n)
            got = eng.mttkrp(n)
            assert rel(got, ref) <= 1e-12, (n, rel(got, ref))


@pytest.mark.parametrize("dims,R", [((20, 16, 12, 10), 8), ((64, 48, 32, 40), 32), ((32, 32, 32, 32), 128)])
def test_dimtree_mttkrp_bf16x3(built, oracle, dims, R):
    T = np.asfortranarray(det_normal(sum(dims) + 2, dims).astype(np.float32))
    F, lam = det_factors(dims, R, seed=R + 2)
    with built.Engine(dims, R, dtype=np.float32, precision="bf16x3", dimtree=True) as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        for n in range(4):
            ref = oracle.mttkrp_krp(T.astype(np.float64), F, n)
            got = eng.mttkrp(n)
            assert rel(got, ref) <= 1e-4, (n, rel(got, ref))


def test_dimtree_fitcheck_trajectory_matches_oracle(built, oracle):
    # full ALS with FitCheck on the dimension-tree engine (FP64) against the oracle's ALS
    rng = np.random.default_rng(11)
    dims, R = (12, 10, 9, 8), 4
    T, _, _ = oracle.lowrank_plus_noise(dims, R, 0.3, 30.0, rng, dtype=np.float64)
    F, lam = det_factors(dims, R, seed=3)
    nrm = float(np.linalg.norm(T))
    chk = built.FitCheck(1e-10, 40, nrm)
    built.als_optimize(T, built.CPD(F, lam), check=chk, alg=built.GB300Normal(precision="fp64", dimtree=True))
    ochk = oracle.FitCheck(1e-10, 40, nrm)
    oracle.als_optimize(T, [f.copy() for f in F], lam.copy(), check=ochk)
    assert len(chk.trajectory) == len(ochk.trajectory)
    assert np.max(np.abs(np.asarray(chk.trajectory) - np.asarray(ochk.trajectory))) <= 1e-8


def test_dimtree_bf16x3_sweeps_track_plain(built, oracle):
    # split-BF16 dimension tree vs the plain split-BF16 path and the FP64 path: same fits
    rng = np.random.default_rng(5)
    dims, R = (40, 36, 32, 28), 8
    T, _, _ = oracle.lowrank_plus_noise(dims, R, 0.3, 30.0, rng)
    F, lam = det_factors(dims, R, seed=9)
    nrm = float(np.linalg.norm(T.astype(np.float64)))
    fits = {}
    for key, prec, dt in (("fp64", "fp64", False), ("plain", "bf16x3", False), ("tree", "bf16x3", True)):
        with built.Engine(dims, R, dtype=np.float32, precision=prec, dimtree=dt) as eng:
            eng.set_tensor(T)
            eng.set_factors(F, lam)
            fits[key] = eng.optimize(built.api._to_device_check(built.FitCheck(0.0, 25, nrm)))
    assert np.max(np.abs(fits["tree"] - fits["fp64"])) < 5e-5
    assert np.max(np.abs(fits["tree"] - fits["plain"])) < 5e-5


def test_dimtree_rejects_other_orders(built):
    with pytest.raises(Exception):
        built.Engine((8, 9, 10), 4, dtype=np.float64, precision="fp64", dimtree=True)

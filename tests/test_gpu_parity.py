"""Parity of the CUDA path (through the C ABI) with the oracle and the golden fixtures.

Tolerances (stated by the engine's specification for the FP64 path):
  * per-call MTTKRP: relative Frobenius error <= 1e-12;
  * per-sweep fit trajectory: absolute difference <= 1e-8;
  * leverage-sample gathers: bit-exact.
"""
import json

import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu

MTTKRP_TOL = 1e-12
FIT_TOL = 1e-8


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


SHAPES = [
    ((12, 13, 7), 5, np.float64),
    ((100, 100, 100), 50, np.float64),  # the reference's CPU-runnable workload
    ((6, 5, 4, 3), 7, np.float64),  # order 4
    ((33, 70), 9, np.float64),  # order 2
    ((1, 17, 9), 3, np.float64),  # unit extent
    ((20, 30, 40), 70, np.float64),  # R > 64: several rank tiles
    ((37, 29, 41), 16, np.float32),  # FP32 storage, FP64 arithmetic
    ((5, 4, 3, 2, 3), 4, np.float64),  # order 5
]


@pytest.mark.parametrize("dims,R,dt", SHAPES)
def test_mttkrp_fp64_parity(built, oracle, dims, R, dt):
    T = np.asfortranarray(det_normal(sum(dims), dims).astype(dt))
    F, lam = det_factors(dims, R, seed=len(dims) + R)
    with built.Engine(dims, R, dtype=dt, precision="fp64") as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        for n in range(len(dims)):
            ref = oracle.mttkrp_krp(T.astype(np.float64), F, n)
            got = eng.mttkrp(n)
            assert rel(got, ref) <= MTTKRP_TOL, (n, rel(got, ref))


def test_grams_and_factor_round_trip(built, oracle):
    dims, R = (11, 9, 8), 6
    F, lam = det_factors(dims, R, seed=4)
    with built.Engine(dims, R) as eng:
        eng.set_tensor(np.asfortranarray(det_normal(1, dims)))
        eng.set_factors(F, lam)
        F2, lam2 = eng.get_factors()
        for a, b in zip(F, F2):
            assert np.array_equal(a, b)
        assert np.array_equal(lam, lam2)
        for n in range(3):
            assert rel(eng.gram(n), F[n].T @ F[n]) < 1e-14


def _run_fitcheck(built, T, F, lam, tol, maxc, graph=True):
    chk = built.FitCheck(tol, maxc, float(np.linalg.norm(T)))
    with built.Engine(T.shape, F[0].shape[1], dtype=T.dtype, graph=graph) as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        c = built.api._to_device_check(chk)
        traj = eng.optimize(c)
        built.api._from_device_check(chk, c, traj, F[0].shape[1], False)
        Ff, lf = eng.get_factors()
    return chk, Ff, lf


@pytest.mark.parametrize("graph", [True, False])
def test_fit_trajectory_small_golden(built, golden_dir, graph):
    g = json.loads((golden_dir / "als_small.json").read_text())
    T = np.asfortranarray(det_normal(g["tensor_seed"], g["dims"]))
    F, lam = det_factors(g["dims"], g["rank"], seed=g["factor_seed"])
    chk, Ff, lf = _run_fitcheck(built, T, F, lam, g["tol"], g["max_counter"], graph=graph)
    assert len(chk.trajectory) == len(g["trajectory"])
    assert np.max(np.abs(np.array(chk.trajectory) - g["trajectory"])) <= FIT_TOL
    assert chk.total_iter == g["total_iter"]
    for a, b in zip(Ff, g["final_factors"]):
        assert rel(a, np.array(b)) < 1e-8
    assert rel(lf, np.array(g["final_lambda"])) < 1e-8


def test_fit_trajectory_c1_golden(built, golden_dir):
    # 100^3 FP64 N(0,1), rank 50, FitCheck(1e-3, 100, norm(T))
    g = json.loads((golden_dir / "als_c1.json").read_text())
    T = np.asfortranarray(det_normal(g["tensor_seed"], g["dims"]))
    F, lam = det_factors(g["dims"], g["rank"], seed=g["factor_seed"])
    chk, _, _ = _run_fitcheck(built, T, F, lam, g["tol"], g["max_counter"])
    assert chk.total_iter == g["total_iter"]
    assert np.max(np.abs(np.array(chk.trajectory) - g["trajectory"])) <= FIT_TOL
    assert abs(chk.final_fit - g["final_fit"]) <= FIT_TOL


def test_per_call_mttkrp_inside_sweep(built, oracle, golden_dir):
    # the first sweep's MTTKRP of every mode, recorded by the oracle: before mode n the
    # factors are the sweep's updated ones for modes < n and the initial ones for modes >= n
    g = json.loads((golden_dir / "als_small.json").read_text())
    T = np.asfortranarray(det_normal(g["tensor_seed"], g["dims"]))
    F, lam = det_factors(g["dims"], g["rank"], seed=g["factor_seed"])
    rec = []
    oracle.als_optimize(T, F, lam, check=oracle.NoCheck(1), record=rec)
    with built.Engine(T.shape, g["rank"]) as eng:
        eng.set_tensor(T)
        for n in range(3):
            state = [rec[0]["factors"][m] if m < n else F[m] for m in range(3)]
            eng.set_factors(state, lam)
            assert rel(eng.mttkrp(n), np.array(g["mttkrp_sweep1"][n])) <= MTTKRP_TOL


def test_overcomplete_rank400_reconstruction(built, oracle):
    # test/cp_als.jl:9-10: rank 400 on 20x30x40 FP64, 100 sweeps -> rel err < 1e-7
    T = np.asfortranarray(det_normal(40, (20, 30, 40)))
    cp = built.random_CPD(T, 400, rng=np.random.default_rng(3))
    opt = built.als_optimize(T, cp)
    assert rel(oracle.reconstruct(opt.factors, opt.lam), T) < 1e-7


def test_rank_deficient_takes_qr_fallback(built, golden_dir):
    g = json.loads((golden_dir / "rank_deficient.json").read_text())
    T = np.asfortranarray(det_normal(g["tensor_seed"], g["dims"]))
    F, lam = det_factors(g["dims"], g["rank"], seed=g["factor_seed"])
    for f in F:
        f[:, 3] = f[:, 2]
    with built.Engine(T.shape, g["rank"]) as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        c = built.api._to_device_check(built.NoCheck(1))
        eng.optimize(c)
        Ff, lf = eng.get_factors()
        assert eng.fallback_count() == g["fallbacks"]
    for a, b in zip(Ff, g["factors_after_sweep1"]):
        assert rel(a, np.array(b)) < 1e-6


def test_nan_tensor_raises_error_nan(built):
    T = np.asfortranarray(det_normal(3, (8, 7, 6)))
    T[2, 3, 4] = np.nan
    cp = built.random_CPD(T, 3)
    with pytest.raises(FloatingPointError, match="Error NAN"):
        built.als_optimize(T, cp, check=built.FitCheck(1e-6, 5, 1.0))


def test_decompose_api_and_rank_adaptive(built, oracle):
    # an exact rank-3 target for which ALS from the default random_CPD start reaches the
    # global optimum on the oracle (plain ALS from random starts can stall in swamps)
    F, _ = det_factors((10, 11, 12), 3, seed=12)
    T = np.asfortranarray(oracle.reconstruct(F, np.array([3.0, 2.0, 1.0])))
    chk = built.FitCheck(1e-10, 200, float(np.linalg.norm(T)))
    cp = built.decompose(T, 3, check=chk)
    assert built.CPDFit(chk) > 0.999
    assert rel(oracle.reconstruct(cp.factors, cp.lam), T) < 1e-3
    cp2 = built.decompose(T, 1e-3, 4, check=built.FitCheck(1e-8, 200, float(np.linalg.norm(T))), start_rank=2)
    assert built.cp_rank(cp2) in (3, 4)
    with pytest.raises(TypeError):
        built.decompose(T, 3, solver=object())


def test_rank_adaptive_decompose_uploads_once(built, oracle):
    """decompose.jl:32-69 on one device copy of T: every rank's handle borrows it, and the
    result equals a loop of als_optimize / increase_cpd_rank that uploads T per rank."""
    F, _ = det_factors((16, 15, 14), 4, seed=13)
    T = np.asfortranarray(oracle.reconstruct(F, np.array([4.0, 3.0, 2.0, 1.0])).astype(np.float32))
    nrm = float(np.linalg.norm(T))
    cp = built.decompose(T, 1e-4, 5, check=built.FitCheck(1e-7, 60, nrm), start_rank=2,
                         rng=np.random.default_rng(5), alg=built.GB300Normal())
    rng = np.random.default_rng(5)
    chk = built.FitCheck(1e-7, 60, nrm)
    ref = built.random_CPD(T, 2, rng)
    for r in range(2, 6):
        ref = built.als_optimize(T, ref, alg=built.GB300Normal(), check=chk, rng=rng)
        chk.iter = 0
        if 1.0 - built.CPDFit(chk) < 1e-4 or r == 5:
            break
        ref = built.increase_cpd_rank(ref, r + 1, rng)
    assert built.cp_rank(cp) == built.cp_rank(ref)
    for a, b in zip(cp.factors, ref.factors):
        np.testing.assert_array_equal(a, b)
    # the borrowed pointer is the owner's
    with built.Engine(T.shape, 1, dtype=np.float32) as owner, built.Engine(T.shape, 3, dtype=np.float32,
                                                                            precision="bf16x3") as e:
        with pytest.raises(built.CpalsError):
            owner.tensor_device_ptr()  # no tensor yet
        owner.set_tensor(T)
        e.set_tensor_from(owner)
        assert e.tensor_device_ptr() == owner.tensor_device_ptr()


# ---------------- randomized path: bit-exact gathers ----------------
@pytest.mark.parametrize("dims,mode", [((100, 150, 200), 0), ((100, 150, 200), 2), ((5, 6, 7, 8), 1),
                                       ((9, 4), 1)])
def test_pivot_hadamard_bit_exact(built, oracle, dims, mode):
    R = 20
    F, lam = det_factors(dims, R, seed=5)
    rng = np.random.default_rng(6)
    others = [d for m, d in enumerate(dims) if m != mode]
    piv = np.stack([rng.integers(1, d + 1, size=333) for d in others], axis=1)
    with built.Engine(dims, R) as eng:
        eng.set_tensor(np.zeros(dims, order="F"))
        eng.set_factors(F, lam)
        got = eng.pivot_hadamard(mode, piv)
    ref = oracle.pivot_hadamard([F[m] for m in range(len(dims)) if m != mode], piv)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_fused_flatten_sample_bit_exact(built, oracle, dt):
    dims = (7, 8, 9, 10)
    T = np.asfortranarray(det_normal(2, dims).astype(dt))
    F, lam = det_factors(dims, 3, seed=5)
    rng = np.random.default_rng(9)
    with built.Engine(dims, 3, dtype=dt) as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        for mode in range(4):
            others = [d for m, d in enumerate(dims) if m != mode]
            piv = np.stack([rng.integers(1, d + 1, size=77) for d in others], axis=1)
            assert np.array_equal(eng.fused_flatten_sample(mode, piv), oracle.fused_flatten_sample(T, mode, piv))
        # single sample, extreme indices
        piv = np.array([[1, 9, 10]])
        assert np.array_equal(eng.fused_flatten_sample(1, piv), oracle.fused_flatten_sample(T, 1, piv))
        piv = np.array([[7, 8, 9]])
        assert np.array_equal(eng.fused_flatten_sample(3, piv), oracle.fused_flatten_sample(T, 3, piv))


def test_gather_rejects_out_of_range_pivots(built):
    dims = (5, 6, 7)
    F, lam = det_factors(dims, 2, seed=1)
    with built.Engine(dims, 2) as eng:
        eng.set_tensor(np.zeros(dims, order="F"))
        eng.set_factors(F, lam)
        for bad in ([[0, 1]], [[6, 1]], [[1, 8]]):
            with pytest.raises(built.CpalsError):
                eng.pivot_hadamard(1, np.array(bad))
            with pytest.raises(built.CpalsError):
                eng.fused_flatten_sample(1, np.array(bad))
        assert eng.pivot_hadamard(1, np.array([[5, 7]])).shape == (1, 2)


def test_leverage_scores_match_qr(built, oracle):
    dims = (40, 13, 9)
    F, lam = det_factors(dims, 6, seed=2)
    with built.Engine(dims, 6) as eng:
        eng.set_tensor(np.zeros(dims, order="F"))
        eng.set_factors(F, lam)
        for n in range(3):
            assert rel(eng.leverage_scores(n), oracle.leverage_score_probabilities(F[n])) < 1e-12


def test_sampled_updates_replay_golden(built, golden_dir, oracle):
    g = json.loads((golden_dir / "lev_small.json").read_text())
    Ft, lt = det_factors(g["dims"], g["rank"], seed=g["truth_seed"])
    T = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F, lam = det_factors(g["dims"], g["rank"], seed=g["factor_seed"])
    for run in g["runs"]:
        with built.Engine(T.shape, g["rank"]) as eng:
            eng.set_tensor(T)
            eng.set_factors(F, lam)
            for step in run["steps"]:
                eng.sampled_update(step["mode"], np.array(step["pivots"]), normal=run["normal"])
                Ff, lf = eng.get_factors()
                assert rel(Ff[step["mode"]], np.array(step["factor"])) < 1e-8
                assert rel(lf, np.array(step["lambda"])) < 1e-8


def test_lev_score_sampled_api(built, oracle):
    dims = (12, 13, 3)
    Ft, lt = det_factors(dims, 5, seed=31)
    T = np.asfortranarray(oracle.reconstruct(Ft, lt))
    # best of five tries (the reference's multiple_tries helper, rand_cp_als.jl:1-14): from
    # this start a sampled run often stalls near 0.12, as the oracle's runs do
    best = 1.0
    for trial in range(5):
        cp = built.CPD(*det_factors(dims, 5, seed=32))
        opt = built.als_optimize(T, cp, alg=built.LevScoreSampled(100), check=built.NoCheck(100), normal=True,
                                 rng=np.random.default_rng(100 + trial))
        best = min(best, rel(oracle.reconstruct(opt.factors, opt.lam), T))
    assert best < 0.1


@pytest.mark.parametrize("prec,dt", [("fp64", np.float64), ("bf16x3", np.float32)])
def test_second_tensor_on_the_same_handle_is_the_one_decomposed(built, prec, dt):
    # the sweep graph survives a new tensor at the same device address; the next optimize
    # must use the new contents (compared with a fresh handle on the second tensor)
    from itensorcpd_gb300 import _lib as L

    dims, R = (24, 20, 18), 4
    Ta = np.asfortranarray(det_normal(31, dims).astype(dt))
    Tb = np.asfortranarray(det_normal(32, dims).astype(dt))
    F, lam = det_factors(dims, R, seed=9)

    def run(eng, T):
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        c = L.CpalsCheck()
        c.kind, c.max_counter, c.ref_norm = L.CHECK_NONE, 4, float(np.linalg.norm(T.astype(np.float64)))
        return eng.optimize(c), eng.get_factors()

    with built.Engine(dims, R, dtype=dt, precision=prec) as e1, built.Engine(dims, R, dtype=dt, precision=prec) as e2:
        run(e1, Ta)
        tr1, (F1, l1) = run(e1, Tb)
        tr2, (F2, l2) = run(e2, Tb)
    assert np.array_equal(tr1, tr2)
    assert np.array_equal(l1, l2)
    for a, b in zip(F1, F2):
        assert np.array_equal(a, b)

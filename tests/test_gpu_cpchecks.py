"""CPDiffCheck and CPAngleCheck on the device against the oracle's restatement
(src/converge_checks/cp_diff_check.jl:20-68, cp_angle_check.jl:20-68).

The device check and the oracle see the same iterates: a second engine runs the same
sweeps one at a time under NoCheck, its factors are read back after every sweep and fed
to the oracle's check.  The sweeps are deterministic, so both engines hold bit-identical
iterates and only the check's own arithmetic differs (summation order).

Tolerances: the fit between consecutive iterates, 1 - sqrt(|a + b - 2c|) / sqrt(a),
cancels to the size of the change; with FP64 sums of different order the trajectories
agree to 1e-7 absolute (fit) and 1e-6 absolute (angle, whose acos amplifies the
cancellation near 0).  Counters, iteration counts and the stopping sweep must be equal.
"""
import ctypes as C

import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu

FIT_ATOL = 1e-7
ANGLE_ATOL = 1e-6


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def lowrank(dims, R, seed, noise=1e-3, dt=np.float64):
    F, lam = det_factors(dims, R, seed)
    T = np.einsum("r," + ",".join(f"{chr(97 + k)}r" for k in range(len(dims))) + "->"
                  + "".join(chr(97 + k) for k in range(len(dims))), lam, *F)
    T = T + noise * np.linalg.norm(T) / np.sqrt(T.size) * det_normal(seed + 99, dims)
    return np.asfortranarray(T.astype(dt))


def device_check(L, kind, tol, max_counter):
    c = L.CpalsCheck()
    c.kind = kind
    c.max_counter = max_counter
    c.tolerance = tol
    c.lastfit = 1.0
    return c


def run_device(built, T, R, F0, lam0, kind, tol, maxc, **eng_kw):
    L = built._lib
    with built.Engine(T.shape, R, dtype=T.dtype, **eng_kw) as e:
        e.set_tensor(T)
        e.set_factors(F0, lam0)
        c = device_check(L, kind, tol, maxc)
        traj = e.optimize(c)
    return c, traj


def run_stepwise(built, oracle_check, T, R, F0, lam0, maxc, **eng_kw):
    L = built._lib
    with built.Engine(T.shape, R, dtype=T.dtype, **eng_kw) as e:
        e.set_tensor(T)
        e.set_factors(F0, lam0)
        for _ in range(maxc):
            nc = L.CpalsCheck()
            nc.kind = L.CHECK_NONE
            nc.max_counter = 1
            e.optimize(nc)
            F, lam = e.get_factors()
            if oracle_check.check_converge(F, lam):
                break
    return oracle_check


def compare(c, traj, oc, atol):
    assert len(traj) == len(oc.trajectory)
    np.testing.assert_allclose(traj, oc.trajectory, rtol=0, atol=atol, equal_nan=True)
    assert np.isnan(traj[0])
    assert c.iter == oc.iter and c.counter == oc.counter and c.total_iter == oc.total_iter
    assert abs(c.final_fit - oc.final_fit) <= atol
    assert abs(c.lastfit - oc.lastfit) <= atol
    assert bool(c.has_prev) == (oc.PrevCP is not None)


CASES = [
    # dims, R, dtype, engine options
    ((30, 35, 40), 6, np.float64, dict(precision="fp64")),
    ((64, 64, 64), 16, np.float32, dict(precision="bf16x3")),
    ((20, 18, 16, 14), 8, np.float64, dict(precision="fp64", dimtree=True)),
    ((40, 50, 30), 70, np.float64, dict(precision="fp64")),  # R > 64: several output tiles
]


@pytest.mark.parametrize("dims,R,dt,kw", CASES)
@pytest.mark.parametrize("which", ["diff", "angle"])
def test_check_matches_oracle(built, oracle, dims, R, dt, kw, which):
    L = built._lib
    T = lowrank(dims, min(R, 8), seed=len(dims) + R, dt=dt)
    F0, lam0 = det_factors(dims, R, seed=7 + R)
    tol = 1e-5 if which == "diff" else 1e-4
    maxc = 25
    kind = L.CHECK_DIFF if which == "diff" else L.CHECK_ANGLE
    c, traj = run_device(built, T, R, F0, lam0, kind, tol, maxc, **kw)
    oc = (oracle.CPDiffCheck if which == "diff" else oracle.CPAngleCheck)(tol, maxc)
    run_stepwise(built, oc, T, R, F0, lam0, maxc, **kw)
    compare(c, traj, oc, FIT_ATOL if which == "diff" else ANGLE_ATOL)


def test_check_converge_entry_on_set_iterates(built, oracle):
    """cpals_check_converge on iterates set from the host, as a sampled solver's loop calls it."""
    L = built._lib
    dims, R = (12, 13, 5), 5
    base, lam = det_factors(dims, R, seed=3)
    for which, cls in (("diff", oracle.CPDiffCheck), ("angle", oracle.CPAngleCheck)):
        oc = cls(1e-3, 6)
        c = device_check(L, L.CHECK_DIFF if which == "diff" else L.CHECK_ANGLE, 1e-3, 6)
        with built.Engine(dims, R, dtype=np.float64, precision="fp64") as e:
            for k in range(6):
                # iterates that approach `base` geometrically, so the check converges
                step = 0.5 ** (2 * k + 1)
                F = [B + step * det_normal(100 * k + m, B.shape) for m, B in enumerate(base)]
                lk = lam * (1 + step)
                e.set_factors(F, lk)
                done, val = e.check_converge(c)
                Fd, ld = e.get_factors()
                odone = oc.check_converge(Fd, ld)
                assert done == odone
                if np.isnan(oc.trajectory[-1]):
                    assert np.isnan(val)
                else:
                    assert abs(val - oc.trajectory[-1]) <= ANGLE_ATOL
                assert c.iter == oc.iter and c.counter == oc.counter
                if done:
                    break
        assert abs(c.final_fit - oc.final_fit) <= ANGLE_ATOL
        assert c.total_iter == oc.total_iter


def test_prev_iterate_moves_between_handles(built, oracle):
    """A check that stopped after storing PrevCP continues on another handle."""
    L = built._lib
    dims, R = (25, 30, 20), 5
    T = lowrank(dims, R, seed=11)
    F0, lam0 = det_factors(dims, R, seed=12)
    ref_c, ref_traj = run_device(built, T, R, F0, lam0, L.CHECK_DIFF, 1e-6, 15, precision="fp64")
    with built.Engine(dims, R, dtype=np.float64, precision="fp64") as a:
        a.set_tensor(T)
        a.set_factors(F0, lam0)
        c = device_check(L, L.CHECK_DIFF, 1e-6, 1)
        a.optimize(c)  # one sweep: PrevCP stored, no reset (cp_diff_check.jl:24-28)
        assert c.has_prev == 1 and c.iter == 1
        Fa, la = a.get_factors()
        Pa, pla = a.get_prev()
        for x, y in zip(Fa, Pa):
            np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(la, pla)
    with built.Engine(dims, R, dtype=np.float64, precision="fp64") as b:
        b.set_tensor(T)
        b.set_factors(Fa, la)
        c.max_counter = 15
        with pytest.raises(built.CpalsError):  # PrevCP claimed but not held by this handle
            b.optimize(c)
        b.set_prev(Pa, pla)
        traj = b.optimize(c)
    np.testing.assert_allclose(traj, ref_traj[1:], rtol=0, atol=FIT_ATOL)
    assert c.total_iter == ref_c.total_iter and c.iter == ref_c.iter


def test_als_optimize_with_diff_check_interpolates_known_low_rank(built, oracle):
    """test/rand_cp_als.jl:73-80 shape: a rank-10 model of an exactly rank-20 tensor under
    CPDiffCheck(1e-5, 100); the GPU and the oracle stop on the same sweep."""
    dims = (20, 25, 30)
    Ft, lt = det_factors(dims, 20, seed=21)
    A = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F0, lam0 = det_factors(dims, 10, seed=22)
    chk = built.CPDiffCheck(1e-5, 100)
    cp = built.als_optimize(A, built.CPD([F.copy() for F in F0], lam0.copy(), dims), check=chk)
    of, ol, oc, _ = oracle.als_optimize(A, F0, lam0, check=oracle.CPDiffCheck(1e-5, 100))
    assert chk.total_iter == oc.total_iter
    assert abs(chk.final_fit - oc.final_fit) <= FIT_ATOL
    err = np.linalg.norm(A - oracle.reconstruct(cp.factors, cp.lam)) / np.linalg.norm(A)
    oerr = np.linalg.norm(A - oracle.reconstruct(of, ol)) / np.linalg.norm(A)
    assert abs(err - oerr) <= 1e-6
    assert chk.PrevCP is None and chk.iter == 0


def test_lev_score_sampled_stops_where_the_check_says(built, oracle):
    """ProjectionAlgorithm.jl:53 passes CPDiffCheck / CPAngleCheck through to the sampled
    solvers (test/rand_cp_als.jl:105-117 runs LevScoreSampled under both).  The loop stops
    on the sweep where the check converges, and its iterate is the one the same loop reaches
    under NoCheck in that many sweeps (same seed, so the same pivots)."""
    dims = (12, 13, 3)
    Ft, lt = det_factors(dims, 5, seed=31)
    T = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F0, lam0 = det_factors(dims, 5, seed=32)

    def run(check):
        return built.als_optimize(T, built.CPD([F.copy() for F in F0], lam0.copy(), dims),
                                  alg=built.LevScoreSampled(100), check=check, rng=np.random.default_rng(5))

    for chk in (built.CPDiffCheck(1e-2, 30), built.CPAngleCheck(1e-2, 30)):
        cp = run(chk)
        k = len(chk.trajectory)
        assert 3 <= k < 30 and chk.total_iter == k and chk.iter == 0 and chk.PrevCP is None
        assert np.isnan(chk.trajectory[0]) and np.all(np.isfinite(chk.trajectory[1:]))
        ref = run(built.NoCheck(k))
        for x, y in zip(cp.factors, ref.factors):
            np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(cp.lam, ref.lam)

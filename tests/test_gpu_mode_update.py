"""The per-mode entry point that a caller-driven sweep loop uses (through the C ABI).

ITensorCPD's optimize (src/optimizers/als_optimizers/optimize.jl:15-32) calls, per mode,
compute_krp, matricize_tensor, solve_ls_problem, row_norm and post_solve, and then
check_converge once per sweep.  An MttkrpAlgorithm plug-in that runs on the device maps those
calls onto cpals_mode_update (one per mode) and cpals_check_converge.  `order` mode updates
and one check must give exactly what one sweep of cpals_optimize gives: the same factors,
lambda, Grams and fit, bit for bit, and the same check state.
"""
import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def fitcheck(L, ref_norm, max_counter, tol=1e-12):
    c = L.CpalsCheck()
    c.kind = L.CHECK_FIT
    c.tolerance = tol
    c.max_counter = max_counter
    c.ref_norm = ref_norm
    c.lastfit = 1.0
    return c


CASES = [
    ((12, 13, 7), 5, np.float64, "fp64", False),
    ((40, 30, 20), 70, np.float64, "fp64", False),  # R > 64
    ((64, 48, 40), 16, np.float32, "bf16x3", False),  # tensor-core MTTKRP
    ((20, 18, 16, 14), 8, np.float32, "bf16x3", True),  # order-4 dimension tree
    ((9, 8, 7, 6), 4, np.float64, "fp64", True),
]


@pytest.mark.parametrize("dims,R,dt,prec,dimtree", CASES)
def test_mode_updates_and_check_equal_one_sweep_bit_for_bit(built, dims, R, dt, prec, dimtree):
    from itensorcpd_gb300 import _lib as L

    T = np.asfortranarray(det_normal(3 + R, dims).astype(dt))
    F0, lam0 = det_factors(dims, R, seed=R + len(dims))
    ref_norm = float(np.linalg.norm(T.astype(np.float64)))
    sweeps = 3
    with built.Engine(dims, R, dtype=dt, precision=prec, dimtree=dimtree) as a, \
            built.Engine(dims, R, dtype=dt, precision=prec, dimtree=dimtree) as b:
        a.set_tensor(T)
        b.set_tensor(T)
        a.set_factors(F0, lam0)
        b.set_factors(F0, lam0)
        ca = fitcheck(L, ref_norm, sweeps)
        traj = a.optimize(ca)
        cb = fitcheck(L, ref_norm, sweeps)
        fits = []
        for s in range(sweeps):
            # (one mode also copies its solution back, as a plug-in keeping host factors does)
            for n in range(len(dims)):
                b.mode_update(n, want_solution=(n == 1))
            conv, fit = b.check_converge(cb)
            fits.append(fit)
            assert not conv
        Fa, la = a.get_factors()
        Fb, lb = b.get_factors()
        assert np.array_equal(np.asarray(traj), np.asarray(fits))
        assert np.array_equal(la, lb)
        for m in range(len(dims)):
            assert np.array_equal(Fa[m], Fb[m]), m
            assert np.array_equal(a.gram(m), b.gram(m)), m
        for f in ("iter", "counter", "lastfit", "final_fit", "total_iter"):
            assert getattr(ca, f) == getattr(cb, f), f


def test_mode_update_returns_the_unnormalised_solution(built):
    dims, R = (15, 11, 9), 4
    T = np.asfortranarray(det_normal(1, dims))
    F0, lam0 = det_factors(dims, R, seed=2)
    with built.Engine(dims, R) as e:
        e.set_tensor(T)
        e.set_factors(F0, lam0)
        X = e.mode_update(0, want_solution=True)
        F, lam = e.get_factors()
        # row_norm (src/math_tools/row_norm.jl:4-24): lambda_r = ||X(:, r)||, F = X / lambda
        assert np.allclose(np.linalg.norm(X, axis=0), lam, rtol=1e-14, atol=0)
        assert np.allclose(X / lam, F[0], rtol=1e-14, atol=1e-15)


def test_check_without_a_last_mode_update_is_out_of_order(built):
    from itensorcpd_gb300 import _lib as L

    dims, R = (6, 5, 4), 2
    with built.Engine(dims, R) as e:
        e.set_tensor(np.asfortranarray(det_normal(4, dims)))
        F0, lam0 = det_factors(dims, R, seed=3)
        e.set_factors(F0, lam0)
        c = fitcheck(L, 1.0, 5)
        with pytest.raises(built.CpalsError):
            e.check_converge(c)  # no mode update has saved the fit's terms
        e.mode_update(0)
        e.mode_update(1)
        with pytest.raises(built.CpalsError):
            e.check_converge(c)  # the last mode has not run
        e.mode_update(2)
        e.check_converge(c)
        with pytest.raises(built.CpalsError):
            e.check_converge(c)  # the terms were used


def test_mode_update_after_a_converged_optimize_still_updates(built):
    from itensorcpd_gb300 import _lib as L

    dims, R = (10, 9, 8), 3
    T = np.asfortranarray(det_normal(6, dims))
    F0, lam0 = det_factors(dims, R, seed=5)
    with built.Engine(dims, R) as e:
        e.set_tensor(T)
        e.set_factors(F0, lam0)
        c = fitcheck(L, float(np.linalg.norm(T)), 200, tol=1e-1)
        e.optimize(c)  # converges, leaving the device check's `done` set
        before, _ = e.get_factors()
        e.mode_update(0)
        after, _ = e.get_factors()
        assert not np.array_equal(before[0], after[0])


@pytest.mark.parametrize("fused,per_mode", [(True, 3), (False, 5)])
def test_a_sweep_launches_per_mode(built, fused, per_mode):
    # per mode: the factorisation, the MTTKRP, then either one cooperative launch for the
    # solve, the Gram, lambda and the normalisation (the fit included on the last mode), or
    # (the default) the solve, the Gram reduction with its finalize and the normalisation;
    # both give the same fits to rounding
    from itensorcpd_gb300 import _lib as L

    dims, R = (40, 30, 20), 6
    T = np.asfortranarray(det_normal(8, dims))
    F0, lam0 = det_factors(dims, R, seed=8)
    with built.Engine(dims, R, fused_tail=fused) as e:
        e.set_tensor(T)
        e.set_factors(F0, lam0)
        c = fitcheck(L, float(np.linalg.norm(T)), 3)
        l0 = e.launch_count()
        fits = e.optimize(c)
        assert e.launch_count() - l0 == 3 * per_mode * len(dims)
    with built.Engine(dims, R, fused_tail=not fused) as e:
        e.set_tensor(T)
        e.set_factors(F0, lam0)
        other = e.optimize(fitcheck(L, float(np.linalg.norm(T)), 3))
    assert np.max(np.abs(np.asarray(fits) - np.asarray(other))) < 1e-12

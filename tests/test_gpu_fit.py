"""The compensated FP64 fit and the device's ||T||^2 (through the C ABI).

FitCheck's fit is 1 - sqrt(|norm(T)^2 + ||X||^2 - 2 |<T, X>||) / norm(T)
(src/converge_checks/fit_check.jl:26-32).  Near fit -> 1 the three terms cancel: a relative
error d in them becomes an error d / (2 rho) in the fit, rho = ||T - X|| / ||T||.  The engine
carries ||T||^2 as a double-double summed exactly on the device, forms <T, X> and ||X||^2
from TwoProduct terms in double-double, and combines them without rounding before the
square root.  What remains is the rounding of the FP64 inputs themselves (the MTTKRP, the
solve's X, the Grams), about eps / rho in the fit.  The tests compare the device's fit with
the residual computed directly from the final factors, ||T - reconstruct(F, lambda)|| / ||T||,
in extended precision (no cancellation: error ~eps), with the bound
    |fit_device - fit_direct| <= 8 eps / rho + 4 eps.
"""
import fractions
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -52


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def exact_sum_squares(x):
    return sum((fractions.Fraction(float(v)) ** 2 for v in np.ravel(x)), fractions.Fraction(0))


def dd_error(hi, lo, exact):
    return abs(fractions.Fraction(hi) + fractions.Fraction(lo) - exact) / exact


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_tensor_norm2_is_exact_to_double_double(built, dt):
    rng = np.random.default_rng(7)
    dims = (23, 17, 11)
    # entries over a wide range of exponents, including FP32 subnormals, zeros and signs
    T = rng.standard_normal(dims) * np.exp2(rng.integers(-30, 30, size=dims))
    T.flat[::97] = 0.0
    T.flat[5] = np.float32(1e-40) if dt == np.float32 else 1e-300
    T = np.asfortranarray(T.astype(dt))
    exact = exact_sum_squares(T)
    with built.Engine(dims, 3, dtype=dt) as eng:
        eng.set_tensor(T)
        nrm, (hi, lo) = eng.tensor_norm()
    # exact but for the bits each square drops below a fixed fraction of the largest square:
    # 2^-78 for FP32 entries, 2^-86 for FP64 (TwoProduct parts): at most n times that, relative
    bound = T.size * (2.0 ** -78 if dt == np.float32 else 2.0 ** -86)
    assert dd_error(hi, lo, exact) < bound
    assert abs(nrm - math.sqrt(float(exact))) <= 2 * EPS * nrm


def test_tensor_norm_of_a_non_finite_tensor_is_refused(built):
    T = np.ones((4, 5, 6), dtype=np.float32, order="F")
    T[1, 2, 3] = np.inf
    with built.Engine(T.shape, 2, dtype=np.float32) as eng:
        eng.set_tensor(T)
        with pytest.raises(FloatingPointError):
            eng.tensor_norm()


def lowrank_plus_noise(dims, R, eta, seed):
    rng = np.random.default_rng(seed)
    F = [rng.standard_normal((d, R)) for d in dims]
    F = [f / np.linalg.norm(f, axis=0) for f in F]
    w = rng.uniform(1.0, 10.0, R)
    T0 = np.einsum("ir,jr,kr,r->ijk", *F, w)
    N = rng.standard_normal(dims)
    T = T0 + eta * np.linalg.norm(T0) * N / np.linalg.norm(N)
    start = [f + 1e-2 * rng.standard_normal(f.shape) for f in F]
    return np.asfortranarray(T), start


def direct_fit(T, F, lam):
    L = np.longdouble
    X = np.einsum("ir,jr,kr,r->ijk", *[f.astype(L) for f in F], lam.astype(L))
    Tl = T.astype(L)
    return float(1 - np.sqrt(np.sum((Tl - X) ** 2)) / np.sqrt(np.sum(Tl * Tl)))


@pytest.mark.parametrize("eta", [1e-3, 1e-5, 1e-7])
def test_fit_near_one_matches_the_direct_residual(built, pkg, eta):
    from itensorcpd_gb300 import _lib as Lb

    dims, R = (40, 50, 60), 5
    T, start = lowrank_plus_noise(dims, R, eta, seed=11)
    with built.Engine(dims, R, dtype=np.float64, precision="fp64") as eng:
        eng.set_tensor(T)
        nrm, _ = eng.tensor_norm()
        eng.set_factors(start, np.ones(R))
        c = Lb.CpalsCheck()
        c.kind = Lb.CHECK_FIT
        c.tolerance = 0.0
        c.max_counter = 25
        c.ref_norm = nrm
        c.lastfit = 1.0
        traj = eng.optimize(c)
        F, lam = eng.get_factors()
    want = direct_fit(T, F, lam)
    rho = 1.0 - want
    assert rho < 3 * eta
    bound = 8 * EPS / rho + 4 * EPS
    assert abs(traj[-1] - want) <= bound, (traj[-1], want, abs(traj[-1] - want), bound)

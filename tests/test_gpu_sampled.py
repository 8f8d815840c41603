"""BlockLevScoreSampled and stop_resample on the device (algorithms/.../randomized/
krp_lev_score_sampled.jl:20-37, 64-106; probability.jl:61-108).

Index drawing stays on the host; the sampled gathers and solves run on the device.  The
replay test feeds the pivots a device run drew to the oracle's sampled steps and compares
the factors (relative Frobenius error <= 1e-8, the sampled-solve parity bound).
"""
import numpy as np
import pytest

from _data import det_factors

pytestmark = pytest.mark.gpu

REPLAY_TOL = 1e-8


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def target(oracle, dims=(12, 13, 3), R=5):
    Ft, lt = det_factors(dims, R, seed=31)
    return np.asfortranarray(oracle.reconstruct(Ft, lt))


@pytest.mark.parametrize("normal", [True, False])
def test_block_sampled_run_replays_through_the_oracle(built, oracle, normal):
    T = target(oracle, (14, 11, 9))
    F0, lam0 = det_factors(T.shape, 5, seed=32)
    seen = []
    cp = built.als_optimize(T, built.CPD([F.copy() for F in F0], lam0.copy(), T.shape),
                            alg=built.BlockLevScoreSampled(60, 3), check=built.NoCheck(4), normal=normal,
                            rng=np.random.default_rng(4), on_pivots=lambda n, p: seen.append((n, p.copy())))
    assert len(seen) == 4 * 3
    F = [f.copy() for f in F0]
    lam = lam0.copy()
    for n, piv in seen:
        others = [F[m] for m in range(3) if m != n]
        S = oracle.pivot_hadamard(others, piv)
        Ts = oracle.fused_flatten_sample(T, n, piv)
        F[n], lam = oracle.row_norm(oracle.sampled_solve(S, Ts, normal))
    for a, b in zip(cp.factors, F):
        assert rel(a, b) <= REPLAY_TOL
    assert rel(cp.lam, lam) <= REPLAY_TOL


def test_block_lev_score_sampled_converges(built, oracle):
    """test/rand_cp_als.jl:219-225: BlockLevScoreSampled(100, 1) and (100, 3) on the exact
    rank-5 12x13x3 target; best of five tries of 100 sweeps below 0.1 relative error."""
    T = target(oracle)
    F0, lam0 = det_factors(T.shape, 5, seed=32)
    for b in (1, 3):
        best = 1.0
        for t in range(5):
            cp = built.als_optimize(T, built.CPD([F.copy() for F in F0], lam0.copy(), T.shape),
                                    alg=built.BlockLevScoreSampled(100, b), check=built.NoCheck(100), normal=True,
                                    rng=np.random.default_rng(100 + t))
            best = min(best, rel(oracle.reconstruct(cp.factors, cp.lam), T))
        assert best < 0.1


@pytest.mark.parametrize("alg_name", ["LevScoreSampled", "BlockLevScoreSampled"])
def test_stop_resample_keeps_the_pivots(built, oracle, alg_name):
    """krp_lev_score_sampled.jl:24-25: a mode draws new pivots while stop_resample < 0 or
    stop_resample > iter(als); stop_resample = 0 keeps compute_als's draw for every sweep,
    stop_resample = 2 draws in the first two sweeps only."""
    T = target(oracle)
    F0, lam0 = det_factors(T.shape, 5, seed=32)
    alg = built.LevScoreSampled(50) if alg_name == "LevScoreSampled" else built.BlockLevScoreSampled(50, 2)
    for stop, fresh_sweeps in ((0, 0), (2, 2), (-1, 5)):
        seen = {n: [] for n in range(3)}
        built.als_optimize(T, built.CPD([F.copy() for F in F0], lam0.copy(), T.shape), alg=alg,
                           check=built.NoCheck(5), normal=True, rng=np.random.default_rng(7), stop_resample=stop,
                           on_pivots=lambda n, p: seen[n].append(p.copy()))
        for n in range(3):
            changes = sum(not np.array_equal(a, b) for a, b in zip(seen[n][:-1], seen[n][1:]))
            # sweeps 1.. reuse the previous pivots unless they draw (draws after the first sweep)
            assert changes == max(0, fresh_sweeps - 1)

"""The randomized path's gathers at the size of the order-4 workload: bit-exact.

The leverage-score sampled ALS on a 128^4 FP32 tensor at rank 128 draws 16384 sampled
Khatri-Rao rows per mode solve, with the indices drawn on the host (1-based, one column per
other mode).  The device gathers them: pivot_hadamard (src/algebra/had_contract.jl:277-295)
and fused_flatten_sample (src/algebra/pivot_mapping.jl:59-85).  Both are copies and products
in a fixed order, so each must equal the oracle's bit for bit at this size, for every mode.
The tensor holds seeded N(0,1) values (the gathers do not depend on the distribution).
"""
import numpy as np
import pytest

from _data import det_factors

pytestmark = pytest.mark.gpu

DIMS = (128, 128, 128, 128)
RANK = 128
NSAMPS = 16384


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def test_gathers_bit_exact_at_128_4_rank128_16384_samples(built, oracle):
    rng = np.random.default_rng(128)
    T = np.asfortranarray(rng.standard_normal(DIMS, dtype=np.float32))
    F, lam = det_factors(DIMS, RANK, seed=31)
    probs = [oracle.leverage_score_probabilities(f) for f in F]
    with built.Engine(DIMS, RANK, dtype=np.float32, precision="fp64") as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        for mode in range(4):
            piv = oracle.sample_factor_matrices(NSAMPS, mode, probs, rng)
            assert piv.shape == (NSAMPS, 3) and piv.min() >= 1 and piv.max() <= 128
            # the extreme coordinates are among the samples
            piv[0, :] = 1
            piv[1, :] = 128
            others = [F[m] for m in range(4) if m != mode]
            assert np.array_equal(eng.pivot_hadamard(mode, piv), oracle.pivot_hadamard(others, piv)), mode
            got = eng.fused_flatten_sample(mode, piv)
            assert got.dtype == np.float32 and got.shape == (128, NSAMPS)
            assert np.array_equal(got, oracle.fused_flatten_sample(T, mode, piv)), mode

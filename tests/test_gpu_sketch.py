"""The sparse sign embedding generator and the sketched matricization on the device.

The generator follows the reference's C generators' rules (src/algebra/sparse_sign.c,
src/algebra/sparsestack.c); its draws come from a counter-based stream, so the checks are
the structure (as test/SEQRCS_test.jl:13-18 checks it), reproducibility per seed, and the
distribution of rows and signs.  The sketched matricization
(src/algebra/pivot_mapping.jl:111-140) must equal the oracle's restatement and the dense
product T_(k) Omega^T within 1e-12 relative (FP64 sums in the reference's entry order).
"""
import numpy as np
import pytest

from _data import det_normal

pytestmark = pytest.mark.gpu

SKETCH_TOL = 1e-12


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def structure(l, n, s, rows1, vals, injective):
    a = 1.0 / np.sqrt(s)
    R = np.asarray(rows1[: n * s]).reshape(n, s) - 1
    assert R.min() >= 0 and R.max() < l
    assert np.all(np.abs(np.abs(vals[: n * s]) - a) < 1e-15)
    assert all(len(set(r)) == s for r in R)
    if injective:
        q, r = divmod(l, s)
        starts = np.array([j * (q + 1) if j < r else r * (q + 1) + (j - r) * q for j in range(s)])
        sizes = np.array([q + 1 if j < r else q for j in range(s)])
        assert np.all(R >= starts[None, :]) and np.all(R < (starts + sizes)[None, :])
    return R


@pytest.mark.parametrize("injective", [False, True])
def test_sparse_sign_structure_and_reproducibility(built, injective):
    """SEQRCS_test.jl:13-18: s nonzeros in every column, values +-1/sqrt(s); the same seed
    gives the same embedding, another seed another one."""
    for (l, n, s) in [(1200, 10000, 8), (50, 300, 4), (7, 40, 7), (13, 25, 5), (5, 9, 9)]:
        rows, vals = built.sparse_sign_matrix(l, n, s, injective=injective, seed=17)
        s_eff = min(s, l)
        structure(l, n, s_eff, rows, vals, injective)
        rows2, vals2 = built.sparse_sign_matrix(l, n, s, injective=injective, seed=17)
        ne = n * s_eff  # the generator clamps s to l (sparse_sign.c); entries past n * s_eff are untouched
        np.testing.assert_array_equal(rows[:ne], rows2[:ne])
        np.testing.assert_array_equal(vals[:ne], vals2[:ne])
        if ne > 64 and s_eff < l:
            rows3, _ = built.sparse_sign_matrix(l, n, s, injective=injective, seed=18)
            assert not np.array_equal(rows[:ne], rows3[:ne])
    om = built.sparse_sign_matrix(120, 500, 6, omega=True, injective=injective, seed=2)
    assert om.shape == (120, 500) and np.all(np.diff(om.indptr) == 6)


def test_sparse_sign_rows_and_signs_are_uniform(built):
    """Rows: each of l rows is hit n s / l times on average (chi-square within 6 sigma of its
    mean); signs: half positive within 6 sigma."""
    l, n, s = 97, 20000, 5
    rows, vals = built.sparse_sign_matrix(l, n, s, seed=23)
    counts = np.bincount(rows - 1, minlength=l)
    e = n * s / l
    chi2 = np.sum((counts - e) ** 2 / e)
    assert abs(chi2 - (l - 1)) < 6 * np.sqrt(2 * (l - 1))
    pos = np.mean(vals > 0)
    assert abs(pos - 0.5) < 6 * np.sqrt(0.25 / (n * s))


@pytest.mark.parametrize("dims,dt", [((3, 6, 8, 2), np.float64), ((30, 40, 20), np.float64), ((33, 17), np.float32),
                                     ((16, 9, 12, 5), np.float32)])
def test_sketched_matricization_matches_oracle(built, oracle, dims, dt):
    """pivot_mapping.jl:117-119: the sketch equals T_(k) Omega^T (and the oracle's
    restatement) in every mode."""
    T = np.asfortranarray(det_normal(sum(dims), dims).astype(dt))
    for k in range(len(dims)):
        n = int(np.prod([d for m, d in enumerate(dims) if m != k]))
        for (l, s, inj) in [(int(round(3 * dims[k] * np.log(dims[k]))) + 2, max(1, int(round(np.log(dims[k])))), False),
                            (7, 3, True)]:
            rows, vals = built.sparse_sign_matrix(l, n, s, injective=inj, seed=k + 1)
            s_eff = min(s, l)
            got = built.sketched_matricization(T, k, l, rows[: n * s_eff], vals[: n * s_eff], s_eff)
            ref = oracle.sketched_matricization(T.astype(np.float64), k, l, rows[: n * s_eff], vals[: n * s_eff], s_eff)
            dense = oracle.unfold(T.astype(np.float64), k) @ oracle.sparse_embedding(l, n, s_eff, rows, vals).T
            scale = max(1.0, np.linalg.norm(dense))
            assert np.linalg.norm(got - ref) <= SKETCH_TOL * scale
            assert np.linalg.norm(got - dense) <= SKETCH_TOL * scale


def test_sketch_keeps_singular_values(built):
    """test/SEQRCS_test.jl:20-28: a 10000 x 10 Gaussian matrix sketched to 1200 rows with 8
    nonzeros per column keeps its singular values within a factor [0.5, 1.5]."""
    m, n, s, l = 10, 10000, 8, 1200
    A = det_normal(77, (n, m))
    rows, vals = built.sparse_sign_matrix(l, n, s, seed=9)
    At = np.asfortranarray(A.T)  # the sketch of A's columns is the mode-0 sketch of A^T
    sk = built.sketched_matricization(At, 0, l, rows, vals, s)  # (m x l) = A^T Omega^T
    ratio = np.linalg.svd(sk.T, compute_uv=False) / np.linalg.svd(A, compute_uv=False)
    assert np.all((0.5 <= ratio) & (ratio <= 1.5))


def test_explicit_omega_forms(built, oracle):
    """pivot_mapping.jl:90-108 and had_contract.jl:300: the forms taking the sparse Omega
    (sparse_sign_matrix(...; omega=true)) give the entry forms' results."""
    dims = (6, 7, 5)
    T = np.asfortranarray(det_normal(41, dims))
    n = 7 * 5
    l, s = 20, 3
    rows, vals = built.sparse_sign_matrix(l, n, s, seed=4)
    om = built.sparse_sign_matrix(l, n, s, seed=4, omega=True)
    np.testing.assert_array_equal(built.sketched_matricization(T, 0, om),
                                  built.sketched_matricization(T, 0, l, rows, vals, s))
    mats = [det_normal(42, (7, 4)), det_normal(43, (5, 4))]
    np.testing.assert_array_equal(built.omega_hadamard(mats, om), built.omega_hadamard(mats, rows, vals, l, s))

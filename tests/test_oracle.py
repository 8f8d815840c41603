"""The oracle pinned against the reference's own known-answer tests (CPU only).

Each test re-expresses one test of ITensorCPD.jl with its literal inputs where the
reference gives them (test/pivot_mapping.jl, test/basic_features.jl, test/cp_als.jl).
"""
import json

import numpy as np
import pytest

from _data import det_factors, det_normal


def test_column_to_multi_coords_literal_pivots(oracle, golden_dir):
    # test/pivot_mapping.jl:6-43: T_matrix[a, pivot] == T[a, coords...] for literal pivots
    for case in json.loads((golden_dir / "index_maps.json").read_text()):
        coords = oracle.column_to_multi_coords(case["pivots"], case["col_dims"])
        assert coords.tolist() == case["coords"]
        dims, k = case["tensor_dims"], case["mode"] - 1
        T = np.asfortranarray(det_normal(5, dims))
        Tm = oracle.unfold(T, k)
        for p, c in zip(case["pivots"], coords):
            idx = list(c - 1)
            idx.insert(k, slice(None))
            assert np.array_equal(Tm[:, p - 1], T[tuple(idx)])


def test_multi_coords_round_trip(oracle):
    # test/pivot_mapping.jl:105-107
    rng = np.random.default_rng(0)
    dims = (100, 150, 200)
    p = rng.integers(1, 100 * 150 * 200 + 1, size=200)
    multi = oracle.column_to_multi_coords(p, dims)
    assert np.array_equal(oracle.multi_coords_to_column(dims, multi), p)


def test_pivot_hadamard_equals_krp_rows(oracle):
    # test/pivot_mapping.jl:46-103: sampled rows of the explicit KRP, exactly
    A = det_normal(1, (100, 20))
    B = det_normal(2, (150, 20))
    C = det_normal(3, (200, 20))
    exact = oracle.khatri_rao([A, B])
    p = np.arange(1, 100 * 150 + 1)
    piv = oracle.column_to_multi_coords(p, (100, 150))
    assert np.array_equal(oracle.pivot_hadamard([A, B], piv), exact)
    rng = np.random.default_rng(1)
    p = rng.integers(1, 100 * 150 * 200 + 1, size=200)
    piv = oracle.column_to_multi_coords(p, (100, 150, 200))
    exact3 = oracle.khatri_rao([A, B, C])
    loop = np.empty((200, 20))
    for s in range(200):
        for r in range(20):
            loop[s, r] = A[piv[s, 0] - 1, r] * B[piv[s, 1] - 1, r] * C[piv[s, 2] - 1, r]
    got = oracle.pivot_hadamard([A, B, C], piv)
    assert np.array_equal(got, loop)
    assert np.array_equal(got, exact3[p - 1])


def test_fused_flatten_sample_equals_fibres(oracle):
    # test/pivot_mapping.jl:103: fibres of the KRP tensor along mode 4
    A, B, C = det_normal(1, (10, 6)), det_normal(2, (15, 6)), det_normal(3, (20, 6))
    Kt = np.reshape(oracle.khatri_rao([A, B, C]), (10, 15, 20, 6), order="F")
    rng = np.random.default_rng(2)
    piv = oracle.column_to_multi_coords(rng.integers(1, 3001, size=50), (10, 15, 20))
    got = oracle.fused_flatten_sample(np.asfortranarray(Kt), 3, piv)
    assert got.shape == (6, 50)
    for s in range(50):
        a, b, c = piv[s] - 1
        assert np.array_equal(got[:, s], Kt[a, b, c, :])
    # a middle mode
    T = np.asfortranarray(det_normal(4, (5, 6, 7, 8)))
    piv = np.stack([rng.integers(1, d + 1, size=9) for d in (5, 7, 8)], axis=1)
    got = oracle.fused_flatten_sample(T, 1, piv)
    for s in range(9):
        assert np.array_equal(got[:, s], T[piv[s, 0] - 1, :, piv[s, 1] - 1, piv[s, 2] - 1])


def test_khatri_rao_matches_loops(oracle):
    # test/basic_features.jl:18-58: had_contract(A, B, r) against explicit loops
    A, B = det_normal(1, (20, 40)), det_normal(2, (30, 40))
    K = oracle.khatri_rao([A, B])
    D = np.empty((20, 30, 40))
    for n in range(40):
        for l_ in range(20):
            for m in range(30):
                D[l_, m, n] = A[l_, n] * B[m, n]
    assert np.linalg.norm(K - D.reshape(600, 40, order="F")) / np.linalg.norm(D) < 1e-7


def test_reconstruct_matches_loops(oracle):
    # test/basic_features.jl:60-92
    A, B, C = det_normal(1, (20, 10)), det_normal(2, (30, 10)), det_normal(3, (40, 10))
    lam = det_normal(4, (10,))
    exact = np.einsum("r,ir,jr,kr->ijk", lam, A, B, C)
    rec = oracle.reconstruct([A, B, C], lam)
    assert abs(1.0 - np.linalg.norm(exact - rec) / np.linalg.norm(exact) - 1.0) <= 5 * np.finfo(float).eps


def test_row_norm_unit_columns(oracle):
    # test/basic_features.jl:1-16
    F, lam = oracle.row_norm(det_normal(7, (20, 30)))
    assert np.allclose(np.sum(F * F, axis=0), 1.0)
    assert np.allclose(lam, np.linalg.norm(det_normal(7, (20, 30)), axis=0))


def test_mttkrp_forms_agree(oracle):
    # KRPFreeNormal (per-r chains) and KRPNormal (explicit KRP) compute the same MTTKRP
    T = np.asfortranarray(det_normal(8, (4, 5, 6, 3)))
    F, _ = det_factors(T.shape, 7, seed=9)
    for n in range(4):
        a = oracle.mttkrp_krp_free(T, F, n)
        b = oracle.mttkrp_krp(T, F, n)
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-13


def test_pivoted_cholesky_solve_and_fallback(oracle):
    # ldiv_solve.jl:13-29: full-rank SPD -> pivoted Cholesky; singular -> pivoted QR
    X = det_normal(3, (30, 6))
    V = X.T @ X
    B = det_normal(4, (6, 9))
    sol, fb = oracle.ldiv_solve(V, B)
    assert not fb
    assert np.allclose(sol, np.linalg.solve(V, B), rtol=1e-10, atol=1e-12)
    X[:, 5] = X[:, 4]
    V = X.T @ X
    sol, fb = oracle.ldiv_solve(V, V @ B)
    assert fb
    assert np.allclose(V @ sol, V @ B, atol=1e-8)


def test_fitcheck_control_flow(oracle):
    # fit_check.jl:24-66: converge after two consecutive |dfit| < tol; iter resets
    chk = oracle.FitCheck(1e-3, 10, 1.0)
    lam = np.array([1.0])
    F = [np.ones((1, 1))]
    seq = []

    def run(inner):
        chk.MttKRP = np.array([[inner]])
        return chk.check_converge(F, lam, [np.ones((1, 1))], verbose=False)

    # ||X||^2 = 1, ref = 1: fit = 1 - sqrt(|2 - 2 inner|), so inner = 1 - (1 - fit)^2 / 2;
    # fits 0, 0.5, 0.9, 0.9995, 0.9999, 0.99995: |dfit| < 1e-3 on the last two sweeps only
    for fit in (0.0, 0.5, 0.9, 0.9995, 0.9999, 0.99995):
        inner = 1.0 - (1.0 - fit) ** 2 / 2.0
        seq.append(run(inner))
    assert seq == [False, False, False, False, False, True]
    assert chk.iter == 0 and chk.total_iter == 6 and chk.counter == 0 and chk.lastfit == 0.0
    with pytest.raises(FloatingPointError):
        run(np.nan)


def test_leverage_scores(oracle):
    F, _ = det_factors((40, 7), 7, seed=5)
    p = oracle.leverage_score_probabilities(F[0])
    assert p.shape == (40,)
    assert np.isclose(p.sum(), 1.0)
    Q, _ = np.linalg.qr(F[0])
    assert np.allclose(p, np.sum(Q * Q, axis=1) / 7)


def test_leverage_scores_wide_factor(oracle):
    # I < R: the thin QR's Q is square and orthogonal, every row scores 1 / I (the device takes
    # them from the leading rank x rank block of the pivoted Cholesky factor, rank = I)
    F, _ = det_factors((40, 90, 80), 70, seed=5)
    p = oracle.leverage_score_probabilities(F[0])
    assert np.allclose(p, 1.0 / 40, rtol=0, atol=1e-14)


def test_golden_fixtures_reproduce(oracle, golden_dir):
    small = json.loads((golden_dir / "als_small.json").read_text())
    T = np.asfortranarray(det_normal(small["tensor_seed"], small["dims"]))
    F, lam = det_factors(small["dims"], small["rank"], seed=small["factor_seed"])
    chk = oracle.FitCheck(small["tol"], small["max_counter"], float(np.linalg.norm(T)))
    oracle.als_optimize(T, F, lam, check=chk)
    assert np.allclose(chk.trajectory, small["trajectory"], rtol=0, atol=1e-12)


def test_cp_als_overcomplete_rank400(oracle):
    # test/cp_als.jl:9-10: 20x30x40 FP64, rank 400, 100 NoCheck sweeps -> rel err < 1e-7
    T = np.asfortranarray(det_normal(40, (20, 30, 40)))
    F, lam = det_factors(T.shape, 400, seed=3)
    Ff, lf, _, _ = oracle.als_optimize(T, F, lam, check=oracle.NoCheck(100))
    assert np.linalg.norm(oracle.reconstruct(Ff, lf) - T) / np.linalg.norm(T) < 1e-7


def test_lev_score_sampled_converges(oracle):
    # test/rand_cp_als.jl:98-121: exact rank-5 12x13x3 target, LevScoreSampled(100);
    # best of three tries (the reference's multiple_tries helper, rand_cp_als.jl:1-14)
    dims = (12, 13, 3)
    Ft, lt = det_factors(dims, 5, seed=31)
    T = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F, lam = det_factors(dims, 5, seed=32)
    best = 1.0
    for trial in range(3):
        Ff, lf = oracle.lev_score_als(T, F, lam, 100, 100, np.random.default_rng(100 + trial), normal=True)
        best = min(best, np.linalg.norm(oracle.reconstruct(Ff, lf) - T) / np.linalg.norm(T))
    assert best < 0.1
    # the sampled system is consistent for an exact target: from the true factors a
    # sampled sweep reproduces them
    Ff, lf = oracle.lev_score_als(T, Ft, lt, 100, 1, np.random.default_rng(7), normal=False)
    assert np.linalg.norm(oracle.reconstruct(Ff, lf) - T) / np.linalg.norm(T) < 1e-10


def test_cp_cp_inner_is_the_dense_inner_product(oracle):
    # cp_contract.jl:32-52 contracted with both lambdas equals <reconstruct(P), reconstruct(F)>
    dims = (6, 5, 4)
    P, lp = det_factors(dims, 3, seed=41)
    F, lf = det_factors(dims, 4, seed=42)
    dense = float(np.sum(oracle.reconstruct(P, lp) * oracle.reconstruct(F, lf)))
    assert abs(oracle.cp_cp_inner(P, lp, F, lf) - dense) <= 1e-12 * abs(dense)
    assert abs(oracle.norm_factors([X.T @ X for X in F], lf) - float(np.sum(oracle.reconstruct(F, lf) ** 2))) <= 1e-10


def test_diff_and_angle_checks_on_a_fixed_iterate(oracle):
    # cp_diff_check.jl / cp_angle_check.jl: the first call stores PrevCP.  An unchanged
    # iterate has fit 1, which already differs from the initial lastfit 1 by less than tol, so
    # CPDiffCheck stops on call 3; its angle 0 differs from the initial lastangle 1, so
    # CPAngleCheck counts from call 3 and stops on call 4.  Both reset their state.
    dims = (7, 6, 5)
    F, lam = det_factors(dims, 3, seed=43)
    for cls, value, calls in ((oracle.CPDiffCheck, 1.0, 3), (oracle.CPAngleCheck, 0.0, 4)):
        chk = cls(1e-6, 10)
        results = [chk.check_converge(F, lam) for _ in range(calls)]
        assert results == [False] * (calls - 1) + [True]
        assert chk.PrevCP is None and chk.iter == 0 and chk.counter == 0 and chk.total_iter == calls
        assert abs(chk.final_fit - value) <= 1e-7
        assert np.isnan(chk.trajectory[0])


def test_diff_check_resets_at_max_counter(oracle):
    # cp_diff_check.jl:58-66: reaching max_counter resets iter, counter, lastfit and PrevCP
    dims = (5, 4, 3)
    chk = oracle.CPDiffCheck(1e-12, 3)
    for k in range(3):
        F, lam = det_factors(dims, 2, seed=50 + k)
        assert chk.check_converge(F, lam) is False
    assert chk.iter == 0 and chk.total_iter == 3 and chk.PrevCP is None and chk.lastfit == 0.0
    assert chk.final_fit == chk.trajectory[-1]


@pytest.mark.parametrize("impl", ["api", "oracle"])
def test_block_sampling_structure_and_block_weights(oracle, pkg, impl):
    # probability.jl:61-108 with I = 13 and block_size 5: two blocks of 6 (13 // 5 = 2,
    # 13 % 5 = 3 > 2 so both are one longer), starting at 1 and 7; index 13 is never drawn
    # inside a block.  Block draws follow the summed leverage weights of each block.
    rng = np.random.default_rng(9)
    probs = [np.abs(rng.standard_normal(d)) for d in (13, 9, 4)]
    sampler = pkg.block_sample_factor_matrices if impl == "api" else oracle.block_sample_factor_matrices
    nsamps, b = 6000, 5
    S = sampler(nsamps, probs, b, 2, np.random.default_rng(1))  # skip mode 2: mode 0 is blocked
    assert S.shape == (nsamps, 2) and S.dtype == np.int64
    assert S[:, 0].min() >= 1 and S[:, 0].max() <= 13 and S[:, 1].min() >= 1 and S[:, 1].max() <= 9
    w = probs[0] / probs[0].sum()
    bprob = np.array([w[0:6].sum(), w[6:12].sum()])
    starts = []
    # 6000 // 5 = 1200 block draws of 6 rows each overflow nsamps after 1000 blocks
    i = 0
    while i < nsamps:
        s0 = S[i, 0]
        assert s0 in (1, 7)
        n = min(6, nsamps - i)
        np.testing.assert_array_equal(S[i:i + n, 0], s0 + np.arange(n))
        assert np.all(S[i:i + n, 1] == S[i, 1])
        starts.append(s0)
        i += n
    assert len(starts) == 1000
    freq = np.mean(np.array(starts) == 1)
    assert abs(freq - bprob[0]) < 4 * np.sqrt(bprob[0] * bprob[1] / len(starts))


@pytest.mark.parametrize("impl", ["api", "oracle"])
def test_block_sampling_fills_the_tail_with_independent_draws(oracle, pkg, impl):
    # block size 4 on a mode of 10: 10 // 4 = 2 blocks, 10 % 4 = 2 so both have 5 indices
    # (starts 1 and 6).  nsamps 11 gives 11 // 4 = 2 block draws, i.e. rows 1-5 and 6-10,
    # and row 11 is an independent draw.  nsamps below the block size gives only
    # independent draws.
    probs = [np.ones(10), np.ones(6), np.ones(3)]
    sampler = pkg.block_sample_factor_matrices if impl == "api" else oracle.block_sample_factor_matrices
    S = sampler(11, probs, 4, 1, np.random.default_rng(2))  # skip mode 1: mode 0 is blocked
    for r0 in (0, 5):
        assert S[r0, 0] in (1, 6)
        np.testing.assert_array_equal(S[r0:r0 + 5, 0], S[r0, 0] + np.arange(5))
        assert np.all(S[r0:r0 + 5, 1] == S[r0, 1])
    assert 1 <= S[10, 0] <= 10 and 1 <= S[10, 1] <= 3
    S = sampler(3, probs, 4, 0, np.random.default_rng(3))  # skip mode 0: mode 1 is blocked
    assert S.shape == (3, 2) and S[:, 0].max() <= 6 and S[:, 1].max() <= 3


def test_block_sampling_rejects_blocks_longer_than_the_mode(pkg):
    with pytest.raises(ValueError):
        pkg.block_sample_factor_matrices(20, [np.ones(3), np.ones(4), np.ones(5)], 5, 2, np.random.default_rng(0))
    with pytest.raises(ValueError):
        pkg.block_sample_factor_matrices(20, [np.ones(3), np.ones(4)], 0, 1, np.random.default_rng(0))


def test_block_lev_score_sampled_converges(oracle):
    # test/rand_cp_als.jl:219-225: BlockLevScoreSampled(100, 1) and (100, 3) on the exact
    # rank-5 12x13x3 target reach a relative error below 0.1 (best of three tries, 100 sweeps)
    dims = (12, 13, 3)
    Ft, lt = det_factors(dims, 5, seed=31)
    T = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F, lam = det_factors(dims, 5, seed=32)
    for b in (1, 3):
        best = min(np.linalg.norm(oracle.reconstruct(*oracle.lev_score_als(
            T, F, lam, 100, 100, np.random.default_rng(100 + t), normal=True, block_size=b)) - T) / np.linalg.norm(T)
            for t in range(3))
        assert best < 0.1


def _embedding_structure(l, n, s, rows0, vals, injective):
    """The structure both reference generators produce (sparse_sign.c, sparsestack.c)."""
    a = 1.0 / np.sqrt(s)
    R = np.asarray(rows0[: n * s]).reshape(n, s)
    assert R.min() >= 0 and R.max() < l
    assert np.all(np.abs(np.abs(np.asarray(vals[: n * s])) - a) < 1e-15)
    assert all(len(set(r)) == s for r in R)  # distinct rows in every column
    if injective:  # one row in each of s near-equal blocks, in block order
        q, r = divmod(l, s)
        starts = np.array([j * (q + 1) if j < r else r * (q + 1) + (j - r) * q for j in range(s)])
        sizes = np.array([q + 1 if j < r else q for j in range(s)])
        assert np.all(R >= starts[None, :]) and np.all(R < (starts + sizes)[None, :])


@pytest.mark.parametrize("injective", [False, True])
def test_reference_sparse_sign_generators_structure(oracle, injective):
    # the reference's own C generators, compiled from its sources by oracle/build_oracle.py:
    # these are the rules the device generator must follow (SEQRCS_test.jl:13-18)
    ref = oracle.load_ref_sparse_sign()
    if ref is None:
        pytest.skip("reference generators not built (no reference checkout)")
    fn = ref[1] if injective else ref[0]
    for (l, n, s) in [(1200, 1000, 8), (50, 300, 4), (7, 40, 7), (13, 25, 5)]:
        rows = np.empty(n * s, np.int32)
        vals = np.empty(n * s)
        cs = np.empty(n + 1, np.int32)
        fn(l, n, s, vals, rows, cs, seed=11)
        np.testing.assert_array_equal(cs, np.arange(n + 1) * s)
        _embedding_structure(l, n, s, rows, vals, injective)


def test_oracle_sketched_matricization_is_the_dense_product(oracle):
    # test/pivot_mapping.jl:110-119 and test/SEQRCS_test.jl:24-25: the sketch equals
    # T_(k) Omega^T; Omega from the reference generator when it is built
    rng = np.random.default_rng(4)
    ref = oracle.load_ref_sparse_sign()
    for dims in [(3, 6, 8, 2), (7, 5), (4, 3, 5)]:
        T = np.asfortranarray(rng.standard_normal(dims))
        for k in range(len(dims)):
            n = int(np.prod([d for m, d in enumerate(dims) if m != k]))
            l, s = 11, 3
            rows = np.empty(n * s, np.int32)
            vals = np.empty(n * s)
            if ref is not None:
                ref[0](l, n, s, vals, rows, np.empty(n + 1, np.int32), seed=5 + k)
            else:
                rows[:] = np.concatenate([rng.choice(l, s, replace=False) for _ in range(n)])
                vals[:] = rng.choice([-1.0, 1.0], n * s) / np.sqrt(s)
            om = oracle.sparse_embedding(l, n, s, rows + 1, vals)
            want = oracle.unfold(T, k) @ om.T
            got = oracle.sketched_matricization(T, k, l, rows + 1, vals, s)
            assert np.linalg.norm(got - want) <= 1e-12 * max(1.0, np.linalg.norm(want))


# ---- column-pivoted QR, omega_hadamard, SE-QRCS (oracle restatements) ----
def _np_sparse_sign(l, n, s, rng):
    """A sparse_sign-layout embedding drawn with numpy (s distinct rows per column), 1-based."""
    rows = np.concatenate([rng.choice(l, size=s, replace=False) for _ in range(n)]).astype(np.int32) + 1
    vals = np.where(rng.random(n * s) < 0.5, -1.0, 1.0) / np.sqrt(s)
    return rows, vals


@pytest.mark.parametrize("shape", [(30, 50), (50, 30), (7, 7), (1, 9), (9, 1), (40, 200)])
def test_qrcp_loop_is_lapack_geqp3(oracle, shape):
    """The step-by-step restatement (the device's rule: largest partial norm, xLAQP2 downdating)
    picks the pivots LAPACK's xGEQP3 picks, and the same R and Q."""
    A = np.random.default_rng(sum(shape)).standard_normal(shape)
    p, rd, R, Q = oracle.qrcp_loop(A)
    Q2, R2, p2 = oracle.qrcp_lapack(A)
    np.testing.assert_array_equal(p, p2)
    np.testing.assert_allclose(R, R2, rtol=0, atol=1e-13 * np.abs(A).max())
    np.testing.assert_allclose(Q, Q2, rtol=0, atol=1e-13)
    np.testing.assert_allclose(rd, np.diag(R2), rtol=1e-13)


def test_qrcp_loop_low_rank_and_early_stop(oracle):
    """Rank 5 plus 1e-9 noise: the same pivots as xGEQP3 throughout; a stopping ratio ends the
    run one step after the last |r_jj| above it (optimizers/.../randomized/qr_lev_score_sampled.jl:28 counts meff)."""
    rng = np.random.default_rng(4)
    A = rng.standard_normal((40, 5)) @ rng.standard_normal((5, 300)) + 1e-9 * rng.standard_normal((40, 300))
    p, rd, _, _ = oracle.qrcp_loop(A)
    _, R2, p2 = oracle.qrcp_lapack(A)
    np.testing.assert_array_equal(p, p2)
    assert oracle.effective_rank(rd, 0.01) == oracle.effective_rank(np.diag(R2), 0.01) == 5
    p3, rd3, _, _ = oracle.qrcp_loop(A, stop_ratio=0.01)
    assert rd3.size == 6 and oracle.effective_rank(rd3, 0.01) == 5
    np.testing.assert_array_equal(p3[:6], p2[:6])
    p4, _, _, _ = oracle.qrcp_loop(A, ncand=100)
    assert set(p4[:40]) <= set(range(1, 101))


def test_oracle_omega_hadamard_is_the_dense_product(oracle):
    """test/pivot_mapping.jl:120-160: omega_hadamard(factors, Omega) = Omega * KRP."""
    rng = np.random.default_rng(5)
    mats = [rng.standard_normal((d, 10)) for d in (3, 6, 8)]
    n = 3 * 6 * 8
    l, s = 31, 3
    rows, vals = _np_sparse_sign(l, n, s, rng)
    got = oracle.omega_hadamard(mats, l, s, rows, vals)
    ref = oracle.sparse_embedding(l, n, s, rows, vals) @ oracle.khatri_rao(mats)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def _qr_error(A, Q, R, p, k):
    return np.linalg.norm(A[:, p - 1] - Q[:, :k] @ R[:k, :], 2) / np.linalg.norm(A, 2)


def test_oracle_seqrcs_reference_property(oracle):
    """test/SEQRCS_test.jl:32-47: for a 50 x 10000 Gaussian matrix, the rank-40 error of SE-QRCS
    (l = 2500, s = 1, t = 40; both subset orders) is within 1e-2 of the pivoted QR's."""
    rng = np.random.default_rng(6)
    A = rng.standard_normal((50, 10000))
    k = 40
    Qa, Ra, pa = oracle.qrcp_lapack(A)
    err_act = _qr_error(A, Qa, Ra, pa, k)
    T = np.asfortranarray(A)
    for use_omega in (False, True):
        rows, vals = _np_sparse_sign(2500, 10000, 1, rng)
        Q, R, p, rd = oracle.seqrcs(T, 0, 2500, 1, 40, rows, vals, use_omega=use_omega)
        assert sorted(p) == list(range(1, 10001))
        assert abs(_qr_error(A, Q, R, p, k) - err_act) <= 1e-2
        np.testing.assert_allclose(np.abs(rd), np.abs(np.diag(R)[: rd.size]), rtol=1e-14)


def test_oracle_seqrcs_of_the_krp(oracle):
    """test/SEQRCS_test.jl:49-64 compares SE-QRCS of a KRP given by its factors with SE-QRCS of
    the explicit KRP matrix (rank-40 errors within 1e-2, each with its own embedding).  With
    the same embedding the two are the same computation (the KRP path selects its subset in
    column order, as the matrix path does with the explicit Omega), so the pivots agree and the
    errors agree to rounding."""
    rng = np.random.default_rng(7)
    mats = [rng.standard_normal((100, 50)), rng.standard_normal((100, 50))]
    K = oracle.khatri_rao(mats)  # 10000 x 50
    Kt = np.asfortranarray(K.T)
    rows, vals = _np_sparse_sign(2500, 10000, 1, rng)
    Q, R, p, _ = oracle.seqrcs(Kt, 0, 2500, 1, 40, rows, vals, use_omega=True)
    Qf, Rf, pf, _ = oracle.seqrcs_krp(mats, 2500, 1, 40, rows, vals)
    np.testing.assert_array_equal(pf, p)
    assert abs(_qr_error(Kt, Qf, Rf, pf, 40) - _qr_error(Kt, Q, R, p, 40)) <= 1e-10


def test_qrcp_golden_pivots(oracle, golden_dir):
    """The committed xGEQP3 pivots (tests/golden/qrcp_pivots.json): scipy's LAPACK and the
    step-by-step restatement both reproduce them."""
    from _data import golden_qrcp_matrix

    for case in json.loads((golden_dir / "qrcp_pivots.json").read_text()):
        A = golden_qrcp_matrix(case)
        k = case["compare"]
        _, R, p = oracle.qrcp_lapack(A)
        p2, rd, _, _ = oracle.qrcp_loop(A)
        np.testing.assert_array_equal(p[:k], case["p"][:k], err_msg=case["name"])
        np.testing.assert_array_equal(p2[:k], case["p"][:k], err_msg=case["name"])
        np.testing.assert_allclose(np.abs(rd[:k]), case["absdiag"][:k], rtol=0, atol=1e-12 * np.linalg.norm(A))


def test_seqrcs_golden(oracle, golden_dir):
    """tests/golden/seqrcs_small.json: SE-QRCS of a seeded tensor with a stored embedding."""
    g = json.loads((golden_dir / "seqrcs_small.json").read_text())
    T = np.asfortranarray(det_normal(g["seed"], g["tensor_dims"]))
    for case in g["cases"]:
        _, _, p, rd = oracle.seqrcs(T, g["mode"], g["l"], g["s"], g["t"], np.asarray(g["rows"]),
                                    np.asarray(g["vals"]), use_omega=case["use_omega"], compute_r=False)
        np.testing.assert_array_equal(p, case["p"])
        np.testing.assert_allclose(np.abs(rd), case["absdiag"], rtol=0, atol=1e-12 * np.linalg.norm(T))


def test_oracle_pivot_solvers_interpolate_a_known_low_rank(oracle):
    """test/rand_cp_als.jl:72-96 on the oracle: a rank-10 model of an exactly rank-20 20x30x40
    tensor under CPDiffCheck(1e-5, 100).  QRPivProjected(1200) and KSEQRCSPivProjected((1),
    (1200,), (1,2,3), 5) (best of up to ten tries, rand_cp_als.jl:1-14) reach errors within 10%
    of exact ALS's."""
    dims = (20, 30, 40)
    Ft, lt = det_factors(dims, 20, seed=21)
    A = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F0, l0 = det_factors(dims, 10, seed=22)

    def err(F, lam):
        return np.linalg.norm(A - oracle.reconstruct(F, lam)) / np.linalg.norm(A)

    Fe, le, _, _ = oracle.als_optimize(A, F0, l0, check=oracle.CPDiffCheck(1e-5, 100))
    exact = err(Fe, le)
    proj, eff, refs = oracle.pivot_solver_setup(A, "qr", end=1200, rng=np.random.default_rng(1))
    assert [p.shape[0] for p in proj] == [1200, 800, 600]
    assert all(sorted(r) == list(range(1, r.size + 1)) for r in refs)
    Fq, lq = oracle.projected_als_check(A, F0, l0, proj, oracle.CPDiffCheck(1e-5, 100))
    assert abs(exact - err(Fq, lq)) / exact < 0.1
    ok = False
    for i in range(10):
        rng = np.random.default_rng(100 + i)
        Fp, lp = oracle.kseqrcs_prelim(A, F0, l0, rng)
        proj, eff, _ = oracle.pivot_solver_setup(A, "kseqrcs", end=1200, random_modes=(1, 2, 3),
                                                 rank_vect={1: 5, 2: 5, 3: 5}, rng=rng, krp_factors=Fp)
        Fk, lk = oracle.projected_als_check(A, F0, l0, proj, oracle.CPDiffCheck(1e-5, 100))
        if abs(exact - err(Fk, lk)) / exact < 0.1:
            ok = True
            break
    assert ok
    # With end = 1200 every mode keeps all its columns, so the runs above equal exact ALS.
    # With fewer pivots the projection is real: 400 pivots per mode (a third to two thirds of
    # the columns) keep both solvers, and 200 keep QRPivProjected, within 10% of exact ALS.
    for kind, end in (("qr", 400), ("qr", 200), ("kseqrcs", 400)):
        rng = np.random.default_rng(5)
        kw = {}
        if kind == "kseqrcs":
            Fp, lp = oracle.kseqrcs_prelim(A, F0, l0, rng)
            kw = dict(random_modes=(1, 2, 3), rank_vect={1: 5, 2: 5, 3: 5}, krp_factors=Fp)
        proj, _, _ = oracle.pivot_solver_setup(A, kind, end=end, rng=rng, **kw)
        assert all(p.shape[0] == end for p in proj)
        F, lam = oracle.projected_als_check(A, F0, l0, proj, oracle.CPDiffCheck(1e-5, 100))
        assert abs(exact - err(F, lam)) / exact < 0.1, (kind, end)


def test_oracle_np_sparse_sign_layouts(oracle):
    """The oracle's numpy embedding follows the generators' two layouts (sparse_sign.c,
    sparsestack.c) and clamps s to l."""
    rng = np.random.default_rng(4)
    for inj in (False, True):
        rows, vals, s = oracle.np_sparse_sign(17, 60, 4, rng, injective=inj)
        R = rows.reshape(60, 4) - 1
        assert s == 4 and R.min() >= 0 and R.max() < 17
        assert all(len(set(r)) == 4 for r in R)
        assert np.all(np.abs(vals) == 0.5)
        if inj:
            q, r = divmod(17, 4)
            starts = [j * (q + 1) if j < r else r * (q + 1) + (j - r) * q for j in range(4)]
            ends = [starts[j] + (q + 1 if j < r else q) for j in range(4)]
            assert all(starts[j] <= R[c, j] < ends[j] for c in range(60) for j in range(4))
    rows, vals, s = oracle.np_sparse_sign(3, 5, 7, rng)
    assert s == 3 and all(sorted(r) == [1, 2, 3] for r in rows.reshape(5, 3))


def test_oracle_pivot_solvers_rank400_against_exact_als(oracle):
    """test/rand_cp_als.jl:38-70 on the oracle: 20x30x40 Gaussian tensor, rank 400,
    FitCheck(1e-6, 20) (not evaluated by the projection solvers: 20 sweeps).  QRPivProjected(800)
    with trunc_tol 0.001 reconstructs within 1e-2 of exact ALS, SEQRCSPivProjected(1, 800,
    (1,2,3), (100,100,100)) within 1e-1 (normal equations; the tall form is the same
    least-squares problem and the GPU tests run it)."""
    dims = (20, 30, 40)
    T = np.asfortranarray(det_normal(5, dims))
    F, lam = det_factors(dims, 400, seed=6)
    nT = float(np.linalg.norm(T))
    Fe, le, _, _ = oracle.als_optimize(T, F, lam, check=oracle.FitCheck(1e-6, 20, nT))
    ref = oracle.reconstruct(Fe, le)
    for kind, tol, bound, kw in (("qr", 0.001, 1e-2, {}),
                                 ("seqrcs", 0.01, 1e-1, dict(random_modes=(1, 2, 3),
                                                             rank_vect={1: 100, 2: 100, 3: 100}))):
        proj, _, _ = oracle.pivot_solver_setup(T, kind, end=800, trunc_tol=tol, rng=np.random.default_rng(2), **kw)
        Fp, lp = oracle.projected_als_check(T, F, lam, proj, oracle.FitCheck(1e-6, 20, nT))
        assert np.linalg.norm(ref - oracle.reconstruct(Fp, lp)) / np.linalg.norm(ref) < bound, kind


@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-10), (np.float32, 2e-5)])
def test_compiled_cpu_baseline_follows_the_oracle(oracle, dt, tol):
    # the C++/OpenMP GEMM-form ALS (the bench's compiled CPU baseline) gives the oracle's fit
    # trajectory: the same algorithm, the MTTKRP in another summation order (and, for FP32
    # tensors, FP32 products)
    import importlib.util

    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    spec = importlib.util.spec_from_file_location("build_oracle", root / "oracle" / "build_oracle.py")
    bo = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bo)
    if bo.build_cpu() is None:
        pytest.skip("g++ not available")
    rng = np.random.default_rng(12)
    dims, R = (23, 19, 17), 6
    T = np.asfortranarray(rng.standard_normal(dims).astype(dt))
    F, lam = oracle.random_factors(dims, R, np.random.default_rng(3))
    ref_norm = float(np.linalg.norm(T.astype(np.float64)))
    chk = oracle.FitCheck(0.0, 8, ref_norm)
    oracle.als_optimize(T.astype(np.float64), F, lam, check=chk, alg="krp", work_dtype=np.float64)
    Fc, lc, fits = oracle.cpu_als_sweeps(T, F, lam, 8, ref_norm, threads=4)
    assert np.max(np.abs(fits - np.asarray(chk.trajectory))) < tol

"""Column-pivoted QR, SE-QRCS and the QR-pivoted projection solvers on the device.

The pivots must be LAPACK xGEQP3's (the reference calls qr(A, ColumnNorm())): on matrices
whose column norms do not tie to rounding the whole permutation is compared for equality,
and R and Q within 1e-12 of ||A||.  SE-QRCS (src/algebra/SEQRCS.jl) is compared with the
oracle's restatement on the same embedding; the solvers follow test/rand_cp_als.jl.
"""
import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu

QR_TOL = 1e-12


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def close_qr(res, Q2, R2, A):
    nrm = np.linalg.norm(A)
    np.testing.assert_allclose(res.R, R2, rtol=0, atol=QR_TOL * nrm)
    np.testing.assert_allclose(res.Q, Q2, rtol=0, atol=1e-10)


@pytest.mark.parametrize("shape", [(30, 50), (50, 30), (7, 7), (1, 9), (9, 1), (64, 3000), (300, 700), (1100, 1200)])
def test_qrcp_matches_lapack(built, oracle, shape):
    """Every step path: columns of at most 128, 512, 1024 rows in registers, longer ones in two passes."""
    A = det_normal(sum(shape), shape)
    res = built.qrcp(A)
    Q2, R2, p2 = oracle.qrcp_lapack(A)
    np.testing.assert_array_equal(res.p, p2)
    assert res.steps == min(shape)
    close_qr(res, Q2, R2, A)
    np.testing.assert_allclose(res.rdiag, np.diag(R2), rtol=0, atol=QR_TOL * np.linalg.norm(A))


def test_qrcp_options_match_the_loop(built, oracle):
    """ncand, max_steps and stop_ratio as the oracle's step-by-step loop runs them."""
    A = det_normal(3, (50, 80))
    for kw in (dict(ncand=30), dict(max_steps=10), dict(ncand=30, max_steps=7)):
        res = built.qrcp(A, **kw)
        p, rd, R, Q = oracle.qrcp_loop(A, kmax=kw.get("max_steps"), ncand=kw.get("ncand"))
        np.testing.assert_array_equal(res.p, p)
        assert res.steps == rd.size
        np.testing.assert_allclose(res.R, R, rtol=0, atol=QR_TOL * np.linalg.norm(A))
        np.testing.assert_allclose(res.Q, Q, rtol=0, atol=1e-10)
    Bm = det_normal(4, (40, 5)) @ det_normal(5, (5, 300)) + 1e-9 * det_normal(6, (40, 300))
    res = built.qrcp(Bm, stop_ratio=0.01)
    p, rd, _, _ = oracle.qrcp_loop(Bm, stop_ratio=0.01)
    assert res.steps == rd.size == 6
    np.testing.assert_array_equal(res.p[:6], p[:6])
    assert sorted(res.p) == list(range(1, 301))
    # the last |r_jj| sits at the noise level: its error is rounding relative to ||A||, not to itself
    np.testing.assert_allclose(res.rdiag, rd, rtol=0, atol=QR_TOL * np.linalg.norm(Bm))


TENSORS = [((12, 13, 7), np.float64), ((6, 5, 7, 4), np.float32), ((40, 9, 11), np.float64)]


@pytest.mark.parametrize("dims,dt", TENSORS)
def test_unfolding_qrcp_matches_lapack(built, oracle, dims, dt):
    T = np.asfortranarray(det_normal(sum(dims), dims).astype(dt))
    T64 = T.astype(np.float64)
    rng = np.random.default_rng(1)
    with built.Engine(dims, 1, dtype=dt, precision="fp64") as e:
        e.set_tensor(T)
        for k in range(len(dims)):
            A = oracle.unfold(T64, k)
            res = e.unfolding_qrcp(k, want_r=True, want_q=True)
            Q2, R2, p2 = oracle.qrcp_lapack(A)
            np.testing.assert_array_equal(res.p, p2)
            close_qr(res, Q2, R2, A)
            cols = rng.choice(A.shape[1], size=max(1, A.shape[1] // 3), replace=False) + 1
            res = e.unfolding_qrcp(k, cols=cols, want_r=True, want_q=True)
            Q2, R2, p2 = oracle.qrcp_lapack(A[:, cols - 1])
            np.testing.assert_array_equal(res.p, p2)
            close_qr(res, Q2, R2, A[:, cols - 1])


def test_krp_qrcp_and_omega_hadamard(built, oracle):
    dims, R = (9, 8, 7), 6
    F, lam = det_factors(dims, R, seed=2)
    with built.Engine(dims, R, dtype=np.float64, precision="fp64") as e:
        e.set_factors(F, lam)
        Fd, _ = e.get_factors()
        for k in range(3):
            others = [Fd[m] for m in range(3) if m != k]
            K = oracle.khatri_rao(others)
            res = e.krp_qrcp(k, want_r=True, want_q=True)
            Q2, R2, p2 = oracle.qrcp_lapack(K.T.copy())
            np.testing.assert_array_equal(res.p[:R], p2[:R])  # past rank R the norms are rounding
            np.testing.assert_allclose(np.abs(res.rdiag), np.abs(np.diag(R2)), rtol=0, atol=1e-12 * np.abs(R2).max())
    # test/pivot_mapping.jl:120-160
    mats = [det_normal(20 + d, (d, 10)) for d in (3, 6, 8)]
    n = 3 * 6 * 8
    for l, s in ((31, 3), (7, 2)):
        rows, vals = built.sparse_sign_matrix(l, n, s, seed=l)
        got = built.omega_hadamard(mats, rows, vals, l, s)
        ref = oracle.omega_hadamard(mats, l, s, rows, vals)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
        dense = oracle.sparse_embedding(l, n, s, rows, vals) @ oracle.khatri_rao(mats)
        np.testing.assert_allclose(got, dense, rtol=0, atol=1e-12 * np.abs(dense).max())


@pytest.mark.parametrize("use_omega", [False, True])
@pytest.mark.parametrize("compute_r", [False, True])
def test_seqrcs_matches_oracle(built, oracle, use_omega, compute_r):
    dims = (20, 30, 40)
    T = np.asfortranarray(det_normal(9, dims))
    for k in range(3):
        m = dims[k]
        n = int(np.prod(dims)) // m
        l, s, t = int(round(3 * m * np.log(m))), int(round(np.log(m))), 8
        rows, vals = built.sparse_sign_matrix(l, n, s, seed=100 + k)
        res = built.SEQRCS(T, k, l, s, t, rows=rows, vals=vals, use_omega=use_omega, compute_r=compute_r)
        Q2, R2, p2, rd2 = oracle.seqrcs(T, k, l, s, t, rows, vals, use_omega=use_omega, compute_r=compute_r)
        np.testing.assert_array_equal(res.p, p2)
        np.testing.assert_allclose(res.rdiag, rd2, rtol=0, atol=QR_TOL * np.linalg.norm(T))
        if compute_r:
            np.testing.assert_allclose(res.R, R2, rtol=0, atol=QR_TOL * np.linalg.norm(T))
            np.testing.assert_allclose(res.Q, Q2, rtol=0, atol=1e-10)


def test_seqrcs_of_the_krp_matches_oracle(built, oracle):
    mats = [det_normal(30 + d, (d, 6)) for d in (12, 9, 5)]
    n = 12 * 9 * 5
    l, s, t = 40, 2, 4
    rows, vals = built.sparse_sign_matrix(l, n, s, seed=5)
    res = built.SEQRCS(mats, l, s, t, rows=rows, vals=vals, compute_r=True)
    Q2, R2, p2, rd2 = oracle.seqrcs_krp(mats, l, s, t, rows, vals, compute_r=True)
    np.testing.assert_array_equal(res.p[: res.nsubset][:6], p2[:6])
    np.testing.assert_array_equal(res.p[res.nsubset:], p2[res.nsubset:])
    np.testing.assert_allclose(np.abs(res.rdiag[:6]), np.abs(rd2[:6]), rtol=0, atol=1e-12)


def qr_error(A, Q, R, p, k):
    return np.linalg.norm(A[:, p - 1] - Q[:, :k] @ R[:k, :], 2) / np.linalg.norm(A, 2)


def test_seqrcs_reference_property(built, oracle):
    """test/SEQRCS_test.jl:32-64: the rank-40 error of SE-QRCS of a 50 x 10000 Gaussian matrix
    (l = 2500, s = 1, t = 40) is within 1e-2 of the pivoted QR's, with either subset order; the
    KRP path equals the explicit-KRP path on the same embedding."""
    A = det_normal(11, (50, 10000))
    Qa, Ra, pa = oracle.qrcp_lapack(A)
    err_act = qr_error(A, Qa, Ra, pa, 40)
    for use_omega in (False, True):
        Q, R, p = built.SEQRCS(np.asfortranarray(A), 0, 2500, 1, 40, use_omega=use_omega, seed=12)
        assert sorted(p) == list(range(1, 10001))
        assert abs(qr_error(A, Q, R, p, 40) - err_act) <= 1e-2
    mats = [det_normal(13, (100, 50)), det_normal(14, (100, 50))]
    Kt = np.asfortranarray(oracle.khatri_rao(mats).T)
    rows, vals = built.sparse_sign_matrix(2500, 10000, 1, seed=15)
    Q, R, p = built.SEQRCS(Kt, 0, 2500, 1, 40, rows=rows, vals=vals, use_omega=True)
    Qf, Rf, pf = built.SEQRCS(mats, 2500, 1, 40, rows=rows, vals=vals)
    np.testing.assert_array_equal(pf[:40], p[:40])
    assert abs(qr_error(Kt, Qf, Rf, pf, 40) - qr_error(Kt, Q, R, p, 40)) <= 1e-8


# ---- the pivot-based solvers (test/rand_cp_als.jl) ----
def rand_problem(R, seed=0, dims=(20, 30, 40)):
    T = np.asfortranarray(det_normal(seed, dims))
    F, lam = det_factors(dims, R, seed=seed + 1)
    return T, F, lam


def recon(cp):
    import cpals_oracle as o

    return o.reconstruct([np.asarray(F, np.float64) for F in cp.factors], np.asarray(cp.lam, np.float64))


def test_compute_als_projectors_match_oracle(built, oracle):
    """Without shuffling, the projectors are the first `end` LAPACK pivots of each unfolding,
    as multi-coordinates; the projected sweeps match the oracle's within 1e-8."""
    T, F, lam = rand_problem(6, seed=3, dims=(8, 9, 10))
    alg = built.QRPivProjected(50)
    als = built.compute_als(T, built.CPD(F, lam), alg=alg, check=built.NoCheck(4), shuffle_pivots=False,
                            rng=np.random.default_rng(1))
    for n in range(3):
        A = oracle.unfold(T, n)
        _, R2, p2 = oracle.qrcp_lapack(A)
        dims_o = [d for m, d in enumerate(T.shape) if m != n]
        ref = oracle.column_to_multi_coords(p2, dims_o)
        np.testing.assert_array_equal(als.additional_items["projects"][n], ref)
        np.testing.assert_array_equal(als.additional_items["projects_tensors"][n], ref[:50])
        assert als.additional_items["effective_ranks"][n] == oracle.effective_rank(np.diag(R2), 0.01)
    cp = built.optimize(built.CPD([f.copy() for f in F], lam.copy()), als)
    of, ol = oracle.projected_als(T, F, lam, als.additional_items["projects_tensors"], 4)
    for x, y in zip(cp.factors, of):
        np.testing.assert_allclose(x, y, rtol=0, atol=1e-8)
    np.testing.assert_allclose(cp.lam, ol, rtol=1e-8)


def test_qr_piv_projected_state_and_update_samples(built):
    """rand_cp_als.jl:20-36."""
    T, F, lam = rand_problem(400)
    check = built.FitCheck(1e-6, 20, float(np.linalg.norm(T)))
    alg = built.QRPivProjected(800)
    als = built.compute_als(T, built.CPD(F, lam), alg=alg, check=check, trunc_tol=4)
    als = built.update_samples(T, als, 900, reshuffle=False)
    assert built.stop(als.mttkrp_alg) == 900 and built.start(als.mttkrp_alg) == 1
    assert isinstance(als.mttkrp_alg, built.QRPivProjected)
    assert als.additional_items["effective_ranks"][0] < 20
    assert [p.shape[0] for p in als.additional_items["projects_tensors"]] == [900, 800, 600]
    cp = built.optimize(built.CPD(F, lam), als)
    assert all(np.all(np.isfinite(f)) for f in cp.factors)


def test_qr_piv_projected_close_to_exact(built):
    """rand_cp_als.jl:38-49: QRPivProjected(800) reconstructs within 1e-2 of the exact ALS."""
    T, F, lam = rand_problem(400, seed=5)
    nT = float(np.linalg.norm(T))
    opt = built.als_optimize(T, built.CPD(F, lam), alg=built.KRPFreeNormal(), check=built.FitCheck(1e-6, 20, nT))
    ref = recon(opt)
    for normal in (True, False):
        got = built.als_optimize(T, built.CPD(F, lam), alg=built.QRPivProjected(800),
                                 check=built.FitCheck(1e-6, 20, nT), shuffle_pivots=True, trunc_tol=0.001,
                                 normal=normal, rng=np.random.default_rng(2))
        assert np.linalg.norm(ref - recon(got)) / np.linalg.norm(ref) < 1e-2


def test_seqrcs_piv_projected(built):
    """rand_cp_als.jl:51-70."""
    T, F, lam = rand_problem(400, seed=7)
    nT = float(np.linalg.norm(T))
    opt = built.als_optimize(T, built.CPD(F, lam), alg=built.KRPFreeNormal(), check=built.FitCheck(1e-6, 20, nT))
    ref = recon(opt)
    alg = built.SEQRCSPivProjected(1, 800, (1, 2, 3), (100, 100, 100))
    als = built.compute_als(T, built.CPD(F, lam), alg=alg, check=built.FitCheck(1e-6, 20, nT))
    als = built.update_samples(T, als, 600, reshuffle=True)
    assert built.stop(als.mttkrp_alg) == 600 and built.start(als.mttkrp_alg) == 1
    assert isinstance(als.mttkrp_alg, built.SEQRCSPivProjected)
    built.optimize(built.CPD(F, lam), als)
    got = built.als_optimize(T, built.CPD(F, lam), alg=built.SEQRCSPivProjected((1,), (800,), (1, 2, 3), (100, 100, 100)),
                             check=built.FitCheck(1e-6, 20, nT), shuffle_pivots=False, rng=np.random.default_rng(3))
    assert np.linalg.norm(ref - recon(got)) / np.linalg.norm(ref) < 1e-1
    got = built.als_optimize(T, built.CPD(F, lam), alg=built.SEQRCSPivProjected((1,), (800,), (1, 2, 3), (20, 20, 20)),
                             check=built.FitCheck(1e-6, 20, nT), shuffle_pivots=True, normal=False, injective=True,
                             rng=np.random.default_rng(4))
    assert np.linalg.norm(ref - recon(got)) / np.linalg.norm(ref) < 1e-1


def multiple_tries(built, A, cp, exact_error, **kw):
    """rand_cp_als.jl:1-14: up to ten attempts; passes when the error is within 10% of the exact ALS's."""
    import cpals_oracle as o

    for i in range(10):
        try:
            got = built.als_optimize(A, built.CPD([f.copy() for f in cp.factors], cp.lam.copy()),
                                     rng=np.random.default_rng(100 + i), **kw)
            err = np.linalg.norm(A - recon(got)) / np.linalg.norm(A)
            return abs(exact_error - err) / exact_error < 0.1
        except Exception:
            if i == 9:
                return False
    return False


def test_pivot_solvers_interpolate_a_known_low_rank(built, oracle):
    """rand_cp_als.jl:72-96: a rank-10 model of an exactly rank-20 tensor under CPDiffCheck."""
    dims = (20, 30, 40)
    Ft, lt = det_factors(dims, 20, seed=21)
    A = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F0, l0 = det_factors(dims, 10, seed=22)
    cp = built.CPD(F0, l0)
    opt = built.als_optimize(A, built.CPD([f.copy() for f in F0], l0.copy()), check=built.CPDiffCheck(1e-5, 100))
    exact_error = np.linalg.norm(A - recon(opt)) / np.linalg.norm(A)
    got = built.als_optimize(A, built.CPD([f.copy() for f in F0], l0.copy()), alg=built.QRPivProjected(1200),
                             check=built.CPDiffCheck(1e-5, 100), rng=np.random.default_rng(1))
    assert abs(exact_error - np.linalg.norm(A - recon(got)) / np.linalg.norm(A)) / exact_error < 0.1
    built.compute_als(A, cp, alg=built.KSEQRCSPivProjected(1, (1200,), (1, 2, 3), 10),
                      check=built.CPDiffCheck(1e-5, 100))
    for kw in (dict(), dict(normal=False), dict(normal=False, injective=True), dict(normal=True, injective=True)):
        assert multiple_tries(built, A, cp, exact_error, alg=built.KSEQRCSPivProjected(1, (1200,), (1, 2, 3), 5),
                              check=built.CPDiffCheck(1e-5, 100), **kw)


def test_device_reproduces_golden_pivots(built, golden_dir):
    """The committed xGEQP3 pivots and SE-QRCS permutations (tests/golden/) from the device."""
    import json

    from _data import golden_qrcp_matrix

    for case in json.loads((golden_dir / "qrcp_pivots.json").read_text()):
        A = golden_qrcp_matrix(case)
        k = case["compare"]
        if "tensor_dims" in case:
            T = np.asfortranarray(det_normal(case["seed"], case["tensor_dims"]))
            with built.Engine(T.shape, 1, dtype=np.float64, precision="fp64") as e:
                e.set_tensor(T)
                res = e.unfolding_qrcp(case["mode"])
        else:
            res = built.qrcp(A)
        np.testing.assert_array_equal(res.p[:k], case["p"][:k], err_msg=case["name"])
        np.testing.assert_allclose(np.abs(res.rdiag[:k]), case["absdiag"][:k], rtol=0,
                                   atol=1e-12 * np.linalg.norm(A))
    g = json.loads((golden_dir / "seqrcs_small.json").read_text())
    T = np.asfortranarray(det_normal(g["seed"], g["tensor_dims"]))
    for case in g["cases"]:
        res = built.SEQRCS(T, g["mode"], g["l"], g["s"], g["t"], rows=np.asarray(g["rows"]), vals=np.asarray(g["vals"]),
                           use_omega=case["use_omega"], compute_r=False)
        np.testing.assert_array_equal(res.p, case["p"])
        np.testing.assert_allclose(np.abs(res.rdiag), case["absdiag"], rtol=0, atol=1e-12 * np.linalg.norm(T))

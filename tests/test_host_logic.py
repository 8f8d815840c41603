"""Host-side logic of the QR-pivoted solvers (no GPU): the algorithm structs, pivot ranges,
effective ranks, the keep-then-shuffle arrangement and update_samples."""
import numpy as np
import pytest


# ---- QR-pivoted solvers: host-side state (algorithms/.../randomized/qr_lev_score_sampled.jl) ----
def test_pivot_solver_structs_and_ranges(pkg):
    api = pkg.api
    a = pkg.QRPivProjected()
    assert (pkg.start(a), pkg.stop(a)) == (1, 0)
    a = pkg.QRPivProjected(800)
    assert (pkg.start(a), pkg.stop(a)) == (1, 800)
    a = pkg.QRPivProjected((20, 30, 40))
    assert (pkg.start(a), pkg.stop(a)) == ((1, 1, 1), (20, 30, 40))
    b = pkg.copy_alg(a, 0, 900)
    assert (pkg.start(b), pkg.stop(b)) == ((1, 1, 1), 900) and pkg.stop(a) == (20, 30, 40)
    s = pkg.SEQRCSPivProjected(1, 800, (1, 2, 3), (100, 100, 100))
    assert s.random_modes == (1, 2, 3) and s.rank_vect == {1: 100, 2: 100, 3: 100}
    s = pkg.SEQRCSPivProjected((1, 1, 1), (800, 800, 600), 2, (100,))
    assert s.random_modes == (2,) and s.rank_vect == {2: 100}
    k = pkg.KSEQRCSPivProjected(1, (1200,), (1, 2, 3), 10)
    assert k.rank_vect == {1: 10, 2: 10, 3: 10}
    c = pkg.copy_alg(k, 0, 600)
    assert isinstance(c, pkg.KSEQRCSPivProjected) and c.random_modes == (1, 2, 3) and pkg.stop(c) == 600
    # optimizers/.../randomized/qr_lev_score_sampled.jl:51-58: end 0 = every column, clamped to the column count
    assert api._pivot_range(pkg.QRPivProjected(), 0, 1200) == (1, 1200)
    assert api._pivot_range(pkg.QRPivProjected(5000), 0, 1200) == (1, 1200)
    assert api._pivot_range(pkg.QRPivProjected((1, 3, 2), (10, 20, 30)), 1, 100) == (3, 20)
    with pytest.raises(AssertionError):
        api._pivot_range(pkg.QRPivProjected(50, 40), 0, 100)


def test_effective_rank_and_arrangement(pkg):
    api = pkg.api
    assert api._effective_rank([10.0, -5.0, 0.2, 0.05], 0.01) == 3  # 0.05 / 10 < 0.01
    assert api._effective_rank([10.0, -5.0, 0.2, 0.05], 0.1) == 2
    assert api._effective_rank([10.0, 1.0], 4) == 0  # rand_cp_als.jl:29 uses trunc_tol = 4
    assert api._effective_rank([0.0, 0.0], 0.01) == 0  # 0/0 is NaN, never above the tolerance
    p = np.arange(1, 21)
    q = api._arrange(p, 5, True, np.random.default_rng(0))
    np.testing.assert_array_equal(q[:5], p[:5])
    assert sorted(q[5:]) == list(range(6, 21)) and not np.array_equal(q[5:], p[5:])
    np.testing.assert_array_equal(api._arrange(p, 5, False, None), p)
    np.testing.assert_array_equal(api._column_to_multi_coords([1, 2, 4, 12], (2, 3, 2)),
                                  [[1, 1, 1], [2, 1, 1], [2, 2, 1], [2, 3, 2]])


def test_update_samples_keeps_or_reshuffles(pkg):
    """update_samples (algorithms/.../randomized/qr_lev_score_sampled.jl:95-149): a new range on the same pivots, or the
    order past meff redrawn."""
    api = pkg.api
    dims = (4, 5, 6)
    T = np.zeros(dims)
    ref, projects, eff = [], [], []
    rng = np.random.default_rng(1)
    for n in range(3):
        dims_o = [d for m, d in enumerate(dims) if m != n]
        p = rng.permutation(int(np.prod(dims_o))) + 1
        ref.append(p)
        eff.append(3)
        projects.append(api._column_to_multi_coords(p, dims_o))
    items = {"ref_projectors": ref, "projects": projects, "projects_tensors": [x[:10] for x in projects],
             "effective_ranks": eff, "normal": True}
    als = pkg.ALS(T, pkg.QRPivProjected(10), items, pkg.NoCheck(5))
    a2 = pkg.update_samples(T, als, 12)
    assert pkg.stop(a2.mttkrp_alg) == 12 and pkg.stop(als.mttkrp_alg) == 10
    for n in range(3):
        np.testing.assert_array_equal(a2.additional_items["projects_tensors"][n], projects[n][:12])
    a3 = pkg.update_samples(T, als, 12, reshuffle=True, rng=np.random.default_rng(2))
    for n in range(3):
        got = a3.additional_items["projects"][n]
        np.testing.assert_array_equal(got[:3], projects[n][:3])
        assert sorted(map(tuple, got.tolist())) == sorted(map(tuple, projects[n].tolist()))
        np.testing.assert_array_equal(a3.additional_items["projects_tensors"][n], got[:12])
    with pytest.raises(AssertionError):
        pkg.update_samples(T, pkg.ALS(T, pkg.LevScoreSampled(4), items, pkg.NoCheck(1)), 5)


def test_explicit_omega_entries(pkg):
    """The explicit-Omega forms (pivot_mapping.jl:90-108, had_contract.jl:300) read a sparse
    Omega back into the generators' entry layout."""
    import scipy.sparse as sp

    rng = np.random.default_rng(3)
    l, n, s = 11, 7, 3
    rows = np.concatenate([np.sort(rng.choice(l, s, replace=False)) for _ in range(n)]).astype(np.int32) + 1
    vals = rng.choice([-1.0, 1.0], n * s) / np.sqrt(s)
    om = sp.csc_matrix((vals, (rows - 1, np.repeat(np.arange(n), s))), shape=(l, n))
    l2, r2, v2, s2 = pkg.api._omega_entries(om)
    assert (l2, s2) == (l, s)
    np.testing.assert_array_equal(r2, rows)
    np.testing.assert_array_equal(v2, vals)
    # a column with one entry fewer
    short = sp.csc_matrix((vals[1:], (rows[1:] - 1, np.repeat(np.arange(n), s)[1:])), shape=(l, n))
    with pytest.raises(ValueError):
        pkg.api._omega_entries(short)


def test_bench_sweeps_to_fit():
    """The bench's sweeps-to-fit report: the first sweep reaching each target, None when none does."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench

    assert bench.sweeps_to_fit([0.1, 0.5, 0.9, 0.95], 0.9) == 3
    assert bench.sweeps_to_fit([0.1, 0.5], 0.99) is None
    rep = bench.sweeps_to_fit_report({"bf16x3": [0.2, 0.8, 0.899, 0.9], "fp64": [0.2, 0.85, 0.9, 0.9]})
    assert rep["absolute"] == {"bf16x3": None, "fp64": None}
    assert rep["relative_target"] == pytest.approx(0.891)
    assert rep["relative"] == {"bf16x3": 3, "fp64": 3}

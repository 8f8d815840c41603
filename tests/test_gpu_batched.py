"""Batched small decompositions (cpals_batch_*) against the oracle, tensor by tensor.

Each tensor of a batch of uneven shapes and ranks must follow the oracle's FP64 ALS from
the same initial factors.  The batched MTTKRP multiplies FP32 tensor entries by FP32 factor
copies with FP32 accumulation inside a slab (compensated FP32 pairs across slabs), so per-sweep fits agree
to ~1e-6 rather than FP64 rounding: the test bounds the final fit after a fixed number of
sweeps by 2e-5, and FitCheck stopping sweeps by +-3 of the oracle's.
"""
import numpy as np
import pytest

from _data import det_factors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


def make_batch(oracle, count, seed, dmin=5, dmax=24, rmin=2, rmax=8):
    rng = np.random.default_rng(seed)
    dims, ranks, Ts, Fs, lams = [], [], [], [], []
    for t in range(count):
        d = tuple(int(x) for x in rng.integers(dmin, dmax + 1, size=3))
        R = int(rng.integers(rmin, rmax + 1))
        T, _, _ = oracle.lowrank_plus_noise(d, R, float(rng.uniform(0, 0.6)), float(rng.uniform(10, 40)), rng)
        F, lam = det_factors(d, R, seed=1000 + t)
        dims.append(d)
        ranks.append(R)
        Ts.append(T)
        Fs.append(F)
        lams.append(lam)
    return dims, ranks, Ts, Fs, lams


def test_batched_fixed_sweeps_match_oracle(built, oracle):
    dims, ranks, Ts, Fs, lams = make_batch(oracle, 40, seed=1)
    norms = [float(np.linalg.norm(T.astype(np.float64))) for T in Ts]
    with built.BatchEngine(dims, ranks, norms) as be:
        be.set_tensors(Ts)
        be.set_factors(Fs, lams)
        sweeps, fits, flags, launches = be.optimize(tol=0.0, max_iter=6)
        out = be.get_factors()
    assert np.all(sweeps == 6) and np.all(flags & 4) and not np.any(flags & 1)
    assert launches > 0
    for t in range(len(Ts)):
        chk = oracle.FitCheck(0.0, 6, norms[t])
        F, lam, chk, _ = oracle.als_optimize(Ts[t].astype(np.float64), Fs[t], lams[t], check=chk)
        assert abs(fits[t] - chk.trajectory[-1]) < 2e-5, (t, fits[t], chk.trajectory[-1])
        # the factors themselves: unit columns and the same reconstruction
        Fg, lg = out[t]
        rec_g = oracle.reconstruct(Fg, lg)
        rec_o = oracle.reconstruct(F, lam)
        assert np.linalg.norm(rec_g - rec_o) / np.linalg.norm(rec_o) < 1e-3, t


def test_batched_fitcheck_stopping(built, oracle):
    dims, ranks, Ts, Fs, lams = make_batch(oracle, 24, seed=2)
    norms = [float(np.linalg.norm(T.astype(np.float64))) for T in Ts]
    with built.BatchEngine(dims, ranks, norms) as be:
        be.set_tensors(Ts)
        be.set_factors(Fs, lams)
        sweeps, fits, flags, _ = be.optimize(tol=1e-5, max_iter=200)
    for t in range(len(Ts)):
        chk = oracle.FitCheck(1e-5, 200, norms[t])
        oracle.als_optimize(Ts[t].astype(np.float64), Fs[t], lams[t], check=chk)
        n_or = len(chk.trajectory)
        assert abs(int(sweeps[t]) - n_or) <= 3, (t, sweeps[t], n_or)
        assert abs(fits[t] - chk.trajectory[-1]) < 1e-4, (t, fits[t], chk.trajectory[-1])


def test_batched_autotune_and_thread_counts(built, oracle):
    dims, ranks, Ts, Fs, lams = make_batch(oracle, 64, seed=3, dmin=16, dmax=40, rmin=4, rmax=16)
    norms = [float(np.linalg.norm(T.astype(np.float64))) for T in Ts]
    res = {}
    with built.BatchEngine(dims, ranks, norms) as be:
        be.set_tensors(Ts)
        nt, ms = be.autotune(Fs, lams, sweeps=2)
        assert nt in (128, 256, 512)
        for threads in (128, 256, 512):
            be.set_threads(threads)
            be.set_factors(Fs, lams)
            _, fits, _, _ = be.optimize(tol=0.0, max_iter=4)
            res[threads] = fits
    # every output element is computed by one thread in a fixed order; only the
    # block-wide sums of the fit depend on the warp count
    assert np.max(np.abs(res[128] - res[512])) < 1e-12
    assert np.max(np.abs(res[256] - res[512])) < 1e-12


def test_batched_split_schedule_matches_one_class(built, oracle):
    # small (12..20) and large (60..96) extents: the small tensors' own layouts allow more CTAs
    # per SM than the large ones', so the autotuner has a split schedule to try; whichever it
    # keeps, every tensor is solved once, as one class solves it (only the fit's block sums
    # depend on the warp count)
    small = make_batch(oracle, 20, seed=7, dmin=12, dmax=20, rmin=2, rmax=6)
    large = make_batch(oracle, 20, seed=8, dmin=60, dmax=96, rmin=4, rmax=16)
    dims, ranks, Ts, Fs, lams = (a + b for a, b in zip(small, large))
    norms = [float(np.linalg.norm(T.astype(np.float64))) for T in Ts]
    with built.BatchEngine(dims, ranks, norms) as be:
        be.set_tensors(Ts)
        be.autotune(Fs, lams, sweeps=2)
        classes, split_ms = be.schedule()
        assert sum(c["tensors"] for c in classes) == len(dims)
        assert split_ms > 0  # more than one size class existed, so the split was timed
        be.set_factors(Fs, lams)
        sw_a, fits_a, _, _ = be.optimize(tol=0.0, max_iter=4)
        be.set_threads(256)
        assert len(be.schedule()[0]) == 1
        be.set_factors(Fs, lams)
        sw_1, fits_1, _, _ = be.optimize(tol=0.0, max_iter=4)
    assert np.array_equal(sw_a, sw_1)
    assert np.max(np.abs(fits_a - fits_1)) < 1e-12


def test_batched_rank_deficient_stays_finite(built, oracle):
    # a tensor whose initial factors repeat a column: V is singular, the sweep stops early
    d, R = (9, 8, 7), 3
    rng = np.random.default_rng(4)
    T, _, _ = oracle.lowrank_plus_noise(d, R, 0.2, 30.0, rng)
    F, lam = det_factors(d, R, seed=5)
    for f in F:
        f[:, 2] = f[:, 1]
    with built.BatchEngine([d], [R], [float(np.linalg.norm(T))]) as be:
        be.set_tensors([T])
        be.set_factors([F], [lam])
        sweeps, fits, flags, _ = be.optimize(tol=0.0, max_iter=3)
    assert flags[0] & 2  # rank-deficient normal equations were met
    assert not (flags[0] & 1) and np.isfinite(fits[0])


def test_batched_rejects_bad_input(built):
    with pytest.raises(Exception):
        built.BatchEngine([(4, 5, 6)], [0], [1.0])
    with pytest.raises(Exception):
        built.BatchEngine([(4, 5, 6)], [3], [0.0])


def test_batched_flat_buffers_match_lists(built, oracle):
    # the flat-buffer calls (one packed FP64 host buffer each way) solve exactly as the lists do
    dims, ranks, Ts, Fs, lams = make_batch(oracle, 12, seed=11)
    norms = [float(np.linalg.norm(T.astype(np.float64))) for T in Ts]
    with built.BatchEngine(dims, ranks, norms) as be:
        be.set_tensors(Ts)
        be.set_factors(Fs, lams)
        _, fits_l, _, _ = be.optimize(tol=0.0, max_iter=3)
        out_l = be.get_factors()
        buf = be.pack_factors(Fs, lams)
        be.set_factors_concat(buf)
        _, fits_c, _, _ = be.optimize(tol=0.0, max_iter=3)
        flat = be.get_factors_concat()
        with pytest.raises(TypeError):
            be.set_factors_concat(buf[:-1])
    assert np.array_equal(fits_l, fits_c)
    for (Fa, la), (Fb, lb) in zip(out_l, be.unpack_factors(flat)):
        assert np.array_equal(la, lb)
        for a, b in zip(Fa, Fb):
            assert np.array_equal(a, b)


def test_batched_one_launch_matches_one_launch_per_sweep(built, oracle):
    # By default one launch runs every tensor to its own stop (a CTA sweeps the tensor it pulls
    # until its check stops it); set_sweeps_per_launch(1) launches one sweep at a time and
    # polls.  Each tensor's sweeps and check are its own, so sweeps, fits, flags and factors
    # agree bit for bit.  Half the batch is exactly rank R and starts at its own factors (it
    # stops within a few sweeps at tol 1e-3: near fit 1 the FP32-product fit terms jitter by
    # ~1e-4, so a tighter tol would not stop it); the other half runs on.
    rng = np.random.default_rng(13)
    dims, ranks, Ts, Fs, lams = [], [], [], [], []
    for t in range(12):
        d = tuple(int(x) for x in rng.integers(8, 21, size=3))
        R = int(rng.integers(2, 6))
        if t % 2 == 0:
            Ft, lt = det_factors(d, R, seed=300 + t)
            T = np.asfortranarray(oracle.reconstruct(Ft, lt)).astype(np.float32)
            F, lam = Ft, lt
        else:
            T, _, _ = oracle.lowrank_plus_noise(d, R, 0.5, 15.0, rng)
            F, lam = det_factors(d, R, seed=400 + t)
        dims.append(d)
        ranks.append(R)
        Ts.append(T)
        Fs.append(F)
        lams.append(lam)
    norms = [float(np.linalg.norm(T.astype(np.float64))) for T in Ts]
    res = {}
    with built.BatchEngine(dims, ranks, norms) as be:
        be.set_tensors(Ts)
        be.set_threads(256)
        for k in (0, 1, 3):
            be.set_sweeps_per_launch(k)
            be.set_factors(Fs, lams)
            sw, fits, flags, launches = be.optimize(tol=1e-3, max_iter=80)
            res[k] = (sw, fits, flags, launches, be.get_factors())
        with pytest.raises(Exception):
            be.set_sweeps_per_launch(-1)
    sw = res[0][0]
    print("sweeps:", sw, "launches:", res[0][3], res[1][3], res[3][3])
    assert np.sum(sw <= 4) >= 5 and np.sum(sw > 6) >= 3
    assert res[0][3] < res[3][3] < res[1][3]
    for k in (1, 3):
        assert np.array_equal(res[k][0], sw) and np.array_equal(res[k][1], res[0][1])
        assert np.array_equal(res[k][2], res[0][2])
        for (Fa, la), (Fb, lb) in zip(res[k][4], res[0][4]):
            assert np.array_equal(la, lb)
            for x, y in zip(Fa, Fb):
                assert np.array_equal(x, y)


def test_batched_tiny_extents_follow_the_oracle(built, oracle):
    # extents 1 to 4 and ranks 1 to 3: one-row slabs, more slab partitions than rows, rank
    # groups wider than the rank
    rng = np.random.default_rng(21)
    dims, ranks, Ts, Fs, lams = [], [], [], [], []
    for t in range(16):
        d = tuple(int(x) for x in rng.integers(1, 5, size=3))
        R = int(rng.integers(1, 4))
        T = np.asfortranarray(rng.standard_normal(d)).astype(np.float32)
        F, lam = det_factors(d, R, seed=500 + t)
        dims.append(d)
        ranks.append(R)
        Ts.append(T)
        Fs.append(F)
        lams.append(lam)
    norms = [float(np.linalg.norm(T.astype(np.float64))) for T in Ts]
    with built.BatchEngine(dims, ranks, norms) as be:
        be.set_tensors(Ts)
        be.set_factors(Fs, lams)
        sweeps, fits, flags, _ = be.optimize(tol=0.0, max_iter=5)
    assert np.all(sweeps == 5) and not np.any(flags & 1) and np.all(np.isfinite(fits))
    compared = 0
    for t in range(len(Ts)):
        chk = oracle.FitCheck(0.0, 5, norms[t])
        oracle.als_optimize(Ts[t].astype(np.float64), Fs[t], lams[t], check=chk)
        if flags[t] & 2:  # a rank-deficient V keeps the basic solution (the oracle's QR differs)
            continue
        if chk.trajectory[-1] > 0.999:
            # an (almost) exactly rank-R tensor: near fit 1 the FP32-product fit terms cancel
            # and the batch's fit carries ~1e-4 of jitter
            assert abs(fits[t] - chk.trajectory[-1]) < 1e-3, (t, dims[t], ranks[t], fits[t])
            continue
        assert abs(fits[t] - chk.trajectory[-1]) < 2e-5, (t, dims[t], ranks[t], fits[t], chk.trajectory[-1])
        compared += 1
    assert compared >= 4


def test_batched_refuses_a_tensor_beyond_shared_memory(built):
    # a 160^3 tensor's per-CTA layout (slab ring, FP32 factors, M, X) exceeds 227 KB
    with pytest.raises(Exception):
        built.BatchEngine([(160, 160, 160)], [8], [1.0])

"""The tcgen05 split-BF16 MTTKRP (precision "bf16x3") through the C ABI.

Two references:
  * an exact CPU emulation of the same arithmetic (BF16 round-to-nearest hi/lo split of
    T and of the FP32 Khatri-Rao tile, the three products Th Kh + Th Kl + Tl Kh summed in
    FP64): the GPU result may differ from it only by FP32 accumulation order,
    tolerance 1e-5 relative Frobenius;
  * the FP64 oracle: the split-BF16 arithmetic itself is accurate to ~2^-16 per
    product, tolerance 1e-4 relative Frobenius (the measured error is printed).
"""
import numpy as np
import pytest

from _data import det_factors, det_normal

pytestmark = pytest.mark.gpu

EMU_TOL = 1e-5
FP64_TOL = 1e-4


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def bf16_rn(x):
    """float32 -> float32 holding the nearest BF16 (ties to even)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def split(x32):
    hi = bf16_rn(x32)
    lo = bf16_rn((x32 - hi).astype(np.float32))
    return hi.astype(np.float64), lo.astype(np.float64)


def bf16_from_f64(x):
    """FP64 -> nearest BF16 (via the nearest FP32, exact for these magnitudes), as float64."""
    return bf16_rn(np.asarray(x, dtype=np.float64).astype(np.float32)).astype(np.float64)


def emulate_mttkrp(oracle, T32, F, n):
    """The kernel's arithmetic.  T is split once into BF16 hi/lo; the fastest reduction
    mode's factor F_f is split from FP64 into BF16 hi/lo; per chunk (64 values of f at a
    fixed outer index o) the three products Th Fh + Th Fl + Tl Fh are formed and then
    scaled by s_o(r), the FP32 product of the outer factor rows (outer modes in mode order)."""
    order = T32.ndim
    R = F[0].shape[1]
    fmode = 1 if n == 0 else 0
    outer = [m for m in range(order) if m not in (n, fmode)]
    s = np.ones((1, R), dtype=np.float32)
    for m in outer:  # later outer modes vary slower; product order = mode order
        s = (s[None, :, :] * np.asarray(F[m], dtype=np.float32)[:, None, :]).reshape(-1, R).astype(np.float32)
    Fh = bf16_from_f64(F[fmode])
    Fl = bf16_from_f64(np.asarray(F[fmode], dtype=np.float64) - Fh)
    perm = [n, fmode] + outer
    Tn = np.reshape(np.transpose(T32, perm), (T32.shape[n], -1), order="F")
    Th, Tl = split(Tn)
    If = T32.shape[fmode]
    M = np.zeros((T32.shape[n], R))
    for o in range(s.shape[0]):
        cols = slice(o * If, (o + 1) * If)
        P = Th[:, cols] @ Fh + Th[:, cols] @ Fl + Tl[:, cols] @ Fh
        M += P * s[o].astype(np.float64)[None, :]
    return M


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


TC_SHAPES = [
    ((12, 13, 7), 5),
    ((70, 65, 9), 20),
    ((6, 5, 4, 3), 7),
    ((33, 70), 9),
    ((1, 17, 9), 3),
    ((130, 20, 3), 33),
    ((64, 64, 64), 64),
    ((200, 96, 80), 96),
    ((40, 50, 60), 200),
    ((128, 128, 64), 128),
]


@pytest.mark.parametrize("dims,R", TC_SHAPES)
def test_mttkrp_bf16x3_against_emulation_and_fp64(built, oracle, dims, R):
    T = np.asfortranarray(det_normal(7 + len(dims), dims).astype(np.float32))
    F, lam = det_factors(dims, R, seed=R)
    with built.Engine(dims, R, dtype=np.float32, precision="bf16x3") as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        for n in range(len(dims)):
            got = eng.mttkrp(n)
            emu = emulate_mttkrp(oracle, T, F, n)
            ref = oracle.mttkrp_krp(T.astype(np.float64), F, n)
            e_emu, e64 = rel(got, emu), rel(got, ref)
            print(f"{dims} R={R} mode {n}: vs emulation {e_emu:.2e}, vs FP64 {e64:.2e}")
            assert e_emu < EMU_TOL
            assert e64 < FP64_TOL


def test_bf16x3_repeated_calls_are_deterministic(built):
    dims, R = (96, 80, 70), 32
    T = np.asfortranarray(det_normal(2, dims).astype(np.float32))
    F, lam = det_factors(dims, R, seed=1)
    with built.Engine(dims, R, dtype=np.float32, precision="bf16x3") as eng:
        eng.set_tensor(T)
        eng.set_factors(F, lam)
        a = [eng.mttkrp(n) for n in range(3)]
        b = [eng.mttkrp(n) for n in range(3)]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_bf16x3_sweeps_track_fp64(built, oracle):
    # low-rank-plus-noise FP32 tensor (congruence 0.5, 20 dB): the mixed-precision ALS
    # tracks the FP64 ALS.  At this size (448 terms in the fit's inner product) the
    # unbiased 4e-6 split-BF16 rounding shows in the reported fit at the 1e-5 level; the
    # 1e-6 agreement is asserted at the 512^3 workload below.
    rng = np.random.default_rng(4)
    T, _, _ = oracle.lowrank_plus_noise((64, 60, 56), 8, 0.5, 20.0, rng)
    F, lam = det_factors(T.shape, 8, seed=6)
    fits = {}
    for prec in ("fp64", "bf16x3"):
        chk = built.FitCheck(0.0, 30, float(np.linalg.norm(T.astype(np.float64))))
        with built.Engine(T.shape, 8, dtype=np.float32, precision=prec) as eng:
            eng.set_tensor(T)
            eng.set_factors(F, lam)
            c = built.api._to_device_check(chk)
            fits[prec] = eng.optimize(c)
    d = np.max(np.abs(fits["fp64"] - fits["bf16x3"]))
    print("max |fit_fp64 - fit_bf16x3| over 30 sweeps:", d, "final", fits["fp64"][-1], fits["bf16x3"][-1])
    assert abs(fits["fp64"][-1] - fits["bf16x3"][-1]) < 2e-5
    assert d < 5e-5


def test_bf16x3_final_fit_matches_fp64_at_512cube(built):
    # The benchmark workload: 512^3 FP32, 64 terms with congruence 0.5, 20 dB noise, rank-64
    # ALS from the same start, each precision run to convergence under FitCheck(1e-7, 400).
    # Target: the same final fit as the plain FP64 GPU ALS within 1e-6.
    from itensorcpd_gb300.synthetic import lowrank_plus_noise

    dims, R = (512, 512, 512), 64
    T, _, _ = lowrank_plus_noise(dims, R, 0.5, 20.0, np.random.default_rng(2024))
    F, lam = det_factors(dims, R, seed=3)
    ref_norm = float(np.linalg.norm(T.reshape(-1).astype(np.float64)))
    final = {}
    for prec in ("bf16x3", "fp64"):
        chk = built.FitCheck(1e-7, 400, ref_norm)
        with built.Engine(dims, R, dtype=np.float32, precision=prec) as eng:
            eng.set_tensor(T)
            eng.set_factors(F, lam)
            c = built.api._to_device_check(chk)
            eng.optimize(c)
            built.api._from_device_check(chk, c, [], R, False)
        final[prec] = (chk.final_fit, chk.total_iter)
    d = abs(final["fp64"][0] - final["bf16x3"][0])
    print("512^3 converged: fp64", final["fp64"], "bf16x3", final["bf16x3"], "diff", d)
    assert d < 1e-6


def _tracking(built, T, F, lam, R, sweeps):
    nrm = float(np.linalg.norm(T.astype(np.float64)))
    fits = {}
    for prec in ("fp64", "bf16x3"):
        with built.Engine(T.shape, R, dtype=np.float32, precision=prec) as eng:
            eng.set_tensor(T)
            eng.set_factors(F, lam)
            fits[prec] = eng.optimize(built.api._to_device_check(built.FitCheck(0.0, sweeps, nrm)))
    return fits


def test_bf16x3_nearly_collinear_factors_fall_back_to_fp64_sweep(built, oracle):
    # two components with column cosines 0.9999 in every mode: V's pivots fall far below
    # 1e-3 of its diagonal, so the FP32 sweep hands over to the FP64 sweep.  The split-BF16
    # MTTKRP's ~1e-7 relative error is amplified by kappa(V) (~1e4 here) in the solve,
    # whatever its precision, so the fits agree to ~1e-4 rather than 1e-6
    rng = np.random.default_rng(21)
    dims, R = (48, 44, 40), 6
    T, _, _ = oracle.lowrank_plus_noise(dims, R, 0.3, 30.0, rng)
    F, lam = det_factors(dims, R, seed=22)
    for f in F:
        f[:, 1] = f[:, 0] + 0.014 * f[:, 1]
        f /= np.linalg.norm(f, axis=0)
    fits = _tracking(built, T, F, lam, R, 12)
    assert np.all(np.isfinite(fits["bf16x3"]))
    assert np.max(np.abs(fits["fp64"] - fits["bf16x3"])) < 1e-3


def test_bf16x3_rank_above_128_tracks_fp64(built, oracle):
    # R > 128: the FP32 sweep is not used (shared-memory limit); FP64 sweep on both engines
    rng = np.random.default_rng(23)
    dims, R = (150, 140, 36), 144
    T, _, _ = oracle.lowrank_plus_noise(dims, 16, 0.2, 30.0, rng)
    F, lam = det_factors(dims, R, seed=24)
    fits = _tracking(built, T, F, lam, R, 4)
    assert np.max(np.abs(fits["fp64"] - fits["bf16x3"])) < 1e-4


def test_bf16x3_rank_deficient_normal_equations(built, oracle):
    # repeated factor columns make V singular: FP32 sweep -> FP64 sweep -> pivoted-QR
    # operator, as on the FP64 engine; both stay finite and agree
    rng = np.random.default_rng(25)
    dims, R = (30, 28, 26), 4
    T, _, _ = oracle.lowrank_plus_noise(dims, R, 0.2, 30.0, rng)
    F, lam = det_factors(dims, R, seed=26)
    for f in F:
        f[:, 3] = f[:, 2]
    fits = _tracking(built, T, F, lam, R, 3)
    assert np.all(np.isfinite(fits["bf16x3"])) and np.all(np.isfinite(fits["fp64"]))
    assert np.max(np.abs(fits["fp64"] - fits["bf16x3"])) < 1e-3


def test_lowmem_engine_matches_the_per_mode_streams(built, oracle):
    # CPALS_FLAG_LOWMEM builds each mode's tile stream into one shared buffer right before its
    # MTTKRP: the same tiles and the same kernel, so the MTTKRPs and a whole graph-replayed
    # FitCheck run equal the engine with one stream per mode bit for bit
    rng = np.random.default_rng(8)
    T, _, _ = oracle.lowrank_plus_noise((72, 60, 50), 8, 0.4, 25.0, rng)
    F, lam = det_factors(T.shape, 8, seed=9)
    out = {}
    for low in (False, True):
        chk = built.FitCheck(1e-7, 20, float(np.linalg.norm(T.astype(np.float64))))
        with built.Engine(T.shape, 8, dtype=np.float32, precision="bf16x3", lowmem=low) as eng:
            eng.set_tensor(T)
            eng.set_factors(F, lam)
            ms = [eng.mttkrp(n) for n in (2, 0, 1)]  # out of order: each call builds its own stream
            fits = eng.optimize(built.api._to_device_check(chk))
            Fo, lo = eng.get_factors()
        out[low] = (ms, fits, Fo, lo)
    for a, b in zip(out[False][0], out[True][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[False][1], out[True][1])
    for a, b in zip(out[False][2], out[True][2]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[False][3], out[True][3])


def test_lowmem_needs_the_plain_split_bf16_engine(built):
    with pytest.raises(Exception):
        built.Engine((8, 9, 10), 4, dtype=np.float32, precision="fp64", lowmem=True)
    with pytest.raises(Exception):
        built.Engine((8, 9, 10, 11), 4, dtype=np.float32, precision="bf16x3", dimtree=True, lowmem=True)

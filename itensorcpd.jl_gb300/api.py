"""User-facing API with the names and argument meaning of ITensorCPD.jl.

``decompose``, ``random_CPD``, ``als_optimize``, ``FitCheck``, ``NoCheck``, ``CPDFit``,
``CPD`` and the algorithm structs behave as in the reference; every sweep runs on the
GPU through libcpals (there is no CPU path).  Arrays are numpy arrays indexed like the
reference's (first index fastest in memory is handled by the binding).
"""
from __future__ import annotations

import copy
import ctypes as C
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .engine import Engine, QRCPResult


# ---------------------------------------------------------------------------
# CPD container (src/cpd.jl:7-46)
# ---------------------------------------------------------------------------
class CPD:
    """Factors F_n (I_n x R) and weights lambda (R), as ``CPD{TargetT}`` (cpd.jl:7-18)."""

    def __init__(self, factors, lam, inds=None):
        self.factors = [np.asarray(F) for F in factors]
        self.lam = np.asarray(lam)
        self.inds = tuple(inds) if inds is not None else tuple(F.shape[0] for F in self.factors)

    @property
    def λ(self):  # noqa: N802 - the reference's field name
        return self.lam

    def __getitem__(self, i):
        return self.factors[i]

    def __len__(self):
        return len(self.factors)

    def __iter__(self):
        return iter(self.factors)

    @property
    def ndims(self):
        return len(self.factors)

    def copy(self):
        return CPD([F.copy() for F in self.factors], self.lam.copy(), self.inds)

    def __eq__(self, other):
        return (
            isinstance(other, CPD)
            and len(self) == len(other)
            and all(np.array_equal(a, b) for a, b in zip(self.factors, other.factors))
            and np.array_equal(self.lam, other.lam)
        )

    @property
    def dtype(self):
        return self.lam.dtype


def cp_rank(cp: CPD) -> int:
    """cpd.jl:29: dimension of the CP rank index."""
    return int(cp.lam.shape[0])


# ---------------------------------------------------------------------------
# Convergence checks (src/converge_checks/)
# ---------------------------------------------------------------------------
class ConvergeAlg:
    pass


@dataclass
class FitCheck(ConvergeAlg):
    """fit_check.jl:5-20: stop when |delta fit| < tolerance on two consecutive sweeps."""

    tolerance: float
    max_counter: int
    ref_norm: float
    iter: int = 0
    counter: int = 0
    lastfit: float = 1.0
    final_fit: float = 0.0
    total_iter: int = 0
    trajectory: list = field(default_factory=list)


@dataclass
class NoCheck(ConvergeAlg):
    """no_check.jl:1-9: run ``max_counter`` sweeps."""

    max_counter: int
    iter: int = 0
    lastfit: float = -1.0


@dataclass
class CPDiffCheck(ConvergeAlg):
    """cp_diff_check.jl:6-18: the fit between consecutive iterates,
    1 - ||T_n - T_{n-1}|| / ||T_{n-1}||, must change by less than ``tolerance`` on two
    consecutive sweeps.  ``PrevCP`` is the previous iterate (a CPD) or None; the engine
    keeps it on the device while it runs."""

    tolerance: float
    max_counter: int
    iter: int = 0
    counter: int = 0
    norm_prev_iter: float = 0.0
    PrevCP: object = None
    lastfit: float = 1.0
    final_fit: float = 0.0
    total_iter: int = 0
    trajectory: list = field(default_factory=list)


@dataclass
class CPAngleCheck(ConvergeAlg):
    """cp_angle_check.jl:6-18: the angle acos(<T_n, T_{n-1}> / (||T_n|| ||T_{n-1}||))
    must change by less than ``tolerance`` on two consecutive sweeps."""

    tolerance: float
    max_counter: int
    iter: int = 0
    counter: int = 0
    norm_prev_iter: float = 0.0
    PrevCP: object = None
    lastangle: float = 1.0
    final_fit: float = 0.0
    total_iter: int = 0
    trajectory: list = field(default_factory=list)


def CPDFit(check) -> float:  # noqa: N802 - reference name
    """fit_check.jl:68, cp_diff_check.jl:73, cp_angle_check.jl:75."""
    return check.final_fit


# ---------------------------------------------------------------------------
# ALS algorithms (src/algorithms/als_algorithms/)
# ---------------------------------------------------------------------------
class MttkrpAlgorithm:
    precision = "fp64"
    dimtree = False


class KRPFreeNormal(MttkrpAlgorithm):
    """Normal-equation ALS, the reference default (standard/tensor.jl:27-49); FP64 MTTKRP on the GPU."""


class KRPNormal(MttkrpAlgorithm):
    """Normal-equation ALS with an explicit KRP in the reference (standard/tensor.jl:10-25).
    On the GPU the KRP is never materialised; the arithmetic is the same FP64 MTTKRP."""


class GB300Normal(MttkrpAlgorithm):
    """Normal-equation ALS with the tcgen05 split-BF16 MTTKRP (FP32 accumulate) and the
    FP64 Gram / Cholesky / fit of the other algorithms.  ``dimtree`` reuses partial
    contractions across modes."""

    def __init__(self, precision: str = "bf16x3", dimtree: bool = False):
        self.precision = precision
        self.dimtree = dimtree


class ProjectionAlgorithm:
    pass


class LevScoreSampled(ProjectionAlgorithm):
    """randomized/krp_lev_score_sampled.jl:9-14: leverage-score sampled ALS with
    ``NSamples`` KRP rows per mode solve (an int or a per-mode tuple)."""

    def __init__(self, n=1):
        self.NSamples = tuple(n) if isinstance(n, (tuple, list)) else (int(n),)

    def nsamples(self, mode: int) -> int:
        return self.NSamples[0] if len(self.NSamples) == 1 else self.NSamples[mode]

    def sample(self, mode: int, probs, rng) -> np.ndarray:
        """project_krp's draw (randomized/krp_lev_score_sampled.jl:20-37)."""
        return sample_factor_matrices(self.nsamples(mode), mode, probs, rng)


class BlockLevScoreSampled(LevScoreSampled):
    """randomized/krp_lev_score_sampled.jl:64-77: leverage-score sampling that draws runs of
    ``Blocks`` consecutive indices of the first sampled mode (an int or a per-mode tuple)."""

    def __init__(self, n=0, m=1):
        super().__init__(n)
        self.Blocks = tuple(m) if isinstance(m, (tuple, list)) else (int(m),)

    def blocks(self, mode: int) -> int:
        return self.Blocks[0] if len(self.Blocks) == 1 else self.Blocks[mode]

    def sample(self, mode: int, probs, rng) -> np.ndarray:
        """project_krp of BlockLevScoreSampled (randomized/krp_lev_score_sampled.jl:80-98)."""
        return block_sample_factor_matrices(self.nsamples(mode), probs, self.blocks(mode), mode, rng)


# ---------------------------------------------------------------------------
# Initial guesses (src/cpd.jl:48-84)
# ---------------------------------------------------------------------------
def _row_norm_host(X):
    lam = np.sqrt(np.sum(X * X, axis=0))
    return X / lam[None, :], lam


def random_factors(dims, rank, rng=None, dtype=np.float64):
    """cpd.jl:48-61: iid N(0,1) I_n x R factors (column-major draw order), each
    column-normalised; lambda is that of the last factor.  ``rng`` defaults to a
    generator seeded with 3, as the reference defaults to MersenneTwister(3)."""
    rng = np.random.default_rng(3) if rng is None else rng
    factors, lam = [], None
    for d in dims:
        X = rng.standard_normal(rank * d).reshape(rank, d).T.astype(dtype)
        F, lam = _row_norm_host(X)
        factors.append(F)
    return factors, lam


def random_CPD(target, rank, rng=None) -> CPD:  # noqa: N802 - reference name
    """cpd.jl:63-84."""
    T = np.asarray(target)
    factors, lam = random_factors(T.shape, int(rank), rng, dtype=T.dtype if T.dtype in (np.float32, np.float64)
                                  else np.float64)
    return CPD(factors, lam, T.shape)


def increase_cpd_rank(cpd: CPD, new_rank: int, rng=None) -> CPD:
    """decompose.jl:71-83: new random factors whose first columns are the old ones."""
    old = cp_rank(cpd)
    if new_rank < old:
        raise ValueError("new rank must be >= the old rank")
    factors, lam = random_factors(cpd.inds, new_rank, rng, dtype=cpd.dtype)
    for old_f, new_f in zip(cpd.factors, factors):
        new_f[:, :old] = old_f
    return CPD(factors, lam, cpd.inds)


# ---------------------------------------------------------------------------
# ALS drivers (src/optimizers/)
# ---------------------------------------------------------------------------
def _to_device_check(check) -> L.CpalsCheck:
    c = L.CpalsCheck()
    if isinstance(check, FitCheck):
        c.kind = L.CHECK_FIT
        c.iter = int(check.iter)
        c.counter = int(check.counter)
        c.max_counter = int(check.max_counter)
        c.tolerance = float(check.tolerance)
        c.ref_norm = float(check.ref_norm)
        c.lastfit = float(check.lastfit)
        c.final_fit = float(check.final_fit)
        c.total_iter = int(check.total_iter)
    elif isinstance(check, NoCheck):
        c.kind = L.CHECK_NONE
        c.iter = int(check.iter)
        c.max_counter = int(check.max_counter)
        c.lastfit = float(check.lastfit)
    elif isinstance(check, (CPDiffCheck, CPAngleCheck)):
        angle = isinstance(check, CPAngleCheck)
        c.kind = L.CHECK_ANGLE if angle else L.CHECK_DIFF
        c.iter = int(check.iter)
        c.counter = int(check.counter)
        c.max_counter = int(check.max_counter)
        c.tolerance = float(check.tolerance)
        c.lastfit = float(check.lastangle if angle else check.lastfit)
        c.final_fit = float(check.final_fit)
        c.total_iter = int(check.total_iter)
        c.norm_prev = float(check.norm_prev_iter)
        c.has_prev = 0 if check.PrevCP is None else 1
    else:
        raise NotImplementedError(f"{type(check).__name__} is not supported by the GPU engine")
    return c


def _prev_in(eng, check):
    """Hand a held PrevCP of a CPDiffCheck / CPAngleCheck to the engine."""
    if isinstance(check, (CPDiffCheck, CPAngleCheck)) and check.PrevCP is not None:
        eng.set_prev(check.PrevCP.factors, check.PrevCP.lam)


def _prev_out(eng, check, c: L.CpalsCheck):
    """Copy the check's state back, PrevCP included (None once the check has reset)."""
    angle = isinstance(check, CPAngleCheck)
    check.iter = c.iter
    check.counter = c.counter
    if angle:
        check.lastangle = c.lastfit
    else:
        check.lastfit = c.lastfit
    check.final_fit = c.final_fit
    check.total_iter = c.total_iter
    check.norm_prev_iter = c.norm_prev
    if c.has_prev:
        fs, lam = eng.get_prev()
        check.PrevCP = CPD(fs, lam, tuple(F.shape[0] for F in fs))
    else:
        check.PrevCP = None


def _print_cross(rank, it0, traj, first_last):
    """The reference's verbose line of cp_diff_check.jl:42-44 / cp_angle_check.jl:44-46."""
    prev = first_last
    for k, f in enumerate(traj, start=1):
        if not np.isnan(f):
            print(f"{rank}\t {it0 + k} \t {f} \t {abs(prev - f)}")
            prev = f


def _from_device_check(check, c: L.CpalsCheck, traj, rank, verbose):
    it0 = check.iter
    prev = check.lastfit
    if isinstance(check, FitCheck):
        check.iter = c.iter
        check.counter = c.counter
        check.lastfit = c.lastfit
        check.final_fit = c.final_fit
        check.total_iter = c.total_iter
        check.trajectory.extend(float(x) for x in traj)
        if verbose:
            for k, f in enumerate(traj, start=1):
                print(f"{rank}\t {it0 + k} \t {f} \t {abs(prev - f)}")
                prev = f
    elif isinstance(check, (CPDiffCheck, CPAngleCheck)):
        prev = check.lastangle if isinstance(check, CPAngleCheck) else check.lastfit
        check.trajectory.extend(float(x) for x in traj)
        if verbose:
            _print_cross(rank, it0, traj, prev)
    else:
        check.iter = c.iter
        if verbose:
            for k in range(len(traj)):
                print(f"{rank}\t {it0 + k + 1}")


def _prepare_target(target):
    T = np.asarray(target)
    if T.dtype not in (np.float32, np.float64):
        if np.iscomplexobj(T):
            raise TypeError("complex tensors are not supported by the GPU engine")
        T = T.astype(np.float64)
    return T


def als_optimize(target, cp: CPD, alg=None, check=None, maxiter=None, verbose=False, device=0, rng=None,
                 normal=None, **kwargs) -> CPD:
    """als_optimizer.jl:15-25 / 37-55: default alg KRPFreeNormal, default check NoCheck(maxiter or 100).
    ``normal`` defaults as the algorithm's compute_als does: false for the leverage-score
    solvers (krp_lev_score_sampled.jl:7, 48), true for the QR-pivoted ones
    (optimizers/.../randomized/qr_lev_score_sampled.jl:9, 88, 186)."""
    T = _prepare_target(target)
    alg = KRPFreeNormal() if alg is None else alg
    check = NoCheck(100 if maxiter is None else maxiter) if check is None else check
    R = cp_rank(cp)
    if isinstance(alg, PivotBasedSolvers):
        if normal is not None:
            kwargs["normal"] = normal
        als = compute_als(T, cp, alg=alg, check=check, rng=rng, device=device, **kwargs)
        return optimize(cp, als, verbose=verbose, device=device)
    if isinstance(alg, ProjectionAlgorithm):
        return _lev_score_optimize(T, cp, alg, check, verbose, device, rng, bool(normal),
                                   stop_resample=int(kwargs.get("stop_resample", -1)),
                                   on_pivots=kwargs.get("on_pivots"))
    source = kwargs.get("tensor_source")  # an Engine holding T on the device (decompose's rank loop)
    with Engine(T.shape, R, dtype=T.dtype, precision=alg.precision, device=device, dimtree=alg.dimtree) as eng:
        if source is not None:
            eng.set_tensor_from(source)
        else:
            eng.set_tensor(T)
        eng.set_factors(cp.factors, cp.lam)
        c = _to_device_check(check)
        _prev_in(eng, check)
        traj = eng.optimize(c)
        factors, lam = eng.get_factors()
        _from_device_check(check, c, traj, R, verbose)
        if isinstance(check, (CPDiffCheck, CPAngleCheck)):
            _prev_out(eng, check, c)
    if T.dtype == np.float32:
        factors = [F.astype(np.float32) for F in factors]
        lam = lam.astype(np.float32)
    return CPD(factors, lam, T.shape)


def sample_factor_matrices(nsamps, skip, probs, rng):
    """probability.jl:23-33: independent weighted draws (1-based) for every mode but ``skip``.
    Index drawing stays on the host; the device gathers are bit-exact for these indices."""
    cols = []
    for m, p in enumerate(probs):
        if m == skip:
            continue
        w = np.abs(p)
        cols.append(rng.choice(len(p), size=nsamps, p=w / w.sum()) + 1)
    return np.asfortranarray(np.stack(cols, axis=1).astype(np.int64))


def _draw(p, size, rng):
    w = np.abs(p)
    return rng.choice(len(p), size=size, p=w / w.sum()) + 1


def block_sample_factor_matrices(nsamps, probs, block_size, skip, rng):
    """probability.jl:61-108: the first sampled mode (mode 0, or mode 1 when ``skip`` is 0)
    is cut into floor(I / block_size) blocks, the first I mod block_size of them one index
    longer, each weighted by its summed probability.  For each of nsamps // block_size
    draws, a block is drawn and expanded into consecutive rows that share one independent
    draw of the other modes; rows past nsamps are dropped, and rows the blocks leave empty
    get independent draws of every mode.  Returns nsamps x (N-1) 1-based indices, in the
    column order of ``sample_factor_matrices``.  Draws stay on the host."""
    N = len(probs)
    block_size = int(block_size)
    if block_size < 1:
        raise ValueError("block size must be positive")
    bf = 1 if skip == 0 else 0
    others = [m for m in range(N) if m != skip and m != bf]
    fast = np.abs(np.asarray(probs[bf], dtype=np.float64))
    nblocks, resid = divmod(len(fast), block_size)
    lens = np.array([block_size + (i < resid) for i in range(nblocks)], dtype=np.int64)
    starts = np.concatenate([[1], 1 + np.cumsum(lens)]).astype(np.int64)  # 1-based block starts
    bprob = np.array([fast[starts[i] - 1:starts[i + 1] - 1].sum() for i in range(nblocks)])
    n_iter = nsamps // block_size
    out = np.empty((nsamps, N - 1), dtype=np.int64)
    m = 0
    if n_iter > 0:
        if nblocks == 0:
            raise ValueError("block size exceeds the extent of the blocked mode")
        other_draws = [_draw(probs[o], n_iter, rng) for o in others]
        blk = rng.choice(nblocks, size=n_iter, p=bprob / bprob.sum())
        for i in range(n_iter):
            if m >= nsamps:
                break
            b = blk[i]
            cnt = min(int(lens[b]), nsamps - m)
            out[m:m + cnt, 0] = starts[b] + np.arange(cnt)
            for j, d in enumerate(other_draws):
                out[m:m + cnt, j + 1] = d[i]
            m += cnt
    if m < nsamps:
        tail = nsamps - m
        for j, mode in enumerate([bf] + others):
            out[m:, j] = _draw(probs[mode], tail, rng)
    return np.asfortranarray(out)


def _sampled_loop(T, cp, alg_name, check, verbose, device, normal, begin, pivots_for, after=None):
    """The sweep loop of the ProjectionAlgorithm solvers (optimize.jl:15-32 with
    randomized/ProjectionAlgorithm.jl:6-68): for every sweep and mode, ``pivots_for(mode, it)``
    gives the mode's pivots (1-based multi-coordinates), ``cpals_sampled_update`` runs
    project_krp / matricize_tensor / solve_ls_problem / row_norm on the device, then
    ``after(mode, eng)``.  ``begin(eng)`` runs once, with the tensor and factors set.  A FitCheck
    is not honoured (ProjectionAlgorithm.jl:30-36: a warning, then max_counter sweeps);
    CPDiffCheck / CPAngleCheck run on the device after every sweep."""
    R = cp_rank(cp)
    N = T.ndim
    if isinstance(check, FitCheck) and check.iter == 0:
        print(f"Warning: FitCheck is not enabled for {alg_name} will run {check.max_counter} iterations.")
    sweeps = max(0, int(check.max_counter) - int(check.iter))
    cross = isinstance(check, (CPDiffCheck, CPAngleCheck))
    with Engine(T.shape, R, dtype=T.dtype, precision="fp64", device=device) as eng:
        eng.set_tensor(T)
        eng.set_factors(cp.factors, cp.lam)
        begin(eng)
        if cross:  # ProjectionAlgorithm.jl:53: these checks run as for the exact solvers
            c = _to_device_check(check)
            _prev_in(eng, check)
            first = check.lastangle if isinstance(check, CPAngleCheck) else check.lastfit
            traj = []
        for s in range(sweeps):
            it = int(c.iter) if cross else int(check.iter) + s
            for n in range(N):
                eng.sampled_update(n, pivots_for(n, it), normal=normal)
                if after is not None:
                    after(n, eng)
            if cross:
                done, val = eng.check_converge(c)
                traj.append(val)
                if done:
                    break
            elif verbose:
                print(f"{R}\t{s + 1}")
        factors, lam = eng.get_factors()
        if cross:
            check.trajectory.extend(traj)
            if verbose:
                _print_cross(R, int(check.iter), traj, first)
            _prev_out(eng, check, c)
    if not cross:
        check.iter = 0
    if T.dtype == np.float32:
        factors = [F.astype(np.float32) for F in factors]
        lam = lam.astype(np.float32)
    return CPD(factors, lam, T.shape)


def _lev_score_optimize(T, cp, alg, check, verbose, device, rng, normal, stop_resample=-1, on_pivots=None):
    """LevScoreSampled / BlockLevScoreSampled: compute_als (optimizers/.../krp_lev_score_sampled.jl:1-40,
    42-80: initial leverage weights and one draw per mode) and the per-mode project_krp /
    matricize_tensor / solve / post_solve of algorithms/.../randomized/krp_lev_score_sampled.jl:20-58,
    80-106.  A mode draws new pivots while stop_resample < 0 or stop_resample > iter(als)
    (the check's iteration count); otherwise it reuses its last pivots.  ``on_pivots(mode,
    pivots)`` (optional) sees every mode's pivots before its solve."""
    rng = np.random.default_rng(3) if rng is None else rng
    N = T.ndim
    state = {}

    def begin(eng):
        state["probs"] = [eng.leverage_scores(n) for n in range(N)]
        state["pivots"] = [alg.sample(n, state["probs"], rng) for n in range(N)]

    def pivots_for(n, it):
        if stop_resample < 0 or stop_resample > it:
            state["pivots"][n] = alg.sample(n, state["probs"], rng)
        if on_pivots is not None:
            on_pivots(n, state["pivots"][n])
        return state["pivots"][n]

    def after(n, eng):
        state["probs"][n] = eng.leverage_scores(n)

    return _sampled_loop(T, cp, type(alg).__name__, check, verbose, device, normal, begin, pivots_for, after)


def sparse_sign_matrix(l, n, s, rows=None, vals=None, *, omega=False, injective=False, seed=0, device=0):
    """SEQRCS.jl:29-39: an l x n sparse sign embedding with s nonzeros per column, generated
    on the device (``cpals_sparse_sign``; counter-based draws keyed by ``seed``).  ``rows``
    (Int32, n * s) and ``vals`` (Float64, n * s) are filled in place when given; rows end
    1-based, as the reference leaves them.  Returns the scipy sparse matrix when ``omega``,
    else (rows, vals)."""
    lib = L.load()
    n, s = int(n), int(s)
    s_eff = min(s, int(l))
    rows = np.empty(n * s, dtype=np.int32) if rows is None else rows
    vals = np.empty(n * s, dtype=np.float64) if vals is None else vals
    if rows.dtype != np.int32 or vals.dtype != np.float64 or rows.size < n * s_eff or vals.size < n * s_eff:
        raise TypeError("rows must be Int32 and vals Float64 arrays of n * s entries")
    colstarts = np.empty(n + 1, dtype=np.int32)
    L.check(lib.cpals_sparse_sign(int(device), int(l), n, s, 1 if injective else 0, int(seed) & (2**64 - 1),
                                  rows.ctypes.data_as(C.POINTER(C.c_int32)), L.dptr(vals),
                                  colstarts.ctypes.data_as(C.POINTER(C.c_int32))), "cpals_sparse_sign")
    rows[: n * s_eff] += 1
    if omega:
        import scipy.sparse as sp

        cols = np.repeat(np.arange(n), s_eff)
        return sp.csc_matrix((vals[: n * s_eff], (rows[: n * s_eff] - 1, cols)), shape=(int(l), n))
    return rows, vals


def _omega_entries(omega):
    """(l, 1-based rows, vals, s) of an explicit sparse embedding (a scipy sparse l x n matrix
    with the same number s of stored entries in every column, as sparse_sign_matrix(...;
    omega=true) builds it), in the column-major entry order the generators write."""
    import scipy.sparse as sp

    if not sp.issparse(omega):
        raise TypeError("omega must be a scipy sparse matrix")
    om = sp.csc_matrix(omega)
    om.sort_indices()
    counts = np.diff(om.indptr)
    if counts.size == 0 or np.any(counts != counts[0]) or counts[0] < 1:
        raise ValueError("every column of omega must hold the same number (>= 1) of entries")
    return om.shape[0], om.indices.astype(np.int32) + 1, om.data.astype(np.float64), int(counts[0])


def sketched_matricization(T, k, l, rows=None, vals=None, s=None, device=0):
    """pivot_mapping.jl:111-140: A_sk = T_(k) Omega^T (I_k x l) for the embedding in 1-based
    ``rows`` / ``vals`` (n * s entries, n the product of the other extents).  ``k`` is the
    0-based mode.  ``sketched_matricization(T, k, omega)`` with a scipy sparse Omega is the
    form of pivot_mapping.jl:90-108.  Runs on the device through
    ``cpals_sketched_matricization``."""
    if rows is None and not isinstance(l, (int, np.integer)):
        l, rows, vals, s = _omega_entries(l)
    T = _prepare_target(T)
    r0 = np.ascontiguousarray(rows, dtype=np.int64) - 1
    if r0.size and (r0.min() < 0 or r0.max() >= int(l)):
        raise ValueError("rows must be 1-based and at most l")
    with Engine(T.shape, 1, dtype=T.dtype, precision="fp64", device=device) as eng:
        eng.set_tensor(T)
        return eng.sketched_matricization(int(k), int(l), r0.astype(np.int32), vals, int(s))


# ---------------------------------------------------------------------------
# Column-pivoted QR, SE-QRCS and the QR-pivoted projection solvers
# (src/algebra/SEQRCS.jl, algorithms/.../randomized/qr_lev_score_sampled.jl,
#  optimizers/.../randomized/qr_lev_score_sampled.jl)
# ---------------------------------------------------------------------------
def qrcp(A, *, ncand=0, max_steps=0, stop_ratio=-1.0, device=0):
    """qr(A, ColumnNorm()) on the device (``cpals_qrcp``): returns a QRCPResult whose
    ``Q, R, p`` are LAPACK xGEQP3's (p 1-based).  ``ncand`` limits the pivots to the first
    columns, ``max_steps`` / ``stop_ratio`` end the factorization early."""
    A = np.asfortranarray(np.asarray(A, dtype=np.float64))
    if A.ndim != 2 or A.size == 0:
        raise ValueError("A must be a nonempty matrix")
    m, n = A.shape
    lib = L.load()
    kcap = min(m, n)
    perm = np.empty(n, dtype=np.int64)
    rdiag = np.empty(kcap, dtype=np.float64)
    steps = np.zeros(1, dtype=np.int64)
    R = np.empty(kcap * n, dtype=np.float64)
    Q = np.empty(m * kcap, dtype=np.float64)
    L.check(lib.cpals_qrcp(int(device), m, n, L.dptr(A), int(ncand), int(max_steps), float(stop_ratio),
                           L.i64ptr(perm), L.dptr(rdiag), L.i64ptr(steps), L.dptr(R), L.dptr(Q)), "cpals_qrcp")
    return QRCPResult.make(perm, rdiag, int(steps[0]), m, n, R, Q)


def _embedding(l, n, s, injective, seed, device):
    """An l x n sparse sign embedding from the device generator: 0-based rows, vals, s_eff."""
    rows, vals = sparse_sign_matrix(l, n, s, injective=injective, seed=seed, device=device)
    s_eff = min(int(s), int(l))
    return rows[: n * s_eff] - 1, vals[: n * s_eff], s_eff


def _other_dims(dims, mode):
    return [d for m, d in enumerate(dims) if m != mode]


def SEQRCS(A, mode=None, l=None, s=None, t=None, *, compute_r=True, use_omega=False, injective=False,  # noqa: N802
           rows=None, vals=None, seed=0, stop_ratio=-1.0, device=0):
    """SE-QRCS (src/algebra/SEQRCS.jl:83-240) on the device.  ``SEQRCS(T, mode, l, s, t)``
    pivots the mode unfolding of the tensor T (``mode`` 0-based); ``SEQRCS(factors, l, s, t)``
    (a list of I_m x R matrices) pivots the transposed Khatri-Rao product of the factors
    (SEQRCS.jl:184-240).  The embedding comes from the device generator (``seed``) unless
    1-based ``rows`` / ``vals`` are given.  Returns a QRCPResult: ``Q, R, p = SEQRCS(...)``; R is
    None unless ``compute_r``, and ``rdiag`` always holds diag(R) of the subset's QR."""
    krp = isinstance(A, (list, tuple))
    if krp:
        l, s, t = mode, l, s
        factors = [np.asarray(F, dtype=np.float64) for F in A]
        R = factors[0].shape[1]
        dims = tuple(F.shape[0] for F in factors) + (1,)
        kmode = len(factors)
    else:
        T = _prepare_target(A)
        dims = T.shape
        kmode = int(mode)
    n = int(np.prod(_other_dims(dims, kmode)))
    if rows is None:
        r0, v, s_eff = _embedding(l, n, s, injective, seed, device)
    else:
        s_eff = min(int(s), int(l))
        r0 = np.ascontiguousarray(rows, dtype=np.int64)[: n * s_eff] - 1
        v = np.ascontiguousarray(vals, dtype=np.float64)[: n * s_eff]
    if krp:
        # the KRP path always selects with the explicit Omega (SEQRCS.jl:205-207): column order
        with Engine(dims, R, dtype=np.float64, precision="fp64", device=device) as eng:
            eng.set_factors(list(factors) + [np.ones((1, R))], np.ones(R))
            return eng.seqrcs(1, kmode, l, r0, v, s_eff, t, sorted_subset=True, compute_r=compute_r,
                              stop_ratio=stop_ratio)
    with Engine(dims, 1, dtype=T.dtype, precision="fp64", device=device) as eng:
        eng.set_tensor(T)
        return eng.seqrcs(0, kmode, l, r0, v, s_eff, t, sorted_subset=use_omega, compute_r=compute_r,
                          stop_ratio=stop_ratio)


def omega_hadamard(factors, rows, vals=None, l=None, s=None, device=0):
    """omega_hadamard (src/algebra/had_contract.jl:300-326): Omega times the Khatri-Rao product
    of ``factors`` (I_m x R matrices, the first index fastest), l x R, for the embedding in
    1-based ``rows`` / ``vals``, or ``omega_hadamard(factors, omega)`` with a scipy sparse Omega."""
    if vals is None:
        l, rows, vals, s = _omega_entries(rows)
    factors = [np.asarray(F, dtype=np.float64) for F in factors]
    R = factors[0].shape[1]
    dims = tuple(F.shape[0] for F in factors) + (1,)
    n = int(np.prod(dims))
    s_eff = min(int(s), int(l))
    r0 = np.ascontiguousarray(rows, dtype=np.int64)[: n * s_eff] - 1
    with Engine(dims, R, dtype=np.float64, precision="fp64", device=device) as eng:
        eng.set_factors(list(factors) + [np.ones((1, R))], np.ones(R))
        return eng.omega_hadamard(len(factors), l, r0, np.asarray(vals, dtype=np.float64)[: n * s_eff], s_eff)


def _range_arg(x):
    if isinstance(x, (tuple, list)):
        return tuple(int(v) for v in x)
    return int(x)


class _PivotBased(ProjectionAlgorithm):
    """Start / End of the pivot range (1-based, inclusive; End 0 = every column), one value
    or one per mode (algorithms/.../randomized/qr_lev_score_sampled.jl:10-22)."""

    def __init__(self, start, end):
        self.Start = _range_arg(start)
        self.End = _range_arg(end)

    def _per_mode(self, v, mode):
        return v if isinstance(v, int) else (v[0] if len(v) == 1 else v[mode])


class QRPivProjected(_PivotBased):
    """algorithms/.../randomized/qr_lev_score_sampled.jl:10-22: projection by the pivots of the column-pivoted QR of each
    mode unfolding.  ``QRPivProjected()`` = (1, 0), ``(n)`` = (1, n), ``((n1, n2, ...))`` =
    per-mode ends from 1, ``(start, end)``."""

    def __init__(self, *args):
        if len(args) == 0:
            start, end = 1, 0
        elif len(args) == 1:
            end = args[0]
            start = tuple(1 for _ in end) if isinstance(end, (tuple, list)) else 1
        else:
            start, end = args
        super().__init__(start, end)


class _RandomModes(_PivotBased):
    def __init__(self, *args):
        if len(args) == 0:
            start, end, rr, rank_vect = 1, 0, None, None
        elif len(args) == 1:
            end = args[0]
            start, rr, rank_vect = (tuple(1 for _ in end) if isinstance(end, (tuple, list)) else 1), None, None
        else:
            start, end = args[0], args[1]
            rr = args[2] if len(args) > 2 else None
            rank_vect = args[3] if len(args) > 3 else None
        super().__init__(start, end)
        if rr is not None and not isinstance(rr, (tuple, list)):
            rr = (rr,)
        self.random_modes = None if rr is None else tuple(int(m) for m in rr)
        if rank_vect is None or isinstance(rank_vect, dict):
            self.rank_vect = rank_vect
        else:
            rv = rank_vect if isinstance(rank_vect, (tuple, list)) else (rank_vect,)
            if len(rv) == 1 and len(self.random_modes) > 1:
                rv = tuple(rv) * len(self.random_modes)  # Dict(rrmodes .=> Tuple(r)) broadcasts a scalar
            self.rank_vect = dict(zip(self.random_modes, (int(r) for r in rv)))


class SEQRCSPivProjected(_RandomModes):
    """algorithms/.../randomized/qr_lev_score_sampled.jl:28-50: QRPivProjected with SE-QRCS pivots on ``random_modes``
    (mode numbers from 1, as in the reference); ``rank_vect`` gives each such mode's sketch
    pivot count t."""


class KSEQRCSPivProjected(_RandomModes):
    """algorithms/.../randomized/qr_lev_score_sampled.jl:61-83: pivots from the Khatri-Rao product of a preliminary
    leverage-score ALS solution (SE-QRCS on ``random_modes``, the KRP's pivoted QR elsewhere)."""


PivotBasedSolvers = (QRPivProjected, SEQRCSPivProjected, KSEQRCSPivProjected)


def start(alg):
    return alg.Start


def stop(alg):
    return alg.End


def copy_alg(alg, new_start=0, new_end=0):
    """algorithms/.../randomized/qr_lev_score_sampled.jl:21-22, 49-50, 82-83: the algorithm with a new pivot range
    (0 keeps the old one)."""
    zero = (lambda v: all(int(x) == 0 for x in v)) if isinstance(new_start, (tuple, list)) else (lambda v: int(v) == 0)
    st = alg.Start if zero(new_start) else _range_arg(new_start)
    zero = (lambda v: all(int(x) == 0 for x in v)) if isinstance(new_end, (tuple, list)) else (lambda v: int(v) == 0)
    en = alg.End if zero(new_end) else _range_arg(new_end)
    out = copy.copy(alg)
    out.Start, out.End = st, en
    return out


class ALS:
    """The ALS state compute_als builds for the pivot-based solvers: the target, the algorithm,
    ``additional_items`` (the reference's extra_args keys) and the check."""

    def __init__(self, target, mttkrp_alg, additional_items, check):
        self.target = target
        self.mttkrp_alg = mttkrp_alg
        self.additional_items = additional_items
        self.check = check


def _pivot_range(alg, mode, dRis):
    """optimizers/.../randomized/qr_lev_score_sampled.jl:51-58: the (start, end) of the pivots a mode keeps."""
    int_end = alg._per_mode(stop(alg), mode)
    int_end = dRis if int_end == 0 else int_end
    int_end = min(int_end, dRis)
    int_start = alg._per_mode(start(alg), mode)
    if not (0 < int_start <= int_end):
        raise AssertionError("int_start > 0 && int_start <= int_end")
    return int_start, int_end


def _effective_rank(rdiag, trunc_tol):
    d = np.abs(np.asarray(rdiag, dtype=np.float64))
    if d.size == 0:
        return 0
    with np.errstate(invalid="ignore", divide="ignore"):
        return int(np.sum(d / d.max() > trunc_tol))


def _arrange(p, meff, shuffle_pivots, rng):
    """p1 = p[1:meff] kept, the rest shuffled (optimizers/.../randomized/qr_lev_score_sampled.jl:40-44)."""
    p = np.asarray(p, dtype=np.int64)
    rest = p[meff:]
    if shuffle_pivots:
        rest = rest[rng.permutation(rest.size)]
    return np.concatenate([p[:meff], rest])


def _column_to_multi_coords(cols1, dims):
    """column_to_multi_coords (pivot_mapping.jl:17-35): 1-based linear column ids of the
    other modes (the first fastest) to 1-based coordinates, one row per id."""
    c = np.asarray(cols1, dtype=np.int64) - 1
    out = np.empty((c.size, len(dims)), dtype=np.int64)
    for k, d in enumerate(dims):
        out[:, k] = c % d + 1
        c = c // d
    return out


def compute_als(target, cp: CPD, alg=None, check=None, *, shuffle_pivots=True, trunc_tol=0.01, normal=True,
                injective=False, guess_num_levs=None, prelim_sample_size=None, prelim_niter=10, rng=None, seed=None,
                device=0, **kwargs) -> ALS:
    """compute_als of the pivot-based solvers (optimizers/.../randomized/qr_lev_score_sampled.jl:1-281):
    per mode, the column-pivoted QR of the mode unfolding (QRPivProjected), SE-QRCS on the
    random modes (SEQRCSPivProjected), or of the Khatri-Rao product of a preliminary
    leverage-score ALS solution (KSEQRCSPivProjected); the effective rank meff (the number of
    |r_jj| / max |r_jj| above trunc_tol); the first meff pivots kept and the rest shuffled; the
    pivots start..end as the mode's projector.  Pivot factorizations run on the device; the
    shuffles and the embedding seeds come from ``rng``."""
    if not isinstance(alg, PivotBasedSolvers):
        raise TypeError("compute_als here builds the pivot-based solvers' state")
    T = _prepare_target(target)
    rng = np.random.default_rng(3) if rng is None else rng
    N = T.ndim
    stop_ratio = float(trunc_tol) if shuffle_pivots else -1.0
    random_modes = tuple(getattr(alg, "random_modes", None) or ())
    rank_sk = getattr(alg, "rank_vect", None)
    ref_pivs, pivots, projectors, eff = [], [], [], []

    def finish(n, res):
        dims_o = _other_dims(T.shape, n)
        dRis = int(np.prod(dims_o))
        ref_pivs.append(np.asarray(res.p, dtype=np.int64).copy())
        meff = _effective_rank(res.rdiag, trunc_tol)
        eff.append(meff)
        p = _arrange(res.p, meff, shuffle_pivots, rng)
        pv = _column_to_multi_coords(p, dims_o)
        pivots.append(pv)
        s0, e0 = _pivot_range(alg, n, dRis)
        projectors.append(pv[s0 - 1: e0].copy())

    def sketch_params(n, int_end):
        m = T.shape[n]
        k_sk = int_end if rank_sk is None else int(rank_sk[n + 1])
        l = int(round(3 * m * np.log(m)))
        s = int(round(np.log(m)))
        return l, max(s, 1), k_sk

    if isinstance(alg, KSEQRCSPivProjected):
        # a preliminary leverage-score ALS puts the factors near T's leverage structure
        # (optimizers/.../randomized/qr_lev_score_sampled.jl:194-202)
        if guess_num_levs is None:
            base = cp
            nsamp = 10 * cp_rank(cp) if prelim_sample_size is None else int(prelim_sample_size)
        else:
            base = random_CPD(T, int(guess_num_levs), rng)
            nsamp = 10 * cp_rank(cp) if prelim_sample_size is None else int(prelim_sample_size)
        upd = als_optimize(T, base, alg=LevScoreSampled(nsamp), check=NoCheck(int(prelim_niter)), normal=True,
                           stop_resample=0, rng=rng, device=device)
        Rk = cp_rank(upd)
        with Engine(T.shape, Rk, dtype=np.float64, precision="fp64", device=device) as eng:
            eng.set_factors([np.asarray(F, dtype=np.float64) for F in upd.factors], np.asarray(upd.lam, np.float64))
            for n in range(N):
                dRis = int(np.prod(_other_dims(T.shape, n)))
                _, int_end = _pivot_range(alg, n, dRis)
                if (n + 1) in random_modes:
                    l, s, k_sk = sketch_params(n, int_end)
                    sd = int(rng.integers(0, 2**63)) if seed is None else int(seed) + n
                    r0, v, s_eff = _embedding(l, dRis, s, injective, sd, device)
                    res = eng.seqrcs(1, n, l, r0, v, s_eff, k_sk, sorted_subset=True, stop_ratio=stop_ratio)
                else:
                    res = eng.krp_qrcp(n, stop_ratio=stop_ratio)
                finish(n, res)
    else:
        with Engine(T.shape, 1, dtype=T.dtype, precision="fp64", device=device) as eng:
            eng.set_tensor(T)
            for n in range(N):
                dRis = int(np.prod(_other_dims(T.shape, n)))
                _, int_end = _pivot_range(alg, n, dRis)
                if isinstance(alg, SEQRCSPivProjected) and (n + 1) in random_modes:
                    l, s, k_sk = sketch_params(n, int_end)
                    sd = int(rng.integers(0, 2**63)) if seed is None else int(seed) + n
                    r0, v, s_eff = _embedding(l, dRis, s, injective, sd, device)
                    res = eng.seqrcs(0, n, l, r0, v, s_eff, k_sk, sorted_subset=False, stop_ratio=stop_ratio)
                else:
                    res = eng.unfolding_qrcp(n, stop_ratio=stop_ratio)
                finish(n, res)
    items = {
        "ref_projectors": ref_pivs,
        "projects": pivots,
        "projects_tensors": projectors,
        "effective_ranks": eff,
        "normal": bool(normal),
    }
    return ALS(T, alg, items, NoCheck(100) if check is None else check)


def update_samples(target, als: ALS, new_num_end, reshuffle=False, new_num_start=0, rng=None) -> ALS:
    """update_samples (algorithms/.../randomized/qr_lev_score_sampled.jl:95-149): the same pivots
    with a new range; ``reshuffle`` redraws the order of the pivots past each mode's effective
    rank."""
    if not isinstance(als.mttkrp_alg, PivotBasedSolvers):
        raise AssertionError("als.mttkrp_alg isa PivotBasedSolvers")
    rng = np.random.default_rng() if rng is None else rng
    T = _prepare_target(target)
    alg = copy_alg(als.mttkrp_alg, new_num_start, new_num_end)
    items = dict(als.additional_items)
    pivots = [p.copy() for p in items["projects"]]
    projectors = []
    for pos, (p, meff) in enumerate(zip(items["ref_projectors"], items["effective_ranks"])):
        dims_o = _other_dims(T.shape, pos)
        if reshuffle:
            pivots[pos] = _column_to_multi_coords(_arrange(p, meff, True, rng), dims_o)
        s0, e0 = _pivot_range(alg, pos, int(np.prod(dims_o)))
        projectors.append(pivots[pos][s0 - 1: e0].copy())
    items["projects"] = pivots
    items["projects_tensors"] = projectors
    return ALS(als.target, alg, items, als.check)


def optimize(cp: CPD, als: ALS, verbose=False, device=0) -> CPD:
    """optimize (optimize.jl:6-35) for an ALS built by compute_als: every sweep solves each
    mode's projected problem at its fixed pivots."""
    T = als.target
    proj = als.additional_items["projects_tensors"]
    return _sampled_loop(T, cp, type(als.mttkrp_alg).__name__, als.check, verbose, device,
                         als.additional_items["normal"], lambda eng: None, lambda n, it: proj[n])


def decompose(A, rank, max_rank=None, *, solver=None, rng=None, alg=None, check=None, maxiter=None, verbose=False,
              start_rank=1, rank_step=1, **kwargs) -> CPD:
    """decompose.jl:1-30 (``decompose(A, rank)``) and, with ``max_rank``, the rank-adaptive
    ``decompose(A, epsilon, max_rank)`` of decompose.jl:32-69 (``rank`` is then epsilon)."""
    if solver is not None:
        raise TypeError("OptimizerError: only the ALS solver is available")
    T = _prepare_target(A)
    if max_rank is None:
        cp = random_CPD(T, int(rank), rng)
        return als_optimize(T, cp, alg=alg, check=check, maxiter=maxiter, verbose=verbose, rng=rng, **kwargs)
    epsilon = float(rank)
    if verbose:
        print(f"Starting with rank: {start_rank}")
    current = int(start_rank)
    cpd = random_CPD(T, current, rng)
    check = FitCheck(1e-3, 100, float(np.linalg.norm(T))) if check is None else check
    # one upload of T for every rank: a rank-1 handle owns the device copy and each rank's
    # handle borrows it (the sampled solvers build their own)
    holder = None
    if not isinstance(alg, ProjectionAlgorithm):
        holder = Engine(T.shape, 1, dtype=T.dtype, precision="fp64", device=kwargs.get("device", 0))
        holder.set_tensor(T)
        kwargs = dict(kwargs, tensor_source=holder)
    try:
        while True:
            cpd = als_optimize(T, cpd, alg=alg, check=check, maxiter=maxiter, verbose=verbose, rng=rng, **kwargs)
            check.iter = 0
            if 1.0 - CPDFit(check) < epsilon:
                return cpd
            current += int(rank_step)
            if verbose:
                print(f"\nIncreasing rank to: {current}")
            if current > int(max_rank):
                print(f"Optimization Failed to converge within rank {max_rank}")
                return cpd
            cpd = increase_cpd_rank(cpd, current, rng)
    finally:
        if holder is not None:
            holder.close()

"""CPU oracle for the normal-equation CP-ALS hot path of ITensorCPD.jl (v0.0.82).

TEST INFRASTRUCTURE ONLY.  This module is the checker, never the product: only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl
reference`` legs of ``bench.py`` may import it.  The shipped engine
(``itensorcpd.jl_gb300``) never calls into it and fails loudly when its CUDA
library is missing.

It restates, in FP64 numpy/scipy, each step of the reference's ALS in the
reference's order.  Every function names the reference file:line it follows
(paths relative to the ITensorCPD.jl repository root).

Parity pinning
--------------
* The reference is Julia, and no Julia toolchain exists on either machine, so
  the reference itself cannot be run to produce fixtures.
* The oracle is pinned instead against the reference's own known-answer tests,
  re-expressed in ``tests/test_oracle.py`` with their literal inputs:
  - index maps (``test/pivot_mapping.jl:4-43`` literal pivot columns,
    ``:105-107`` round trip);
  - loop-defined ``had_contract`` / ``pivot_hadamard`` / ``fused_flatten_sample``
    (``test/pivot_mapping.jl:46-103``, ``test/basic_features.jl:18-58``);
  - ``reconstruct`` against explicit loops (``test/basic_features.jl:60-92``);
  - ``row_norm`` unit columns (``test/basic_features.jl:1-16``);
  - end-to-end residual bounds of ``test/cp_als.jl:1-54`` (20x30x40, rank 400).
* Bit-level agreement with Julia is **not** pinned for two things:
  - the ``MersenneTwister`` random streams (initial factors are always supplied
    by the caller instead);
  - the contraction order chosen inside ITensors.jl.
  Both are pinned to tolerance only.
* The pivot solvers and SE-QRCS take pivots from LinearAlgebra's qr(A, ColumnNorm()), which
  is LAPACK xGEQP3, a third-party routine (no Manifest.toml pins its version).
  - ``qrcp_lapack`` calls the same routine through scipy.
  - ``qrcp_loop`` restates it one step at a time: the largest partial norm with ties to the
    first position, xLAQP2's norm downdate with the sqrt(eps) recompute, and xLARFG's
    reflector.
  - ``tests/test_oracle.py`` checks that the loop gives xGEQP3's pivots exactly, and its R
    and Q to rounding.
  - The sparse sign generators are pinned by the reference's own C sources: ``build_oracle.py``
    compiles them into ``_ref/``, and the tests check the layouts against them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.linalg import lapack

# ITensorCPD.jl src/ITensorCPD.jl:2 -- tolerance of the pivoted Cholesky.
CHOLESKY_EPSILON = 1e-6


# ---------------------------------------------------------------------------
# Factor initialisation and normalisation
# ---------------------------------------------------------------------------
def row_norm(X: np.ndarray):
    """src/math_tools/row_norm.jl:4-24: lambda_r = sqrt(sum_i X(i,r)^2), F = X ./ lambda."""
    lam = np.sqrt(np.sum(X * X, axis=0))
    return X / lam[None, :], lam


def random_factors(dims, rank, rng: np.random.Generator):
    """src/cpd.jl:48-61.

    One iid N(0,1) I_n x R matrix per mode, filled in column-major draw order as
    Julia's ``randn`` fills it.  Each is column-normalised; the returned lambda
    is that of the LAST factor (the loop variable ``l`` survives the loop).
    """
    factors, lam = [], None
    for d in dims:
        X = rng.standard_normal(rank * d).reshape(rank, d).T.copy()
        F, lam = row_norm(X)
        factors.append(F)
    return factors, lam


def gram(F: np.ndarray) -> np.ndarray:
    """post_solve, src/algorithms/als_algorithms/standard/tensor.jl:22-25, 46-49: G = F^T F."""
    return F.T @ F


def hadamard_of_grams(grams, skip: int) -> np.ndarray:
    """compute_krp, src/algorithms/als_algorithms/standard/MttkrpAlgorithm.jl:18-31.

    Starts from ones and multiplies the Grams of every mode but ``skip``, in mode order.
    """
    V = np.ones_like(grams[0])
    for i, G in enumerate(grams):
        if i == skip:
            continue
        V = V * G
    return V


# ---------------------------------------------------------------------------
# MTTKRP
# ---------------------------------------------------------------------------
def mttkrp_krp_free(T: np.ndarray, factors, mode: int) -> np.ndarray:
    """matricize_tensor(::KRPFreeNormal), standard/tensor.jl:32-44 with
    had_contract(list, r), src/algebra/had_contract.jl:72-124.

    For every rank column r, T is contracted with the vectors F_m[:, r] of every
    other mode (R independent tensor-times-vector chains, each streaming all of T).
    """
    N = T.ndim
    R = factors[0].shape[1]
    dims = T.shape
    M = np.empty((dims[mode], R))
    Tf = np.asfortranarray(T)
    for r in range(R):
        # trailing modes (last first) then leading modes (first first): each step is a
        # matrix-vector product on a column-major view, the first one streams all of T
        x = Tf
        for m in reversed(range(mode + 1, N)):
            x = np.reshape(x, (-1, dims[m]), order="F") @ factors[m][:, r]
        for m in range(mode):
            x = factors[m][:, r] @ np.reshape(x, (dims[m], -1), order="F")
        M[:, r] = np.reshape(x, -1)
    return M


def khatri_rao(mats) -> np.ndarray:
    """had_contract(factors, r) of the KRPNormal path, standard/tensor.jl:12-20.

    Rows are indexed by the multi-index of ``mats`` with the FIRST matrix's row
    index fastest (column-major fusion of the remaining modes).
    """
    R = mats[0].shape[1]
    K = np.ones((1, R))
    for A in mats:  # first matrix fastest => later matrices vary slowest
        K = (A[:, None, :] * K[None, :, :]).reshape(-1, R)
    return K


def unfold(T: np.ndarray, mode: int) -> np.ndarray:
    """Mode-n unfolding T_(n): I_n x prod(other dims), other modes fused column-major."""
    return np.reshape(np.moveaxis(T, mode, 0), (T.shape[mode], -1), order="F")


def mttkrp_krp(T: np.ndarray, factors, mode: int) -> np.ndarray:
    """matricize_tensor(::KRPNormal), standard/tensor.jl:12-20: T_(n) * KRP."""
    others = [factors[m] for m in range(T.ndim) if m != mode]
    return unfold(T, mode) @ khatri_rao(others)


# ---------------------------------------------------------------------------
# Normal-equation solve
# ---------------------------------------------------------------------------
def _qr_pivoted_solve(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """``qr(A, ColumnNorm()) \\ B`` (Julia LinearAlgebra, QRPivoted ldiv!).

    Column-pivoted Householder QR; numerical rank is cut where the trailing
    R diagonal falls below rcond = min(m, n) * eps relative to |R_11| (Julia
    estimates this incrementally with LAPACK laic1); the truncated system is then
    solved for its minimum-norm solution (Julia: tzrzf + ormrz).
    """
    import scipy.linalg as sla

    m, n = A.shape
    Q, Rm, piv = sla.qr(A, pivoting=True, mode="economic")
    rcond = min(m, n) * np.finfo(np.float64).eps
    d = np.abs(np.diag(Rm))
    rnk = 1
    while rnk < min(m, n) and d[rnk] > rcond * d[0]:
        rnk += 1
    C = Q.T @ B
    Y, *_ = np.linalg.lstsq(Rm[:rnk, :], C[:rnk], rcond=None)
    X = np.empty_like(Y)
    X[piv] = Y
    return X


def pstrf_upper(V: np.ndarray, tol: float = CHOLESKY_EPSILON):
    """LAPACK dpstrf('U', V, tol) as called by ``cholesky(Hermitian(V), RowMaximum(), tol)``.

    Returns (U, piv (0-based), rank): P^T V P = U^T U.
    """
    c, piv, rank, info = lapack.dpstrf(np.array(V, dtype=np.float64, order="F"), tol=tol, lower=0)
    return np.triu(c), piv - 1, int(rank)


def ldiv_solve(A: np.ndarray, B: np.ndarray):
    """ldiv_solve!(A, B; factorizeA=true), src/algebra/ldiv_solve.jl:13-29.

    Square A: pivoted Cholesky (RowMaximum, tol = 1e-6, check = true); a rank
    deficient factor throws, and the catch falls back to column-pivoted QR.
    Non-square A: pivoted QR least squares.
    Returns (X, used_fallback).
    """
    if A.shape[0] == A.shape[1]:
        U, piv, rank = pstrf_upper(A)
        if rank == A.shape[0] and np.all(np.isfinite(U)):
            # CholeskyPivoted ldiv!: permute rows, potrs, inverse-permute.
            Bp = B[piv]
            Y = np.linalg.solve(U.T, Bp)
            Y = np.linalg.solve(U, Y)
            X = np.empty_like(Y)
            X[piv] = Y
            return X, False
        return _qr_pivoted_solve(A, B), True
    return _qr_pivoted_solve(A, B), True


def solve_ls_problem(V: np.ndarray, M: np.ndarray):
    """solve_ls_problem(::MttkrpAlgorithm), MttkrpAlgorithm.jl:34-41: X^T = V \\ M^T."""
    Xt, fb = ldiv_solve(V, M.T)
    return Xt.T.copy(), fb


# ---------------------------------------------------------------------------
# Convergence checks
# ---------------------------------------------------------------------------
def norm_factors(grams, lam) -> float:
    """src/converge_checks/converge_checks.jl:5-11: lambda^T (G_1 o G_2 o ...) lambda."""
    had = grams[0].copy()
    for G in grams[1:]:
        had = had * G
    return float(lam @ had @ lam)


@dataclass
class FitCheck:
    """src/converge_checks/fit_check.jl:5-20 (mutable struct FitCheck)."""

    tolerance: float
    max_counter: int
    ref_norm: float
    iter: int = 0
    counter: int = 0
    lastfit: float = 1.0
    final_fit: float = 0.0
    total_iter: int = 0
    MttKRP: np.ndarray | None = None
    trajectory: list = field(default_factory=list)

    def check_converge(self, factors, lam, grams, verbose=False) -> bool:
        """fit_check.jl:24-66."""
        self.iter += 1
        inner = float(np.sum(self.MttKRP * (factors[-1] * lam[None, :])))
        fact_square = norm_factors(grams, lam)
        norm_res = math.sqrt(abs(self.ref_norm * self.ref_norm + fact_square - 2 * abs(inner)))
        curr_fit = 1.0 - norm_res / self.ref_norm
        dfit = abs(self.lastfit - curr_fit)
        self.lastfit = curr_fit
        self.trajectory.append(curr_fit)
        if verbose:
            print(f"{lam.shape[0]}\t {self.iter} \t {curr_fit} \t {dfit}")
        if math.isnan(curr_fit):
            raise FloatingPointError("Error NAN")
        if dfit < self.tolerance:
            self.counter += 1
            if self.counter >= 2:
                self.total_iter = self.iter
                self.iter = 0
                self.counter = 0
                self.final_fit = self.lastfit
                self.lastfit = 0.0
                return True
        else:
            self.counter = 0
        if self.iter >= self.max_counter:
            self.total_iter = self.iter
            self.iter = 0
            self.counter = 0
            self.final_fit = self.lastfit
            self.lastfit = 0.0
        return False


def cp_cp_inner(prev_factors, prev_lam, factors, lam) -> float:
    """<T_prev, T_curr> as the checks form it: prev_lam^T (P_1^T F_1 o P_2^T F_2 o ...) lam
    (cp_cp_contract, src/algebra/cp_contract.jl:32-52, contracted with both lambdas,
    cp_diff_check.jl:31)."""
    inner = np.ones((prev_lam.shape[0], lam.shape[0]))
    for P, F in zip(prev_factors, factors):
        inner = inner * (P.T @ F)
    return float(prev_lam @ inner @ lam)


def _factor_grams(factors):
    return [F.T @ F for F in factors]


@dataclass
class CPDiffCheck:
    """src/converge_checks/cp_diff_check.jl:6-18 (mutable struct CPDiffCheck)."""

    tolerance: float
    max_counter: int
    iter: int = 0
    counter: int = 0
    norm_prev_iter: float = 0.0
    PrevCP: tuple | None = None  # (factors, lam) of the previous iterate
    lastfit: float = 1.0
    final_fit: float = 0.0
    total_iter: int = 0
    trajectory: list = field(default_factory=list)

    def check_converge(self, factors, lam, grams=None, verbose=False) -> bool:
        """cp_diff_check.jl:20-68."""
        self.iter += 1
        if self.PrevCP is None:
            self.PrevCP = ([F.copy() for F in factors], lam.copy())
            self.norm_prev_iter = norm_factors(_factor_grams(factors), lam)
            self.trajectory.append(float("nan"))
            return False
        inner = cp_cp_inner(self.PrevCP[0], self.PrevCP[1], factors, lam)
        fact_square = norm_factors(_factor_grams(factors), lam)
        norm_res = math.sqrt(abs(self.norm_prev_iter + fact_square - 2 * abs(inner)))
        curr_fit = 1.0 - norm_res / math.sqrt(abs(self.norm_prev_iter))
        dfit = abs(self.lastfit - curr_fit)
        self.lastfit = curr_fit
        self.PrevCP = ([F.copy() for F in factors], lam.copy())
        self.norm_prev_iter = fact_square
        self.trajectory.append(curr_fit)
        if verbose:
            print(f"{lam.shape[0]}\t {self.iter} \t {curr_fit} \t {dfit}")
        return self._count(dfit)

    def _count(self, delta) -> bool:
        """The counter logic shared by both checks (cp_diff_check.jl:46-66)."""
        if delta < self.tolerance:
            self.counter += 1
            if self.counter >= 2:
                self._reset()
                return True
        else:
            self.counter = 0
        if self.iter >= self.max_counter:
            self._reset()
        return False

    def _reset(self):
        self.total_iter = self.iter
        self.iter = 0
        self.counter = 0
        self.final_fit = self.lastfit
        self.lastfit = 0.0
        self.PrevCP = None


@dataclass
class CPAngleCheck(CPDiffCheck):
    """src/converge_checks/cp_angle_check.jl:6-18; ``lastfit`` plays ``lastangle``."""

    def check_converge(self, factors, lam, grams=None, verbose=False) -> bool:
        """cp_angle_check.jl:20-68."""
        self.iter += 1
        if self.PrevCP is None:
            self.PrevCP = ([F.copy() for F in factors], lam.copy())
            self.norm_prev_iter = math.sqrt(norm_factors(_factor_grams(factors), lam))
            self.trajectory.append(float("nan"))
            return False
        numer = cp_cp_inner(self.PrevCP[0], self.PrevCP[1], factors, lam)
        norm_curr = math.sqrt(norm_factors(_factor_grams(factors), lam))
        theta = numer / (norm_curr * self.norm_prev_iter)
        theta = 1.0 if theta > 1.0 else theta
        curr_angle = math.acos(theta) if -1.0 <= theta else float("nan")
        dangle = abs(self.lastfit - curr_angle)
        self.lastfit = curr_angle
        self.PrevCP = ([F.copy() for F in factors], lam.copy())
        self.norm_prev_iter = norm_curr
        self.trajectory.append(curr_angle)
        if verbose:
            print(f"{lam.shape[0]}\t {self.iter} \t {curr_angle} \t {dangle}")
        return self._count(dangle)


@dataclass
class NoCheck:
    """src/converge_checks/no_check.jl:1-20."""

    max_counter: int
    iter: int = 0
    lastfit: float = -1.0

    def check_converge(self, factors, lam, grams, verbose=False) -> bool:
        self.iter += 1
        if verbose:
            print(f"{lam.shape[0]}\t {self.iter}")
        if self.iter == self.max_counter:
            self.iter = 0
            return True
        return False


# ---------------------------------------------------------------------------
# ALS driver
# ---------------------------------------------------------------------------
def als_optimize(T, factors, lam, check=None, maxiter=None, alg="krp", verbose=False, record=None,
                 work_dtype=np.float64):
    """als_optimize -> compute_als -> optimize.

    src/optimizers/als_optimizers/als_optimizer.jl:15-25, 37-55 (defaults: NoCheck(100)),
    optimizers/als_optimizers/standard/tensor.jl:3-14 (initial Grams),
    src/optimizers/als_optimizers/optimize.jl:6-35 (sweep loop).

    ``alg`` = "krp_free" (KRPFreeNormal, the reference default) or "krp" (KRPNormal);
    both compute the same MTTKRP and differ only in rounding order.
    ``record`` (optional list) receives per-sweep dicts with the MTTKRP of every
    mode, for per-call parity checks.  ``work_dtype`` is the factors' element type
    (the reference keeps the target's element type, cpd.jl:63-78; FP64 by default
    here for parity work).
    Returns (factors, lam, check, n_fallbacks).
    """
    if check is None:
        check = NoCheck(100 if maxiter is None else maxiter)
    mttkrp = mttkrp_krp_free if alg == "krp_free" else mttkrp_krp
    factors = [np.array(F, dtype=work_dtype) for F in factors]
    lam = np.array(lam, dtype=work_dtype)
    N = T.ndim
    grams = [gram(F) for F in factors]
    it = check.iter
    n_fallbacks = 0
    while it < check.max_counter:
        M = None
        rec = {"mttkrp": []}
        for n in range(N):
            V = hadamard_of_grams(grams, n)
            M = mttkrp(T, factors, n)
            rec["mttkrp"].append(M)
            X, fb = solve_ls_problem(V.astype(np.float64), M.astype(np.float64))
            n_fallbacks += int(fb)
            factors[n], lam = row_norm(X.astype(work_dtype))
            grams[n] = gram(factors[n])
        if record is not None:
            rec["factors"] = [F.copy() for F in factors]
            rec["lam"] = lam.copy()
            record.append(rec)
        if isinstance(check, FitCheck):
            check.MttKRP = M  # save_mttkrp, fit_check.jl:22
        if check.check_converge(factors, lam, grams, verbose):
            break
        it += 1
    return factors, lam, check, n_fallbacks


def reconstruct(factors, lam) -> np.ndarray:
    """src/algebra/reconstruct.jl:2-9: lambda * had_contract(factors, r)."""
    K = khatri_rao(factors) * lam[None, :]
    dims = [F.shape[0] for F in factors]
    return np.reshape(K.sum(axis=1), dims, order="F")


# ---------------------------------------------------------------------------
# Randomized leverage-score path
# ---------------------------------------------------------------------------
def column_to_multi_coords(col_indices, dims) -> np.ndarray:
    """src/algebra/pivot_mapping.jl:17-35 (1-based in and out, first mode fastest)."""
    col = np.asarray(col_indices, dtype=np.int64) - 1
    out = np.empty((col.shape[0], len(dims)), dtype=np.int64)
    rem = col.copy()
    for j, d in enumerate(dims):
        out[:, j] = rem % d + 1
        rem //= d
    return out


def multi_coords_to_column(sizes, pivots) -> np.ndarray:
    """src/algebra/pivot_mapping.jl:42-47."""
    sizes = list(sizes)
    strides = [int(np.prod(sizes[: len(sizes) - s])) for s in range(1, len(sizes) + 1)]
    piv = np.asarray(pivots, dtype=np.int64)
    return ((piv[:, ::-1] - 1) * np.asarray(strides)[None, :]).sum(axis=1) + 1


def pivot_hadamard(mats, pivots) -> np.ndarray:
    """src/algebra/had_contract.jl:277-295.

    prod = ones(nsamps, R); prod .*= F_m[pivots[:, m], :] for each matrix in order.
    The left-to-right product order is what the device gather reproduces bit for bit.
    """
    piv = np.asarray(pivots, dtype=np.int64)
    prod = np.ones((piv.shape[0], mats[0].shape[1]), dtype=mats[0].dtype)
    for j, F in enumerate(mats):
        prod *= F[piv[:, j] - 1, :]
    return prod


def fused_flatten_sample(T: np.ndarray, k: int, pivots) -> np.ndarray:
    """src/algebra/pivot_mapping.jl:59-85: As(:, s) = T[p_1, ..., :, ..., p_{N-1}] (mode k free)."""
    piv = np.asarray(pivots, dtype=np.int64) - 1
    idx = []
    j = 0
    for m in range(T.ndim):
        if m == k:
            idx.append(np.arange(T.shape[k])[:, None])
        else:
            idx.append(piv[None, :, j])
            j += 1
    return np.asfortranarray(T[tuple(idx)])  # I_k x nsamps


def leverage_score_probabilities(F: np.ndarray) -> np.ndarray:
    """src/math_tools/probability.jl:3-10: row sums of |Q|^2 over min(dims), Q from thin QR."""
    Q, _ = np.linalg.qr(F, mode="reduced")
    return np.sum(Q * Q, axis=1) / min(F.shape)


def sample_factor_matrices(nsamps, skip, probs, rng: np.random.Generator) -> np.ndarray:
    """src/math_tools/probability.jl:23-33 (1-based indices; weighted draws per other mode).

    StatsBase's stream is not reproducible here; the draws come from ``rng``.
    """
    cols = []
    for m, p in enumerate(probs):
        if m == skip:
            continue
        w = np.abs(p) / np.sum(np.abs(p))
        cols.append(rng.choice(len(p), size=nsamps, p=w) + 1)
    return np.stack(cols, axis=1).astype(np.int64)


def block_sample_factor_matrices(nsamps, probs, block_size, skip, rng) -> np.ndarray:
    """probability.jl:61-108, loop for loop (1-based output, ``skip`` 0-based).

    The blocked mode is the first sampled one.  Its indices are cut into
    nblocks = I // block_size blocks, the first I % block_size one longer
    (probability.jl:71-82); each of nsamps // block_size iterations draws the other modes
    once (sample_single_col_from_factors, :17-19) and one block, and writes the block's
    consecutive indices with those draws until nsamps rows are written (:86-100); rows left
    empty get independent draws of every sampled mode (:101-105)."""
    N = len(probs)
    sampled = np.zeros((nsamps, N - 1), dtype=np.int64)
    bf = 1 if skip == 0 else 0
    blocked = np.abs(np.asarray(probs[bf], dtype=np.float64))
    size_fast = len(blocked)
    nblocks, resid = size_fast // block_size, size_fast % block_size
    block_prob, block_starts = [], [1]
    m = 1
    for i in range(1, nblocks + 1):
        ln = block_size + (1 if i <= resid else 0)
        block_prob.append(blocked[m - 1:m - 1 + ln].sum())
        m += ln
        block_starts.append(m)

    def draw(p):
        w = np.abs(p) / np.sum(np.abs(p))
        return int(rng.choice(len(p), p=w)) + 1

    def single_col():
        return [draw(probs[k]) for k in range(N) if k != skip]

    m = 1
    for _ in range(nsamps // block_size):
        other = single_col()
        bp = np.array(block_prob)
        b = int(rng.choice(len(bp), p=bp / bp.sum())) + 1
        start, end = block_starts[b - 1], block_starts[b]
        for j in range(1, end - start + 1):
            if m > nsamps:
                m += 1
                break
            sampled[m - 1, :] = [start + j - 1] + other[1:]
            m += 1
    for i in range(m, nsamps + 1):
        sampled[i - 1, :] = single_col()
    return sampled


def sampled_solve(S: np.ndarray, Ts: np.ndarray, normal: bool):
    """solve_ls_problem(::ProjectionAlgorithm), randomized/ProjectionAlgorithm.jl:57-68.

    normal: (S^T S) X = (Ts S)^T; otherwise the tall problem S X = Ts^T.
    Returns the I_n x R solution.
    """
    if normal:
        Xt, _ = ldiv_solve(S.T @ S, (Ts @ S).T)
    else:
        Xt, _ = ldiv_solve(S, Ts.T)
    return Xt.T.copy()


def lev_score_als(T, factors, lam, nsamps, sweeps, rng, normal=False, record=None, block_size=None,
                  stop_resample=-1):
    """LevScoreSampled path: optimizers/.../randomized/krp_lev_score_sampled.jl:1-40 and
    algorithms/.../randomized/krp_lev_score_sampled.jl:20-58, run for a fixed number of sweeps
    (a FitCheck is not honoured, ProjectionAlgorithm.jl:30-51).  With stop_resample < 0 every
    mode draws new pivots every sweep; otherwise compute_als draws once per mode up front
    and a sweep s draws again only while stop_resample > s (krp_lev_score_sampled.jl:24-25).
    ``record`` receives the per-mode pivots so a device run can replay them.
    ``block_size`` switches to BlockLevScoreSampled's draw (probability.jl:61-108).
    """
    factors = [np.array(F, dtype=np.float64) for F in factors]
    N = T.ndim
    probs = [leverage_score_probabilities(F) for F in factors]

    def draw(n):
        if block_size is None:
            return sample_factor_matrices(nsamps, n, probs, rng)
        return block_sample_factor_matrices(nsamps, probs, block_size, n, rng)

    held = [draw(n) for n in range(N)] if stop_resample >= 0 else [None] * N
    for sweep in range(sweeps):
        for n in range(N):
            if stop_resample < 0 or stop_resample > sweep:
                held[n] = draw(n)
            piv = held[n]
            others = [factors[m] for m in range(N) if m != n]
            S = pivot_hadamard(others, piv)
            Ts = fused_flatten_sample(T, n, piv)
            X = sampled_solve(S, Ts, normal)
            factors[n], lam = row_norm(X)
            probs[n] = leverage_score_probabilities(factors[n])
            if record is not None:
                record.append({"mode": n, "pivots": piv, "factor": factors[n].copy(), "lam": lam.copy()})
    return factors, lam


# ---------------------------------------------------------------------------
# Sparse sign embeddings and the sketched matricization
# ---------------------------------------------------------------------------
def sparse_embedding(l, n, s, rows1, vals) -> np.ndarray:
    """The dense l x n Omega of an embedding given as the reference leaves it after
    sparse_sign_matrix (SEQRCS.jl:29-39): column c's s entries at rows1[c*s : c*s+s] (1-based)
    with values vals[c*s : c*s+s]."""
    om = np.zeros((l, n))
    cols = np.repeat(np.arange(n), s)
    np.add.at(om, (np.asarray(rows1[: n * s], dtype=np.int64) - 1, cols), np.asarray(vals[: n * s]))
    return om


def sketched_matricization(T, k, l, rows1, vals, s) -> np.ndarray:
    """src/algebra/pivot_mapping.jl:111-140, step for step (k 0-based, rows1 1-based).

    The entries are grouped by output column in entry order (dict_rows); entry p belongs to
    column alpha = p div s + (p mod s > 0) of Omega (1-based p), whose fibre starts at
    transform_alpha_to_vectorized_tensor_position (pivot_mapping.jl:52-55); output column j
    is the dot product of the fibres at each mode-k index with the entries' values."""
    v = np.asarray(T).reshape(-1, order="F")
    didx = T.shape[k]
    stride = int(np.prod(T.shape[:k], dtype=np.int64))
    As = np.zeros((didx, l))
    groups = {j: [] for j in range(1, l + 1)}
    for p, j in enumerate(np.asarray(rows1), start=1):
        groups[int(j)].append(p)
    for j in range(1, l + 1):
        nzs = np.asarray(groups[j], dtype=np.int64)
        if nzs.size == 0:
            continue
        alpha = nzs // s + (nzs % s > 0)
        tt = (alpha - 1) // stride
        pos = tt * stride * didx + (alpha - tt * stride)  # 1-based positions
        m2 = np.asarray(vals)[nzs - 1]
        for i in range(didx):
            As[i, j - 1] = np.dot(v[pos - 1 + stride * i], m2)
    return As


def load_ref_sparse_sign():
    """The reference's own generators, compiled by build_oracle.py into _ref/ (None when the
    reference checkout was not available to build them).  Returns (sparse_sign, sparsestack),
    each called as f(l, n, zeta, vals, rows, colstarts) on numpy arrays, as SEQRCS.jl:41-60
    calls them; their rand() stream is srand-seeded by the caller."""
    import ctypes
    from pathlib import Path

    lib_path = Path(__file__).resolve().parent / "_ref" / "libsparse_sign.so"
    if not lib_path.exists():
        return None
    lib = ctypes.CDLL(str(lib_path))
    libc = ctypes.CDLL(None)
    argt = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]

    def wrap(fn):
        fn.argtypes = argt
        fn.restype = None

        def call(l, n, zeta, vals, rows, colstarts, seed=1):
            libc.srand(ctypes.c_uint(seed))
            fn(int(l), int(n), int(zeta), vals.ctypes.data_as(argt[3]), rows.ctypes.data_as(argt[4]),
               colstarts.ctypes.data_as(argt[5]))
        return call

    return wrap(lib.sparse_sign), wrap(lib.sparsestack)


def cpu_als_sweeps(T, factors, lam, sweeps, ref_norm=None, threads=0):
    """The compiled CPU baseline (cpals_cpu.cpp: order-3 normal-equation ALS with the MTTKRP
    in GEMM form, KRPNormal, OpenMP), built by build_oracle.py into _build/.  Returns
    (factors, lam, fits) after `sweeps` sweeps from the given start, or None when the
    library has not been built."""
    import ctypes
    from pathlib import Path

    lib_path = Path(__file__).resolve().parent / "_build" / "libcpals_cpu.so"
    if not lib_path.exists() or T.ndim != 3:
        return None
    lib = ctypes.CDLL(str(lib_path))
    dp = ctypes.POINTER(ctypes.c_double)
    lib.cpu_als_sweeps.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                                   dp, dp, ctypes.c_int, ctypes.c_double, dp, ctypes.c_int]
    lib.cpu_als_sweeps.restype = ctypes.c_int
    Tc = np.asfortranarray(T)
    dtype = 0 if Tc.dtype == np.float64 else 1
    if Tc.dtype not in (np.float64, np.float32):
        Tc = np.asfortranarray(Tc, dtype=np.float64)
        dtype = 0
    dims = np.asarray(Tc.shape, dtype=np.int64)
    R = factors[0].shape[1]
    buf = np.concatenate([np.asarray(F, dtype=np.float64).reshape(-1, order="F") for F in factors])
    lm = np.array(lam, dtype=np.float64)
    fits = np.full(max(1, sweeps), np.nan)
    rn = float(np.linalg.norm(Tc.reshape(-1).astype(np.float64))) if ref_norm is None else float(ref_norm)
    st = lib.cpu_als_sweeps(dtype, Tc.ctypes.data, dims.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(R),
                            buf.ctypes.data_as(dp), lm.ctypes.data_as(dp), int(sweeps), rn,
                            fits.ctypes.data_as(dp), int(threads))
    if st != 0:
        raise ValueError("cpu_als_sweeps rejected its arguments")
    out, o = [], 0
    for d in Tc.shape:
        out.append(buf[o:o + d * R].reshape(d, R, order="F").copy())
        o += d * R
    return out, lm, fits[:sweeps]


# ---------------------------------------------------------------------------
# Column-pivoted QR, SE-QRCS, omega_hadamard, the pivot-based solvers
# ---------------------------------------------------------------------------
def qrcp_lapack(A):
    """qr(A, ColumnNorm()) as the reference calls it (LinearAlgebra's pivoted QR is LAPACK
    xGEQP3; scipy binds the same routine): Q (m x k), R (k x n), p (1-based), k = min(m, n)."""
    import scipy.linalg

    Q, R, p = scipy.linalg.qr(np.asarray(A, dtype=np.float64), mode="economic", pivoting=True)
    return Q, R, p.astype(np.int64) + 1


def qrcp_loop(A, kmax=None, ncand=None, stop_ratio=-1.0):
    """Businger-Golub QR with column pivoting, one step at a time, with xGEQP3's pivot rule
    (largest partial norm, the first position on ties) and xLAQP2's norm downdating with its
    sqrt(eps) recompute safeguard; reflectors in xLARFG's convention.  Pivots are chosen
    among the first ``ncand`` columns; ``kmax`` steps at most; the run ends after the first
    step with |r_jj| <= stop_ratio |r_00| (stop_ratio >= 0).  Returns (p 1-based, rdiag,
    R (k x n), Q (m x k)).  Small cases only."""
    A = np.array(A, dtype=np.float64)
    m, n = A.shape
    ncand = n if ncand is None or ncand <= 0 else min(int(ncand), n)
    kmax = min(m, ncand) if kmax is None or kmax <= 0 else min(int(kmax), m, ncand)
    perm = np.arange(n)
    vn1 = np.sqrt(np.sum(A * A, axis=0))
    vn2 = vn1.copy()
    tol3z = math.sqrt(np.finfo(np.float64).eps)
    rdiag, taus = [], []
    for j in range(kmax):
        p = j + int(np.argmax(vn1[j:ncand]))
        if p != j:
            A[:, [j, p]] = A[:, [p, j]]
            perm[[j, p]] = perm[[p, j]]
            vn1[p], vn2[p] = vn1[j], vn2[j]
        alpha = A[j, j]
        x = A[j + 1:, j]
        s2 = float(x @ x)
        if s2 > 0.0:
            beta = -math.copysign(math.sqrt(alpha * alpha + s2), alpha)
            tau = (beta - alpha) / beta
            A[j + 1:, j] = x * (1.0 / (alpha - beta))
        else:
            beta, tau = alpha, 0.0
        A[j, j] = beta
        rdiag.append(beta)
        taus.append(tau)
        if j + 1 < n:
            v = np.concatenate([[1.0], A[j + 1:, j]])
            w = v @ A[j:, j + 1:]
            A[j:, j + 1:] -= tau * np.outer(v, w)
            c = np.arange(j + 1, ncand)
            c = c[vn1[c] != 0.0]
            if c.size:
                temp = np.maximum(1.0 - (np.abs(A[j, c]) / vn1[c]) ** 2, 0.0)
                temp2 = temp * (vn1[c] / vn2[c]) ** 2
                rec = temp2 <= tol3z
                cr = c[rec]
                if j + 1 < m:
                    vn1[cr] = np.sqrt(np.sum(A[j + 1:, cr] ** 2, axis=0))
                else:
                    vn1[cr] = 0.0
                vn2[cr] = vn1[cr]
                ck = c[~rec]
                vn1[ck] = vn1[ck] * np.sqrt(temp[~rec])
        if stop_ratio >= 0.0 and not (abs(beta) > stop_ratio * abs(rdiag[0])):
            break
    k = len(rdiag)
    R = np.triu(A[:k, :])
    Q = np.eye(m, k)
    for j in range(k - 1, -1, -1):
        v = np.concatenate([[1.0], A[j + 1:, j]])
        Q[j:, j:] -= taus[j] * np.outer(v, v @ Q[j:, j:])
    return perm + 1, np.array(rdiag), R, Q


def _embedding_row_lists(l, n, s, rows1):
    """Columns of Omega (0-based, ascending) with an entry in each row."""
    lists = [[] for _ in range(l)]
    r = np.asarray(rows1[: n * s], dtype=np.int64).reshape(n, s) - 1
    for c in range(n):
        for j in r[c]:
            lists[int(j)].append(c)
    return lists


def seqrcs_subset(l, n, s, rows1, psk1, use_omega) -> np.ndarray:
    """The SE-QRCS column subset (1-based) for sketch pivots psk1 (1-based rows of Omega):
    use_omega, the columns of omega[p_sk, :] with a nonzero, in column order
    (SEQRCS.jl:109-111, 205-207); otherwise, for each pivot row in order, the columns
    holding it, ascending, with repeats dropped (SEQRCS.jl:158-159)."""
    r = np.asarray(rows1[: n * s], dtype=np.int64).reshape(n, s) - 1
    if use_omega:
        sel = set(int(p) - 1 for p in psk1)
        return np.asarray([c + 1 for c in range(n) if any(int(j) in sel for j in r[c])], dtype=np.int64)
    lists = _embedding_row_lists(l, n, s, rows1)
    subset, seen = [], set()
    for p in psk1:
        for c in lists[int(p) - 1]:
            if c not in seen:
                seen.add(c)
                subset.append(c + 1)
    return np.asarray(subset, dtype=np.int64)


def seqrcs(T, k, l, s, t, rows1, vals, use_omega=False, compute_r=True):
    """SE-QRCS of the mode-k unfolding (src/algebra/SEQRCS.jl:89-182; k 0-based): the first t
    pivots of the pivoted QR of the sketch T_(k) Omega^T; the columns of Omega with an entry
    in those rows (use_omega: in column order, SEQRCS.jl:109-111; else for each pivot row in
    order, its columns ascending, first occurrence kept, SEQRCS.jl:158-159); the pivoted QR
    of those columns of T_(k); p = vcat(subset[p_subset], the other columns).  With
    compute_r, R = hcat(R_subset, Q^T A_rem).  Returns (Q, R, p 1-based, diag(R_subset))."""
    A = unfold(np.asarray(T, dtype=np.float64), k)
    n = A.shape[1]
    Ask = sketched_matricization(np.asarray(T, dtype=np.float64), k, l, rows1, vals, s)
    _, _, psk = qrcp_lapack(Ask)
    subset = seqrcs_subset(l, n, s, rows1, psk[:t], use_omega) - 1
    rem = np.setdiff1d(np.arange(n), subset)
    if subset.size == 0:
        return None, None, rem + 1, np.zeros(0)
    Q, R, ps = qrcp_lapack(A[:, subset])
    p = np.concatenate([subset[ps - 1], rem]) + 1
    rd = np.diag(R).copy()
    if compute_r:
        R = np.hstack([R, Q.T @ A[:, rem]])
    return Q, R, p, rd


def omega_hadamard(mats, l, s, rows1, vals) -> np.ndarray:
    """src/algebra/had_contract.jl:300-326: row j of the l x R result is the sum over Omega's
    row j (columns ascending) of the signed Khatri-Rao rows, each the product of the factor
    rows in order."""
    dims = [F.shape[0] for F in mats]
    n = int(np.prod(dims))
    R = mats[0].shape[1]
    lists = _embedding_row_lists(l, n, s, rows1)
    val = {}
    r = np.asarray(rows1[: n * s], dtype=np.int64).reshape(n, s) - 1
    v = np.asarray(vals[: n * s]).reshape(n, s)
    for c in range(n):
        for q in range(s):
            val[(int(r[c, q]), c)] = v[c, q]
    out = np.zeros((l, R))
    for j in range(l):
        cols = np.asarray(lists[j], dtype=np.int64)
        if cols.size == 0:
            continue
        piv = column_to_multi_coords(cols + 1, dims)
        kr = pivot_hadamard(mats, piv)
        signs = np.array([val[(j, int(c))] for c in cols])
        out[j] = np.sum(kr * signs[:, None], axis=0)
    return out


def seqrcs_krp(mats, l, s, t, rows1, vals, compute_r=True):
    """SE-QRCS of the transposed Khatri-Rao product of ``mats`` (src/algebra/SEQRCS.jl:184-240):
    the sketch omega_hadamard(mats, Omega), the first t pivots of the pivoted QR of its
    transpose, the columns of Omega with an entry in those rows (column order), the pivoted QR
    of those KRP rows transposed, p = vcat(subset[p_subset], the rest).  Returns (Q, R, p
    1-based, diag(R_subset))."""
    dims = [F.shape[0] for F in mats]
    n = int(np.prod(dims))
    Ask = omega_hadamard(mats, l, s, rows1, vals)
    _, _, psk = qrcp_lapack(Ask.T.copy())
    subset = seqrcs_subset(l, n, s, rows1, psk[:t], True) - 1
    rem = np.setdiff1d(np.arange(n), subset)
    if subset.size == 0:
        return None, None, rem + 1, np.zeros(0)
    K = khatri_rao(mats)  # n x R, rows in column_to_multi_coords order
    Q, R, ps = qrcp_lapack(K[subset].T.copy())
    p = np.concatenate([subset[ps - 1], rem]) + 1
    rd = np.diag(R).copy()
    if compute_r:
        R = np.hstack([R, Q.T @ K[rem].T])
    return Q, R, p, rd


def effective_rank(rdiag, trunc_tol) -> int:
    """meff = sum(abs.(dr) ./ maximum(abs.(dr)) .> trunc_tol) (optimizers/.../randomized/qr_lev_score_sampled.jl:28)."""
    d = np.abs(np.asarray(rdiag, dtype=np.float64))
    if d.size == 0:
        return 0
    with np.errstate(invalid="ignore", divide="ignore"):
        return int(np.sum(d / d.max() > trunc_tol))


def projected_als(T, factors, lam, projectors, sweeps, normal=True, record=None):
    """The pivot-based solvers' sweeps (optimize.jl:15-32 with algorithms/.../randomized/qr_lev_score_sampled.jl:151-166
    and ProjectionAlgorithm.jl:57-68): every mode solves its projected least-squares problem
    at fixed pivots (``projectors[n]``, 1-based multi-coordinates) and row-normalizes."""
    factors = [np.array(F, dtype=np.float64) for F in factors]
    N = T.ndim
    for _ in range(sweeps):
        for n in range(N):
            others = [factors[m] for m in range(N) if m != n]
            S = pivot_hadamard(others, projectors[n])
            Ts = fused_flatten_sample(T, n, projectors[n])
            X = sampled_solve(S, Ts, normal)
            factors[n], lam = row_norm(X)
            if record is not None:
                record.append({"mode": n, "factor": factors[n].copy(), "lam": lam.copy()})
    return factors, lam


def np_sparse_sign(l, n, s, rng, injective=False):
    """A sparse sign embedding drawn with numpy in the layouts of the reference's C generators
    (src/algebra/sparse_sign.c: s distinct uniform rows per column; sparsestack.c: one uniform
    row in each of s near-equal blocks), values +-1/sqrt(s), rows 1-based; s is clamped to l."""
    s = min(int(s), int(l))
    if injective:
        q, r = divmod(l, s)
        starts = np.array([j * (q + 1) if j < r else r * (q + 1) + (j - r) * q for j in range(s)])
        sizes = np.array([q + 1 if j < r else q for j in range(s)])
        rows = (starts[None, :] + (rng.random((n, s)) * sizes[None, :]).astype(np.int64)).reshape(-1)
    else:
        rows = np.concatenate([rng.choice(l, size=s, replace=False) for _ in range(n)])
    vals = np.where(rng.random(n * s) < 0.5, -1.0, 1.0) / np.sqrt(s)
    return rows.astype(np.int64) + 1, vals, s


def kseqrcs_prelim(T, factors, lam, rng, prelim_niter=10, nsamps=None):
    """The preliminary solve of KSEQRCSPivProjected's compute_als
    (optimizers/.../randomized/qr_lev_score_sampled.jl:194-202): LevScoreSampled(10 R),
    NoCheck(prelim_niter), normal equations, stop_resample = 0."""
    R = factors[0].shape[1]
    return lev_score_als(T, factors, lam, 10 * R if nsamps is None else nsamps, prelim_niter, rng, normal=True,
                         stop_resample=0)


def pivot_solver_setup(T, kind, start=1, end=0, random_modes=(), rank_vect=None, trunc_tol=0.01,
                       shuffle_pivots=True, injective=False, rng=None, krp_factors=None):
    """compute_als of the QR-pivoted solvers (optimizers/.../randomized/qr_lev_score_sampled.jl:1-281):
    kind "qr" (QRPivProjected: pivoted QR of each unfolding), "seqrcs" (SEQRCSPivProjected:
    SE-QRCS on the 1-based ``random_modes``), "kseqrcs" (KSEQRCSPivProjected: SE-QRCS of the KRP
    of ``krp_factors`` on the random modes, its pivoted QR elsewhere).  Per mode: meff = the
    count of |r_jj| / max |r_jj| above trunc_tol, p[1:meff] kept and the rest shuffled, the
    pivots as 1-based multi-coordinates, and rows start..end (end 0 = all, clamped) as the
    projector.  Returns (projectors, effective ranks, 1-based column pivots)."""
    rng = np.random.default_rng(3) if rng is None else rng
    N = T.ndim
    projectors, effs, refs = [], [], []
    for n in range(N):
        dims_o = [d for m, d in enumerate(T.shape) if m != n]
        dRis = int(np.prod(dims_o))
        e = end if isinstance(end, int) else (end[0] if len(end) == 1 else end[n])
        int_end = dRis if e == 0 else min(e, dRis)
        st = start if isinstance(start, int) else (start[0] if len(start) == 1 else start[n])
        assert 0 < st <= int_end
        m = T.shape[n]
        rand = (n + 1) in tuple(random_modes or ())
        if rand:
            l, s = int(round(3 * m * np.log(m))), max(1, int(round(np.log(m))))
            t = int_end if rank_vect is None else int(rank_vect[n + 1])
            rows1, vals, s = np_sparse_sign(l, dRis, s, rng, injective)
        if kind == "qr" or (kind == "seqrcs" and not rand):
            _, R, p = qrcp_lapack(unfold(T, n))
            dr = np.diag(R)
        elif kind == "seqrcs":
            _, _, p, dr = seqrcs(T, n, l, s, t, rows1, vals, use_omega=False, compute_r=False)
        elif rand:
            others = [krp_factors[k] for k in range(N) if k != n]
            _, _, p, dr = seqrcs_krp(others, l, s, t, rows1, vals, compute_r=False)
        else:
            others = [krp_factors[k] for k in range(N) if k != n]
            _, R, p = qrcp_lapack(khatri_rao(others).T.copy())
            dr = np.diag(R)
        refs.append(np.asarray(p, dtype=np.int64))
        meff = effective_rank(dr, trunc_tol)
        effs.append(meff)
        rest = np.asarray(p[meff:], dtype=np.int64)
        if shuffle_pivots:
            rest = rest[rng.permutation(rest.size)]
        pp = np.concatenate([np.asarray(p[:meff], dtype=np.int64), rest])
        projectors.append(column_to_multi_coords(pp, dims_o)[st - 1: int_end])
    return projectors, effs, refs


def projected_als_check(T, factors, lam, projectors, check, normal=True):
    """optimize (optimize.jl:15-32) for a pivot-based solver: projected sweeps at fixed pivots
    until a CPDiffCheck / CPAngleCheck stops them, or check.max_counter sweeps under a FitCheck
    or NoCheck, which the projection solvers do not evaluate (ProjectionAlgorithm.jl:30-51)."""
    factors = [np.array(F, dtype=np.float64) for F in factors]
    cross = isinstance(check, CPDiffCheck)
    for _ in range(int(check.max_counter)):
        factors, lam = projected_als(T, factors, lam, projectors, 1, normal)
        if cross and check.check_converge(factors, lam):
            break
    return factors, lam


# ---------------------------------------------------------------------------
# Synthetic low-rank-plus-noise generator (the benchmark workloads' tensors)
# ---------------------------------------------------------------------------
def congruent_factor(dim, rank, congruence, rng) -> np.ndarray:
    """I x R factor with unit columns and pairwise column inner product ``congruence``.

    iid N(0,1) entries are orthonormalised (QR), then mixed by the transposed
    Cholesky factor of C = (1 - c) I + c 11^T, so A^T A = C exactly.
    """
    Z = rng.standard_normal((dim, rank))
    C = (1.0 - congruence) * np.eye(rank) + congruence * np.ones((rank, rank))
    L = np.linalg.cholesky(C)
    if rank <= dim:
        Q, _ = np.linalg.qr(Z)
        return Q @ L.T
    # rank > dim: A^T A = C cannot hold; unit iid columns mixed by L, renormalised
    A = (Z / np.linalg.norm(Z, axis=0)) @ L.T
    return A / np.linalg.norm(A, axis=0)


def lowrank_plus_noise(dims, rank, congruence, snr_db, rng, wmin=1.0, wmax=10.0, dtype=np.float32):
    """Sum of ``rank`` weighted rank-1 terms (weights U[wmin, wmax]) plus iid Gaussian
    noise at ``snr_db``.  Returns (T column-major, true factors, weights)."""
    facs = [congruent_factor(d, rank, congruence, rng) for d in dims]
    w = rng.uniform(wmin, wmax, size=rank)
    A0 = facs[0] * w[None, :]
    K = khatri_rao(facs[1:])
    S = (A0 @ K.T).astype(dtype)  # I_1 x prod(rest), column-major fusion
    sn = float(np.linalg.norm(S))
    noise = rng.standard_normal(S.shape).astype(dtype)
    nn = float(np.linalg.norm(noise))
    S += noise * dtype(sn / nn / (10.0 ** (snr_db / 20.0)))
    T = np.reshape(S, dims, order="F")
    return np.asfortranarray(T), facs, w

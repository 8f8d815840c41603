"""Generate the golden fixtures under tests/golden/ (run from the repo root:
``python tests/golden/make_golden.py``).

The reference (Julia) cannot run on either machine, so the fixtures come from:
  * literal inputs of the reference's own tests, with answers defined independently of
    the oracle (Julia column-major reshape == numpy ``unravel_index(order="F")``,
    explicit loops) -- test/pivot_mapping.jl:4-43, 46-107;
  * the oracle (tests pin the oracle against the reference's known-answer tests first)
    run on inputs from ``det_normal``, a platform-independent generator, so the GPU machine
    regenerates exactly the same inputs without shipping large arrays.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))

import cpals_oracle as oracle  # noqa: E402
from _data import det_factors, det_normal  # noqa: E402


def index_maps():
    # test/pivot_mapping.jl:6-43, literal pivot columns and dims
    cases = [
        {"tensor_dims": [4, 5, 6, 3], "mode": 1, "col_dims": [5, 6, 3],
         "pivots": [1, 4, 7, 12, 29, 30, 8, 21, 17, 42, 62, 86, 72]},
        {"tensor_dims": [3, 6, 8, 2], "mode": 3, "col_dims": [3, 6, 2],
         "pivots": [1, 3, 7, 14, 29, 30, 10, 22, 35, 8, 11]},
    ]
    for c in cases:
        coords = np.stack(np.unravel_index(np.asarray(c["pivots"]) - 1, c["col_dims"], order="F"), axis=1) + 1
        c["coords"] = coords.tolist()
    return cases


def als_small():
    dims, R = (12, 13, 7), 5
    T = np.asfortranarray(det_normal(11, dims))
    F, lam = det_factors(dims, R, seed=3)
    rec = []
    chk = oracle.FitCheck(1e-10, 8, float(np.linalg.norm(T)))
    Ff, lf, chk, fb = oracle.als_optimize(T, F, lam, check=chk, record=rec)
    return {
        "dims": list(dims), "rank": R, "tensor_seed": 11, "factor_seed": 3,
        "tol": 1e-10, "max_counter": 8,
        "trajectory": chk.trajectory, "total_iter": chk.total_iter, "final_fit": chk.final_fit,
        "mttkrp_sweep1": [m.tolist() for m in rec[0]["mttkrp"]],
        "final_factors": [f.tolist() for f in Ff], "final_lambda": lf.tolist(), "fallbacks": fb,
    }


def als_c1():
    # The reference's CPU-runnable workload: 100^3 FP64 N(0,1), rank 50,
    # FitCheck(1e-3, 100, norm(T)), random_CPD initial factors.
    dims, R = (100, 100, 100), 50
    T = np.asfortranarray(det_normal(1, dims))
    F, lam = det_factors(dims, R, seed=3)
    chk = oracle.FitCheck(1e-3, 100, float(np.linalg.norm(T)))
    _, _, chk, fb = oracle.als_optimize(T, F, lam, check=chk)
    return {"dims": list(dims), "rank": R, "tensor_seed": 1, "factor_seed": 3, "tol": 1e-3, "max_counter": 100,
            "trajectory": chk.trajectory, "total_iter": chk.total_iter, "final_fit": chk.final_fit,
            "fallbacks": fb}


def rank_deficient():
    # Duplicated factor columns make every Hadamard of Grams singular: the pivoted
    # Cholesky stops early and the solve takes the pivoted-QR path (ldiv_solve.jl:17-22).
    dims, R = (9, 8, 7), 4
    T = np.asfortranarray(det_normal(21, dims))
    F, lam = det_factors(dims, R, seed=22)
    for f in F:
        f[:, 3] = f[:, 2]
    rec = []
    chk = oracle.NoCheck(1)
    Ff, lf, _, fb = oracle.als_optimize(T, F, lam, check=chk, record=rec)
    return {"dims": list(dims), "rank": R, "tensor_seed": 21, "factor_seed": 22, "fallbacks": fb,
            "factors_after_sweep1": [f.tolist() for f in Ff], "lambda": lf.tolist()}


def lev_small():
    # test/rand_cp_als.jl:98-121: 12x13x3 exact rank-5 target, LevScoreSampled.
    dims, R = (12, 13, 3), 5
    Ft, lt = det_factors(dims, R, seed=31)
    T = np.asfortranarray(oracle.reconstruct(Ft, lt))
    F, lam = det_factors(dims, R, seed=32)
    out = {"dims": list(dims), "rank": R, "truth_seed": 31, "factor_seed": 32, "runs": []}
    for normal, nsamps in ((True, 100), (False, 100)):
        rec = []
        Ff, lf = oracle.lev_score_als(T, F, lam, nsamps, 3, np.random.default_rng(33), normal=normal, record=rec)
        out["runs"].append({
            "normal": normal, "nsamps": nsamps,
            "steps": [{"mode": r["mode"], "pivots": r["pivots"].tolist(), "factor": r["factor"].tolist(),
                       "lambda": r["lam"].tolist()} for r in rec],
            "rel_error": float(np.linalg.norm(oracle.reconstruct(Ff, lf) - T) / np.linalg.norm(T)),
        })
    return out


def qrcp_pivots():
    # qr(A, ColumnNorm()) (LAPACK xGEQP3, which the pivot solvers and SEQRCS call) on seeded
    # matrices: Gaussian, a mode-1 unfolding, and rank 5 with 1e-9 noise (first 6 pivots only;
    # the rest sit at the noise level).  Pivots 1-based, |diag(R)|.
    out = []
    for name, seed, shape in (("gauss_30x50", 51, (30, 50)), ("gauss_64x40", 52, (64, 40)),
                              ("gauss_1x9", 53, (1, 9))):
        A = det_normal(seed, shape)
        _, R, p = oracle.qrcp_lapack(A)
        out.append({"name": name, "seed": seed, "shape": list(shape), "p": p.tolist(),
                    "absdiag": np.abs(np.diag(R)).tolist(), "compare": p.size})
    dims = (8, 9, 10)
    T = np.asfortranarray(det_normal(54, dims))
    _, R, p = oracle.qrcp_lapack(oracle.unfold(T, 1))
    out.append({"name": "unfold_8x9x10_mode1", "seed": 54, "tensor_dims": list(dims), "mode": 1, "p": p.tolist(),
                "absdiag": np.abs(np.diag(R)).tolist(), "compare": p.size})
    A = det_normal(55, (40, 5)) @ det_normal(56, (5, 300)) + 1e-9 * det_normal(57, (40, 300))
    _, R, p = oracle.qrcp_lapack(A)
    out.append({"name": "rank5_noise_40x300", "seeds": [55, 56, 57], "shape": [40, 300], "p": p.tolist(),
                "absdiag": np.abs(np.diag(R)).tolist(), "compare": 6})
    return out


def seqrcs_small():
    # SEQRCS.jl:139-182 (subset in pivot order) on a seeded 20x30x10 tensor, mode 0,
    # l = round(3 m ln m) = 180, s = round(ln m) = 3, t = 8, with a stored embedding of the
    # sparse_sign layout (3 distinct rows per column, +-1/sqrt(3)).
    dims, k = (20, 30, 10), 0
    T = np.asfortranarray(det_normal(61, dims))
    m = dims[k]
    n = int(np.prod(dims)) // m
    l, s, t = int(round(3 * m * np.log(m))), int(round(np.log(m))), 8
    rng = np.random.default_rng(62)
    rows = np.concatenate([rng.choice(l, size=s, replace=False) for _ in range(n)]).astype(np.int64) + 1
    vals = np.where(rng.random(n * s) < 0.5, -1.0, 1.0) / np.sqrt(s)
    out = {"tensor_dims": list(dims), "seed": 61, "mode": k, "l": l, "s": s, "t": t,
           "rows": rows.tolist(), "vals": vals.tolist(), "cases": []}
    for use_omega in (False, True):
        _, _, p, rd = oracle.seqrcs(T, k, l, s, t, rows, vals, use_omega=use_omega, compute_r=False)
        out["cases"].append({"use_omega": use_omega, "p": p.tolist(), "absdiag": np.abs(rd).tolist()})
    return out


def main():
    (HERE / "index_maps.json").write_text(json.dumps(index_maps()))
    (HERE / "als_small.json").write_text(json.dumps(als_small()))
    (HERE / "als_c1.json").write_text(json.dumps(als_c1()))
    (HERE / "rank_deficient.json").write_text(json.dumps(rank_deficient()))
    (HERE / "lev_small.json").write_text(json.dumps(lev_small()))
    (HERE / "qrcp_pivots.json").write_text(json.dumps(qrcp_pivots()))
    (HERE / "seqrcs_small.json").write_text(json.dumps(seqrcs_small()))
    for p in sorted(HERE.glob("*.json")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()

"""Platform-independent synthetic inputs for the tests.

``det_normal`` hashes (seed, index) with SplitMix64 and applies Box-Muller, so the
same arrays come out on x86 and Arm with any numpy version (up to libm rounding of
log/cos, 1e-16 relative).
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)


def _splitmix(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + _G
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def det_uniform(seed: int, n: int) -> np.ndarray:
    idx = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = _splitmix(idx * np.uint64(2) + np.uint64(seed) * np.uint64(0x100000001B3))
    return ((x >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def det_normal(seed: int, shape) -> np.ndarray:
    """iid N(0,1) array of ``shape`` in column-major fill order."""
    n = int(np.prod(shape))
    u = det_uniform(seed, 2 * ((n + 1) // 2))
    u1, u2 = u[0::2], u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])[:n]
    return np.reshape(z, shape, order="F")


def det_factors(dims, rank, seed):
    """random_factors (src/cpd.jl:48-61) with det_normal draws: unit columns, lambda of the last."""
    factors, lam = [], None
    for k, d in enumerate(dims):
        X = det_normal(seed * 1000 + k, (d, rank))
        lam = np.sqrt(np.sum(X * X, axis=0))
        factors.append(X / lam[None, :])
    return factors, lam


def golden_qrcp_matrix(case):
    """The matrix of one qrcp_pivots.json case, rebuilt from its seeds."""
    if "tensor_dims" in case:
        T = np.asfortranarray(det_normal(case["seed"], case["tensor_dims"]))
        k = case["mode"]
        return np.reshape(np.moveaxis(T, k, 0), (T.shape[k], -1), order="F")
    if "seeds" in case:  # rank 5 (40 x 5 times 5 x 300) plus 1e-9 noise
        a, b, c = case["seeds"]
        return det_normal(a, (40, 5)) @ det_normal(b, (5, 300)) + 1e-9 * det_normal(c, (40, 300))
    return det_normal(case["seed"], case["shape"])

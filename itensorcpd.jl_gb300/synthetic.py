"""Seeded synthetic tensors with the benchmark workloads' structure.

A sum of ``rank`` weighted rank-1 terms whose factor columns have unit norm and a set
pairwise congruence (inner product), plus iid Gaussian noise at a set SNR.  Nothing
here runs on the ALS path; it only makes inputs.
"""
from __future__ import annotations

import numpy as np


def congruent_factor(dim, rank, congruence, rng):
    """dim x rank, unit columns, A^T A = (1 - c) I + c 11^T (orthonormalised draws mixed by
    the transposed Cholesky factor of the congruence matrix)."""
    Z = rng.standard_normal((dim, rank))
    C = (1.0 - congruence) * np.eye(rank) + congruence * np.ones((rank, rank))
    if rank <= dim:
        Q, _ = np.linalg.qr(Z)
        return Q @ np.linalg.cholesky(C).T
    # more columns than rows: the congruence can hold only approximately; unit-norm iid
    # columns mixed by the same Cholesky factor, renormalised
    A = (Z / np.linalg.norm(Z, axis=0)) @ np.linalg.cholesky(C).T
    return A / np.linalg.norm(A, axis=0)


def _khatri_rao(mats):
    R = mats[0].shape[1]
    K = np.ones((1, R))
    for A in mats:
        K = (A[:, None, :] * K[None, :, :]).reshape(-1, R)
    return K


def lowrank_plus_noise(dims, rank, congruence, snr_db, rng, wmin=1.0, wmax=10.0, dtype=np.float32, out=None):
    """Column-major tensor of ``dims`` (written into ``out`` if given, e.g. pinned memory).
    Returns (T, true factors, weights)."""
    facs = [congruent_factor(d, rank, congruence, rng) for d in dims]
    w = rng.uniform(wmin, wmax, size=rank)
    A0 = (facs[0] * w[None, :]).astype(dtype)
    K = _khatri_rao(facs[1:]).astype(dtype)
    S = A0 @ K.T  # I_1 x prod(rest): column-major fusion of modes 2..N
    sn = float(np.linalg.norm(S))
    noise = rng.standard_normal(S.shape, dtype=np.float32).astype(dtype, copy=False)
    nn = float(np.linalg.norm(noise))
    noise *= dtype(sn / nn / (10.0 ** (snr_db / 20.0)))
    S += noise
    del noise
    T = np.reshape(S, dims, order="F")
    if out is not None:
        out[...] = T
        T = out
    return np.asfortranarray(T), facs, w

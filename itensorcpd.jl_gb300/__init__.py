"""GB300-native CP-ALS engine with ITensorCPD.jl's API.

The compute path is libcpals.so (hand-written CUDA for sm_103a, C ABI in
include/cpals.h); this package is the host side that mirrors the reference's
``decompose`` / ``random_CPD`` / ``als_optimize`` / ``FitCheck`` / ``CPDiffCheck`` /
``CPAngleCheck`` / ``CPD`` interface.
"""
from ._lib import CpalsError, load
from .api import (
    BlockLevScoreSampled,
    CPD,
    CPAngleCheck,
    CPDFit,
    CPDiffCheck,
    ConvergeAlg,
    FitCheck,
    GB300Normal,
    KRPFreeNormal,
    KRPNormal,
    LevScoreSampled,
    MttkrpAlgorithm,
    NoCheck,
    ProjectionAlgorithm,
    als_optimize,
    cp_rank,
    decompose,
    increase_cpd_rank,
    random_CPD,
    random_factors,
    block_sample_factor_matrices,
    sample_factor_matrices,
    sketched_matricization,
    sparse_sign_matrix,
    ALS,
    KSEQRCSPivProjected,
    QRPivProjected,
    SEQRCS,
    SEQRCSPivProjected,
    compute_als,
    copy_alg,
    omega_hadamard,
    optimize,
    qrcp,
    start,
    stop,
    update_samples,
)
from .batched import BatchEngine
from .engine import Engine, QRCPResult
from . import warmstart
from .warmstart import WarmStartMLP

__all__ = [
    "BatchEngine", "BlockLevScoreSampled", "CPAngleCheck", "CPD", "CPDFit", "CPDiffCheck", "ConvergeAlg", "CpalsError", "Engine", "FitCheck", "GB300Normal", "KRPFreeNormal", "KRPNormal",
    "LevScoreSampled", "MttkrpAlgorithm", "NoCheck", "ProjectionAlgorithm", "als_optimize", "cp_rank", "decompose",
    "increase_cpd_rank", "load", "random_CPD", "random_factors", "sample_factor_matrices", "block_sample_factor_matrices", "sparse_sign_matrix", "sketched_matricization", "WarmStartMLP", "warmstart",
    "ALS", "KSEQRCSPivProjected", "QRCPResult", "QRPivProjected", "SEQRCS", "SEQRCSPivProjected", "compute_als",
    "copy_alg", "omega_hadamard", "optimize", "qrcp", "start", "stop", "update_samples",
]

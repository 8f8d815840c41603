"""ctypes binding of libcpals.so (the C ABI declared in include/cpals.h)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libcpals.so"

CPALS_OK = 0
CPALS_E_ARG = -1
CPALS_E_CUDA = -2
CPALS_E_NAN = -3
CPALS_E_STATE = -4
CPALS_E_UNSUPPORTED = -5
CPALS_E_DEVICE = -6

DTYPE_F64 = 0
DTYPE_F32 = 1
MTTKRP_FP64 = 0
MTTKRP_BF16X3 = 1
FLAG_NO_GRAPH = 1
FLAG_DIMTREE = 2
FLAG_LOWMEM = 4
FLAG_FUSED_TAIL = 8
CHECK_NONE = 0
CHECK_FIT = 1
CHECK_DIFF = 2
CHECK_ANGLE = 3


class CpalsCheck(C.Structure):
    """Mirror of ``cpals_check`` (include/cpals.h)."""

    _fields_ = [
        ("kind", C.c_int32),
        ("iter", C.c_int32),
        ("counter", C.c_int32),
        ("max_counter", C.c_int32),
        ("tolerance", C.c_double),
        ("ref_norm", C.c_double),
        ("lastfit", C.c_double),
        ("final_fit", C.c_double),
        ("total_iter", C.c_int32),
        ("sweeps_run", C.c_int32),
        ("norm_prev", C.c_double),
        ("has_prev", C.c_int32),
        ("reserved", C.c_int32),
    ]


# name -> (restype, argtypes); every exported entry point of include/cpals.h
_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)
SIGNATURES = {
    "cpals_version": (C.c_int, []),
    "cpals_status_string": (C.c_char_p, [C.c_int]),
    "cpals_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int, _I64P, C.c_int64, C.c_int, C.c_int, C.c_int]),
    "cpals_destroy": (C.c_int, [_P]),
    "cpals_set_tensor": (C.c_int, [_P, _P]),
    "cpals_set_tensor_device": (C.c_int, [_P, _P]),
    "cpals_tensor_device": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "cpals_set_factors": (C.c_int, [_P, C.POINTER(_DP), _DP]),
    "cpals_get_factors": (C.c_int, [_P, C.POINTER(_DP), _DP]),
    "cpals_get_gram": (C.c_int, [_P, C.c_int, _DP]),
    "cpals_mttkrp": (C.c_int, [_P, C.c_int, _DP]),
    "cpals_optimize": (C.c_int, [_P, C.POINTER(CpalsCheck), _DP, C.c_int64]),
    "cpals_check_converge": (C.c_int, [_P, C.POINTER(CpalsCheck), C.POINTER(C.c_int), _DP]),
    "cpals_get_prev": (C.c_int, [_P, C.POINTER(_DP), _DP]),
    "cpals_set_prev": (C.c_int, [_P, C.POINTER(_DP), _DP]),
    "cpals_sparse_sign": (C.c_int, [C.c_int, C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_uint64,
                                    C.POINTER(C.c_int32), _DP, C.POINTER(C.c_int32)]),
    "cpals_sketched_matricization": (C.c_int, [_P, C.c_int, C.c_int64, C.c_int, C.POINTER(C.c_int32), _DP, _DP]),
    "cpals_qrcp": (C.c_int, [C.c_int, C.c_int64, C.c_int64, _DP, C.c_int64, C.c_int64, C.c_double, _I64P, _DP,
                             _I64P, _DP, _DP]),
    "cpals_unfolding_qrcp": (C.c_int, [_P, C.c_int, C.c_int64, _I64P, C.c_int64, C.c_int64, C.c_double, _I64P,
                                       _DP, _I64P, _DP, _DP]),
    "cpals_krp_qrcp": (C.c_int, [_P, C.c_int, C.c_int64, _I64P, C.c_int64, C.c_int64, C.c_double, _I64P, _DP,
                                 _I64P, _DP, _DP]),
    "cpals_omega_hadamard": (C.c_int, [_P, C.c_int, C.c_int64, C.c_int, C.POINTER(C.c_int32), _DP, _DP]),
    "cpals_seqrcs_subset": (C.c_int, [C.c_int64, C.c_int64, C.c_int, C.POINTER(C.c_int32), C.c_int64, _I64P, C.c_int,
                                      _I64P, _I64P]),
    "cpals_seqrcs": (C.c_int, [_P, C.c_int, C.c_int, C.c_int64, C.c_int, C.POINTER(C.c_int32), _DP, C.c_int64,
                               C.c_int, C.c_int, C.c_double, _I64P, _DP, _I64P, _I64P, _DP, _DP]),
    "cpals_fallback_count": (C.c_int, [_P, _I64P]),
    "cpals_synchronize": (C.c_int, [_P]),
    "cpals_timer_start": (C.c_int, [_P]),
    "cpals_timer_stop": (C.c_int, [_P, _DP]),
    "cpals_set_profiling": (C.c_int, [_P, C.c_int]),
    "cpals_profile_read": (C.c_int, [_P, _DP, _I64P]),
    "cpals_launch_count": (C.c_int, [_P, _I64P]),
    "cpals_set_cluster_sweep_min_rank": (C.c_int, [C.c_int]),
    "cpals_mttkrp_fp64_noalloc": (C.c_int, [C.c_int, _I64P, C.c_int64, C.c_int, C.c_int, _P, C.POINTER(_DP), _DP,
                                            _P]),
    "cpals_mode_update": (C.c_int, [_P, C.c_int, _DP]),
    "cpals_profile_read_sampled": (C.c_int, [_P, _DP, _DP, _I64P]),
    "cpals_tensor_norm": (C.c_int, [_P, _DP, _DP]),
    "cpals_pivot_hadamard": (C.c_int, [_P, C.c_int, _I64P, C.c_int64, _DP]),
    "cpals_fused_flatten_sample": (C.c_int, [_P, C.c_int, _I64P, C.c_int64, _P]),
    "cpals_leverage_scores": (C.c_int, [_P, C.c_int, _DP]),
    "cpals_sampled_update": (C.c_int, [_P, C.c_int, _I64P, C.c_int64, C.c_int]),
    "cpals_batch_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int64, _I64P, _I64P, _DP]),
    "cpals_batch_destroy": (C.c_int, [_P]),
    "cpals_batch_set_tensors": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "cpals_batch_set_norms": (C.c_int, [_P, _DP]),
    "cpals_batch_set_factors": (C.c_int, [_P, _DP]),
    "cpals_batch_get_factors": (C.c_int, [_P, _DP]),
    "cpals_batch_set_threads": (C.c_int, [_P, C.c_int]),
    "cpals_batch_set_sweeps_per_launch": (C.c_int, [_P, C.c_int]),
    "cpals_batch_optimize": (C.c_int, [_P, C.c_double, C.c_int, C.POINTER(C.c_int), _DP, C.POINTER(C.c_int),
                                       _I64P]),
    "cpals_batch_autotune": (C.c_int, [_P, _DP, C.c_int, C.POINTER(C.c_int), _DP]),
    "cpals_batch_schedule": (C.c_int, [_P, C.POINTER(C.c_int), _I64P, _DP]),
    "cpals_synth_lowrank": (C.c_int, [C.c_int, C.c_int, _I64P, C.c_int64, _DP, _DP, C.c_double, C.c_uint64, _P]),
    "cpals_mlp_create": (C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(C.c_int)]),
    "cpals_mlp_destroy": (C.c_int, [_P]),
    "cpals_mlp_num_params": (C.c_int64, [_P]),
    "cpals_mlp_set_params": (C.c_int, [_P, _FP]),
    "cpals_mlp_get_params": (C.c_int, [_P, _FP]),
    "cpals_mlp_forward": (C.c_int, [_P, _FP, C.c_int, _FP]),
    "cpals_mlp_gradients": (C.c_int, [_P, _FP, _FP, C.c_int, _FP, _DP]),
    "cpals_mlp_set_dataset": (C.c_int, [_P, _FP, _FP, C.c_int64]),
    "cpals_mlp_train": (C.c_int, [_P, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_float, _DP]),
    "cpals_mlp_train_stats": (C.c_int, [_P, C.c_int, _DP, _DP]),
}

_lib = None


class CpalsError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} (status {status})")


def load(path: Path | None = None):
    """Load libcpals.so.  Raises if the library has not been built: there is no CPU fallback."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"libcpals.so not found at {p}; build it first (python -c 'import __graft_entry__ as g; g.build()')"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load().cpals_status_string(status).decode()
    except Exception:  # library missing: still give a readable message
        return "unknown"


def check(status: int, what: str):
    if status != CPALS_OK:
        raise CpalsError(status, what)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def i64ptr(a: np.ndarray):
    return a.ctypes.data_as(_I64P)

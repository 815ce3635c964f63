"""ctypes access to libamfls_gb300.so (the C ABI declared in include/amfls_gpu.h).

The library is built in-tree by amfls_solver_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

from .build import LIB

_lib = None

METRICS, COUNTERS, TIMINGS, TRACE_FLOAT, TRACE_INT = 21, 36, 9, 29, 4


class Options(ctypes.Structure):
    _fields_ = [("regularization", ctypes.c_double), ("tolerance", ctypes.c_double),
                ("failure_probability", ctypes.c_double), ("maximum_epochs", ctypes.c_int),
                ("maximum_basis_size", ctypes.c_int), ("seed", ctypes.c_uint64),
                ("stream", ctypes.c_uint64), ("maximum_depth", ctypes.c_int),
                ("maximum_auxiliary_width", ctypes.c_int), ("auxiliary_width", ctypes.c_int),
                ("stop_early", ctypes.c_int), ("time_operators", ctypes.c_int),
                ("use_graphs", ctypes.c_int), ("reduced_basis", ctypes.c_int)]


class BaselineOptions(ctypes.Structure):
    """amfls_gpu_baseline_options: LsqrOptions / LsmrOptions."""
    _fields_ = [("regularization", ctypes.c_double), ("tolerance", ctypes.c_double),
                ("maximum_iterations", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("iterations", ctypes.c_int),
                ("depth", ctypes.c_int), ("auxiliary_width", ctypes.c_int),
                ("basis_rank", ctypes.c_int), ("status", ctypes.c_int),
                ("stop_reason", ctypes.c_int), ("metrics", ctypes.c_double * METRICS),
                ("counters", ctypes.c_longlong * COUNTERS),
                ("timings", ctypes.c_double * TIMINGS), ("trace_rows", ctypes.c_int),
                ("kernel_launches", ctypes.c_longlong),
                ("reduced_basis_levels", ctypes.c_longlong),
                ("reduced_basis_fallbacks", ctypes.c_longlong)]


class ValidationModel(ctypes.Structure):
    _fields_ = [("operator_norm_upper_bound", ctypes.c_double),
                ("operator_norm_lower_bound", ctypes.c_double),
                ("apply_rounding_steps", ctypes.c_longlong),
                ("apply_transpose_rounding_steps", ctypes.c_longlong)]


APPLY_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                            ctypes.c_void_p, ctypes.c_void_p)
COST_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_void_p, ctypes.c_int)


class Callbacks(ctypes.Structure):
    _fields_ = [("context", ctypes.c_void_p), ("apply", APPLY_FN),
                ("apply_transpose", APPLY_FN), ("relative_block_product_cost", COST_FN),
                ("has_validation_model", ctypes.c_int),
                ("validation_model", ValidationModel)]


# every symbol include/amfls_gpu.h declares
EXPORTED = [
    "amfls_gpu_default_options", "amfls_gpu_last_error", "amfls_gpu_csr_operator_create",
    "amfls_gpu_dense_operator_create", "amfls_gpu_operator_destroy", "amfls_gpu_operator_rows",
    "amfls_gpu_operator_cols", "amfls_gpu_operator_apply", "amfls_gpu_operator_apply_transpose",
    "amfls_gpu_operator_relative_block_product_cost",
    "amfls_gpu_operator_validation_error_model", "amfls_gpu_solve_amfls",
    "amfls_gpu_solve_fixed_rbgk", "amfls_gpu_dense_apply_transpose_noalloc",
    "amfls_gpu_reduced_operator_create", "amfls_gpu_solve_amfls_mixed",
    "amfls_gpu_policy_initial_params", "amfls_gpu_policy_create", "amfls_gpu_policy_destroy",
    "amfls_gpu_policy_forward", "amfls_gpu_policy_gradient", "amfls_gpu_policy_train",
    "amfls_gpu_solve_amfls_controlled", "amfls_gpu_solve_amfls_batch",
    "amfls_gpu_callback_operator_create", "amfls_gpu_default_baseline_options",
    "amfls_gpu_solve_lsqr", "amfls_gpu_solve_lsmr", "amfls_gpu_solve_amfls_replay",
    "amfls_gpu_probe_reorthogonalization", "amfls_gpu_csr_operator_schedule",
    "amfls_gpu_probe_reorthogonalization_reduced",
]

POLICY_FEATURES = 11
POLICY_INPUTS = 12
POLICY_PARAMS = 1505
DECISION_COLUMNS = 15


class NativeError(RuntimeError):
    pass


def library_path() -> Path:
    return Path(os.environ.get("AMFLS_GB300_LIBRARY", str(LIB)))


def load():
    """Load (not build) the native library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.is_file():
        raise NativeError(
            f"libamfls_gb300.so not found at {path}; build it with "
            "`python -m amfls_solver_gb300.build` (nvcc, sm_103a)")
    lib = ctypes.CDLL(str(path))
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.amfls_gpu_last_error.restype = ctypes.c_char_p
    lib.amfls_gpu_default_options.argtypes = [ctypes.POINTER(Options)]
    lib.amfls_gpu_default_options.restype = None
    lib.amfls_gpu_csr_operator_create.argtypes = [I, I, P, P, P, ctypes.c_int64, P,
                                                  ctypes.POINTER(P)]
    lib.amfls_gpu_dense_operator_create.argtypes = [I, I, P, I, P, ctypes.POINTER(P)]
    lib.amfls_gpu_operator_destroy.argtypes = [P]
    lib.amfls_gpu_operator_rows.argtypes = [P]
    lib.amfls_gpu_operator_cols.argtypes = [P]
    lib.amfls_gpu_operator_apply.argtypes = [P, P, I, P, P]
    lib.amfls_gpu_operator_apply_transpose.argtypes = [P, P, I, P, P]
    lib.amfls_gpu_operator_relative_block_product_cost.argtypes = [P, I]
    lib.amfls_gpu_operator_relative_block_product_cost.restype = D
    lib.amfls_gpu_operator_validation_error_model.argtypes = [P, ctypes.POINTER(ValidationModel)]
    lib.amfls_gpu_dense_apply_transpose_noalloc.argtypes = [I, I, P, P, P, P]
    for name in ("amfls_gpu_solve_amfls", "amfls_gpu_solve_fixed_rbgk"):
        getattr(lib, name).argtypes = [P, P, ctypes.POINTER(Options), P, ctypes.POINTER(Result),
                                       P, P, I, P]
    lib.amfls_gpu_default_baseline_options.argtypes = [ctypes.POINTER(BaselineOptions)]
    lib.amfls_gpu_default_baseline_options.restype = None
    for name in ("amfls_gpu_solve_lsqr", "amfls_gpu_solve_lsmr"):
        getattr(lib, name).argtypes = [P, P, ctypes.POINTER(BaselineOptions), P,
                                       ctypes.POINTER(Result), P, P, I, P]
    lib.amfls_gpu_reduced_operator_create.argtypes = [P, I, P, ctypes.POINTER(P)]
    lib.amfls_gpu_solve_amfls_mixed.argtypes = [P, P, P, ctypes.POINTER(Options), D, I, P,
                                                ctypes.POINTER(Result), P, P, I, P]
    U64 = ctypes.c_uint64
    lib.amfls_gpu_policy_initial_params.argtypes = [U64, P, I]
    lib.amfls_gpu_policy_create.argtypes = [P, I, ctypes.POINTER(P)]
    lib.amfls_gpu_policy_destroy.argtypes = [P]
    lib.amfls_gpu_policy_forward.argtypes = [P, I, P, I, P, P]
    lib.amfls_gpu_policy_gradient.argtypes = [P, I, P, P, I, P, P, P]
    lib.amfls_gpu_policy_train.argtypes = [P, I, P, P, I, I, D, P, P, P]
    lib.amfls_gpu_callback_operator_create.argtypes = [I, I, ctypes.POINTER(Callbacks), P,
                                                       ctypes.POINTER(P)]
    lib.amfls_gpu_solve_amfls_batch.argtypes = [I, P, P, ctypes.POINTER(Options), P,
                                                ctypes.POINTER(Result), P, I, P]
    lib.amfls_gpu_solve_amfls_controlled.argtypes = [P, P, ctypes.POINTER(Options), P, D, U64,
                                                     P, I, P, P, ctypes.POINTER(Result), P, P,
                                                     I, P]
    lib.amfls_gpu_solve_amfls_replay.argtypes = [P, P, ctypes.POINTER(Options), P, I, P, I, P,
                                                 P, P, ctypes.POINTER(Result), P, P, I, P]
    lib.amfls_gpu_probe_reorthogonalization.argtypes = [I, I, I, P, P]
    lib.amfls_gpu_csr_operator_schedule.argtypes = [P, P, P]
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        raise NativeError(f"amfls_gpu error {rc}: {load().amfls_gpu_last_error().decode()}")


def default_options() -> Options:
    """Reference defaults; AMFLS_GB300_USE_GRAPHS=0 in the environment turns the
    per-interval CUDA graph off (same kernels, launched one by one)."""
    o = Options()
    load().amfls_gpu_default_options(ctypes.byref(o))
    if os.environ.get("AMFLS_GB300_USE_GRAPHS", "1") == "0":
        o.use_graphs = 0
    return o

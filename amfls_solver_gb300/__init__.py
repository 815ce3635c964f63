"""GB300-native AMFLS: adaptive-width block Golub-Kahan least squares on sm_103a.

Drop-in for the reference's python/amfls package on CUDA tensors:
``run_amfls``, ``run_fixed_rbgk``, ``run_lsqr``, ``run_lsmr``, ``SolveResult``,
``load_library`` and ``torch.ops.amfls.run_amfls`` / ``run_fixed_rbgk`` /
``run_lsqr`` / ``run_lsmr`` with the reference's schemas,
plus the mixed-precision form ``run_amfls_mixed`` (FP32 / BF16 inner solves
refined in FP64), batched solves ``run_amfls_batch`` and, in
``amfls_solver_gb300.learned``, the learned width controller.
The compute path is the native library libamfls_gb300.so (C ABI in
include/amfls_gpu.h); importing this package never falls back to the CPU.
"""
from .binding import (
    DeviceOperator,
    SolveResult,
    load_library,
    register_torch_ops,
    run_amfls,
    run_amfls_batch,
    run_amfls_mixed,
    run_fixed_rbgk,
    run_lsmr,
    run_lsqr,
    solve_amfls,
    solve_amfls_replay,
)

__all__ = [
    "DeviceOperator",
    "SolveResult",
    "load_library",
    "register_torch_ops",
    "run_amfls",
    "run_amfls_batch",
    "run_amfls_mixed",
    "run_fixed_rbgk",
    "run_lsmr",
    "run_lsqr",
    "solve_amfls",
    "solve_amfls_replay",
]

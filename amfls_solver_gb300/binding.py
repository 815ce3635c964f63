"""PyTorch binding of the GB300 AMFLS solver (CUDA tensors).

Mirrors the reference's python/amfls/binding.py (SolveResult :9-90,
load_library :92-97, _decode :159-255, run_amfls :259-290) and its torch op
``torch.ops.amfls.run_amfls`` (bindings/torch/torch_binding.cpp:510-516,
same schema string and 8-tuple), registered here for the CUDA and
SparseCsrCUDA dispatch keys.  When the reference's CPU library is loaded in
the same process the op already exists; only the CUDA kernels are added, so
one op dispatches to the reference on CPU tensors and to this library on
CUDA tensors.
"""
from __future__ import annotations

import ctypes
import dataclasses
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _native

TRACE_CAPACITY = 16384

RUN_AMFLS_SCHEMA = (
    "run_amfls(Tensor matrix, Tensor b, float regularization, float tolerance, "
    "float failure_probability, int maximum_epochs=0, int maximum_depth=0, "
    "int maximum_auxiliary_width=0, int maximum_basis_size=0, "
    "int seed=0, int stream=0) -> "
    "(Tensor, Tensor, Tensor, Tensor, Tensor, Tensor, int, int)")
RUN_FIXED_RBGK_SCHEMA = (
    "run_fixed_rbgk(Tensor matrix, Tensor b, float regularization, float tolerance, "
    "float failure_probability, int auxiliary_width, int maximum_depth, "
    "int maximum_basis_size, int seed, int stream) -> "
    "(Tensor, Tensor, Tensor, Tensor, Tensor, Tensor, int, int)")
# torch_binding.cpp:522-529
RUN_LSQR_SCHEMA = (
    "run_lsqr(Tensor matrix, Tensor b, float regularization, float tolerance, "
    "int maximum_iterations=0) -> "
    "(Tensor, Tensor, Tensor, Tensor, Tensor, Tensor, int, int)")
RUN_LSMR_SCHEMA = (
    "run_lsmr(Tensor matrix, Tensor b, float regularization, float tolerance, "
    "int maximum_iterations=0) -> "
    "(Tensor, Tensor, Tensor, Tensor, Tensor, Tensor, int, int)")


@dataclass(frozen=True)
class SolveResult:
    solution: torch.Tensor
    objective: float
    residual_norm: float
    augmented_residual_norm: float
    normal_residual_norm: float
    solution_norm: float
    solution_energy_norm: float
    operator_norm_lower_bound: float
    augmented_operator_norm_lower_bound: float
    compatible_backward_error_upper_bound: float
    least_squares_backward_error_upper_bound: float
    backward_error_upper_bound: float
    relative_normal_residual_upper_bound: float
    energy_error_upper_bound: float
    relative_energy_error_upper_bound: float
    objective_gap_upper_bound: float
    ridge_base_energy_error_upper_bound: float | None
    ridge_corrected_energy_error_upper_bound: float | None
    ridge_correction_gamma: float | None
    ridge_correction_z_h_z: float | None
    ridge_correction_two_abs_z_t_q: float | None
    ridge_correction_q_norm_squared: float | None
    a_columns: int
    at_columns: int
    a_block_calls: int
    at_block_calls: int
    search_a_columns: int
    search_at_columns: int
    validation_a_columns: int
    validation_at_columns: int
    iterations: int
    depth: int
    auxiliary_width: int
    basis_rank: int
    sketch_a_columns: int
    sketch_at_columns: int
    sketch_a_block_calls: int
    sketch_at_block_calls: int
    iterative_a_columns: int
    iterative_at_columns: int
    iterative_a_block_calls: int
    iterative_at_block_calls: int
    gaussian_random_columns: int
    gaussian_random_values: int
    search_a_block_calls: int
    search_at_block_calls: int
    validation_a_block_calls: int
    validation_at_block_calls: int
    base_validation_a_columns: int
    base_validation_at_columns: int
    base_validation_a_block_calls: int
    base_validation_at_block_calls: int
    ridge_correction_a_columns: int
    ridge_correction_at_columns: int
    ridge_correction_a_block_calls: int
    ridge_correction_at_block_calls: int
    gaussian_random_block_requests: int
    ridge_correction_disposition: int
    total_seconds: float
    a_seconds: float
    at_seconds: float
    orthogonalization_seconds: float
    projected_solve_seconds: float
    validation_seconds: float
    other_seconds: float
    base_validation_seconds: float
    ridge_correction_validation_seconds: float
    trace: torch.Tensor
    trace_float: torch.Tensor
    trace_int: torch.Tensor
    status: int
    stop_reason: int
    # GB300 extras (not in the reference's result): width-one levels whose
    # first reorthogonalisation pass ran on the reduced copy of the basis, and
    # how many of them redid it in FP64
    reduced_basis_levels: int = 0
    reduced_basis_fallbacks: int = 0

    @property
    def success(self) -> bool:
        return self.status == 0

    @property
    def search_vector_work(self) -> int:
        return self.search_a_columns + self.search_at_columns


_METRIC_NAMES = [
    "objective", "residual_norm", "augmented_residual_norm", "normal_residual_norm",
    "solution_norm", "solution_energy_norm", "operator_norm_lower_bound",
    "augmented_operator_norm_lower_bound", "compatible_backward_error_upper_bound",
    "least_squares_backward_error_upper_bound", "backward_error_upper_bound",
    "relative_normal_residual_upper_bound", "energy_error_upper_bound",
    "relative_energy_error_upper_bound", "objective_gap_upper_bound",
    "ridge_base_energy_error_upper_bound", "ridge_corrected_energy_error_upper_bound",
    "ridge_correction_gamma", "ridge_correction_z_h_z", "ridge_correction_two_abs_z_t_q",
    "ridge_correction_q_norm_squared"]
_COUNTER_NAMES = [
    "a_columns", "at_columns", "a_block_calls", "at_block_calls", "search_a_columns",
    "search_at_columns", "validation_a_columns", "validation_at_columns", "iterations", "depth",
    "auxiliary_width", "basis_rank", "sketch_a_columns", "sketch_at_columns",
    "sketch_a_block_calls", "sketch_at_block_calls", "iterative_a_columns",
    "iterative_at_columns", "iterative_a_block_calls", "iterative_at_block_calls",
    "gaussian_random_columns", "gaussian_random_values", "search_a_block_calls",
    "search_at_block_calls", "validation_a_block_calls", "validation_at_block_calls",
    "base_validation_a_columns", "base_validation_at_columns", "base_validation_a_block_calls",
    "base_validation_at_block_calls", "ridge_correction_a_columns", "ridge_correction_at_columns",
    "ridge_correction_a_block_calls", "ridge_correction_at_block_calls",
    "gaussian_random_block_requests", "ridge_correction_disposition"]
_TIMING_NAMES = [
    "total_seconds", "a_seconds", "at_seconds", "orthogonalization_seconds",
    "projected_solve_seconds", "validation_seconds", "other_seconds", "base_validation_seconds",
    "ridge_correction_validation_seconds"]


# ------------------------------------------------------------ operators ----

def _stream_handle(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class DeviceOperator:
    """A device MatrixOperator (CSR or dense) owned by the native library.

    CSR inputs are copied and validated (like the reference's
    SparseCsrOperator constructor); dense inputs are referenced in place, so
    the tensor is kept alive by this object.
    """

    def __init__(self, matrix: torch.Tensor):
        lib = _native.load()
        if matrix.device.type != "cuda":
            raise ValueError("the GB300 binding supports CUDA tensors only")
        if matrix.dtype != torch.float64:
            raise ValueError("matrix must use torch.float64")
        if matrix.dim() != 2 or matrix.shape[0] <= 0 or matrix.shape[1] <= 0:
            raise ValueError("matrix must have shape (m,n) with m, n > 0")
        if matrix.shape[0] > 2**31 - 1 or matrix.shape[1] > 2**31 - 1:
            raise ValueError("matrix exceeds the LP64 dimension limit")
        self.rows, self.cols = int(matrix.shape[0]), int(matrix.shape[1])
        handle = ctypes.c_void_p()
        stream = _stream_handle(matrix.device)
        with torch.cuda.device(matrix.device):
            if matrix.layout == torch.sparse_csr:
                crow = matrix.crow_indices().to(torch.int64).contiguous()
                col = matrix.col_indices().to(torch.int64).contiguous()
                val = matrix.values().contiguous()
                if crow.numel() != self.rows + 1:
                    raise ValueError("CSR row offsets must have length rows + 1")
                if col.numel() != val.numel():
                    raise ValueError("CSR column indices and values must be equally sized")
                _native.check(lib.amfls_gpu_csr_operator_create(
                    self.rows, self.cols, crow.data_ptr(), col.data_ptr(), val.data_ptr(),
                    val.numel(), stream, ctypes.byref(handle)))
                self._keep = None
            elif matrix.layout == torch.strided:
                # a column-major view (the transpose of a contiguous tensor) is
                # used in place; anything else is made row-major contiguous
                column_major = (not matrix.is_contiguous()) and matrix.t().is_contiguous()
                dense = matrix if column_major else matrix.contiguous()
                _native.check(lib.amfls_gpu_dense_operator_create(
                    self.rows, self.cols, dense.data_ptr(), int(column_major), stream,
                    ctypes.byref(handle)))
                self._keep = dense
            else:
                raise ValueError("matrix must use dense strided or sparse CSR storage")
        self.handle = handle
        self.device = matrix.device

    @classmethod
    def from_callbacks(cls, rows: int, cols: int, apply, apply_transpose, *,
                       validation_model=None, relative_block_product_cost=None,
                       device: torch.device | None = None) -> "DeviceOperator":
        """A matrix-free operator (the reference's custom MatrixOperator).

        apply(x, y) must write y = A x and apply_transpose(y, x) x = A^T y,
        where x (cols, s) and y (rows, s) are float64 CUDA tensors viewing
        the solver's column-major blocks; they run with torch's current
        stream set to the solver's stream.  validation_model is
        (norm_upper, norm_lower, apply_steps, transpose_steps) or None (then
        no solve certifies success).  A callback that raises makes the solve
        fail with an error."""
        dev = device or torch.device("cuda", torch.cuda.current_device())

        def view(ptr, nrows, s):
            class _Block:  # column-major nrows x s float64 block at ptr
                __cuda_array_interface__ = {"shape": (nrows, s), "typestr": "<f8",
                                            "data": (ptr, False), "version": 2,
                                            "strides": (8, 8 * nrows)}
            return torch.as_tensor(_Block(), device=dev)

        def solver_stream(handle):
            # the solver's stream as a torch stream: a NULL handle is the
            # legacy default stream, which is torch's default stream (an
            # ExternalStream over 0 would be a different stream, unordered
            # with the solver's kernels)
            if not handle:
                return torch.cuda.default_stream(dev)
            return torch.cuda.ExternalStream(handle, device=dev)

        def wrap(fn, in_rows, out_rows):
            def call(_ctx, src, s, dst, stream):
                try:
                    with torch.cuda.stream(solver_stream(stream)):
                        fn(view(src, in_rows, s), view(dst, out_rows, s))
                    return 0
                except Exception:  # reported to the solver as a failed product
                    return 1
            return _native.APPLY_FN(call)

        op = cls.__new__(cls)
        op.rows, op.cols, op.device = int(rows), int(cols), dev
        cb = _native.Callbacks()
        cb.context = None
        cb.apply = wrap(apply, op.cols, op.rows)
        cb.apply_transpose = wrap(apply_transpose, op.rows, op.cols)
        cb.relative_block_product_cost = (
            _native.COST_FN(lambda _c, s: float(relative_block_product_cost(int(s))))
            if relative_block_product_cost else _native.COST_FN())
        if validation_model is not None:
            cb.has_validation_model = 1
            cb.validation_model = _native.ValidationModel(*validation_model)
        handle = ctypes.c_void_p()
        with torch.cuda.device(dev):
            _native.check(_native.load().amfls_gpu_callback_operator_create(
                op.rows, op.cols, ctypes.byref(cb), _stream_handle(dev), ctypes.byref(handle)))
        op.handle = handle
        op._keep = cb  # the callbacks must outlive the operator
        return op

    @classmethod
    def from_csr_arrays(cls, rows, cols, row_offsets, column_indices, values):
        """CSR operator from device tensors (int64 offsets/indices, float64 values)."""
        t = torch.sparse_csr_tensor(row_offsets, column_indices, values, size=(rows, cols))
        return cls(t)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _native.load().amfls_gpu_operator_destroy(h)
            except Exception:
                pass
            self.handle = None

    def apply(self, x: torch.Tensor, transpose: bool = False) -> torch.Tensor:
        """Y = A X (or X = A^T Y) for a column-major block given as (k, s) or (k,)."""
        lib = _native.load()
        vec = x.dim() == 1
        xs = x.reshape(-1, 1) if vec else x
        s = xs.shape[1]
        xc = xs.t().contiguous()  # column-major storage of the block
        out_rows = self.cols if transpose else self.rows
        yc = torch.empty((s, out_rows), dtype=torch.float64, device=x.device)
        fn = lib.amfls_gpu_operator_apply_transpose if transpose else lib.amfls_gpu_operator_apply
        _native.check(fn(self.handle, xc.data_ptr(), s, yc.data_ptr(), _stream_handle(x.device)))
        y = yc.t()
        return y.reshape(-1) if vec else y

    def tile_schedule(self):
        """CSR operators: ({"A": "row vector" | "chains" | "row blocks",
        "A^T": ...}, timings in microseconds {(side, tiling): us} of the
        construction-time autotuner's tile candidates, empty where it did not
        run)."""
        chains = (ctypes.c_int * 2)()
        us = (ctypes.c_double * 4)()
        _native.check(_native.load().amfls_gpu_csr_operator_schedule(self.handle, chains, us))
        names = ("A", "A^T")
        kinds = {0: "row blocks", 1: "chains", 2: "row vector"}
        choice = {names[i]: kinds[int(chains[i])] for i in range(2)}
        times = {f"{names[i // 2]} {'chains' if i % 2 else 'row blocks'}": us[i]
                 for i in range(4) if us[i] > 0}
        return choice, times

    def validation_error_model(self):
        m = _native.ValidationModel()
        _native.check(_native.load().amfls_gpu_operator_validation_error_model(
            self.handle, ctypes.byref(m)))
        return (m.operator_norm_upper_bound, m.operator_norm_lower_bound,
                m.apply_rounding_steps, m.apply_transpose_rounding_steps)

    def relative_block_product_cost(self, block_cols: int) -> float:
        return _native.load().amfls_gpu_operator_relative_block_product_cost(
            self.handle, block_cols)

    def reduced(self, values: str = "fp32") -> "DeviceOperator":
        """The same matrix with values rounded to FP32 or BF16 (products in
        FP32); part of the mixed-precision form.  Keeps this operator alive."""
        codes = {"fp32": 1, "bf16": 2}
        if values not in codes:
            raise ValueError("values must be 'fp32' or 'bf16'")
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(_native.load().amfls_gpu_reduced_operator_create(
                self.handle, codes[values], _stream_handle(self.device), ctypes.byref(handle)))
        op = DeviceOperator.__new__(DeviceOperator)
        op.rows, op.cols, op.device = self.rows, self.cols, self.device
        op.handle = handle
        op._keep = self  # a reduced CSR operator shares the source's index arrays
        op.values = values
        return op


# --------------------------------------------------------------- solves ----

def _with_extras(result: SolveResult, res) -> SolveResult:
    """The GB300 counters of a native result struct added to a decoded result."""
    return dataclasses.replace(result, reduced_basis_levels=int(res.reduced_basis_levels),
                               reduced_basis_fallbacks=int(res.reduced_basis_fallbacks))


def _solve_raw(algorithm: str, op: DeviceOperator, b: torch.Tensor, options, native=None):
    """options: _native.Options (amfls, fixed_rbgk) or _native.BaselineOptions
    (lsqr, lsmr); `native` (a list) receives the native result struct."""
    lib = _native.load()
    if b.device != op.device:
        raise ValueError("matrix and b must be on the same CUDA device")
    b = b.contiguous()
    x = torch.empty(op.cols, dtype=torch.float64, device=b.device)
    res = _native.Result()
    tf = np.zeros((TRACE_CAPACITY, 29))
    ti = np.zeros((TRACE_CAPACITY, 4), dtype=np.int64)
    fn = getattr(lib, f"amfls_gpu_solve_{algorithm}")
    with torch.cuda.device(b.device):
        _native.check(fn(op.handle, b.data_ptr(), ctypes.byref(options), x.data_ptr(),
                         ctypes.byref(res), tf.ctypes.data, ti.ctypes.data, TRACE_CAPACITY,
                         _stream_handle(b.device)))
    rows = min(res.trace_rows, TRACE_CAPACITY)
    if native is not None:
        native.append(res)
    return (x,
            torch.tensor(list(res.metrics), dtype=torch.float64),
            torch.tensor(list(res.counters), dtype=torch.int64),
            torch.tensor(list(res.timings), dtype=torch.float64),
            torch.from_numpy(tf[:rows].copy()),
            torch.from_numpy(ti[:rows].copy()),
            int(res.status), int(res.stop_reason))


def _uint64(v: int) -> int:
    return int(v) & (2**64 - 1)


def _reduced_storage(reduced_basis) -> int:
    """reduced_basis argument -> options.reduced_basis: False / 0 off,
    True / "fp32" / 1 an FP32 copy of the basis, "fp16" / 2 an FP16 copy."""
    codes = {False: 0, None: 0, 0: 0, True: 1, 1: 1, "fp32": 1, 2: 2, "fp16": 2}
    try:
        return codes[reduced_basis]
    except (KeyError, TypeError):
        raise ValueError("reduced_basis must be False, True, 'fp32' or 'fp16'") from None


def solve_amfls(op: DeviceOperator, b: torch.Tensor, *, regularization: float = 0.0,
                tolerance: float = 1e-8, failure_probability: float = 1e-6,
                maximum_epochs: int = 0, maximum_depth: int = 0,
                maximum_auxiliary_width: int = 0, maximum_basis_size: int = 0, seed: int = 0,
                stream: int = 0, reduced_basis=False) -> SolveResult:
    """AMFLS on an existing DeviceOperator (CSR, dense, reduced or callback),
    the reference's C++ entry amfls::solve_amfls(op, b, options)
    (include/amfls/amfls.hpp:22-25).  reduced_basis (not a reference option:
    True or "fp32", "fp16") runs the first reorthogonalisation pass of
    width-one levels on an FP32 or FP16 copy of the right basis, the sweeps
    of the mixed form's restart cycles; a single solve of an ill-conditioned
    problem to FP64 accuracy can stall with it (the certificate reports
    that)."""
    if b.device != op.device or b.dtype != torch.float64 or b.dim() != 1 or b.numel() != op.rows:
        raise ValueError("b must be a float64 CUDA vector of length rows on the operator's device")
    o = _native.default_options()
    o.regularization = float(regularization)
    o.tolerance = float(tolerance)
    o.failure_probability = float(failure_probability)
    o.maximum_epochs = int(maximum_epochs)
    o.maximum_depth = int(maximum_depth)
    o.maximum_auxiliary_width = int(maximum_auxiliary_width)
    o.maximum_basis_size = int(maximum_basis_size)
    o.seed = _uint64(seed)
    o.stream = _uint64(stream)
    o.reduced_basis = _reduced_storage(reduced_basis)
    native = []
    return _with_extras(_decode(_solve_raw("amfls", op, b, o, native)), native[0])


def solve_amfls_replay(op: DeviceOperator, b: torch.Tensor, replay, *,
                       regularization: float = 0.0, tolerance: float = 1e-8,
                       failure_probability: float = 1e-6, maximum_epochs: int = 0,
                       maximum_depth: int = 0, maximum_auxiliary_width: int = 0,
                       maximum_basis_size: int = 0, seed: int = 0, stream: int = 0,
                       reduced_basis=False):
    """AMFLS in schedule-replay mode: the width decisions at the controller's
    decision sites (amfls.cpp:323-354) take the candidate bits in `replay`
    (a sequence of 0/1) instead of the timing-driven cost gate's, so a
    widening solve recorded on the reference is reproduced whatever the
    timings.  Returns (SolveResult, decisions, overrun): the bit taken at
    every decision site and the number of sites beyond the list.  A test
    mode; no counterpart in the reference's API.  reduced_basis as in
    solve_amfls."""
    if b.device != op.device or b.dtype != torch.float64 or b.dim() != 1 or b.numel() != op.rows:
        raise ValueError("b must be a float64 CUDA vector of length rows on the operator's device")
    o = _native.default_options()
    o.regularization = float(regularization)
    o.tolerance = float(tolerance)
    o.failure_probability = float(failure_probability)
    o.maximum_epochs = int(maximum_epochs)
    o.maximum_depth = int(maximum_depth)
    o.maximum_auxiliary_width = int(maximum_auxiliary_width)
    o.maximum_basis_size = int(maximum_basis_size)
    o.seed = _uint64(seed)
    o.stream = _uint64(stream)
    o.reduced_basis = _reduced_storage(reduced_basis)
    rp = np.ascontiguousarray(np.asarray(list(replay), dtype=np.int32))
    cap = 1 << 16
    dec = np.zeros(cap, dtype=np.int32)
    count = ctypes.c_int(0)
    over = ctypes.c_longlong(0)
    b = b.contiguous()
    x = torch.empty(op.cols, dtype=torch.float64, device=b.device)
    res = _native.Result()
    tf = np.zeros((TRACE_CAPACITY, 29))
    ti = np.zeros((TRACE_CAPACITY, 4), dtype=np.int64)
    with torch.cuda.device(b.device):
        _native.check(_native.load().amfls_gpu_solve_amfls_replay(
            op.handle, b.data_ptr(), ctypes.byref(o), rp.ctypes.data, int(rp.shape[0]),
            dec.ctypes.data, cap, ctypes.byref(count), ctypes.byref(over), x.data_ptr(),
            ctypes.byref(res), tf.ctypes.data, ti.ctypes.data, TRACE_CAPACITY,
            _stream_handle(b.device)))
    rows = min(res.trace_rows, TRACE_CAPACITY)
    result = _decode((x, torch.tensor(list(res.metrics), dtype=torch.float64),
                      torch.tensor(list(res.counters), dtype=torch.int64),
                      torch.tensor(list(res.timings), dtype=torch.float64),
                      torch.from_numpy(tf[:rows].copy()), torch.from_numpy(ti[:rows].copy()),
                      int(res.status), int(res.stop_reason)))
    return result, dec[:min(count.value, cap)].copy(), int(over.value)


def run_amfls_batch(problems, *, workers: int = 16, regularization=0.0, tolerance=1e-8,
                    failure_probability: float = 1e-6, maximum_epochs: int = 0,
                    maximum_depth: int = 0, maximum_auxiliary_width: int = 0,
                    maximum_basis_size: int = 0, seed: int = 0, stream: int = 0):
    """Solve many independent problems concurrently on the current GPU.

    `problems` is a sequence of (matrix, b) with matrix a CUDA tensor or a
    DeviceOperator; `regularization` and `tolerance` may be scalars or one
    value per problem.  Returns (results, seconds, wall_seconds): a
    SolveResult per problem (empty traces), each problem's wall time and the
    batch's.  No counterpart in the reference."""
    problems = list(problems)
    count = len(problems)
    ops = [m if isinstance(m, DeviceOperator) else DeviceOperator(m) for m, _ in problems]
    bs = [b.contiguous() for _, b in problems]
    for op, b in zip(ops, bs):
        if b.device != op.device or b.dtype != torch.float64 or b.numel() != op.rows:
            raise ValueError("each b must be a float64 CUDA vector of its matrix's row count")
    def per(v):
        return list(v) if np.ndim(v) else [v] * count
    regs, tols = per(regularization), per(tolerance)
    opts = (_native.Options * max(1, count))()
    for i in range(count):
        o = _native.default_options()
        o.regularization = float(regs[i])
        o.tolerance = float(tols[i])
        o.failure_probability = float(failure_probability)
        o.maximum_epochs = int(maximum_epochs)
        o.maximum_depth = int(maximum_depth)
        o.maximum_auxiliary_width = int(maximum_auxiliary_width)
        o.maximum_basis_size = int(maximum_basis_size)
        o.seed = _uint64(seed)
        o.stream = _uint64(stream)
        opts[i] = o
    xs = [torch.empty(op.cols, dtype=torch.float64, device=op.device) for op in ops]
    P = ctypes.c_void_p
    h_ops = (P * max(1, count))(*[op.handle.value for op in ops])
    h_b = (P * max(1, count))(*[b.data_ptr() for b in bs])
    h_x = (P * max(1, count))(*[x.data_ptr() for x in xs])
    res = (_native.Result * max(1, count))()
    secs = np.zeros(max(1, count))
    wall = ctypes.c_double()
    torch.cuda.synchronize()
    _native.check(_native.load().amfls_gpu_solve_amfls_batch(
        count, h_ops, h_b, opts, h_x, res, secs.ctypes.data, int(workers), ctypes.byref(wall)))
    empty_f, empty_i = torch.zeros((0, 29), dtype=torch.float64), torch.zeros((0, 4), dtype=torch.int64)
    results = [_decode((xs[i], torch.tensor(list(res[i].metrics), dtype=torch.float64),
                        torch.tensor(list(res[i].counters), dtype=torch.int64),
                        torch.tensor(list(res[i].timings), dtype=torch.float64), empty_f, empty_i,
                        int(res[i].status), int(res[i].stop_reason))) for i in range(count)]
    return results, secs[:count].copy(), wall.value


def run_amfls_mixed(matrix, b: torch.Tensor, *, values: str = "fp32",
                    inner_tolerance: float = 1e-6, maximum_refinements: int = 8,
                    regularization: float = 0.0, tolerance: float = 1e-8,
                    failure_probability: float = 1e-6, maximum_epochs: int = 0,
                    maximum_depth: int = 0, maximum_auxiliary_width: int = 0,
                    maximum_basis_size: int = 0, seed: int = 0, stream: int = 0,
                    reduced: "DeviceOperator | None" = None,
                    reduced_basis=False) -> SolveResult:
    """Mixed-precision AMFLS: inner solves refined in FP64; the certified
    FP64 validation on the original matrix decides termination.  `values`
    is the inner products' precision ("fp32", "bf16", or "fp64" for inner
    solves on the FP64 operator itself); `reduced_basis` (True or "fp32",
    "fp16") runs the inner solves' first reorthogonalisation pass on an FP32
    or FP16 copy of the basis.
    With maximum_depth set and a tiny inner_tolerance every inner solve is
    one restart cycle of maximum_depth levels.  `matrix` is a CUDA tensor or
    a DeviceOperator; `reduced` reuses an existing reduced operator.  Work
    limits apply to each inner solve.  No counterpart in the reference."""
    op = matrix if isinstance(matrix, DeviceOperator) else DeviceOperator(matrix)
    if b.device != op.device or b.dtype != torch.float64 or b.dim() != 1 or b.numel() != op.rows:
        raise ValueError("b must be a float64 CUDA vector of length rows on the matrix's device")
    if reduced is not None:
        low = reduced
    elif values == "fp64":
        low = op
    else:
        low = op.reduced(values)
    o = _native.default_options()
    o.regularization = float(regularization)
    o.tolerance = float(tolerance)
    o.failure_probability = float(failure_probability)
    o.maximum_epochs = int(maximum_epochs)
    o.maximum_depth = int(maximum_depth)
    o.maximum_auxiliary_width = int(maximum_auxiliary_width)
    o.maximum_basis_size = int(maximum_basis_size)
    o.seed = _uint64(seed)
    o.stream = _uint64(stream)
    o.reduced_basis = _reduced_storage(reduced_basis)
    b = b.contiguous()
    x = torch.empty(op.cols, dtype=torch.float64, device=b.device)
    res = _native.Result()
    tf = np.zeros((TRACE_CAPACITY, 29))
    ti = np.zeros((TRACE_CAPACITY, 4), dtype=np.int64)
    with torch.cuda.device(b.device):
        _native.check(_native.load().amfls_gpu_solve_amfls_mixed(
            op.handle, low.handle, b.data_ptr(), ctypes.byref(o), float(inner_tolerance),
            int(maximum_refinements), x.data_ptr(), ctypes.byref(res), tf.ctypes.data,
            ti.ctypes.data, TRACE_CAPACITY, _stream_handle(b.device)))
    rows = min(res.trace_rows, TRACE_CAPACITY)
    return _with_extras(_decode((x, torch.tensor(list(res.metrics), dtype=torch.float64),
                                 torch.tensor(list(res.counters), dtype=torch.int64),
                                 torch.tensor(list(res.timings), dtype=torch.float64),
                                 torch.from_numpy(tf[:rows].copy()),
                                 torch.from_numpy(ti[:rows].copy()),
                                 int(res.status), int(res.stop_reason))), res)


def _run_amfls_impl(matrix, b, regularization, tolerance, failure_probability,
                    maximum_epochs=0, maximum_depth=0, maximum_auxiliary_width=0,
                    maximum_basis_size=0, seed=0, stream=0):
    _check_inputs(matrix, b)
    op = DeviceOperator(matrix)
    o = _native.default_options()
    o.regularization = float(regularization)
    o.tolerance = float(tolerance)
    o.failure_probability = float(failure_probability)
    o.maximum_epochs = int(maximum_epochs)
    o.maximum_depth = int(maximum_depth)
    o.maximum_auxiliary_width = int(maximum_auxiliary_width)
    o.maximum_basis_size = int(maximum_basis_size)
    o.seed = _uint64(seed)
    o.stream = _uint64(stream)
    return _solve_raw("amfls", op, b, o)


def _run_fixed_rbgk_impl(matrix, b, regularization, tolerance, failure_probability,
                         auxiliary_width, maximum_depth, maximum_basis_size, seed, stream):
    _check_inputs(matrix, b)
    op = DeviceOperator(matrix)
    o = _native.default_options()
    o.regularization = float(regularization)
    o.tolerance = float(tolerance)
    o.failure_probability = float(failure_probability)
    o.auxiliary_width = int(auxiliary_width)
    o.maximum_depth = int(maximum_depth)
    o.maximum_basis_size = int(maximum_basis_size)
    o.seed = _uint64(seed)
    o.stream = _uint64(stream)
    return _solve_raw("fixed_rbgk", op, b, o)


def _run_baseline_impl(algorithm, matrix, b, regularization, tolerance, maximum_iterations=0):
    _check_inputs(matrix, b)
    op = DeviceOperator(matrix)
    o = _native.BaselineOptions()
    _native.load().amfls_gpu_default_baseline_options(ctypes.byref(o))
    o.regularization = float(regularization)
    o.tolerance = float(tolerance)
    o.maximum_iterations = int(maximum_iterations)
    return _solve_raw(algorithm, op, b, o)


def _run_lsqr_impl(matrix, b, regularization, tolerance, maximum_iterations=0):
    return _run_baseline_impl("lsqr", matrix, b, regularization, tolerance, maximum_iterations)


def _run_lsmr_impl(matrix, b, regularization, tolerance, maximum_iterations=0):
    return _run_baseline_impl("lsmr", matrix, b, regularization, tolerance, maximum_iterations)


_LIBS = []
_OPS = {"run_amfls": (RUN_AMFLS_SCHEMA, "_run_amfls_impl"),
        "run_fixed_rbgk": (RUN_FIXED_RBGK_SCHEMA, "_run_fixed_rbgk_impl"),
        "run_lsqr": (RUN_LSQR_SCHEMA, "_run_lsqr_impl"),
        "run_lsmr": (RUN_LSMR_SCHEMA, "_run_lsmr_impl")}


def _op_exists(name: str) -> bool:
    try:
        getattr(torch.ops.amfls, name)
        return True
    except (AttributeError, RuntimeError):
        return False


def register_torch_ops() -> None:
    """Register torch.ops.amfls.{run_amfls, run_fixed_rbgk, run_lsqr, run_lsmr}
    for CUDA tensors (reference: torch_binding.cpp:511-611)."""
    if _LIBS:
        return
    defined = {n: _op_exists(n) for n in _OPS}
    if not all(defined.values()):
        lib_def = torch.library.Library("amfls", "FRAGMENT")
        for name, (schema, _) in _OPS.items():
            if not defined[name]:
                lib_def.define(schema)
        _LIBS.append(lib_def)
    lib_impl = torch.library.Library("amfls", "IMPL")
    for key in ("CUDA", "SparseCsrCUDA"):
        for name, (_, impl) in _OPS.items():
            lib_impl.impl(name, globals()[impl], key)
    _LIBS.append(lib_impl)


def load_library(path: str | Path | None = None) -> Path:
    """Load libamfls_gb300.so and register the torch ops (reference: binding.py:92-97)."""
    import os

    if path is not None:
        os.environ["AMFLS_GB300_LIBRARY"] = str(Path(path).expanduser().resolve())
    _native.load()
    register_torch_ops()
    return _native.library_path()


# --------------------------------------------------------- python API ----

def _check_inputs(matrix: torch.Tensor, b: torch.Tensor) -> None:
    if matrix.device.type != "cuda" or b.device.type != "cuda":
        raise ValueError("the GB300 binding supports CUDA tensors only")
    if matrix.dtype != torch.float64 or b.dtype != torch.float64:
        raise ValueError("matrix and b must use torch.float64")
    if matrix.layout not in (torch.strided, torch.sparse_csr):
        raise ValueError("matrix must use dense strided or sparse CSR storage")
    if b.layout != torch.strided:
        raise ValueError("b must use dense strided storage")
    if matrix.ndim != 2 or b.ndim != 1 or matrix.shape[0] != b.shape[0]:
        raise ValueError("matrix must have shape (m,n) and b must have shape (m,)")


def _canonical_uint64_to_int64_transport(value: int, name: str) -> int:
    if isinstance(value, bool) or not isinstance(value, int):
        raise ValueError(f"{name} must be an integer in [0, 2**64 - 1]")
    if value < 0 or value >= 1 << 64:
        raise ValueError(f"{name} must be an integer in [0, 2**64 - 1]")
    return value if value < 1 << 63 else value - (1 << 64)


def _decode(raw) -> SolveResult:
    if not isinstance(raw, (tuple, list)) or len(raw) != 8:
        raise RuntimeError("AMFLS binding result must be an eight-item tuple")
    solution, metrics, counters, timings, trace_float, trace_int, status, reason = raw
    if metrics.shape != (21,) or counters.shape != (36,) or timings.shape != (9,):
        raise RuntimeError("AMFLS binding result tensors have the wrong shape")
    if trace_float.ndim != 2 or trace_float.shape[1] != 29 or \
            tuple(trace_int.shape) != (trace_float.shape[0], 4):
        raise RuntimeError("AMFLS binding trace tensors have the wrong shape")
    fields = {"solution": solution}
    m = metrics.tolist()
    c = counters.tolist()
    t = timings.tolist()
    fields.update({k: float(m[i]) for i, k in enumerate(_METRIC_NAMES)})
    fields.update({k: int(c[i]) for i, k in enumerate(_COUNTER_NAMES)})
    fields.update({k: float(t[i]) for i, k in enumerate(_TIMING_NAMES)})
    fields.update(trace=trace_float[:, :18], trace_float=trace_float, trace_int=trace_int,
                  status=int(status), stop_reason=int(reason))
    return SolveResult(**fields)


def run_amfls(matrix: torch.Tensor, b: torch.Tensor, *, regularization: float = 0.0,
              tolerance: float = 1e-8, failure_probability: float = 1e-6,
              maximum_epochs: int = 0, maximum_depth: int = 0,
              maximum_auxiliary_width: int = 0, maximum_basis_size: int = 0, seed: int = 0,
              stream: int = 0) -> SolveResult:
    """AMFLS on CUDA tensors (reference: python/amfls/binding.py:259-290)."""
    _check_inputs(matrix, b)
    register_torch_ops()
    return _decode(torch.ops.amfls.run_amfls(
        matrix, b, regularization, tolerance, failure_probability, maximum_epochs,
        maximum_depth, maximum_auxiliary_width, maximum_basis_size,
        _canonical_uint64_to_int64_transport(seed, "seed"),
        _canonical_uint64_to_int64_transport(stream, "stream")))


def run_fixed_rbgk(matrix: torch.Tensor, b: torch.Tensor, *, auxiliary_width: int,
                   maximum_depth: int, maximum_basis_size: int = 0,
                   regularization: float = 0.0, tolerance: float = 1e-8,
                   failure_probability: float = 1e-6, seed: int = 0,
                   stream: int = 0) -> SolveResult:
    """Fixed-width randomized block Golub-Kahan (reference: binding.py:293-322)."""
    _check_inputs(matrix, b)
    register_torch_ops()
    return _decode(torch.ops.amfls.run_fixed_rbgk(
        matrix, b, regularization, tolerance, failure_probability, auxiliary_width,
        maximum_depth, maximum_basis_size,
        _canonical_uint64_to_int64_transport(seed, "seed"),
        _canonical_uint64_to_int64_transport(stream, "stream")))


def run_lsqr(matrix: torch.Tensor, b: torch.Tensor, *, regularization: float = 0.0,
             tolerance: float = 1e-8, maximum_iterations: int = 0) -> SolveResult:
    """Scalar LSQR, every checkpoint certified (reference: binding.py:325-342)."""
    _check_inputs(matrix, b)
    register_torch_ops()
    return _decode(torch.ops.amfls.run_lsqr(matrix, b, regularization, tolerance,
                                            maximum_iterations))


def run_lsmr(matrix: torch.Tensor, b: torch.Tensor, *, regularization: float = 0.0,
             tolerance: float = 1e-8, maximum_iterations: int = 0) -> SolveResult:
    """Scalar LSMR, every checkpoint certified (reference: binding.py:345-362)."""
    _check_inputs(matrix, b)
    register_torch_ops()
    return _decode(torch.ops.amfls.run_lsmr(matrix, b, regularization, tolerance,
                                            maximum_iterations))

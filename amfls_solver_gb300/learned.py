"""Learned width controller (no counterpart in the reference).

The reference's AMFLS decides when to widen its block (inject the next
dyadic block of Gaussian seeds) with a cost-gated heuristic
(src/algorithms/amfls/amfls_internal.hpp, decision sites amfls.cpp:319-359).
Here a small MLP, trained and run by the library's own CUDA kernels, scores
the two choices at each such decision from the controller's own features:

  0 log10(certificate / tol)           6 log2(1 + increment)
  1 recent decades per level           7 free basis fraction
  2 log10 operator s per level         8 free depth fraction
  3 log10 local s per level            9 matched-horizon plan active
  4 log10 block-cost ratio            10 the heuristic's own choice
  5 log2(1 + current width)

plus the action (0 stay, 1 widen), and predicts how good that action is;
at run time the controller widens when the score for widening is higher,
and the FP64 certificate still decides termination.  Two training sources:

* counterfactual_dataset: the plain controller's own traces.  At each of
  the heuristic's decision sites the solve is replayed with the opposite
  choice (schedule replay) and timed; the target is the log speed-up of an
  action over the heuristic's (0 for the heuristic's own).  Both actions are
  seen in exactly the same state, so the score is not confounded by when
  decisions happen.
* dataset(collect_decisions(...)): exploration solves whose decisions are
  randomised; the target is the rate at which the certificate fell after
  the decision (decades per second, compressed as asinh(rate / scale)).
  Early decisions see fast certificate decay whatever the action, so this
  target mixes the state into the action's value.

    data = counterfactual_dataset(training_problems)   # or dataset(collect_decisions(...))
    policy = WidthPolicy.train(data.inputs, data.targets, epochs=2000)
    result, decisions = solve_controlled(matrix, b, policy=policy, tolerance=1e-10)
    rows = compare_controllers(held_out_problems, policy)

On this GPU the reference's cost gate, which prices local block algebra at
a CPU's BLAS-3 rates, widens dense solves whose wider levels then run
slower here (FP64 block reorthogonalisation is bound by the FP64 FMA rate
and each block level synchronises with the host for its rank decisions);
the trained policy learns from the measured rates when staying at width one
finishes sooner.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native
from .binding import TRACE_CAPACITY, DeviceOperator, _decode, _stream_handle, _uint64

F = _native.POLICY_FEATURES
IN = _native.POLICY_INPUTS
P = _native.POLICY_PARAMS
COLS = _native.DECISION_COLUMNS


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _stream():
    return torch.cuda.current_stream().cuda_stream if torch.cuda.is_available() else None


def initial_params(seed: int = 0) -> np.ndarray:
    p = np.zeros(P)
    _native.check(_native.load().amfls_gpu_policy_initial_params(_uint64(seed), _ptr(p), P))
    return p


def forward(params: np.ndarray, inputs: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(inputs, dtype=np.float64)
    out = np.zeros(x.shape[0])
    _native.check(_native.load().amfls_gpu_policy_forward(_ptr(p), P, _ptr(x), x.shape[0],
                                                          _ptr(out), _stream()))
    return out


def gradient(params: np.ndarray, inputs: np.ndarray, targets: np.ndarray):
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(inputs, dtype=np.float64)
    y = np.ascontiguousarray(targets, dtype=np.float64)
    g = np.zeros(P)
    loss = ctypes.c_double()
    _native.check(_native.load().amfls_gpu_policy_gradient(
        _ptr(p), P, _ptr(x), _ptr(y), x.shape[0], _ptr(g), ctypes.byref(loss), _stream()))
    return loss.value, g


class WidthPolicy:
    """Trained parameters plus the device object the solver calls."""

    def __init__(self, params: np.ndarray):
        self.params = np.ascontiguousarray(params, dtype=np.float64).copy()
        if self.params.shape != (P,):
            raise ValueError(f"a policy has {P} parameters")
        h = ctypes.c_void_p()
        _native.check(_native.load().amfls_gpu_policy_create(_ptr(self.params), P,
                                                             ctypes.byref(h)))
        self.handle = h
        self.losses = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _native.load().amfls_gpu_policy_destroy(h)
            except Exception:
                pass
            self.handle = None

    @classmethod
    def train(cls, inputs: np.ndarray, targets: np.ndarray, *, epochs: int = 3000,
              learning_rate: float = 3e-3, seed: int = 0) -> "WidthPolicy":
        """Full-batch Adam from seeded initial parameters, on the GPU."""
        p = initial_params(seed)
        x = np.ascontiguousarray(inputs, dtype=np.float64)
        y = np.ascontiguousarray(targets, dtype=np.float64)
        first, last = ctypes.c_double(), ctypes.c_double()
        _native.check(_native.load().amfls_gpu_policy_train(
            _ptr(p), P, _ptr(x), _ptr(y), x.shape[0], int(epochs), float(learning_rate),
            ctypes.byref(first), ctypes.byref(last), _stream()))
        policy = cls(p)
        policy.losses = (first.value, last.value)
        return policy

    def scores(self, features: np.ndarray) -> np.ndarray:
        """(n, 2): predicted score of staying and of widening."""
        f = np.atleast_2d(np.asarray(features, dtype=np.float64))
        x = np.zeros((2 * f.shape[0], IN))
        x[0::2, :F] = f
        x[1::2, :F] = f
        x[1::2, F] = 1.0
        return forward(self.params, x).reshape(-1, 2)


def solve_controlled(matrix, b: torch.Tensor, *, policy: WidthPolicy | None = None,
                     exploration: float = 0.0, exploration_seed: int = 0,
                     decision_capacity: int = 4096, regularization: float = 0.0,
                     tolerance: float = 1e-8, failure_probability: float = 1e-6,
                     maximum_epochs: int = 0, maximum_depth: int = 0,
                     maximum_auxiliary_width: int = 0, maximum_basis_size: int = 0,
                     seed: int = 0, stream: int = 0):
    """AMFLS with its width decisions taken by `policy` (or the heuristic),
    optionally randomised; returns (SolveResult, decision log (rows x 15))."""
    op = matrix if isinstance(matrix, DeviceOperator) else DeviceOperator(matrix)
    if b.device != op.device or b.dtype != torch.float64 or b.dim() != 1 or b.numel() != op.rows:
        raise ValueError("b must be a float64 CUDA vector of length rows on the matrix's device")
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
    b = b.contiguous()
    x = torch.empty(op.cols, dtype=torch.float64, device=b.device)
    res = _native.Result()
    tf = np.zeros((TRACE_CAPACITY, 29))
    ti = np.zeros((TRACE_CAPACITY, 4), dtype=np.int64)
    log = np.zeros((decision_capacity, COLS))
    rows = ctypes.c_int()
    with torch.cuda.device(b.device):
        _native.check(_native.load().amfls_gpu_solve_amfls_controlled(
            op.handle, b.data_ptr(), ctypes.byref(o), policy.handle if policy else None,
            float(exploration), _uint64(exploration_seed), _ptr(log), decision_capacity,
            ctypes.byref(rows), x.data_ptr(), ctypes.byref(res), tf.ctypes.data, ti.ctypes.data,
            TRACE_CAPACITY, _stream_handle(b.device)))
    n = min(res.trace_rows, TRACE_CAPACITY)
    result = _decode((x, torch.tensor(list(res.metrics), dtype=torch.float64),
                      torch.tensor(list(res.counters), dtype=torch.int64),
                      torch.tensor(list(res.timings), dtype=torch.float64),
                      torch.from_numpy(tf[:n].copy()), torch.from_numpy(ti[:n].copy()),
                      int(res.status), int(res.stop_reason)))
    return result, log[:min(rows.value, decision_capacity)].copy()


@dataclass
class Dataset:
    inputs: np.ndarray   # (n, 12): features and action
    targets: np.ndarray  # (n,): asinh(rate / scale)
    scale: float


def dataset(logs, scale: float | None = None) -> Dataset:
    """Training pairs from decision logs: rows with a measured rate."""
    rows = np.concatenate([np.asarray(l).reshape(-1, COLS) for l in logs], axis=0)
    rows = rows[rows[:, 14] > 0]
    if rows.shape[0] == 0:
        raise ValueError("no decision with a measured rate")
    rate = rows[:, 13]
    if scale is None:
        scale = float(np.median(np.abs(rate))) or 1.0
    x = np.concatenate([rows[:, :F], rows[:, 11:12]], axis=1)
    return Dataset(x, np.arcsinh(rate / scale), scale)


def collect_decisions(problems, *, exploration: float = 0.4, exploration_seeds=(1, 2)):
    """Decision logs of exploration solves: `problems` yields (matrix or
    DeviceOperator, b, options dict); each is solved once per exploration
    seed with that share of its width decisions replaced by a fair coin."""
    logs = []
    for matrix, b, options in problems:
        op = matrix if isinstance(matrix, DeviceOperator) else DeviceOperator(matrix)
        for es in exploration_seeds:
            _, log = solve_controlled(op, b, exploration=exploration, exploration_seed=es,
                                      **options)
            logs.append(log)
    return logs


def counterfactual_dataset(problems, *, max_sites: int = 8) -> Dataset:
    """Training pairs from the plain controller's own traces, without the
    confounding of random exploration: for each problem the heuristic solve
    is logged (its features at every decision site) and timed; then, for
    each of its first `max_sites` decision sites, the solve is replayed with
    the heuristic's bits up to that site and the opposite bit there
    (amfls_gpu_solve_amfls_replay; later sites follow the heuristic again)
    and timed.  The site's features with the heuristic's action get target
    0, with the opposite action log(t_heuristic / t_flipped): the log
    speed-up that choice would have brought.  A policy trained on these
    scores picks, at each site, the action predicted to finish sooner."""
    import time

    from .binding import solve_amfls_replay

    xs, ys = [], []
    for matrix, b, options in problems:
        op = matrix if isinstance(matrix, DeviceOperator) else DeviceOperator(matrix)
        solve_controlled(op, b, **options)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, log = solve_controlled(op, b, **options)
        torch.cuda.synchronize()
        t_h = time.perf_counter() - t0
        bits = [int(v) for v in log[:, 11]] if len(log) else []
        for i in range(min(len(bits), max_sites)):
            replay = bits[:i] + [1 - bits[i]]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            solve_amfls_replay(op, b, replay, **options)
            torch.cuda.synchronize()
            t_f = time.perf_counter() - t0
            f = log[i, :F]
            xs.append(np.concatenate([f, [bits[i]]]))
            ys.append(0.0)
            xs.append(np.concatenate([f, [1 - bits[i]]]))
            ys.append(float(np.log(t_h / t_f)))
    if not xs:
        raise ValueError("no decision site in the training problems")
    return Dataset(np.asarray(xs), np.asarray(ys), 1.0)


def compare_controllers(problems, policy: WidthPolicy):
    """Time-to-tol of the heuristic and of `policy` on each problem (host
    wall clock around each synchronous solve, after one untimed warm-up
    solve of each): rows of (heuristic SolveResult, seconds, learned
    SolveResult, seconds)."""
    import time

    rows = []
    for matrix, b, options in problems:
        op = matrix if isinstance(matrix, DeviceOperator) else DeviceOperator(matrix)
        solve_controlled(op, b, **options)
        solve_controlled(op, b, policy=policy, **options)
        out = []
        for pol in (None, policy):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r, _ = solve_controlled(op, b, policy=pol, **options)
            torch.cuda.synchronize()
            out += [r, time.perf_counter() - t0]
        rows.append(tuple(out))
    return rows

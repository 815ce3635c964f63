"""Test infrastructure: ctypes access to the reference build in oracle/_ref/.

``oracle/_ref/libamfls_ref.so`` is the reference's own AMFLS code compiled by
``make -C oracle ref`` (only where the reference sources exist).  It is used to
generate the golden fixtures under tests/golden/ and, where present, to pin the
oracle.  Nothing in the product imports this module.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_ref" / "libamfls_ref.so"
_lib = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_D = ctypes.c_double


def available() -> bool:
    return LIB_PATH.is_file()


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(LIB_PATH))
        _lib.ref_last_error.restype = ctypes.c_char_p
        _lib.ref_solve.argtypes = [
            _I, _I, _I, _I, _P, _P, _P, _I64, _P, _D, _D, _D, _I, _I, _I, _I,
            _U64, _U64, _I, _P, _P, _P, _P, _P, _P, _I, _P, _P, _P]
        _lib.ref_apply.argtypes = [_I, _I, _I, _P, _P, _P, _I64, _I, _P, _I, _P]
        _lib.ref_validation_model.argtypes = [_I, _I, _I, _P, _P, _P, _I64, _P, _P]
        _lib.ref_gaussian_matrix.argtypes = [_I, _I, _U64, _U64, _U64, _P]
        _lib.ref_norm_interval.argtypes = [_P, _I64, _P]
        _lib.ref_norm_interval.restype = None
        _lib.ref_set_width_replay.argtypes = [_P, _I]
        _lib.ref_set_width_replay.restype = None
        _lib.ref_width_decisions.argtypes = [_P, _P, _I, ctypes.POINTER(ctypes.c_longlong)]
        _lib.ref_width_decisions.restype = _I
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _operator_args(problem, custom=False):
    """(kind, rows, cols, offsets, indices, values, nnz, keep-alive list);
    custom=True puts a CSR matrix behind a custom MatrixOperator (kind 3)."""
    if hasattr(problem, "row_offsets"):
        off = np.ascontiguousarray(problem.row_offsets, dtype=np.int64)
        col = np.ascontiguousarray(problem.column_indices, dtype=np.int64)
        val = np.ascontiguousarray(problem.values, dtype=np.float64)
        return (3 if custom else 0), problem.rows, problem.cols, off, col, val, val.shape[0], \
            [off, col, val]
    a = problem.matrix
    if a.flags.c_contiguous:
        return 1, a.shape[0], a.shape[1], None, None, a, a.size, [a]
    a = np.asfortranarray(a)
    return 2, a.shape[0], a.shape[1], None, None, a, a.size, [a]


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().ref_last_error().decode())


_ALGORITHMS = {"amfls": 0, "fixed_rbgk": 1, "lsqr": 2, "lsmr": 3}


def solve(problem, *, algorithm="amfls", regularization=0.0, tolerance=1e-8,
          failure_probability=1e-6, maximum_epochs=0, maximum_depth=0,
          maximum_auxiliary_width=0, maximum_basis_size=0, seed=0, stream=0,
          auxiliary_width=4, maximum_iterations=0, trace_capacity=4096, replay=None,
          custom=False):
    """algorithm: amfls, fixed_rbgk, lsqr or lsmr (the last two take
    regularization, tolerance and maximum_iterations only).

    The AMFLS result carries ``decisions`` (the candidate bit of every width
    decision the controller took, amfls.cpp:323-354), ``horizons`` (their
    matched horizons) and ``replay_overrun``.  ``replay`` (a sequence of 0/1)
    makes the controller take those decisions in order instead of its
    timing-driven ones (sites beyond the list keep the reference's choice and
    are counted in ``replay_overrun``).  custom=True solves through a custom
    MatrixOperator over the CSR matrix (no extended-precision validation
    products)."""
    if algorithm in ("lsqr", "lsmr"):
        maximum_depth = maximum_iterations
    kind, m, n, off, col, val, nnz, keep = _operator_args(problem, custom)
    b = np.ascontiguousarray(problem.b, dtype=np.float64)
    x = np.zeros(n)
    metrics = np.zeros(21)
    counters = np.zeros(36, dtype=np.int64)
    timings = np.zeros(9)
    tf = np.zeros((trace_capacity, 29))
    ti = np.zeros((trace_capacity, 4), dtype=np.int64)
    rows = ctypes.c_int(0)
    status = ctypes.c_int(0)
    reason = ctypes.c_int(0)
    rp = np.ascontiguousarray(np.asarray(replay if replay is not None else [], dtype=np.int32))
    lib().ref_set_width_replay(_ptr(rp), rp.shape[0] if replay is not None else -1)
    _check(lib().ref_solve(
        _ALGORITHMS[algorithm], kind, m, n, _ptr(off), _ptr(col),
        _ptr(val), nnz, _ptr(b), regularization, tolerance, failure_probability,
        maximum_epochs, maximum_depth, maximum_auxiliary_width,
        maximum_basis_size, seed, stream, auxiliary_width, _ptr(x),
        _ptr(metrics), _ptr(counters), _ptr(timings), _ptr(tf), _ptr(ti),
        trace_capacity, ctypes.byref(rows), ctypes.byref(status),
        ctypes.byref(reason)))
    lib().ref_set_width_replay(None, -1)
    r = min(rows.value, trace_capacity)
    cap = 1 << 16
    dec = np.zeros(cap, dtype=np.int32)
    hor = np.zeros(cap, dtype=np.int32)
    over = ctypes.c_longlong(0)
    nd = lib().ref_width_decisions(_ptr(dec), _ptr(hor), cap, ctypes.byref(over))
    return dict(solution=x, metrics=metrics, counters=counters, timings=timings,
                trace_float=tf[:r].copy(), trace_int=ti[:r].copy(),
                status=status.value, stop_reason=reason.value,
                decisions=dec[:min(nd, cap)].copy(), horizons=hor[:min(nd, cap)].copy(),
                replay_overrun=int(over.value))


def apply(problem, x, transpose=False):
    kind, m, n, off, col, val, nnz, keep = _operator_args(problem)
    x = np.asfortranarray(x, dtype=np.float64)
    s = 1 if x.ndim == 1 else x.shape[1]
    out = np.zeros((n if transpose else m, s), order="F")
    _check(lib().ref_apply(kind, m, n, _ptr(off), _ptr(col), _ptr(val), nnz,
                           1 if transpose else 0, _ptr(x), s, _ptr(out)))
    return out[:, 0] if x.ndim == 1 else out


def validation_model(problem):
    kind, m, n, off, col, val, nnz, keep = _operator_args(problem)
    model = np.zeros(2)
    steps = np.zeros(2, dtype=np.int64)
    _check(lib().ref_validation_model(kind, m, n, _ptr(off), _ptr(col), _ptr(val),
                                      nnz, _ptr(model), _ptr(steps)))
    return model, steps


def gaussian_matrix(rows, cols, seed, stream, first_column):
    out = np.zeros((rows, cols), order="F")
    _check(lib().ref_gaussian_matrix(rows, cols, seed, stream, first_column, _ptr(out)))
    return out


def norm_interval(values):
    v = np.ascontiguousarray(values, dtype=np.float64)
    out = np.zeros(2)
    lib().ref_norm_interval(_ptr(v), v.shape[0], _ptr(out))
    return out

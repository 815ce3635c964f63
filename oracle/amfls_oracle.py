"""Test infrastructure: the AMFLS oracle, a CPU restatement of the reference.

This module is the checker for the GPU implementation and nothing else: only
tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s cpu_baseline leg may
import it.  It restates doloMing/amfls_solver's adaptive-width block
Golub-Kahan least-squares solve with numpy + scipy (scipy's BLAS/LAPACK
wrappers call the same routines the reference calls: dgemv, dgemm, dnrm2,
ddot, dgesdd, dgelsy) and with the C half in amfls_oracle.c for the
elementwise arithmetic (CSR products, directed rounding, validation).

Parity is pinned against the reference's own outputs: tests/golden/ holds
fixtures produced by the reference build (oracle/_ref, see oracle/Makefile)
and tests/test_oracle.py checks this restatement against them.

Reference map (paths relative to the reference repository):
  solve_amfls ................ src/algorithms/amfls/amfls.cpp:57-661
  width controller ........... src/algorithms/amfls/amfls_internal.hpp:14-674
  checkpoint schedule ........ src/algorithms/mathematics/krylov/certificate_checkpoint_schedule.hpp:15-131
  BlockGolubKahanWorkspace ... src/algorithms/mathematics/krylov/krylov_workspace.cpp:335-963
  orthogonalize_and_factor ... krylov_workspace.cpp:63-310
  stable_ridge_filter ........ krylov_workspace.cpp:312-331
  step audits ................ krylov_workspace.cpp:965-979
  solve_fixed_rbgk ........... src/algorithms/fixed_rbgk/fixed_rbgk.cpp:18-209
  result layout .............. bindings/torch/result_tensors.hpp:12-156
"""
from __future__ import annotations

import ctypes
import math
import subprocess
import time
from pathlib import Path

import numpy as np
import scipy.linalg as sla
from scipy.linalg import blas as sblas

EPS = float(np.finfo(np.float64).eps)
INF = math.inf
INT_MAX = 2**31 - 1
_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "liboracle.so"
_lib = None


# ------------------------------------------------------------ C half ----

class _OrcOperator(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("rows", ctypes.c_int), ("cols", ctypes.c_int),
                ("row_offsets", ctypes.c_void_p), ("column_indices", ctypes.c_void_p),
                ("values", ctypes.c_void_p), ("nonzeros", ctypes.c_int64)]


class _OrcModel(ctypes.Structure):
    _fields_ = [("norm_upper", ctypes.c_double), ("norm_lower", ctypes.c_double),
                ("apply_steps", ctypes.c_longlong), ("transpose_steps", ctypes.c_longlong)]


_VALIDATION_DOUBLES = [
    "objective", "residual_norm", "augmented_residual_norm", "normal_residual_norm",
    "solution_norm", "solution_energy_norm", "operator_norm_lower_bound",
    "augmented_operator_norm_lower_bound", "compatible_backward_error_upper_bound",
    "least_squares_backward_error_upper_bound", "backward_error_upper_bound",
    "relative_normal_residual_upper_bound", "energy_error_upper_bound",
    "relative_energy_error_upper_bound", "objective_gap_upper_bound",
    "ridge_base_energy_error_upper_bound", "ridge_corrected_energy_error_upper_bound",
    "ridge_correction_gamma", "ridge_correction_z_h_z", "ridge_correction_two_abs_z_t_q",
    "ridge_correction_q_norm_squared"]


class _OrcValidation(ctypes.Structure):
    _fields_ = ([(name, ctypes.c_double) for name in _VALIDATION_DOUBLES] +
                [("status", ctypes.c_int), ("stop_reason", ctypes.c_int),
                 ("ridge_correction_disposition", ctypes.c_int),
                 ("calls", ctypes.c_int * 6)])


def build_library() -> Path:
    """Compile the C half (gcc) if it is missing; returns its path."""
    if not _LIB_PATH.is_file():
        subprocess.run(["make", "-s", "-C", str(_HERE), "restatement"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build_library()))
        P = ctypes.c_void_p
        _lib.orc_apply.argtypes = [P, P, ctypes.c_int, P]
        _lib.orc_apply_transpose.argtypes = [P, P, ctypes.c_int, P]
        _lib.orc_model_of.argtypes = [P, P]
        _lib.orc_gaussian_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                             ctypes.c_uint64, ctypes.c_uint64, P]
        _lib.orc_norm_interval.argtypes = [P, ctypes.c_int64, P, P]
        _lib.orc_binary64_gamma.argtypes = [ctypes.c_longlong]
        _lib.orc_binary64_gamma.restype = ctypes.c_double
        _lib.orc_validate.argtypes = [P, P, P, P, ctypes.c_double, ctypes.c_double, P]
    return _lib


def gaussian_matrix(rows, cols, seed, stream, first_column):
    out = np.zeros((rows, cols), order="F")
    lib().orc_gaussian_matrix(rows, cols, seed & (2**64 - 1), stream & (2**64 - 1),
                              first_column, out.ctypes.data)
    return out


def norm_interval(v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    lo, hi = ctypes.c_double(), ctypes.c_double()
    lib().orc_norm_interval(v.ctypes.data, v.shape[0], ctypes.byref(lo), ctypes.byref(hi))
    return lo.value, hi.value


class Operator:
    """CSR or dense operator with the reference's MatrixOperator contract
    (include/amfls/matrix_operator.hpp:29-89)."""

    def __init__(self, problem, custom=False):
        """custom=True puts a CSR matrix behind a custom MatrixOperator: the
        same products and model but no extended-precision validation
        products (the interface defaults, matrix_operator.hpp:62-88)."""
        if hasattr(problem, "row_offsets"):
            self.kind = 3 if custom else 0
            self._keep = [np.ascontiguousarray(problem.row_offsets, dtype=np.int64),
                          np.ascontiguousarray(problem.column_indices, dtype=np.int64),
                          np.ascontiguousarray(problem.values, dtype=np.float64)]
            off, col, val = self._keep
            self.rows, self.cols = int(problem.rows), int(problem.cols)
            self._spec = _OrcOperator(self.kind, self.rows, self.cols, off.ctypes.data,
                                      col.ctypes.data, val.ctypes.data, val.shape[0])
        else:
            a = problem.matrix
            self.rows, self.cols = int(a.shape[0]), int(a.shape[1])
            if a.flags.c_contiguous:
                self.kind = 1
            else:
                a = np.asfortranarray(a)
                self.kind = 2
            self._keep = [a]
            self._spec = _OrcOperator(self.kind, self.rows, self.cols, None, None,
                                      a.ctypes.data, a.size)
        self._model = _OrcModel()
        lib().orc_model_of(ctypes.byref(self._spec), ctypes.byref(self._model))

    def relative_block_product_cost(self, block_cols):
        # CSR keeps the interface default (one unit per vector); both dense
        # operators charge one shared pass (dense_operator.cpp:100-105).
        if block_cols <= 0:
            return INF
        return float(block_cols) if self.kind in (0, 3) else 1.0

    def model(self):
        m = self._model
        return m.norm_upper, m.norm_lower, m.apply_steps, m.transpose_steps

    def _dense_product(self, v, transpose):
        """The reference's BLAS calls: column-major DenseOperator always uses
        dgemm (dense_operator.cpp:165-185); RowMajorDenseOperator uses dgemv
        for one column and dgemm otherwise on the transposed (n x m
        column-major) view of its buffer (row_major_dense_operator.cpp:183-260)."""
        a = self._keep[0]
        v = np.asfortranarray(v.reshape(v.shape[0], -1), dtype=np.float64)
        if self.kind == 2:  # a is m x n Fortran-ordered
            return sblas.dgemm(1.0, a, v, trans_a=1 if transpose else 0)
        at = a.T  # n x m Fortran-ordered view of the row-major buffer
        if v.shape[1] == 1:
            out = sblas.dgemv(1.0, at, v[:, 0], trans=0 if transpose else 1)
            return np.asfortranarray(out.reshape(-1, 1))
        return sblas.dgemm(1.0, at, v, trans_a=0 if transpose else 1)

    def apply(self, x):
        if self.kind not in (0, 3):
            return self._dense_product(np.asarray(x, dtype=np.float64), False)
        x = np.asfortranarray(x, dtype=np.float64)
        s = 1 if x.ndim == 1 else x.shape[1]
        y = np.zeros((self.rows, s), order="F")
        lib().orc_apply(ctypes.byref(self._spec), x.ctypes.data, s, y.ctypes.data)
        return y

    def apply_transpose(self, y):
        if self.kind not in (0, 3):
            return self._dense_product(np.asarray(y, dtype=np.float64), True)
        y = np.asfortranarray(y, dtype=np.float64)
        s = 1 if y.ndim == 1 else y.shape[1]
        x = np.zeros((self.cols, s), order="F")
        lib().orc_apply_transpose(ctypes.byref(self._spec), y.ctypes.data, s, x.ctypes.data)
        return x

    def validate(self, b, x, regularization, tolerance):
        out = _OrcValidation()
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        lib().orc_validate(ctypes.byref(self._spec), ctypes.byref(self._model), b.ctypes.data,
                           x.ctypes.data, regularization, tolerance, ctypes.byref(out))
        res = {name: getattr(out, name) for name in _VALIDATION_DOUBLES}
        res["status"] = out.status
        res["stop_reason"] = out.stop_reason
        res["ridge_correction_disposition"] = out.ridge_correction_disposition
        res["calls"] = list(out.calls)
        return res


# -------------------------------------------------------- statistics ----

_STAT_INTS = [
    "a_columns", "at_columns", "a_block_calls", "at_block_calls", "search_a_columns",
    "search_at_columns", "validation_a_columns", "validation_at_columns",
    "sketch_a_columns", "sketch_at_columns", "sketch_a_block_calls", "sketch_at_block_calls",
    "iterative_a_columns", "iterative_at_columns", "iterative_a_block_calls",
    "iterative_at_block_calls", "gaussian_random_columns", "gaussian_random_values",
    "search_a_block_calls", "search_at_block_calls", "validation_a_block_calls",
    "validation_at_block_calls", "base_validation_a_columns", "base_validation_at_columns",
    "base_validation_a_block_calls", "base_validation_at_block_calls",
    "ridge_correction_a_columns", "ridge_correction_at_columns",
    "ridge_correction_a_block_calls", "ridge_correction_at_block_calls",
    "gaussian_random_block_requests"]
_STAT_FLOATS = ["total_seconds", "a_seconds", "at_seconds", "orthogonalization_seconds",
                "projected_solve_seconds", "validation_seconds", "base_validation_seconds",
                "ridge_correction_validation_seconds"]


class Statistics:
    def __init__(self):
        for k in _STAT_INTS:
            setattr(self, k, 0)
        for k in _STAT_FLOATS:
            setattr(self, k, 0.0)

    def copy(self):
        s = Statistics()
        s.__dict__.update(self.__dict__)
        return s


# ------------------------------------------------- small LAPACK shims ----

def _nrm2(v):
    v = np.ravel(v, order="F")
    return 0.0 if v.shape[0] == 0 else float(sblas.dnrm2(v))


def _dot(a, b):
    return float(sblas.ddot(np.ravel(a), np.ravel(b)))


def _gemm(a, b, trans_a=False, trans_b=False):
    if a.shape[0] == 0 or b.shape[0] == 0 or a.shape[1] == 0 or b.shape[1] == 0:
        r = a.shape[1] if trans_a else a.shape[0]
        c = b.shape[0] if trans_b else b.shape[1]
        return np.zeros((r, c), order="F")
    return sblas.dgemm(1.0, a, b, trans_a=trans_a, trans_b=trans_b)


def _gemm_update(c, a, b, trans_b=False):
    """c -= a @ b (or a @ b.T); returns c (Fortran)."""
    if a.shape[1] == 0 or c.size == 0:
        return c
    return sblas.dgemm(-1.0, a, b, beta=1.0, c=c, trans_b=trans_b, overwrite_c=True)


def _thin_svd(a):
    u, s, vt = sla.svd(a, full_matrices=False, lapack_driver="gesdd", check_finite=False)
    return np.asfortranarray(u), s, np.asfortranarray(vt)


# ------------------------------------------------ orthogonalisation ----

def _rank_cutoff(scale, m, n, kb, cols):
    if not (scale >= 0.0) or not math.isfinite(scale):
        return INF
    return 64.0 * EPS * max(1, m, n, kb, cols) * scale


class _Factor:
    pass


def orthogonalize_and_factor(block, basis, maximum_rank, m, n, scale, tracked_prefix,
                             retain, stats):
    """krylov_workspace.cpp:82-310."""
    t0 = time.perf_counter()
    rows, cols = block.shape
    kb = basis.shape[1]
    retain_scalar = cols != 1 or retain
    coeff = np.zeros((kb if retain_scalar else 0, cols), order="F")
    coeff_finite = True
    if cols == 1 and kb > 0:
        x = np.asfortranarray(block[:, 0]).copy()
        before = _nrm2(x)
        acc = np.zeros(kb)

        def one_pass(x):
            pc = sblas.dgemv(1.0, basis, x, trans=1)
            if retain_scalar:
                coeff[:, 0] += pc
            else:
                acc[:] += pc
            return sblas.dgemv(-1.0, basis, pc, beta=1.0, y=x, overwrite_y=True)

        x = one_pass(x)
        after = _nrm2(x)
        if math.isfinite(before) and math.isfinite(after) and after < math.sqrt(0.5) * before:
            x = one_pass(x)
            after = _nrm2(x)
        if not retain_scalar:
            coeff_finite = bool(np.all(np.isfinite(acc)))
        block = np.asfortranarray(x.reshape(rows, 1))
    else:
        block = np.asfortranarray(block)
        if kb > 0:
            for _ in range(2):
                pc = _gemm(basis, block, trans_a=True)
                coeff += pc
                block = _gemm_update(block, basis, pc)
        after = _nrm2(block)
    f = _Factor()
    f.cutoff = _rank_cutoff(scale, m, n, kb, cols)
    finite = math.isfinite(scale) and math.isfinite(after) and coeff_finite and \
        bool(np.all(np.isfinite(coeff)))
    f.coefficients = coeff
    f.q = np.zeros((rows, 0), order="F")
    f.factor = np.zeros((0, cols), order="F")
    f.discarded = after
    f.tracked = 0.0
    f.positive_below = False
    f.nonfinite = not finite
    if not finite:
        f.discarded = INF
        f.tracked = INF if tracked_prefix > 0 else 0.0
    elif maximum_rank == 0 or cols == 0:
        for c in range(tracked_prefix):
            f.tracked = math.hypot(f.tracked, _nrm2(block[:, c]))
    elif cols == 1:
        rn = after
        if math.isfinite(rn) and rn > f.cutoff:
            inv = 1.0 / rn
            f.q = np.asfortranarray(block * inv)
            f.factor = np.full((1, 1), rn, order="F")
            f.discarded = 0.0
            f.tracked = 0.0
        elif math.isfinite(rn) and 0.0 < rn <= f.cutoff and maximum_rank > 0:
            f.positive_below = True
            if tracked_prefix == 1:
                f.tracked = rn
    else:
        u, s, vt = _thin_svd(block)
        rank = 0
        while rank < s.shape[0] and rank < maximum_rank and math.isfinite(s[rank]) and \
                s[rank] > f.cutoff:
            rank += 1
        if rank < s.shape[0] and rank < maximum_rank:
            first = s[rank]
            f.positive_below = math.isfinite(first) and 0.0 < first <= f.cutoff
        if rank > 0:
            f.q = np.asfortranarray(u[:, :rank])
            f.factor = np.asfortranarray(s[:rank, None] * vt[:rank, :])
        f.discarded = 0.0
        for idx in range(rank, s.shape[0]):
            f.discarded = math.hypot(f.discarded, s[idx])
            w = 0.0
            for c in range(tracked_prefix):
                w = math.hypot(w, vt[idx, c])
            f.tracked = math.hypot(f.tracked, s[idx] * w)
    stats.orthogonalization_seconds += time.perf_counter() - t0
    return f


def stable_ridge_filter(sigma, lam):
    """sigma / (sigma^2 + lam) without overflow (krylov_workspace.cpp:312-331)."""
    if not (sigma > 0.0) or not (lam > 0.0):
        return 0.0
    root = math.sqrt(lam)
    if not (root > 0.0) or not math.isfinite(root):
        return sigma / (sigma * sigma + lam)
    if sigma <= root:
        r = sigma / root
        return (r / (1.0 + r * r)) / root
    inv = root / sigma
    return (1.0 / sigma) / (1.0 + inv * inv)


def _new_audit():
    return dict(requested_injected_columns=0, retained_injected_columns=0, left_input_width=0,
                retained_right_width=0, retained_next_left_width=0, basis_rank_before=0,
                basis_rank_after=0, right_rank_cutoff=0.0, right_discarded_residual_norm=0.0,
                right_active_discarded_residual_norm=0.0, left_rank_cutoff=0.0,
                left_discarded_residual_norm=0.0, right_rank_loss=False, left_rank_loss=False,
                right_positive_finite_below_cutoff=False,
                left_positive_finite_below_cutoff=False, right_nonfinite_residual=False,
                left_nonfinite_residual=False, right_basis_cap_truncation=False,
                left_basis_cap_truncation=False)


def step_has_numerical_rank_truncation(a):
    return (a["right_rank_loss"] and a["right_positive_finite_below_cutoff"] and
            a["right_active_discarded_residual_norm"] > 0.0) or \
        (a["left_rank_loss"] and a["left_positive_finite_below_cutoff"])


def step_has_nonfinite_breakdown(a):
    return a["right_nonfinite_residual"] or a["left_nonfinite_residual"]


# ---------------------------------------------------------- workspace ----

class Workspace:
    """Variable-width block Golub-Kahan process (krylov_workspace.hpp:93-189)."""

    def __init__(self, op, b, regularization, maximum_basis_size, stats):
        self.op, self.stats = op, stats
        self.m, self.n = op.rows, op.cols
        self.b = np.ascontiguousarray(b, dtype=np.float64).copy()
        if not np.all(np.isfinite(self.b)):
            raise ValueError("block Golub-Kahan right-hand side must be finite")
        self.bnorm = _nrm2(self.b)
        self.reg = regularization
        mn = min(self.m, self.n)
        self.basis_limit = min(maximum_basis_size, mn) if maximum_basis_size > 0 else mn
        self.U = np.zeros((self.m, 0), order="F")
        self.P = np.zeros((self.m, 0), order="F")
        self._V = np.zeros((self.n, 8), order="F")
        self.k = 0
        self._T = np.zeros((min(self.basis_limit + 1, 8), 8), order="F")
        self.g = []
        self.active = (0, 0)
        self.prev_right = (0, 0)
        self.coupling = np.zeros((0, 0), order="F")
        self.pending_requested = 0
        self.pending_retained = 0
        self.depth = 0
        self.initialized = False
        self.reliable = True
        self.audit = _new_audit()

    # -- storage helpers
    @property
    def V(self):
        return self._V[:, :self.k]

    def _append_v(self, q):
        need = self.k + q.shape[1]
        if need > self._V.shape[1]:
            cap = max(need, 2 * self._V.shape[1])
            nv = np.zeros((self.n, cap), order="F")
            nv[:, :self.k] = self._V[:, :self.k]
            self._V = nv
        self._V[:, self.k:need] = q
        self.k = need

    def _ensure_t(self, rows, cols):
        limit = self.basis_limit + 1
        if rows > limit:
            raise RuntimeError("block Golub-Kahan projected row limit was exceeded")
        r, c = self._T.shape
        if rows > r:
            nr = max(1, r)
            while nr < rows:
                nr = limit if nr > limit // 2 else 2 * nr
        else:
            nr = r
        nc = c if cols <= c else max(cols, 2 * c)
        if (nr, nc) != (r, c):
            t = np.zeros((nr, nc), order="F")
            t[:r, :c] = self._T
            self._T = t

    def projected_operator(self):
        return np.asfortranarray(self._T[:len(self.g), :self.k])

    # -- operator calls
    def _apply_search(self, x):
        t0 = time.perf_counter()
        y = self.op.apply(x)
        s = self.stats
        s.a_seconds += time.perf_counter() - t0
        s.a_columns += x.shape[1]
        s.search_a_columns += x.shape[1]
        s.a_block_calls += 1
        s.search_a_block_calls += 1
        return y

    def _apply_transpose_search(self, y):
        t0 = time.perf_counter()
        x = self.op.apply_transpose(y)
        s = self.stats
        s.at_seconds += time.perf_counter() - t0
        s.at_columns += y.shape[1]
        s.search_at_columns += y.shape[1]
        s.at_block_calls += 1
        s.search_at_block_calls += 1
        return x

    def can_advance(self):
        return self.initialized and self.reliable and \
            self.U.shape[1] + self.P.shape[1] > 0 and self.k < self.basis_limit

    def active_left_width(self):
        return self.active[1]

    def initialize(self, aux):
        """krylov_workspace.cpp:470-503."""
        if self.initialized:
            raise RuntimeError("block Golub-Kahan workspace is already initialized")
        self.initialized = True
        self.audit = _new_audit()
        t0 = time.perf_counter()
        if math.isfinite(self.bnorm) and self.bnorm > 0.0 and self.basis_limit > 0:
            inv = 1.0 / self.bnorm
            self.U = np.asfortranarray((self.b * inv).reshape(self.m, 1))
            self.g.append(self.bnorm)
            self.active = (0, 1)
        self.stats.orthogonalization_seconds += time.perf_counter() - t0
        if self.bnorm > 0.0 and aux.shape[1] > 0:
            self.append_left_seed(aux)

    def append_left_seed(self, seed):
        """krylov_workspace.cpp:505-587."""
        if not self.initialized:
            raise RuntimeError("block Golub-Kahan workspace is not initialized")
        if not self.reliable:
            raise RuntimeError("cannot continue block Golub-Kahan after numerical truncation")
        if self.pending_requested == 0 and self.P.shape[1] == 0:
            self.audit = _new_audit()
        c = seed.shape[1]
        self.pending_requested += c
        self.audit["requested_injected_columns"] = self.pending_requested
        self.audit["retained_injected_columns"] = self.pending_retained
        if c == 0:
            return 0
        available = max(0, self.basis_limit - self.k - self.U.shape[1] - self.P.shape[1])
        max_rank = min(available, self.m - self.U.shape[1] - self.P.shape[1], c)
        if max_rank <= 0:
            return 0
        local = self.U if self.P.shape[1] == 0 else np.asfortranarray(np.hstack([self.U, self.P]))
        scale = _nrm2(seed)
        f = orthogonalize_and_factor(np.asfortranarray(seed), local, max_rank, self.m, self.n,
                                     scale, 0, False, self.stats)
        kept = f.q.shape[1]
        if kept <= 0:
            return 0
        self.P = f.q if self.P.shape[1] == 0 else np.asfortranarray(np.hstack([self.P, f.q]))
        self.pending_retained += kept
        self.audit["retained_injected_columns"] = self.pending_retained
        return kept

    def advance_level(self):
        """krylov_workspace.cpp:589-831."""
        a = _new_audit()
        a["requested_injected_columns"] = self.pending_requested
        a["retained_injected_columns"] = self.pending_retained
        a["basis_rank_before"] = a["basis_rank_after"] = self.k
        a["left_input_width"] = self.U.shape[1] + self.P.shape[1]
        self.audit = a
        if not self.can_advance():
            return False
        old_right, old_left, aw = self.k, len(self.g), self.U.shape[1]
        combined = self.U if self.P.shape[1] == 0 else np.asfortranarray(np.hstack([self.U, self.P]))
        rres = self._apply_transpose_search(combined)
        self.P = np.zeros((self.m, 0), order="F")
        self.pending_requested = self.pending_retained = 0
        rscale = _nrm2(rres)
        pf, pw = self.prev_right
        if pw > 0 and aw > 0:
            coup = self.coupling
            if combined.shape[1] != aw:
                ext = np.zeros((combined.shape[1], pw), order="F")
                ext[:aw, :] = coup
                coup = ext
            rres = _gemm_update(rres, np.asfortranarray(self._V[:, pf:pf + pw]),
                                np.asfortranarray(coup), trans_b=True)
        max_rr = min(combined.shape[1], self.basis_limit - self.k)
        rf = orthogonalize_and_factor(rres, self.V, max_rr, self.m, self.n, rscale, aw, False,
                                      self.stats)
        rw = rf.q.shape[1]
        a["retained_right_width"] = rw
        a["right_rank_cutoff"] = rf.cutoff
        a["right_discarded_residual_norm"] = rf.discarded
        a["right_active_discarded_residual_norm"] = rf.tracked
        a["right_positive_finite_below_cutoff"] = rf.positive_below
        a["right_nonfinite_residual"] = rf.nonfinite
        a["right_rank_loss"] = rw < max_rr
        a["right_basis_cap_truncation"] = max_rr < combined.shape[1]
        if step_has_numerical_rank_truncation(a) or step_has_nonfinite_breakdown(a):
            self.reliable = False
        if rw == 0:
            self.U = np.zeros((self.m, 0), order="F")
            self.active = (old_left, 0)
            self.prev_right = (self.k, 0)
            self.coupling = np.zeros((0, 0), order="F")
            return False
        new_right = rf.q
        lres = self._apply_search(new_right)
        lscale = _nrm2(lres)
        act = rf.factor if rf.factor.shape[1] == aw else np.asfortranarray(rf.factor[:, :aw])
        if aw > 0:
            lres = _gemm_update(lres, self.U, act, trans_b=True)
        max_lr = min(rw, self.m - old_left, self.basis_limit + 1 - old_left)
        lf = orthogonalize_and_factor(lres, self.U, max_lr, self.m, self.n, lscale, 0, True,
                                      self.stats)
        nlw = lf.q.shape[1]
        a["retained_next_left_width"] = nlw
        a["left_rank_cutoff"] = lf.cutoff
        a["left_discarded_residual_norm"] = lf.discarded
        a["left_positive_finite_below_cutoff"] = lf.positive_below
        a["left_nonfinite_residual"] = lf.nonfinite
        a["left_rank_loss"] = nlw < max_lr
        a["left_basis_cap_truncation"] = max_lr < rw
        if step_has_numerical_rank_truncation(a) or step_has_nonfinite_breakdown(a):
            self.reliable = False
        if lf.nonfinite:
            return False
        if self.k * 1 + rw > 0 and self.n * (self.k + rw) > INT_MAX:
            raise OverflowError("matrix is too large for the LP64 backend")
        self._append_v(new_right)
        self._ensure_t(old_left + nlw, old_right + rw)
        af = self.active[0]
        for j in range(rw):
            for r in range(aw):
                self._T[af + r, old_right + j] = act[j, r] + lf.coefficients[r, j]
            for r in range(nlw):
                self._T[old_left + r, old_right + j] = lf.factor[r, j]
        self.U = lf.q
        for j in range(nlw):
            self.g.append(_dot(self.U[:, j], self.b))
        self.active = (old_left, nlw)
        self.prev_right = (old_right, rw)
        self.coupling = lf.factor
        self.depth += 1
        a["basis_rank_after"] = self.k
        return True

    def evaluate(self, tolerance, epoch, auxiliary_width):
        """krylov_workspace.cpp:833-925."""
        if not self.initialized:
            raise RuntimeError("block Golub-Kahan workspace is not initialized")
        if not (0.0 < tolerance < 1.0):
            raise ValueError("block Golub-Kahan tolerance must lie strictly between zero and one")
        t0 = time.perf_counter()
        if self.k > 0:
            t = self.projected_operator()
            g = np.asarray(self.g)
            rtol = min(0.5, 64.0 * EPS * max(t.shape[0], t.shape[1]))
            if self.reg == 0.0:
                y = sla.lstsq(t, g, cond=rtol, lapack_driver="gelsy", check_finite=False)[0]
            else:
                u, s, vt = _thin_svd(t)
                spec = np.array([stable_ridge_filter(s[i], self.reg) * _dot(u[:, i], g)
                                 for i in range(s.shape[0])])
                y = np.array([float(np.sum(vt[:, c].astype(np.longdouble) *
                                           spec.astype(np.longdouble)))
                              for c in range(self.k)])
            x = _gemm(np.asfortranarray(self.V), np.asfortranarray(y.reshape(-1, 1)))[:, 0]
        else:
            x = np.zeros(self.n)
        self.stats.projected_solve_seconds += time.perf_counter() - t0
        r = validate_candidate(self.op, self.b, x, self.reg, tolerance, self.stats)
        r["depth"] = self.depth
        r["auxiliary_width"] = auxiliary_width
        r["basis_rank"] = self.k
        r["trace"] = [_trace_record(r, epoch)]
        return r


def validate_candidate(op, b, x, regularization, tolerance, stats):
    """candidate_validation.cpp:1176-1378, through the C half."""
    t0 = time.perf_counter()
    v = op.validate(b, x, regularization, tolerance)
    dt = time.perf_counter() - t0
    c = v.pop("calls")
    base_a, base_at = c[0] + c[2], c[1] + c[3]
    corr_a, corr_at = c[4], c[5]
    share = dt / max(1, sum(c))
    s = stats
    s.a_columns += base_a + corr_a
    s.at_columns += base_at + corr_at
    s.a_block_calls += base_a + corr_a
    s.at_block_calls += base_at + corr_at
    s.validation_a_columns += base_a + corr_a
    s.validation_at_columns += base_at + corr_at
    s.validation_a_block_calls += base_a + corr_a
    s.validation_at_block_calls += base_at + corr_at
    s.base_validation_a_columns += base_a
    s.base_validation_at_columns += base_at
    s.base_validation_a_block_calls += base_a
    s.base_validation_at_block_calls += base_at
    s.ridge_correction_a_columns += corr_a
    s.ridge_correction_at_columns += corr_at
    s.ridge_correction_a_block_calls += corr_a
    s.ridge_correction_at_block_calls += corr_at
    s.a_seconds += share * (base_a + corr_a)
    s.at_seconds += share * (base_at + corr_at)
    s.base_validation_seconds += share * (base_a + base_at)
    s.ridge_correction_validation_seconds += share * (corr_a + corr_at)
    s.validation_seconds = s.base_validation_seconds + s.ridge_correction_validation_seconds
    v["solution"] = np.array(x, dtype=np.float64)
    v["statistics"] = stats.copy()
    return v


def candidate_validation_failed_numerically(r):
    return r["status"] == 4 or r["stop_reason"] == 7


_TRACE_DOUBLES = [
    "objective", "residual_norm", "augmented_residual_norm", "normal_residual_norm",
    "operator_norm_lower_bound", "compatible_backward_error_upper_bound",
    "least_squares_backward_error_upper_bound", "backward_error_upper_bound",
    "relative_normal_residual_upper_bound", "relative_energy_error_upper_bound",
    "solution_norm", "solution_energy_norm", "augmented_operator_norm_lower_bound",
    "energy_error_upper_bound", "objective_gap_upper_bound",
    "ridge_base_energy_error_upper_bound", "ridge_corrected_energy_error_upper_bound",
    "ridge_correction_gamma", "ridge_correction_z_h_z", "ridge_correction_two_abs_z_t_q",
    "ridge_correction_q_norm_squared"]


def _trace_record(r, epoch):
    s = r["statistics"]
    head = [epoch, r.get("depth", 0), r.get("auxiliary_width", 0), r.get("basis_rank", 0),
            s.a_columns, s.at_columns, s.a_block_calls, s.at_block_calls]
    return dict(floats=[float(v) for v in head] + [r[k] for k in _TRACE_DOUBLES],
                ints=[r["status"], r["stop_reason"], 1 if r["status"] == 0 else 0,
                      r["ridge_correction_disposition"]])


def validate_common_inputs(op, b, regularization, tolerance):
    if op.rows <= 0 or op.cols <= 0:
        raise ValueError("operator dimensions must be positive")
    if not math.isfinite(regularization) or regularization < 0.0:
        raise ValueError("regularization must be finite and nonnegative")
    if not math.isfinite(tolerance) or tolerance <= 0.0 or tolerance >= 1.0:
        raise ValueError("tolerance must lie strictly between zero and one")
    if not np.all(np.isfinite(b)):
        raise ValueError("right-hand side must be finite")


# ------------------------------------------------- checkpoint cadence ----

def is_certificate_checkpoint(iteration, regularization):
    if iteration <= 1:
        return True
    odd = iteration
    while odd % 2 == 0:
        odd //= 2
    return odd == 1 or (regularization == 0.0 and odd == 3)


class CheckpointSchedule:
    """certificate_checkpoint_schedule.hpp:37-131."""

    def __init__(self, regularization, tolerance):
        self.reg, self.tol = regularization, tolerance
        self.predicted = INT_MAX
        self.prev_iter = 0
        self.prev_compat = self.prev_ls = self.prev_energy = 0.0
        self.has_prev = False

    def should_evaluate(self, it):
        return is_certificate_checkpoint(it, self.reg) or it >= self.predicted

    @staticmethod
    def _crossing(prev, cur, prev_it, cur_it, tol):
        if not (prev > cur) or not (cur > tol) or not (tol > 0.0) or not math.isfinite(prev) \
                or not math.isfinite(cur) or not math.isfinite(tol):
            return INT_MAX
        LD = np.longdouble
        dist = np.log(LD(cur)) - np.log(LD(tol))
        contraction = np.log(LD(prev)) - np.log(LD(cur))
        offset = np.ceil(LD(cur_it - prev_it) * dist / contraction)
        if not (offset > 0) or not np.isfinite(offset) or offset > INT_MAX - cur_it:
            return INT_MAX
        return cur_it + int(offset)

    def record(self, it, r):
        self.predicted = INT_MAX
        static = is_certificate_checkpoint(it, self.reg)
        if static and self.has_prev and it > self.prev_iter:
            if self.reg > 0.0:
                self.predicted = self._crossing(self.prev_energy,
                                                r["relative_energy_error_upper_bound"],
                                                self.prev_iter, it, self.tol)
            else:
                self.predicted = min(
                    self._crossing(self.prev_compat, r["compatible_backward_error_upper_bound"],
                                   self.prev_iter, it, self.tol),
                    self._crossing(self.prev_ls, r["least_squares_backward_error_upper_bound"],
                                   self.prev_iter, it, self.tol))
        self.prev_iter = it
        self.prev_compat = r["compatible_backward_error_upper_bound"]
        self.prev_ls = r["least_squares_backward_error_upper_bound"]
        self.prev_energy = r["relative_energy_error_upper_bound"]
        self.has_prev = True


# --------------------------------------------------- width controller ----

DBL_MAX = float(np.finfo(np.float64).max)


class ProgressHistory:
    def __init__(self):
        self.contr = [0.0, 0.0]
        self.level_contr = [0.0, 0.0]
        self.levels = [0, 0]
        self.op_s = [INF, INF]
        self.local_s = [INF, INF]
        self.count = 0
        self.prior_contr = 0.0
        self.prior_levels = 0
        self.width = -1


def record_deepen_progress(h, prev, cur, start_w, end_w, levels, op_s, local_s):
    """amfls_internal.hpp:35-144 (long double arithmetic kept as float64 here)."""
    if start_w <= 0 or end_w <= 0 or start_w != end_w:
        h.__init__()
        return
    if h.width != start_w:
        h.__init__()
        h.width = start_w
    if levels <= 0 or not (prev > 0.0) or not (cur > 0.0) or not math.isfinite(prev) or \
            not math.isfinite(cur):
        return
    LD = np.longdouble
    progress_ld = np.log(LD(prev)) - np.log(LD(cur)) if prev > cur else LD(0.0)
    if not (progress_ld >= 0.0) or not np.isfinite(progress_ld):
        return
    progress = float(progress_ld)
    lvl = progress_ld / LD(levels)
    lvl_d = float(min(lvl, LD(DBL_MAX))) if lvl > 0.0 and np.isfinite(lvl) else 0.0
    fin = op_s >= 0.0 and local_s >= 0.0 and math.isfinite(op_s) and math.isfinite(local_s) \
        and op_s + local_s > 0.0 and math.isfinite(op_s + local_s)
    lop = op_s / levels if fin else INF
    lloc = local_s / levels if fin else INF
    if h.count < 2:
        i = h.count
        h.contr[i], h.level_contr[i], h.levels[i] = progress, lvl_d, levels
        h.op_s[i], h.local_s[i] = lop, lloc
        h.count += 1
    else:
        pooled = np.longdouble(h.prior_contr) + np.longdouble(h.contr[0])
        if h.prior_levels > INT_MAX - h.levels[0] or not np.isfinite(pooled) or pooled > DBL_MAX:
            h.prior_contr, h.prior_levels = INF, INT_MAX
        else:
            h.prior_contr = float(pooled)
            h.prior_levels += h.levels[0]
        h.contr = [h.contr[1], progress]
        h.level_contr = [h.level_contr[1], lvl_d]
        h.levels = [h.levels[1], levels]
        h.op_s = [h.op_s[1], lop]
        h.local_s = [h.local_s[1], lloc]


def next_dyadic_increment(active, generated, max_generated, available):
    """amfls_internal.hpp:151-181."""
    if active <= 0 or generated < 0 or max_generated <= generated or active > generated + 1 \
            or available <= 0:
        return 0
    max_active = active + max_generated - generated
    nxt = max_active if active > max_active // 2 else min(2 * active, max_active)
    if nxt <= active:
        return 0
    req = nxt - active
    return req if req <= available and req <= INT_MAX else 0


def _ceil_ratio(a, b):
    return 0 if a <= 0 or b <= 0 else 1 + (a - 1) // b


def feedback_feasible_increment(rank, limit, frontier, levels):
    """amfls_internal.hpp:193-207."""
    if rank < 0 or limit < rank or frontier < 0 or levels <= 0:
        return 0
    return max(0, (limit - rank) // levels - frontier)


class WidthDecision:
    def __init__(self):
        self.recent = self.prior = self.remaining = 0.0
        self.forecast = self.incumbent_levels = self.target_levels = 0
        self.target_remaining = self.matched_horizon = 0
        self.inc_s = self.tgt_s = INF
        self.history_mature = self.prior_mature = False
        self.recent_slowdown = self.persistent_slowdown = self.stalled = False
        self.long_horizon = self.necessary = self.costs_mature = False
        self.width_depth_ok = True
        self.pass_reduction = self.feasible = self.finite_cert = False
        self.finite_boundary = self.candidate = False


def _cost_gate(d, aw, tw, lop, lloc, count, inc_cost, tgt_cost):
    """amfls_internal.hpp:238-325."""
    if d.incumbent_levels <= 0 or d.target_levels <= 0 or aw <= 0 or tw <= aw or count != 2 \
            or not (inc_cost > 0.0) or not (tgt_cost > 0.0) or not math.isfinite(inc_cost) \
            or not math.isfinite(tgt_cost):
        return
    LD = np.longdouble
    wr = LD(tw) / LD(aw)
    wr2 = wr * wr
    ratio = LD(tgt_cost) / LD(inc_cost)
    inc_op_cost = LD(d.incumbent_levels) * LD(inc_cost)
    tgt_op_cost = LD(d.target_levels) * LD(tgt_cost)
    best_inc, worst_tgt, ok = LD(INF), LD(0.0), True
    for i in range(count):
        o, l = LD(lop[i]), LD(lloc[i])
        if not (o >= 0.0) or not (l >= 0.0) or not np.isfinite(o) or not np.isfinite(l) \
                or not (o + l > 0.0):
            ok = False
            break
        inc = LD(d.incumbent_levels) * (o + l)
        tl = l * wr2
        tgt = LD(d.target_levels) * (o * ratio + tl) + tl
        if not np.isfinite(inc) or not np.isfinite(tgt):
            ok = False
            break
        best_inc = min(best_inc, inc)
        worst_tgt = max(worst_tgt, tgt)
    if ok:
        ok = best_inc <= DBL_MAX and worst_tgt <= DBL_MAX
        if ok:
            d.inc_s, d.tgt_s = float(best_inc), float(worst_tgt)
    d.costs_mature = ok
    d.pass_reduction = d.width_depth_ok and d.target_levels < d.incumbent_levels and \
        tgt_op_cost < inc_op_cost and d.costs_mature and d.tgt_s < d.inc_s


def horizon_candidate(inc, horizon, depth, max_depth, rank, limit, aw, lop, lloc, count,
                      inc_cost=1.0, tgt_cost=1.0, balance=False):
    """amfls_internal.hpp:332-392."""
    d = WidthDecision()
    d.feasible = inc > 0 and aw > 0 and inc <= INT_MAX - aw
    d.finite_boundary = depth >= 0 and max_depth >= depth and rank >= 0 and limit >= rank and \
        aw > 0 and horizon > 0 and horizon <= limit - rank
    if not d.feasible or not d.finite_boundary:
        return d
    tw = aw + inc
    d.target_remaining = min(max_depth - depth, (limit - rank) // tw)
    d.matched_horizon = int(min(horizon, d.target_remaining * tw))
    d.incumbent_levels = _ceil_ratio(d.matched_horizon, aw)
    d.target_levels = _ceil_ratio(d.matched_horizon, tw)
    if d.target_levels < 2:
        return d
    d.width_depth_ok = (not balance) or d.target_levels > tw
    _cost_gate(d, aw, tw, lop, lloc, count, inc_cost, tgt_cost)
    d.candidate = d.pass_reduction
    return d


def initial_candidate(inc, cert, tol, depth, max_depth, rank, limit, aw, h, inc_cost=1.0,
                      tgt_cost=1.0):
    """amfls_internal.hpp:399-552."""
    d = WidthDecision()
    d.finite_cert = cert > 0.0 and tol > 0.0 and cert > tol and math.isfinite(cert) and \
        math.isfinite(tol)
    d.history_mature = h.width == aw and h.count >= 2
    if not d.finite_cert or not d.history_mature or depth < 0 or max_depth < depth or \
            rank < 0 or limit < rank or aw <= 0 or inc <= 0 or inc > INT_MAX - aw:
        return d
    LD = np.longdouble
    recent_levels = h.levels[0] + h.levels[1]
    recent_progress = LD(h.contr[0]) + LD(h.contr[1])
    if recent_levels <= 0 or not (recent_progress >= 0.0) or not np.isfinite(recent_progress):
        return d
    d.stalled = recent_progress == 0.0
    d.recent = 0.0 if d.stalled else float(recent_progress / LD(recent_levels))
    d.remaining = math.log(cert) - math.log(tol)
    if (not d.stalled and (not (d.recent > 0.0) or not math.isfinite(d.recent))) or \
            not (d.remaining > 0.0) or not math.isfinite(d.remaining):
        return d
    if not d.stalled:
        raw = LD(d.remaining) / LD(d.recent)
        if not (raw > 0.0) or not np.isfinite(raw):
            return d
        d.forecast = INT_MAX if raw >= INT_MAX else max(1, int(np.ceil(raw)))
    d.prior_mature = h.prior_levels > 0 and h.prior_contr > 0.0 and math.isfinite(h.prior_contr)
    if d.prior_mature:
        d.prior = h.prior_contr / h.prior_levels
        d.persistent_slowdown = math.isfinite(d.prior) and h.level_contr[0] > 0.0 and \
            h.level_contr[1] > 0.0 and h.level_contr[0] < d.prior and h.level_contr[1] < d.prior
    remaining_basis = limit - rank
    tw = aw + inc
    tr = min(max_depth - depth, remaining_basis // tw)
    raw_h = tw * tr if d.stalled else aw * d.forecast
    horizon = int(min(raw_h, remaining_basis))
    c = horizon_candidate(inc, horizon, depth, max_depth, rank, limit, aw, h.op_s, h.local_s, 2,
                          inc_cost, tgt_cost)
    c.finite_cert, c.history_mature = d.finite_cert, d.history_mature
    c.prior_mature, c.persistent_slowdown = d.prior_mature, d.persistent_slowdown
    c.stalled, c.recent, c.prior = d.stalled, d.recent, d.prior
    c.remaining, c.forecast = d.remaining, d.forecast
    c.long_horizon = c.target_remaining > 0 and (c.stalled or d.forecast > c.target_remaining)
    positive = h.level_contr[0] > 0.0 and h.level_contr[1] > 0.0
    c.recent_slowdown = positive and h.level_contr[1] < 0.5 * h.level_contr[0]
    established_stall = c.stalled and (aw > 1 or c.prior_mature)
    scalar_needed = aw == 1 and positive and (c.recent_slowdown or (
        c.prior_mature and (c.persistent_slowdown or c.long_horizon)))
    block_needed = aw > 1 and (positive or established_stall) and (
        c.persistent_slowdown or c.long_horizon or c.pass_reduction)
    c.necessary = scalar_needed or block_needed
    c.candidate = c.candidate and c.necessary
    return c


class HorizonPlan:
    def __init__(self):
        self.end = -1
        self.origin = -1
        self.width = -1
        self.start_cert = INF
        self.op_s = [INF, INF]
        self.local_s = [INF, INF]
        self.count = 0


def remaining_horizon(p, rank):
    if p.end < 0 or rank < 0 or rank >= p.end:
        return 0
    return p.end - rank


def extend_to_limit(p, rank, limit):
    if p.end < 0 or rank < 0 or limit <= rank or rank < p.end:
        return False
    p.end = limit
    return True


def horizon_stalled(p, cert):
    return p.start_cert > 0.0 and cert > 0.0 and math.isfinite(p.start_cert) and \
        math.isfinite(cert) and math.log(p.start_cert) - math.log(cert) < math.log(2.0)


def start_plan(p, rank, limit, horizon, origin, target, cert):
    if rank < 0 or limit < rank or horizon <= 0 or horizon > limit - rank or origin <= 0 or \
            target <= 0 or not (cert > 0.0) or not math.isfinite(cert):
        p.__init__()
        return False
    p.__init__()
    p.end, p.origin, p.width, p.start_cert = rank + horizon, origin, target, cert
    return True


def reset_plan_costs(p, width):
    p.width = width
    p.op_s = [INF, INF]
    p.local_s = [INF, INF]
    p.count = 0


def record_plan_cost(p, start_w, end_w, levels, op_s, local_s):
    if p.end < 0 or start_w <= 0 or start_w != end_w or start_w != p.width or levels <= 0 or \
            op_s < 0.0 or local_s < 0.0 or not math.isfinite(op_s) or \
            not math.isfinite(local_s) or not (op_s + local_s > 0.0) or p.count >= 2:
        return False
    p.op_s[p.count] = op_s / levels
    p.local_s[p.count] = local_s / levels
    p.count += 1
    return True


# -------------------------------------------------------------- solve ----

def _default_epochs(dim):
    epochs, covered = 1, 1
    while covered < dim and epochs < 30:
        covered *= 2
        epochs += 1
    return epochs


def _certificate(r, reg):
    return r["relative_energy_error_upper_bound"] if reg > 0.0 else r["backward_error_upper_bound"]


def solve_amfls(problem, regularization=0.0, tolerance=1e-8, failure_probability=1e-6,
                maximum_epochs=0, maximum_depth=0, maximum_auxiliary_width=0,
                maximum_basis_size=0, seed=0, stream=0, replay=None, custom=False):
    """amfls.cpp:57-661. Returns the result dict in the torch binding's layout.
    custom=True solves a CSR problem through a custom MatrixOperator (see
    Operator)."""
    op = Operator(problem, custom=custom)
    b = np.ascontiguousarray(problem.b, dtype=np.float64)
    return solve_amfls_operator(op, b, regularization, tolerance, failure_probability,
                                maximum_epochs, maximum_depth, maximum_auxiliary_width,
                                maximum_basis_size, seed, stream, replay=replay)


def solve_amfls_operator(op, b, regularization=0.0, tolerance=1e-8, failure_probability=1e-6,
                         maximum_epochs=0, maximum_depth=0, maximum_auxiliary_width=0,
                         maximum_basis_size=0, seed=0, stream=0, replay=None):
    """The controller of amfls.cpp:57-661.  The result also carries
    ``decisions``: the candidate bit of every width decision taken at the
    reference's decision sites (amfls.cpp:323-354).  ``replay`` (a sequence
    of 0/1) substitutes those bits in order for the timing-driven ones, the
    schedule-replay mode that makes widening solves reproducible; sites
    beyond the list keep their own decision and are counted in
    ``replay_overrun``."""
    reg, tol = regularization, tolerance
    decisions = []
    overrun = 0
    validate_common_inputs(op, b, reg, tol)
    if not math.isfinite(failure_probability) or not (0.0 < failure_probability < 1.0):
        raise ValueError("failure_probability must lie strictly between zero and one")
    if min(maximum_epochs, maximum_depth, maximum_auxiliary_width, maximum_basis_size) < 0:
        raise ValueError("work limits must be nonnegative")
    t_start = time.perf_counter()
    stats = Statistics()
    ws = Workspace(op, b, reg, maximum_basis_size, stats)
    dim = min(op.rows, op.cols)
    max_depth = min(maximum_depth, dim) if maximum_depth > 0 else dim
    cap = max(0, ws.basis_limit - 1)
    max_aux = min(maximum_auxiliary_width if maximum_auxiliary_width > 0 else cap, cap)
    max_epochs = maximum_epochs if maximum_epochs > 0 else _default_epochs(dim)
    trace = []
    sched = CheckpointSchedule(reg, tol)
    st = dict(evals=0, last_depth=-1, aux=0, result=None, best=None, best_cert=INF, has=False)

    def record(cand, train):
        if cand["depth"] == st["last_depth"]:
            raise RuntimeError("AMFLS evaluated one checkpoint more than once")
        st["last_depth"] = cand["depth"]
        if train:
            sched.record(cand["depth"], cand)
        trace.append(cand["trace"][0])
        st["evals"] += 1
        cert = _certificate(cand, reg)
        better = (not st["has"]) or (math.isfinite(cert) and not math.isfinite(st["best_cert"])) \
            or cert < st["best_cert"]
        if better:
            st["best_cert"], st["best"] = cert, cand
        st["has"] = True
        st["result"] = cand

    def evaluate(train):
        record(ws.evaluate(tol, st["evals"], st["aux"]), train)

    def finish(final, status=None, reason=None):
        final = dict(final)
        if status is not None:
            final["status"], final["stop_reason"] = status, reason
        final["iterations"] = ws.depth
        final["trace"] = list(trace)
        stats.total_seconds = time.perf_counter() - t_start
        final["statistics"] = stats.copy()
        out = pack(final, op.cols)
        out["decisions"] = np.array(decisions, dtype=np.int32)
        out["replay_overrun"] = overrun
        return out

    def finish_at_limit(status, reason):
        return finish(st["result"] if reg > 0.0 else st["best"], status, reason)

    ws.initialize(np.zeros((op.rows, 0), order="F"))
    if ws.can_advance() and max_depth > 0:
        ws.advance_level()
    evaluate(True)
    res = st["result"]
    if candidate_validation_failed_numerically(res) or res["status"] == 0:
        return finish(res)
    truncated = step_has_numerical_rank_truncation(ws.audit)
    broke = step_has_nonfinite_breakdown(ws.audit)
    hist = ProgressHistory()
    plan = HorizonPlan()
    epoch = 0
    generated = 0
    bhat = None
    bhat_ready = False
    feedback = False
    fb_target = stage_rank = stage_origin = stage_target = 0

    def gaussian_block(cols, first):
        nonlocal bhat, bhat_ready
        rnd = gaussian_matrix(op.rows, cols, seed, stream, first)
        if not bhat_ready:
            nb = _nrm2(b)
            if nb != 0.0:
                bhat = b / nb
            bhat_ready = True
        if bhat is None:
            return rnd
        for c in range(cols):
            coef = _dot(bhat, rnd[:, c])
            rnd[:, c] -= coef * bhat
        return rnd

    while True:
        if broke:
            return finish_at_limit(4, 7)
        if ws.k >= ws.basis_limit:
            return finish_at_limit(2, 5)
        if ws.depth >= max_depth:
            return finish_at_limit(1, 3)
        if truncated:
            return finish_at_limit(3, 6)
        interval_cert = _certificate(st["result"], reg)
        frontier = ws.active_left_width()
        avail_inc = max(0, max(0, ws.basis_limit - ws.k) - frontier)
        width_cap = min(avail_inc, max(0, max_aux - st["aux"]))
        full_fb = max_depth - ws.depth >= 2
        fb_depth = ws.depth + 2 if full_fb else ws.depth
        fb_inc = feedback_feasible_increment(ws.k, ws.basis_limit, frontier,
                                             fb_depth - ws.depth) if full_fb else 0
        feasible_cap = min(width_cap, fb_inc)
        if plan.end >= 0 and remaining_horizon(plan, ws.k) == 0:
            plan.__init__()
        rem = remaining_horizon(plan, ws.k)
        horizon_active = rem > 0
        collecting = horizon_active and not feedback and plan.count < 2
        ready = not feedback and not collecting
        stage_ok = ready and epoch < max_epochs
        inc = next_dyadic_increment(frontier, st["aux"], max_aux, feasible_cap) if stage_ok else 0
        requested = 0
        req_horizon = 0
        if stage_ok and inc > 0:
            tw = frontier + inc
            if horizon_active:
                d = horizon_candidate(inc, rem, ws.depth, max_depth, ws.k, ws.basis_limit,
                                      frontier, plan.op_s, plan.local_s, plan.count,
                                      op.relative_block_product_cost(frontier),
                                      op.relative_block_product_cost(tw), plan.origin > 1)
            else:
                d = initial_candidate(inc, interval_cert, tol, ws.depth, max_depth, ws.k,
                                      ws.basis_limit, frontier, hist,
                                      op.relative_block_product_cost(frontier),
                                      op.relative_block_product_cost(tw))
            if replay is not None:
                if len(decisions) < len(replay):
                    d.candidate = bool(replay[len(decisions)])
                else:
                    overrun += 1
            decisions.append(1 if d.candidate else 0)
            if d.candidate:
                requested = inc
                if not horizon_active:
                    req_horizon = d.matched_horizon
        if horizon_active and ready and requested == 0:
            plan.__init__()
        if requested > 0:
            fb_target = fb_depth
            stage_rank = ws.k
            stage_origin = plan.origin if horizon_active else frontier
            stage_target = frontier + requested
            hist.__init__()
            sched = CheckpointSchedule(reg, tol)
            rnd = gaussian_block(requested, generated)
            stats.gaussian_random_block_requests += 1
            stats.gaussian_random_columns += requested
            stats.gaussian_random_values += op.rows * requested
            generated += requested
            st["aux"] += requested
            epoch += 1
            ws.append_left_seed(rnd)
            advanced = ws.advance_level() if ws.can_advance() else False
            if advanced:
                if req_horizon > 0:
                    start_plan(plan, stage_rank, ws.basis_limit, req_horizon, stage_origin,
                               stage_target, interval_cert)
                else:
                    reset_plan_costs(plan, stage_target)
                truncated = step_has_numerical_rank_truncation(ws.audit)
                broke = step_has_nonfinite_breakdown(ws.audit)
                exhausted = remaining_horizon(plan, ws.k) == 0
                terminal = ws.k >= ws.basis_limit or ws.depth >= max_depth or not ws.can_advance()
                if terminal or exhausted:
                    evaluate(False)
                    res = st["result"]
                    if candidate_validation_failed_numerically(res) or res["status"] == 0:
                        return finish(res)
                reliable = not truncated and not broke and ws.k > stage_rank and \
                    ws.active_left_width() == stage_target
                extended = exhausted and horizon_stalled(plan, _certificate(st["result"], reg)) \
                    and extend_to_limit(plan, ws.k, ws.basis_limit)
                if not reliable or (exhausted and not extended):
                    plan.__init__()
                    feedback = False
                else:
                    feedback = True
            else:
                truncated = step_has_numerical_rank_truncation(ws.audit)
                broke = step_has_nonfinite_breakdown(ws.audit)
                feedback = False
                plan.__init__()
            continue

        if ws.can_advance():
            d0, k0 = ws.depth, ws.k
            matched = (not feedback) and remaining_horizon(plan, k0) > 0 and plan.count < 2
            if feedback:
                target = fb_target
            elif matched:
                target = min(d0 + 1, max_depth)
            else:
                target = d0 + 1
                while target < max_depth and not sched.should_evaluate(target):
                    target += 1
            t0 = time.perf_counter()
            a0, at0 = stats.a_seconds, stats.at_seconds
            while ws.can_advance() and ws.depth < target:
                ok = ws.advance_level()
                truncated = step_has_numerical_rank_truncation(ws.audit)
                broke = step_has_nonfinite_breakdown(ws.audit)
                if not ok or truncated or broke:
                    break
            span = time.perf_counter() - t0
            op_s = max(0.0, stats.a_seconds - a0 + stats.at_seconds - at0)
            local_s = max(0.0, span - op_s)
            if ws.depth > d0:
                pair_done = matched and plan.count == 1
                exhausts = (feedback or matched) and remaining_horizon(plan, ws.k) == 0
                terminal = ws.k >= ws.basis_limit or ws.depth >= max_depth or not ws.can_advance()
                if (not feedback and not matched) or pair_done or exhausts or terminal:
                    evaluate(not feedback and not matched)
                    res = st["result"]
                    if candidate_validation_failed_numerically(res) or res["status"] == 0:
                        return finish(res)
                if feedback and ws.depth >= fb_target:
                    feedback = False
                    ok_fb = not truncated and not broke and ws.k > k0 and ws.k > stage_rank and \
                        frontier == stage_target and ws.active_left_width() == stage_target
                    rec = ok_fb and record_plan_cost(plan, frontier, ws.active_left_width(),
                                                     ws.depth - d0, op_s, local_s)
                    exh = remaining_horizon(plan, ws.k) == 0
                    ext = exh and horizon_stalled(plan, _certificate(st["result"], reg)) and \
                        extend_to_limit(plan, ws.k, ws.basis_limit)
                    if not rec or (exh and not ext):
                        plan.__init__()
                elif matched:
                    ok_c = not truncated and not broke and ws.k > k0 and \
                        frontier == ws.active_left_width()
                    rec = ok_c and record_plan_cost(plan, frontier, ws.active_left_width(),
                                                    ws.depth - d0, op_s, local_s)
                    exh = remaining_horizon(plan, ws.k) == 0
                    ext = exh and horizon_stalled(plan, _certificate(st["result"], reg)) and \
                        extend_to_limit(plan, ws.k, ws.basis_limit)
                    if not rec or (exh and not ext):
                        plan.__init__()
                elif not feedback:
                    record_deepen_progress(hist, interval_cert, _certificate(st["result"], reg),
                                           frontier, ws.active_left_width(), ws.depth - d0,
                                           op_s, local_s)
                continue
            if feedback or matched:
                feedback = False
                plan.__init__()
            continue
        reason = 2
        if not feedback and epoch >= max_epochs and st["aux"] < max_aux and avail_inc > 0:
            reason = 4
        return finish_at_limit(1, reason)


def solve_fixed_rbgk(problem, regularization=0.0, tolerance=1e-8, failure_probability=1e-6,
                     auxiliary_width=4, maximum_depth=32, maximum_basis_size=0, seed=0,
                     stream=0, stop_early=True):
    """fixed_rbgk.cpp:18-209."""
    op = Operator(problem)
    b = np.ascontiguousarray(problem.b, dtype=np.float64)
    reg, tol = regularization, tolerance
    validate_common_inputs(op, b, reg, tol)
    if not math.isfinite(failure_probability) or not (0.0 < failure_probability < 1.0):
        raise ValueError("failure_probability must lie strictly between zero and one")
    if auxiliary_width < 0:
        raise ValueError("auxiliary_width must be nonnegative")
    if maximum_depth <= 0:
        raise ValueError("maximum_depth must be positive")
    if maximum_basis_size < 0:
        raise ValueError("maximum_basis_size must be nonnegative")
    t_start = time.perf_counter()
    stats = Statistics()
    ws = Workspace(op, b, reg, maximum_basis_size, stats)
    aux = 0 if ws.bnorm == 0.0 else min(auxiliary_width, max(0, ws.basis_limit - 1))
    trace = []
    sched = CheckpointSchedule(reg, tol)
    st = dict(result=None, depth=0, evaluated=-1)

    def evaluate():
        r = ws.evaluate(tol, 0, aux)
        sched.record(st["depth"], r)
        st["evaluated"] = st["depth"]
        trace.append(r["trace"][0])
        st["result"] = r

    def terminal_eval():
        if st["evaluated"] != st["depth"]:
            evaluate()
        return candidate_validation_failed_numerically(st["result"])

    seed_block = np.zeros((op.rows, aux), order="F")
    if aux > 0:
        seed_block = gaussian_matrix(op.rows, aux, seed, stream, 0)
        stats.gaussian_random_block_requests += 1
        stats.gaussian_random_columns += aux
        stats.gaussian_random_values += op.rows * aux
    ws.initialize(seed_block)
    if ws.can_advance():
        ws.advance_level()
    st["depth"] = ws.depth
    evaluate()
    truncated = step_has_numerical_rank_truncation(ws.audit)
    broke = step_has_nonfinite_breakdown(ws.audit)

    def set_status(status, reason):
        r = dict(st["result"])
        if r["status"] != 0:
            r["status"], r["stop_reason"] = status, reason
        st["result"] = r

    while True:
        r = st["result"]
        if candidate_validation_failed_numerically(r):
            break
        if r["status"] == 0 and stop_early:
            break
        if broke:
            if terminal_eval():
                break
            st["result"] = dict(st["result"], status=4, stop_reason=7)
            break
        if ws.k >= ws.basis_limit:
            if not terminal_eval():
                set_status(2, 5)
            break
        if st["depth"] >= maximum_depth:
            if not terminal_eval():
                set_status(1, 3)
            break
        if truncated:
            if not terminal_eval():
                set_status(3, 6)
            break
        if not ws.can_advance():
            if not terminal_eval():
                set_status(1, 2)
            break
        ok = ws.advance_level()
        truncated = step_has_numerical_rank_truncation(ws.audit)
        broke = step_has_nonfinite_breakdown(ws.audit)
        if not ok:
            if not ws.audit["right_rank_loss"] and not broke:
                raise RuntimeError("failed fixed extension did not report rank loss")
            continue
        st["depth"] = ws.depth
        term = st["depth"] >= maximum_depth or ws.k >= ws.basis_limit or not ws.can_advance() \
            or truncated or broke
        if sched.should_evaluate(st["depth"]) or term:
            evaluate()
    final = dict(st["result"])
    final["iterations"] = st["depth"]
    final["depth"] = st["depth"]
    final["trace"] = trace
    stats.total_seconds = time.perf_counter() - t_start
    final["statistics"] = stats.copy()
    return pack(final, op.cols)


def pack(r, cols):
    """Result in the torch binding's tensor layout (result_tensors.hpp:12-156)."""
    s = r["statistics"]
    metrics = np.array([r[k] for k in _VALIDATION_DOUBLES], dtype=np.float64)
    counters = np.array(
        [s.a_columns, s.at_columns, s.a_block_calls, s.at_block_calls, s.search_a_columns,
         s.search_at_columns, s.validation_a_columns, s.validation_at_columns,
         r.get("iterations", 0), r.get("depth", 0), r.get("auxiliary_width", 0),
         r.get("basis_rank", 0), s.sketch_a_columns, s.sketch_at_columns,
         s.sketch_a_block_calls, s.sketch_at_block_calls, s.iterative_a_columns,
         s.iterative_at_columns, s.iterative_a_block_calls, s.iterative_at_block_calls,
         s.gaussian_random_columns, s.gaussian_random_values, s.search_a_block_calls,
         s.search_at_block_calls, s.validation_a_block_calls, s.validation_at_block_calls,
         s.base_validation_a_columns, s.base_validation_at_columns,
         s.base_validation_a_block_calls, s.base_validation_at_block_calls,
         s.ridge_correction_a_columns, s.ridge_correction_at_columns,
         s.ridge_correction_a_block_calls, s.ridge_correction_at_block_calls,
         s.gaussian_random_block_requests, r["ridge_correction_disposition"]], dtype=np.int64)
    other = max(0.0, s.total_seconds - s.a_seconds - s.at_seconds -
                s.orthogonalization_seconds - s.projected_solve_seconds)
    timings = np.array([s.total_seconds, s.a_seconds, s.at_seconds,
                        s.orthogonalization_seconds, s.projected_solve_seconds,
                        s.validation_seconds, other, s.base_validation_seconds,
                        s.ridge_correction_validation_seconds])
    tf = np.array([t["floats"] for t in r["trace"]], dtype=np.float64).reshape(-1, 29)
    ti = np.array([t["ints"] for t in r["trace"]], dtype=np.int64).reshape(-1, 4)
    x = np.asarray(r["solution"], dtype=np.float64)
    if x.shape[0] != cols:
        raise RuntimeError("oracle solution has the wrong size")
    return dict(solution=x, metrics=metrics, counters=counters, timings=timings,
                trace_float=tf, trace_int=ti, status=int(r["status"]),
                stop_reason=int(r["stop_reason"]))

"""Test infrastructure: CPU restatement of the reference's scalar LSQR and LSMR.

The checker for the GPU's ``amfls_gpu_solve_lsqr`` / ``amfls_gpu_solve_lsmr``;
only tests and bench's CPU legs use it, never the product.  It follows
src/algorithms/lsqr/lsqr.cpp:84-281 and src/algorithms/lsmr/lsmr.cpp:112-351
step by step in the reference's own arithmetic: dnrm2 norms, separate
multiply and subtract in every vector update (the reference is built
without FMA contraction), libm hypot for the rotations, the reference's CSR
and BLAS products through ``amfls_oracle.Operator``, and the certified
validation and checkpoint schedule of ``amfls_oracle`` at every checkpoint.
Pinned against fixtures produced by the reference itself
(tests/golden/baseline_*.npz, written by tests/golden/make_golden.py).
"""
from __future__ import annotations

import math
import time

import numpy as np

from oracle.amfls_oracle import (CheckpointSchedule, Operator, Statistics, _nrm2, _trace_record,
                                 candidate_validation_failed_numerically, pack,
                                 validate_candidate, validate_common_inputs)


def _finite(v):
    return bool(np.all(np.isfinite(v)))


class _Search:
    """apply_search / apply_transpose_search (lsqr.cpp:20-50): one column per
    call, counted as search work."""

    def __init__(self, op, stats):
        self.op, self.stats = op, stats

    def apply(self, v):
        t0 = time.perf_counter()
        out = np.ravel(self.op.apply(v), order="F").copy()
        s = self.stats
        s.a_seconds += time.perf_counter() - t0
        s.a_columns += 1
        s.a_block_calls += 1
        s.search_a_columns += 1
        s.search_a_block_calls += 1
        return out

    def apply_transpose(self, u):
        t0 = time.perf_counter()
        out = np.ravel(self.op.apply_transpose(u), order="F").copy()
        s = self.stats
        s.at_seconds += time.perf_counter() - t0
        s.at_columns += 1
        s.at_block_calls += 1
        s.search_at_columns += 1
        s.search_at_block_calls += 1
        return out


def _validate_iterate(op, b, x, reg, tol, iteration, stats):
    """validate_iterate (lsqr.cpp:59-78): the certified validation of x with
    iterations = depth = basis rank = iteration, epoch 0, width 0."""
    r = validate_candidate(op, b, x, reg, tol, stats)
    r["iterations"] = r["depth"] = r["basis_rank"] = iteration
    r["auxiliary_width"] = 0
    return r


def _finish(r, trace, stats, t_start, cols):
    r = dict(r)
    r["trace"] = trace
    stats.total_seconds = time.perf_counter() - t_start
    r["statistics"] = stats.copy()
    return pack(r, cols)


def _check_iterations(maximum_iterations):
    if maximum_iterations < 0:
        raise ValueError("maximum_iterations must be nonnegative")


def solve_lsqr(problem, regularization=0.0, tolerance=1e-8, maximum_iterations=0):
    """solve_lsqr (lsqr.cpp:84-281).  Returns the torch binding's layout."""
    op = Operator(problem)
    b = np.ascontiguousarray(problem.b, dtype=np.float64)
    return solve_lsqr_operator(op, b, regularization, tolerance, maximum_iterations)


def solve_lsqr_operator(op, b, regularization=0.0, tolerance=1e-8, maximum_iterations=0):
    reg, tol = regularization, tolerance
    validate_common_inputs(op, b, reg, tol)
    _check_iterations(maximum_iterations)
    max_it = maximum_iterations if maximum_iterations > 0 else min(op.rows, op.cols)
    t_start = time.perf_counter()
    stats = Statistics()
    search = _Search(op, stats)

    u = b.copy()
    beta = _nrm2(u)
    x = np.zeros(op.cols)
    if beta > 0.0:
        u = u * (1.0 / beta)
    v = search.apply_transpose(u)
    alpha = _nrm2(v)
    if alpha > 0.0:
        v = v * (1.0 / alpha)
    w = v.copy()
    rhobar, phibar = alpha, beta
    damp = math.sqrt(reg)
    trace = []
    sched = CheckpointSchedule(reg, tol)
    result = None

    def evaluate(iteration):
        nonlocal result
        result = _validate_iterate(op, b, x, reg, tol, iteration, stats)
        sched.record(iteration, result)
        trace.append(_trace_record(result, 0))

    if not math.isfinite(beta) or not math.isfinite(alpha) or alpha == 0.0:
        evaluate(0)
        if candidate_validation_failed_numerically(result) or result["status"] == 0 or \
                alpha == 0.0:
            return _finish(result, trace, stats, t_start, op.cols)

    for it in range(1, max_it + 1):
        av = search.apply(v)
        av = av - alpha * u
        beta = _nrm2(av)
        if beta > 0.0:
            av = av * (1.0 / beta)
        rhobar1 = float(np.hypot(rhobar, damp))
        cs1 = 1.0 if rhobar1 == 0.0 else rhobar / rhobar1
        phibar *= cs1
        rho = float(np.hypot(rhobar1, beta))
        cs = 1.0 if rho == 0.0 else rhobar1 / rho
        sn = 0.0 if rho == 0.0 else beta / rho
        phi = cs * phibar
        phibar = sn * phibar
        finite = all(math.isfinite(t) for t in (beta, rhobar1, cs1, rho, cs, sn, phi, phibar))
        if rho != 0.0:
            update = phi / rho
            finite = finite and math.isfinite(update)
            x = x + update * w
        finite = finite and _finite(x)
        u = av

        breakdown = beta == 0.0
        checkpoint = sched.should_evaluate(it) or breakdown or not finite or it == max_it
        evaluated = False
        if checkpoint:
            evaluate(it)
            evaluated = True
            if candidate_validation_failed_numerically(result) or result["status"] == 0:
                break
            if not finite:
                result = dict(result, status=4, stop_reason=7)
                break
            if breakdown:
                result = dict(result, status=1, stop_reason=2)
                break
            if it == max_it:
                result = dict(result, status=1, stop_reason=3)
                break

        atu = search.apply_transpose(u)
        atu = atu - beta * v
        next_alpha = _nrm2(atu)
        cont = math.isfinite(next_alpha) and _finite(atu)
        if next_alpha > 0.0 and math.isfinite(next_alpha):
            atu = atu * (1.0 / next_alpha)
        theta = sn * next_alpha
        next_rhobar = -cs * next_alpha
        recurrence = theta / rho
        cont = cont and math.isfinite(theta) and math.isfinite(next_rhobar) and \
            math.isfinite(recurrence)
        if cont and next_alpha > 0.0:
            w = atu - recurrence * w
            cont = _finite(w)
        if not cont or next_alpha == 0.0:
            if not evaluated:
                evaluate(it)
                if candidate_validation_failed_numerically(result) or result["status"] == 0:
                    break
            result = dict(result, status=1 if cont else 4, stop_reason=2 if cont else 7)
            break
        alpha, rhobar = next_alpha, next_rhobar
        v = atu
    return _finish(result, trace, stats, t_start, op.cols)


def _givens(first, second):
    """symmetric_givens (lsmr.cpp:17-27): (cosine, sine, radius)."""
    radius = float(np.hypot(first, second))
    if radius == 0.0:
        return 1.0, 0.0, 0.0
    return first / radius, second / radius, radius


def solve_lsmr(problem, regularization=0.0, tolerance=1e-8, maximum_iterations=0):
    """solve_lsmr (lsmr.cpp:112-351), Fong and Saunders (2011) section 5.2 with
    damp^2 = regularization.  Returns the torch binding's layout."""
    op = Operator(problem)
    b = np.ascontiguousarray(problem.b, dtype=np.float64)
    return solve_lsmr_operator(op, b, regularization, tolerance, maximum_iterations)


def solve_lsmr_operator(op, b, regularization=0.0, tolerance=1e-8, maximum_iterations=0):
    reg, tol = regularization, tolerance
    validate_common_inputs(op, b, reg, tol)
    _check_iterations(maximum_iterations)
    max_it = maximum_iterations if maximum_iterations > 0 else min(op.rows, op.cols)
    t_start = time.perf_counter()
    stats = Statistics()
    search = _Search(op, stats)

    u = b.copy()
    beta = _nrm2(u)
    if beta > 0.0 and math.isfinite(beta):
        u = u * (1.0 / beta)
    v = search.apply_transpose(u)
    alpha = _nrm2(v)
    if alpha > 0.0 and math.isfinite(alpha):
        v = v * (1.0 / alpha)
    x = np.zeros(op.cols)
    h = v.copy()
    hbar = np.zeros(op.cols)
    alphabar, zetabar = alpha, alpha * beta
    rho = rhobar = cbar = 1.0
    sbar = 0.0
    damp = math.sqrt(reg)
    trace = []
    sched = CheckpointSchedule(reg, tol)
    result = None

    initial_breakdown = not math.isfinite(beta) or not math.isfinite(alpha)
    if initial_breakdown or alpha == 0.0:
        result = _validate_iterate(op, b, x, reg, tol, 0, stats)
        sched.record(0, result)
        trace.append(_trace_record(result, 0))
        initial_breakdown = initial_breakdown or candidate_validation_failed_numerically(result)
        if initial_breakdown:
            result = dict(result, status=4, stop_reason=7)
        elif alpha == 0.0 and result["status"] != 0:
            result = dict(result, status=1, stop_reason=2)
        if result["status"] == 0 or initial_breakdown or alpha == 0.0:
            return _finish(result, trace, stats, t_start, op.cols)

    for it in range(1, max_it + 1):
        av = search.apply(v)
        valid = _finite(av)
        av = av - alpha * u
        beta = _nrm2(av)
        valid = valid and math.isfinite(beta)
        if beta > 0.0 and math.isfinite(beta):
            av = av * (1.0 / beta)
        if beta == 0.0:
            atu = np.zeros(op.cols)
            alpha = 0.0
        else:
            atu = search.apply_transpose(av)
            atu = atu - beta * v
            alpha = _nrm2(atu)
            valid = valid and math.isfinite(alpha)
            if alpha > 0.0 and math.isfinite(alpha):
                atu = atu * (1.0 / alpha)

        c_damp, s_damp, r_damp = _givens(alphabar, damp)
        rho_old = rho
        c_bi, s_bi, rho = _givens(r_damp, beta)
        theta_new = s_bi * alpha
        alphabar = c_bi * alpha
        rhobar_old = rhobar
        theta_bar = sbar * rho
        rho_temp = cbar * rho
        cbar, sbar, rhobar = _givens(rho_temp, theta_new)
        zeta = cbar * zetabar
        zetabar = -sbar * zetabar
        hbar_den = rho_old * rhobar_old
        sol_den = rho * rhobar
        valid = valid and all(math.isfinite(t) for t in (
            c_damp, s_damp, r_damp, c_bi, s_bi, rho, theta_new, alphabar, theta_bar, rho_temp,
            cbar, sbar, rhobar, zeta, zetabar, hbar_den, sol_den)) and \
            hbar_den != 0.0 and sol_den != 0.0 and rho != 0.0
        if valid:
            hbar_rec = theta_bar * rho / hbar_den
            sol_update = zeta / sol_den
            h_rec = theta_new / rho
            valid = math.isfinite(hbar_rec) and math.isfinite(sol_update) and \
                math.isfinite(h_rec)
            next_hbar = h - hbar_rec * hbar
            next_x = x + sol_update * next_hbar
            next_h = atu - h_rec * h
            valid = valid and _finite(next_hbar) and _finite(next_x) and _finite(next_h)
            if valid:
                hbar, x, h = next_hbar, next_x, next_h
        u, v = av, atu

        exact_breakdown = alpha == 0.0 or beta == 0.0
        if not (sched.should_evaluate(it) or not valid or exact_breakdown or it == max_it):
            continue
        result = _validate_iterate(op, b, x, reg, tol, it, stats)
        sched.record(it, result)
        trace.append(_trace_record(result, 0))
        if candidate_validation_failed_numerically(result):
            break
        if not valid:
            result = dict(result, status=4, stop_reason=7)
            break
        if result["status"] == 0:
            break
        if exact_breakdown:
            result = dict(result, status=1, stop_reason=2)
            break
        if it == max_it:
            result = dict(result, status=1, stop_reason=3)
    return _finish(result, trace, stats, t_start, op.cols)

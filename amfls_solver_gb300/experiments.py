"""Dense experiment runner on the GPU solver (the reference's comparative
study, experiments/runners/run_comparative_study.py, restated for AMFLS).

The reference re-runs its dense test families from a JSON suite
(experiments/configs/large_dense_*.json): each case names a shape, a rank,
a singular-value spectrum, a coherence and a right-hand-side kind; each
instance seed regenerates one problem with a known reference solution.
This module restates the problem generator (make_problem, :283-383, with
orthonormal_columns :193-212 and singular_values :215-280) and the
external diagnostics (diagnostics, :577-654), drives the GPU run_amfls with
the study's options (run_method, :553-565; the algorithm seed of
method_seed, :1093-1108) and returns rows with the reference CSV's field
names, so the dense instances can be re-run on a GB300 as a regression
suite against the reference's recorded rows.

    python -m amfls_solver_gb300.experiments SUITE.json [--cases a,b]
           [--seeds 101,102] [--out rows.csv]

Problems are built with torch on the CPU from a seeded torch.Generator, as
in the reference, then moved to the GPU; the solve itself runs only on the
GPU (run_amfls on a CUDA tensor).
"""
from __future__ import annotations

import argparse
import csv
import json
import math
import sys
import time

import torch

ROW_FIELDS = [
    "suite", "case", "instance_seed", "algorithm_seed", "method", "m", "n", "rank",
    "coherence", "spectrum", "rhs", "regularization", "regularization_ratio", "tolerance",
    "success", "external_success", "status", "stop_reason", "objective",
    "reference_objective", "relative_objective_gap", "residual_norm", "normal_residual_norm",
    "compatible_backward_error_external", "least_squares_backward_error_external",
    "backward_error_external", "relative_energy_error_external", "reported_accuracy_upper",
    "relative_solution_error", "relative_null_component", "a_columns", "at_columns",
    "a_block_calls", "at_block_calls", "search_vector_work", "validation_vector_work",
    "gaussian_random_columns", "gaussian_random_block_requests", "iterations", "depth",
    "auxiliary_width", "basis_rank", "kernel_seconds", "wall_seconds"]


def orthonormal_columns(rows: int, columns: int, generator: torch.Generator,
                        coherence: str) -> torch.Tensor:
    """run_comparative_study.py:193-212: coordinate columns (coherent) or a
    sign-fixed QR of a Gaussian block (haar)."""
    if coherence == "coherent":
        q = torch.zeros((rows, columns), dtype=torch.float64)
        idx = torch.arange(columns)
        q[idx, idx] = 1.0
        return q
    if coherence != "haar":
        raise ValueError(f"unknown coherence: {coherence}")
    g = torch.randn((rows, columns), generator=generator, dtype=torch.float64)
    q, r = torch.linalg.qr(g, mode="reduced")
    s = torch.sign(torch.diagonal(r))
    s[s == 0.0] = 1.0
    return q * s


def singular_values(case: dict, rank: int) -> torch.Tensor:
    """run_comparative_study.py:215-280: the case's spectrum."""
    kind = str(case["spectrum"])
    i = torch.arange(rank, dtype=torch.float64)
    if kind == "flat":
        return torch.ones(rank, dtype=torch.float64)
    if kind in ("outliers", "separated_outliers"):
        count = min(int(case.get("outlier_count", 1)), rank)
        top = float(case.get("outlier_ratio", 1.0e4))
        vals = torch.linspace(1.0, float(case.get("tail_minimum", 0.2)), rank,
                              dtype=torch.float64)
        if kind == "outliers" or count == 1:
            vals[:count] = top
        else:
            vals[:count] = torch.logspace(math.log10(top),
                                          math.log10(float(case.get("smallest_outlier_ratio",
                                                                    10.0))),
                                          count, dtype=torch.float64)
        return vals
    if kind == "clusters":
        vals = torch.full((rank,), 0.1, dtype=torch.float64)
        first = min(rank, max(1, rank // 16))
        second = min(rank, max(first + 1, rank // 2))
        vals[:first] = 100.0
        vals[first:second] = 1.0
        return vals
    if kind == "polynomial":
        return (i + 1.0).pow(-float(case.get("alpha", 1.0)))
    if kind in ("exponential", "numerical"):
        end = float(case.get("endpoint", 1.0e-8)) if kind == "exponential" else \
            float(case["endpoint"])
        if rank == 1:
            return torch.ones(1, dtype=torch.float64)
        return torch.logspace(0.0, math.log10(end), rank, dtype=torch.float64)
    if kind == "smooth":
        if rank == 1:
            return torch.ones(1, dtype=torch.float64)
        return torch.exp(-4.0 * (i / float(rank - 1)).pow(1.5))
    if kind == "precision_two_mode":
        vals = torch.ones(rank, dtype=torch.float64)
        vals[-1] = float(case["two_mode_small_singular_value"])
        return vals
    raise ValueError(f"unknown spectrum: {kind}")


def make_problem(case: dict, seed: int) -> dict:
    """run_comparative_study.py:283-383: A = U diag(sigma) V^T (or its
    coordinate form), b from the case's right-hand-side kind, lambda =
    ratio * sigma_1^2, and the exact (shrunk) reference solution."""
    m, n, rank = int(case["m"]), int(case["n"]), int(case["rank"])
    if rank <= 0 or rank > min(m, n):
        raise ValueError(f"invalid rank {rank} for shape ({m},{n})")
    gen = torch.Generator(device="cpu").manual_seed(seed)
    coherence = str(case.get("coherence", "haar"))
    left = orthonormal_columns(m, rank, gen, coherence)
    right = orthonormal_columns(n, rank, gen, coherence)
    sigma = singular_values(case, rank)
    if coherence == "coherent":
        a = torch.zeros((m, n), dtype=torch.float64)
        idx = torch.arange(rank)
        a[idx, idx] = sigma
    else:
        a = ((left * sigma) @ right.T).contiguous()
    coef = torch.randn(rank, generator=gen, dtype=torch.float64)
    rhs = str(case["rhs"])
    ratio_reg = float(case.get("regularization_ratio", 0.0))
    exact_inconsistent = (coherence == "coherent" and rhs == "inconsistent"
                          and rank < min(m, n) and ratio_reg == 0.0)
    if exact_inconsistent:
        coef = torch.sign(coef)
        coef[coef == 0.0] = 1.0
    if rhs == "top_loaded":
        coef[max(1, rank // 8):] = 0.0
    elif rhs == "tail_loaded":
        coef[:max(0, rank - max(1, rank // 8))] = 0.0
    elif rhs == "outlier_orthogonal":
        coef[:min(int(case.get("outlier_count", 1)), rank)] = 0.0
    elif rhs == "energy_balanced":
        reg = ratio_reg * float(sigma[0]) ** 2
        coef = (sigma.square() + reg).rsqrt()
        signs = torch.sign(torch.randn(rank, generator=gen, dtype=torch.float64))
        signs[signs == 0.0] = 1.0
        coef *= signs
    elif rhs not in ("random", "consistent", "inconsistent"):
        raise ValueError(f"unknown right-hand side: {rhs}")
    signal = left @ (sigma * coef)
    b = signal.clone()
    if rhs == "inconsistent":
        if rank >= m:
            raise ValueError("an inconsistent case requires rank < m")
        if exact_inconsistent:
            noise = torch.zeros(m, dtype=torch.float64)
            noise[rank:] = torch.randn(m - rank, generator=gen, dtype=torch.float64)
        else:
            noise = torch.randn(m, generator=gen, dtype=torch.float64)
            noise -= left @ (left.T @ noise)
        nn = float(torch.linalg.vector_norm(noise))
        if nn == 0.0:
            raise RuntimeError("failed to construct an inconsistent component")
        b += float(case.get("noise_ratio", 0.05)) * float(torch.linalg.vector_norm(signal)) * \
            noise / nn
    reg = ratio_reg * float(sigma[0]) ** 2
    reference = right @ (sigma.square() / (sigma.square() + reg) * coef)
    bn = float(torch.linalg.vector_norm(b))
    if bn == 0.0:
        raise ValueError("right-hand side cannot be zero")
    if exact_inconsistent:
        _, e = math.frexp(bn)
        scale = math.ldexp(1.0, -e)
        b *= scale
        reference *= scale
    else:
        b /= bn
        reference /= bn
    res = a @ reference - b
    return {"matrix": a, "b": b.contiguous(), "reference": reference.contiguous(),
            "row_basis": right, "operator_norm": float(sigma[0]), "regularization": reg,
            "reference_objective": float(res @ res + reg * (reference @ reference))}


def _ratio(num: float, den: float) -> float:
    if num == 0.0:
        return 0.0
    return math.inf if den == 0.0 else num / den


def diagnostics(problem: dict, solution: torch.Tensor, tolerance: float) -> dict:
    """run_comparative_study.py:577-654: external backward error (lambda = 0)
    or relative energy error (lambda > 0) against the exact reference
    solution, the minimum-norm check and the objective gap, in float64 on the
    CPU."""
    a, b, ref = problem["matrix"], problem["b"], problem["reference"]
    reg, norm_a = float(problem["regularization"]), float(problem["operator_norm"])
    x = solution
    r = a @ x - b
    normal = a.T @ r + reg * x
    rn, nn = float(torch.linalg.vector_norm(r)), float(torch.linalg.vector_norm(normal))
    xn, bn = float(torch.linalg.vector_norm(x)), float(torch.linalg.vector_norm(b))
    aug_r = math.sqrt(rn * rn + reg * xn * xn)
    aug_n = math.sqrt(norm_a * norm_a + reg)
    compat = _ratio(aug_r, aug_n * xn + bn)
    lsq = _ratio(nn, aug_n * aug_r)
    backward = min(compat, lsq)
    err = x - ref
    en, refn = float(torch.linalg.vector_norm(err)), float(torch.linalg.vector_norm(ref))
    ea, ra = float(torch.linalg.vector_norm(a @ err)), float(torch.linalg.vector_norm(a @ ref))
    energy = _ratio(math.sqrt(ea * ea + reg * en * en), math.sqrt(ra * ra + reg * refn * refn))
    primary = energy if reg > 0.0 else backward
    slack = 256.0 * torch.finfo(torch.float64).eps + 1.0e-7 * tolerance
    objective = float(r @ r + reg * (x @ x))
    ref_obj = float(problem["reference_objective"])
    basis = problem["row_basis"]
    if reg > 0.0 or basis.shape[1] >= a.shape[1]:
        null_rel, min_norm_ok = 0.0, True
    else:
        null_rel = _ratio(float(torch.linalg.vector_norm(x - basis @ (basis.T @ x))), refn)
        min_norm_ok = null_rel <= tolerance + slack
    return {"external_success": int(primary <= tolerance + slack and min_norm_ok),
            "objective": objective,
            "relative_objective_gap": (objective - ref_obj) / max(ref_obj,
                                                                  torch.finfo(torch.float64).tiny),
            "residual_norm": rn, "normal_residual_norm": nn,
            "compatible_backward_error_external": compat,
            "least_squares_backward_error_external": lsq, "backward_error_external": backward,
            "relative_energy_error_external": energy,
            "relative_solution_error": _ratio(en, refn), "relative_null_component": null_rel}


def run_case(suite: dict, case: dict, instance_seed: int, device="cuda") -> dict:
    """One AMFLS row: the instance, the GPU solve with the suite's options
    (run_method's AMFLS branch), the diagnostics."""
    from .binding import run_amfls

    problem = make_problem(case, instance_seed)
    algorithm_seed = instance_seed + int(suite["algorithm_seed_offset"])
    tol = float(suite["tolerance"])
    a = problem["matrix"].to(device)
    b = problem["b"].to(device)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    r = run_amfls(a, b, regularization=float(problem["regularization"]), tolerance=tol,
                  failure_probability=float(suite["failure_probability"]),
                  maximum_epochs=int(suite["maximum_epochs"]),
                  maximum_depth=int(suite["maximum_depth"]),
                  maximum_auxiliary_width=int(suite["maximum_auxiliary_width"]),
                  maximum_basis_size=int(suite["maximum_basis_size"]), seed=algorithm_seed)
    torch.cuda.synchronize(device)
    wall = time.perf_counter() - t0
    values = diagnostics(problem, r.solution.cpu(), tol)
    reg = float(problem["regularization"])
    row = {"suite": suite["suite"], "case": case["name"], "instance_seed": instance_seed,
           "algorithm_seed": algorithm_seed, "method": "amfls", "m": case["m"], "n": case["n"],
           "rank": case["rank"], "coherence": case.get("coherence", "haar"),
           "spectrum": case["spectrum"], "rhs": case["rhs"], "regularization": reg,
           "regularization_ratio": float(case.get("regularization_ratio", 0.0)),
           "tolerance": tol, "success": int(r.success), "status": r.status,
           "stop_reason": r.stop_reason, "reference_objective": problem["reference_objective"],
           "reported_accuracy_upper": (r.relative_energy_error_upper_bound if reg > 0.0
                                       else r.backward_error_upper_bound),
           "a_columns": r.a_columns, "at_columns": r.at_columns,
           "a_block_calls": r.a_block_calls, "at_block_calls": r.at_block_calls,
           "search_vector_work": r.search_a_columns + r.search_at_columns,
           "validation_vector_work": r.validation_a_columns + r.validation_at_columns,
           "gaussian_random_columns": r.gaussian_random_columns,
           "gaussian_random_block_requests": r.gaussian_random_block_requests,
           "iterations": r.iterations, "depth": r.depth, "auxiliary_width": r.auxiliary_width,
           "basis_rank": r.basis_rank, "kernel_seconds": r.total_seconds, "wall_seconds": wall}
    row.update(values)
    return row


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("suite", help="a suite JSON in the reference's experiment-config format")
    ap.add_argument("--cases", default="", help="comma-separated case names (default: all)")
    ap.add_argument("--seeds", default="", help="comma-separated instance seeds (default: all)")
    ap.add_argument("--out", default="", help="CSV file for the rows (default: stdout)")
    args = ap.parse_args(argv)
    with open(args.suite) as f:
        suite = json.load(f)
    names = set(filter(None, args.cases.split(",")))
    seeds = [int(s) for s in args.seeds.split(",") if s] or list(suite["instance_seeds"])
    out = open(args.out, "w", newline="") if args.out else sys.stdout
    writer = csv.DictWriter(out, fieldnames=ROW_FIELDS, extrasaction="ignore")
    writer.writeheader()
    for case in suite["cases"]:
        if names and case["name"] not in names:
            continue
        for seed in seeds:
            writer.writerow(run_case(suite, case, seed))
            out.flush()
    if out is not sys.stdout:
        out.close()


if __name__ == "__main__":
    main()

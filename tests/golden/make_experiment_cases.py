"""Generate tests/golden/experiment_cases.json from the reference's own
experiment suite (run where the reference checkout exists).

    python tests/golden/make_experiment_cases.py

For the four dense suites of the reference's comparative study
(experiments/configs/large_dense_*.json) it keeps the suite options, every
case, and, for instance seeds 101 and 102, the reference's recorded AMFLS row
of experiments/results/formal_100_v2/<suite>.csv (status, stop reason,
certified and external success, depth, auxiliary width, basis rank, reported
accuracy).  It also pins the restated generator and diagnostics
(amfls_solver_gb300.experiments) against the reference's own functions
(run_comparative_study.py make_problem :283-383 and diagnostics :577-654),
run here: the SHA-256 of the reference's arrays for each instance, and the
reference's diagnostics of a fixed perturbation of the exact solution.
The AMFLS library is never loaded (only the runner's Python functions are
imported).
"""
from __future__ import annotations

import csv
import hashlib
import importlib.util
import json
import os
import sys
from pathlib import Path

import torch

REFERENCE = Path(os.environ.get("AMFLS_REFERENCE", "/root/reference"))
OUT = Path(__file__).resolve().parent / "experiment_cases.json"
SUITES = ["large_dense_spectral_coverage_v1", "large_dense_ordinary_v2",
          "large_dense_ridge_v1", "large_dense_geometry_rank_v1"]
SEEDS = [101, 102]
KEEP = ["success", "external_success", "status", "stop_reason", "depth", "auxiliary_width",
        "basis_rank", "reported_accuracy_upper", "kernel_seconds", "a_columns", "at_columns"]


def digest(problem):
    h = hashlib.sha256()
    for k in ("matrix", "b", "reference"):
        h.update(problem[k].contiguous().numpy().tobytes())
    return h.hexdigest()


class _Result:  # the two fields diagnostics() reads
    def __init__(self, solution):
        self.solution = solution


def main():
    sys.path.insert(0, str(REFERENCE / "python"))
    spec = importlib.util.spec_from_file_location(
        "reference_runner", REFERENCE / "experiments/runners/run_comparative_study.py")
    runner = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(runner)
    out = {"seeds": SEEDS, "suites": []}
    for name in SUITES:
        suite = json.loads((REFERENCE / f"experiments/configs/{name}.json").read_text())
        rows = {}
        with open(REFERENCE / f"experiments/results/formal_100_v2/{name}.csv") as f:
            for r in csv.DictReader(f):
                if r["method"] == "amfls" and int(r["instance_seed"]) in SEEDS:
                    rows[(r["case"], int(r["instance_seed"]))] = {k: r[k] for k in KEEP}
        entry = {k: suite[k] for k in ("suite", "tolerance", "failure_probability",
                                       "algorithm_seed_offset", "maximum_depth",
                                       "maximum_auxiliary_width", "maximum_epochs",
                                       "maximum_basis_size")}
        entry["cases"] = suite["cases"]
        entry["instances"] = []
        for case in suite["cases"]:
            for seed in SEEDS:
                p = runner.make_problem(case, seed)
                x = p["reference"] + 1e-9 * torch.ones_like(p["reference"])
                diag = runner.diagnostics(p, _Result(x), float(suite["tolerance"]))
                entry["instances"].append({
                    "case": case["name"], "seed": seed, "digest": digest(p),
                    "regularization": p["regularization"],
                    "diagnostics_of_perturbed_reference": {
                        k: float(v) for k, v in diag.items()},
                    "reference_row": rows[(case["name"], seed)]})
        out["suites"].append(entry)
        print(name, len(entry["instances"]), "instances")
    OUT.write_text(json.dumps(out, indent=1))
    print("wrote", OUT)


if __name__ == "__main__":
    main()

"""The restated experiment runner (amfls_solver_gb300.experiments) against the
reference's own runner functions, through tests/golden/experiment_cases.json
(made by tests/golden/make_experiment_cases.py from the reference's
run_comparative_study.py): the generated instances are the same bytes as the
reference's make_problem (:283-383) on this platform, and the external
diagnostics (:577-654) of a fixed perturbation of the exact solution agree.
No GPU is used."""
import hashlib
import json
import platform

import pytest
import torch

from conftest import GOLDEN
from amfls_solver_gb300 import experiments as ex

CASES = json.loads((GOLDEN / "experiment_cases.json").read_text())


def _instances():
    for suite in CASES["suites"]:
        cases = {c["name"]: c for c in suite["cases"]}
        for inst in suite["instances"]:
            yield suite, cases[inst["case"]], inst


@pytest.mark.parametrize("suite,case,inst", list(_instances()),
                         ids=lambda v: v["case"] + "-" + str(v["seed"]) if "seed" in v else "")
def test_generator_and_diagnostics_match_reference(suite, case, inst):
    p = ex.make_problem(case, inst["seed"])
    assert p["regularization"] == inst["regularization"]
    if platform.machine() in ("x86_64", "AMD64"):  # the fixture's platform
        h = hashlib.sha256()
        for k in ("matrix", "b", "reference"):
            h.update(p[k].contiguous().numpy().tobytes())
        assert h.hexdigest() == inst["digest"]
    x = p["reference"] + 1e-9 * torch.ones_like(p["reference"])
    got = ex.diagnostics(p, x, float(suite["tolerance"]))
    want = inst["diagnostics_of_perturbed_reference"]
    for k, v in want.items():
        assert got[k] == pytest.approx(v, rel=1e-9, abs=1e-300), k

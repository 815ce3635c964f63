"""CPU: the oracle's LSQR and LSMR restatements pinned against fixtures that
the reference itself produced (tests/golden/baseline_*.npz).

The restatement repeats the reference's arithmetic (dnrm2, unfused vector
updates, libm hypot, the reference's CSR order and BLAS calls), so the
iterates and the solution are bit-identical; the certified bounds in the
trace agree to rounding of the validation's extended-precision steps.
"""
import numpy as np
import pytest

from conftest import BASELINE_FIXTURES, golden_options, load_golden
from oracle import baselines


@pytest.mark.parametrize("name", BASELINE_FIXTURES)
def test_oracle_baseline_matches_reference(name):
    data, prob = load_golden(name)
    opts = golden_options(data)
    solve = baselines.solve_lsqr if opts.pop("algorithm") == "lsqr" else baselines.solve_lsmr
    r = solve(prob, **opts)
    assert (r["status"], r["stop_reason"]) == (int(data["status"]), int(data["stop_reason"]))
    np.testing.assert_array_equal(r["counters"], data["counters"])
    np.testing.assert_array_equal(r["trace_int"], data["trace_int"])
    np.testing.assert_array_equal(r["solution"], data["solution"])
    np.testing.assert_allclose(r["trace_float"][:, :8], data["trace_float"][:, :8], rtol=0)
    np.testing.assert_allclose(r["trace_float"], data["trace_float"], rtol=1e-11, atol=1e-300,
                               equal_nan=True)
    np.testing.assert_allclose(r["metrics"], data["metrics"], rtol=1e-11, atol=1e-300,
                               equal_nan=True)


def test_baseline_fixtures_cover_each_outcome():
    """Certified successes (both solvers), the iteration limit, an explicit
    iteration cap and the zero right-hand side are all represented."""
    outcomes = {}
    for name in BASELINE_FIXTURES:
        data, _ = load_golden(name)
        outcomes.setdefault(name.split("_")[1], set()).add(
            (int(data["status"]), int(data["stop_reason"])))
    for alg in ("lsqr", "lsmr"):
        assert {(0, 9), (0, 10), (1, 3), (0, 1)} <= outcomes[alg]


def test_baseline_rejects_negative_iteration_limit():
    data, prob = load_golden(BASELINE_FIXTURES[0])
    with pytest.raises(ValueError):
        baselines.solve_lsqr(prob, maximum_iterations=-1)
    with pytest.raises(ValueError):
        baselines.solve_lsmr(prob, maximum_iterations=-1)

"""The oracle (oracle/amfls_oracle.{c,py}) against the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference build; these
tests pin the CPU restatement before it is trusted as the GPU checker.  On
x86-64 (the machine that made the fixtures) the CSR paths agree bit for bit;
elsewhere long double and libm differ in the last bits, hence the small
relative tolerances.
"""
import numpy as np
import pytest

from conftest import CUSTOM_FIXTURES, GOLDEN, SOLVE_FIXTURES, golden_options, load_golden
from oracle import amfls_oracle as orc

ULP_TOL = 1e-14


def test_csr_products_match_reference():
    data, prob = load_golden("csr_products")
    op = orc.Operator(prob)
    np.testing.assert_array_equal(op.apply(data["x"][:, 0])[:, 0], data["ax1"])
    np.testing.assert_array_equal(op.apply_transpose(data["y"][:, 0])[:, 0], data["aty1"])
    np.testing.assert_array_equal(op.apply(data["x"]), data["ax3"])
    np.testing.assert_array_equal(op.apply_transpose(data["y"]), data["aty3"])


def test_csr_ragged_products_and_model():
    data, prob = load_golden("csr_ragged")
    op = orc.Operator(prob)
    np.testing.assert_array_equal(op.apply(data["x"])[:, 0], data["ax1"])
    np.testing.assert_array_equal(op.apply_transpose(data["y"])[:, 0], data["aty1"])
    up, lo, sa, st = op.model()
    np.testing.assert_allclose([up, lo], data["model"], rtol=ULP_TOL)
    assert [sa, st] == list(data["steps"])


@pytest.mark.parametrize("name", ["csr_products", "dense_model_rm", "dense_model_cm"])
def test_validation_model_matches_reference(name):
    data, prob = load_golden(name)
    up, lo, sa, st = orc.Operator(prob).model()
    np.testing.assert_allclose([up, lo], data["model"], rtol=ULP_TOL)
    assert [sa, st] == list(data["steps"])


def test_gaussian_stream_matches_reference():
    data = dict(np.load(GOLDEN / "gaussian.npz"))
    for i, (rows, cols, seed, stream, first) in enumerate(data["params"]):
        g = orc.gaussian_matrix(int(rows), int(cols), int(seed), int(stream), int(first))
        np.testing.assert_allclose(g, data[f"g{i}"], rtol=1e-15, atol=0)


def test_norm_interval_matches_reference():
    data = dict(np.load(GOLDEN / "norm_interval.npz"))
    for i, (lo, hi) in enumerate(data["bounds"]):
        got = orc.norm_interval(data[f"v{i}"])
        np.testing.assert_allclose(got, [lo, hi], rtol=ULP_TOL)
        v = data[f"v{i}"]
        if np.all(np.abs(v) < 1e150):
            exact = float(np.sqrt(np.sum(np.longdouble(v) ** 2)))
            assert got[0] <= exact <= got[1]


@pytest.mark.parametrize("name", SOLVE_FIXTURES)
def test_oracle_solve_matches_reference(name, gelsy_ranks):
    data, prob = load_golden(name)
    opts = golden_options(data)
    if opts.pop("algorithm", "amfls") == "fixed_rbgk":
        r = orc.solve_fixed_rbgk(prob, **opts)
    else:
        r = orc.solve_amfls(prob, **opts)
    assert r["status"] == int(data["status"])
    assert r["stop_reason"] == int(data["stop_reason"])
    if r["counters"][10] == data["counters"][10]:  # same width history
        np.testing.assert_array_equal(r["counters"], data["counters"])
        assert r["trace_int"].shape == data["trace_int"].shape
        np.testing.assert_array_equal(r["trace_int"], data["trace_int"])
    x, xr = r["solution"], data["solution"]
    scale = max(np.linalg.norm(xr), 1e-300)
    assert np.linalg.norm(x - xr) <= 1e-9 * scale
    # Certified bounds.  The oracle's CSR products repeat the reference's FMA
    # order exactly and its dense products make the reference's BLAS calls
    # (same OpenBLAS here), so the bounds agree to rounding.  On another BLAS
    # build the dense bounds near convergence would sit at a different
    # rounding floor.
    rel = 1e-6
    for idx in (8, 9, 10, 13):
        a, b = r["metrics"][idx], data["metrics"][idx]
        if np.isfinite(b):
            assert abs(a - b) <= rel * abs(b) + 1e-13, (idx, a, b)
        else:
            assert a == b
    # every projected solve had full column rank in dgelsy's sense, where the
    # GPU's QR recurrence gives the same solution
    assert all(rank == shape[1] for shape, rank in gelsy_ranks), gelsy_ranks


@pytest.mark.parametrize("name", CUSTOM_FIXTURES)
def test_oracle_custom_operator_solve_matches_reference(name):
    """A CSR matrix behind a custom MatrixOperator (the reference driver's
    forwarding operator: no extended-precision validation products,
    matrix_operator.hpp:62-88): the oracle's kind-3 operator reproduces the
    reference's counters, trace and solution."""
    data, prob = load_golden(name)
    r = orc.solve_amfls(prob, custom=True, **golden_options(data))
    assert (r["status"], r["stop_reason"]) == (int(data["status"]), int(data["stop_reason"]))
    np.testing.assert_array_equal(r["counters"], data["counters"])
    np.testing.assert_array_equal(r["trace_int"], data["trace_int"])
    xr = data["solution"]
    assert np.linalg.norm(r["solution"] - xr) <= 1e-9 * max(np.linalg.norm(xr), 1e-300)

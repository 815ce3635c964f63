"""GPU tests of matrix-free operators over user callbacks (the reference's
custom MatrixOperator, include/amfls/matrix_operator.hpp:29-89): a solve
through callbacks that multiply by a dense matrix must certify like the
built-in dense operator with the same validation model; without a model no
solve certifies success (matrix_operator.hpp:17-20); a failing callback is
an error, not a status."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def dense_problem():
    from amfls_solver_gb300 import problems

    return problems.scaled_dense(1500, 200, decades=3.0, seed=8, column_major=True)


def callbacks_for(a):
    def apply(x, y):
        y.copy_(a @ x)

    def apply_t(y, x):
        x.copy_(a.t() @ y)
    return apply, apply_t


def test_callback_operator_solves_like_the_dense_operator():
    import amfls_solver_gb300 as amfls

    prob = dense_problem()
    x_true = np.random.default_rng(3).standard_normal(prob.cols)
    bh = prob.matrix @ x_true + 1e-10 * np.random.default_rng(4).standard_normal(prob.rows)
    a = torch.from_numpy(np.ascontiguousarray(prob.matrix.T)).cuda().t()
    b = torch.from_numpy(bh).cuda()
    dense = amfls.DeviceOperator(a)
    apply, apply_t = callbacks_for(a)
    cb = amfls.DeviceOperator.from_callbacks(prob.rows, prob.cols, apply, apply_t,
                                             validation_model=dense.validation_error_model())
    assert cb.validation_error_model() == dense.validation_error_model()
    assert cb.relative_block_product_cost(4) == 4.0  # the interface default
    x = torch.randn(prob.cols, 3, dtype=torch.float64, device="cuda")
    torch.testing.assert_close(cb.apply(x), a @ x)
    tol = 1e-10
    ref = amfls.solve_amfls(dense, b, tolerance=tol)
    got = amfls.solve_amfls(cb, b, tolerance=tol)
    assert ref.status == 0 and ref.auxiliary_width == 0
    # the width controller sees device times, so a run over slower callback
    # products may widen and fill the 200-column basis first; at width one
    # it is the same process and must certify
    if got.auxiliary_width == 0:
        assert (got.status, got.depth) == (ref.status, ref.depth)
    if got.status != 0:
        assert got.status == 2 and got.auxiliary_width > 0
        return
    assert got.backward_error_upper_bound <= tol
    s = np.linalg.svd(prob.matrix, compute_uv=False)
    cond = s[0] / s[-1]
    xr, xg = ref.solution.cpu().numpy(), got.solution.cpu().numpy()
    assert np.linalg.norm(xg - xr) <= 4 * cond * tol * np.linalg.norm(xr)


def test_callback_operator_without_model_never_certifies():
    import amfls_solver_gb300 as amfls

    prob = dense_problem()
    a = torch.from_numpy(np.ascontiguousarray(prob.matrix.T)).cuda().t()
    apply, apply_t = callbacks_for(a)
    cb = amfls.DeviceOperator.from_callbacks(prob.rows, prob.cols, apply, apply_t)
    r = amfls.solve_amfls(cb, torch.from_numpy(prob.b).cuda(), regularization=1e-6,
                          tolerance=1e-2, maximum_depth=30)
    assert r.status != 0
    assert not np.isfinite(r.relative_energy_error_upper_bound)


def test_failing_callback_is_an_error():
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import _native

    def broken(x, y):
        raise RuntimeError("user product failed")

    cb = amfls.DeviceOperator.from_callbacks(40, 10, broken, broken,
                                             validation_model=(1.0, 0.5, 2, 2))
    with pytest.raises(_native.NativeError, match="custom operator"):
        amfls.solve_amfls(cb, torch.ones(40, dtype=torch.float64, device="cuda"))

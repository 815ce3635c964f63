"""GPU tests of the mixed-precision form (no counterpart in the reference).

Reduced operators: FP32- or BF16-rounded values, x rounded to FP32, FP32
accumulation.  Each product entry must lie within
    (u_v + (L + 3) 2^-24) (|A| |x|)_i,   u_v = 2^-24 (FP32) or 2^-8 (BF16),
of the FP64 product (L the longest row, or column, of the summed dimension),
with a factor 2 of slack.

Mixed solves: the certified FP64 validation on the original matrix decides
termination, so a success must also pass the host float64 checks that the
FP64 parity tests apply (backward error, or energy error against an exact
dense ridge solution, at most tol), and x must agree with the FP64 oracle's
solution to the accuracy the problem determines.
"""
import numpy as np
import pytest
import torch

from oracle import amfls_oracle as orc
from test_gpu_parity import check_solution, csr_tensor, skewed_csr

pytestmark = pytest.mark.gpu

U32 = 2.0 ** -24


@pytest.fixture(scope="module")
def amfls():
    import amfls_solver_gb300 as m

    m.load_library()
    return m


def reduced_bound(absa, x, L, values):
    uv = U32 if values == "fp32" else 2.0 ** -8
    return 2.0 * (uv + (L + 3) * U32) * (absa @ np.abs(x)) + 1e-300


@pytest.mark.parametrize("chains", ["0", "1"])
@pytest.mark.parametrize("values", ["fp32", "bf16"])
def test_reduced_csr_products(amfls, monkeypatch, values, chains):
    """Row blocks (chains="0") and chain groups (chains="1") of the shared
    single-column tables."""
    monkeypatch.setenv("AMFLS_GB300_CSR_CHAINS", chains)
    prob = skewed_csr(m=3000, n=3000)
    a = prob.to_dense()
    op = amfls.DeviceOperator(csr_tensor(prob))
    low = op.reduced(values)
    rng = np.random.default_rng(11)
    Lr = int(np.diff(prob.row_offsets).max())
    Lc = int(np.bincount(prob.column_indices, minlength=prob.cols).max())
    for s in (1, 3, 8):
        x = rng.standard_normal((prob.cols, s))
        y = rng.standard_normal((prob.rows, s))
        ax = low.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        aty = low.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()
        for c in range(s):
            assert np.all(np.abs(ax[:, c] - a @ x[:, c]) <= reduced_bound(np.abs(a), x[:, c], Lr, values))
            assert np.all(np.abs(aty[:, c] - a.T @ y[:, c]) <=
                          reduced_bound(np.abs(a.T), y[:, c], Lc, values))
    up, lo, sa, st = op.validation_error_model()
    rup, rlo, rsa, rst = low.validation_error_model()
    assert rup >= up and rlo <= lo
    assert (rsa, rst) == ((sa + 1) * 2 ** 29, (st + 1) * 2 ** 29)


@pytest.mark.parametrize("layout", ["row", "col"])
@pytest.mark.parametrize("values", ["fp32", "bf16"])
def test_reduced_dense_products(amfls, layout, values):
    rng = np.random.default_rng(5)
    m, n = 1003, 301  # contiguous extents that are not multiples of the vector width
    a = rng.standard_normal((m, n))
    t = torch.from_numpy(a).cuda() if layout == "row" else torch.from_numpy(a.T.copy()).cuda().t()
    op = amfls.DeviceOperator(t)
    low = op.reduced(values)
    for s in (1, 2, 5, 8, 11):
        x = rng.standard_normal((n, s))
        y = rng.standard_normal((m, s))
        ax = low.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        aty = low.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()
        for c in range(s):
            assert np.all(np.abs(ax[:, c] - a @ x[:, c]) <= reduced_bound(np.abs(a), x[:, c], n, values))
            assert np.all(np.abs(aty[:, c] - a.T @ y[:, c]) <=
                          reduced_bound(np.abs(a.T), y[:, c], m, values))


def _oracle_x(prob, reg, tol):
    r = orc.solve_amfls(prob, regularization=reg, tolerance=tol)
    return np.asarray(r["solution"])


# (noise, lambda, tol): a nearly consistent least-squares problem at 1e-10
# and a ridge problem at 1e-6, each above the level where residual
# correction with FP32 inner solves stops contracting (for the ridge problem
# the correction residual tends to [A x - b; sqrt(lambda) x], which is not
# small, and the inner solves stop relative to it).
@pytest.mark.parametrize("noise,reg,tol", [(1e-10, 0.0, 1e-10), (1e-6, 1e-4, 1e-6)])
def test_mixed_csr_solve_is_certified_in_fp64(amfls, noise, reg, tol):
    from amfls_solver_gb300 import problems

    prob = problems.scaled_uniform_csr(3000, 800, per_row=10, decades=3.0, noise=noise, seed=3)
    mat, b = csr_tensor(prob), torch.from_numpy(prob.b).cuda()
    r = amfls.run_amfls_mixed(mat, b, values="fp32", inner_tolerance=1e-6,
                              maximum_refinements=8, regularization=reg, tolerance=tol)
    assert r.status == 0
    cert = r.backward_error_upper_bound if reg == 0.0 else r.relative_energy_error_upper_bound
    assert cert <= tol
    check_solution(prob, r.solution.cpu().numpy(), _oracle_x(prob, reg, tol), reg, tol, True)


def test_mixed_dense(amfls):
    """Dense column-major operator: a consistent least-squares problem is
    certified at 1e-10; a ridge problem with an inconsistent b asked for
    1e-10, far below what FP32 correction steps can reach there, switches to
    FP64 inner solves once the FP32 steps stop contracting (trace column 2),
    and its outcome must be honest: a success passes the host checks against
    the oracle, a failure reports a certificate above the tolerance."""
    from amfls_solver_gb300 import problems

    prob = problems.scaled_dense(2000, 300, decades=3.0, seed=2, column_major=True)
    t = torch.from_numpy(np.ascontiguousarray(prob.matrix.T)).cuda().t()
    op = amfls.DeviceOperator(t)
    low = op.reduced("fp32")
    x_true = np.random.default_rng(4).standard_normal(300)
    prob.b = prob.matrix @ x_true
    b = torch.from_numpy(prob.b).cuda()
    r = amfls.run_amfls_mixed(op, b, reduced=low, inner_tolerance=1e-6, maximum_refinements=8,
                              tolerance=1e-10)
    assert r.status == 0 and r.backward_error_upper_bound <= 1e-10
    check_solution(prob, r.solution.cpu().numpy(), _oracle_x(prob, 0.0, 1e-10), 0.0, 1e-10, True)
    b_inc = torch.from_numpy(np.random.default_rng(6).standard_normal(2000)).cuda()
    deep = amfls.run_amfls_mixed(op, b_inc, reduced=low, inner_tolerance=1e-6,
                                 maximum_refinements=12, regularization=1e-6, tolerance=1e-10)
    steps = deep.trace_float.numpy()
    assert steps[0, 2] == 0 and steps[-1, 2] == 1  # FP32 first, FP64 after the stall
    if deep.status == 0:
        assert deep.relative_energy_error_upper_bound <= 1e-10
        prob.b = b_inc.cpu().numpy()
        check_solution(prob, deep.solution.cpu().numpy(), _oracle_x(prob, 1e-6, 1e-10), 1e-6,
                       1e-10, True)
    else:
        assert deep.relative_energy_error_upper_bound > 1e-10


def test_mixed_bf16_on_a_consistent_well_conditioned_problem(amfls):
    from amfls_solver_gb300 import problems

    tol = 1e-10
    prob = problems.scaled_uniform_csr(4000, 500, per_row=12, decades=0.5, noise=0.0, seed=9)
    r = amfls.run_amfls_mixed(csr_tensor(prob), torch.from_numpy(prob.b).cuda(), values="bf16",
                              inner_tolerance=1e-3, maximum_refinements=16, tolerance=tol)
    assert r.status == 0 and r.backward_error_upper_bound <= tol
    check_solution(prob, r.solution.cpu().numpy(), _oracle_x(prob, 0.0, tol), 0.0, tol, True)

"""GPU tests of the row-vector CSR products (csr_vector.cuh), forced with
AMFLS_GB300_CSR_VECTOR=1 (large sides choose them by timing).

Rows are binned by length (1-32 lanes per row) and sorted longest first
within a bin; a row of fewer than 32 nonzeros is one lane's sequential FMA
chain in storage order, the reference's order (sparse_csr_operator.cpp:
203-235), so those entries must be bit-identical to the oracle's; every entry
lies within gamma_{2L+2} (|A| |x|)_i of the oracle's (L the row length), the
reference's rounding model for one product.  A solve through the fused
products must reproduce the oracle's status, stop reason and depth like the
tiled products do.
"""
import numpy as np
import pytest
import torch

from oracle import amfls_oracle as orc
from test_gpu_parity import chain_csr, csr_tensor, product_bound, skewed_csr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def amfls():
    import amfls_solver_gb300 as m

    m.load_library()
    return m


@pytest.mark.parametrize("make", [chain_csr, skewed_csr])
def test_vector_products_against_oracle(amfls, monkeypatch, make):
    monkeypatch.setenv("AMFLS_GB300_CSR_VECTOR", "1")
    prob = make()
    op = amfls.DeviceOperator(csr_tensor(prob))
    choice, _ = op.tile_schedule()
    assert choice == {"A": "row vector", "A^T": "row vector"}
    ref = orc.Operator(prob)
    rng = np.random.default_rng(9)
    x = rng.standard_normal((prob.cols, 1))
    y = rng.standard_normal((prob.rows, 1))
    ax = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()[:, 0]
    aty = op.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()[:, 0]
    ax_ref = ref.apply(np.asfortranarray(x))[:, 0]
    aty_ref = ref.apply_transpose(np.asfortranarray(y))[:, 0]
    lens = np.diff(prob.row_offsets)
    clens = np.bincount(prob.column_indices, minlength=prob.cols)
    assert np.array_equal(ax[lens < 32], ax_ref[lens < 32])
    assert np.array_equal(aty[clens < 32], aty_ref[clens < 32])
    assert np.all(np.abs(ax - ax_ref) <= 2 * product_bound(prob, x[:, 0], False))
    assert np.all(np.abs(aty - aty_ref) <= 2 * product_bound(prob, y[:, 0], True))
    assert np.all(ax[lens == 0] == 0.0)
    again = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()[:, 0]
    assert np.array_equal(ax, again)
    # multi-column products keep the tiles; their first column agrees
    X = np.asfortranarray(rng.standard_normal((prob.cols, 3)))
    AX = op.apply(torch.from_numpy(X).cuda()).cpu().numpy()
    AX_ref = ref.apply(X)
    for c in range(3):
        assert np.all(np.abs(AX[:, c] - AX_ref[:, c]) <= 2 * product_bound(prob, X[:, c], False))


@pytest.mark.parametrize("values", ["fp32", "bf16"])
def test_vector_reduced_products(amfls, monkeypatch, values):
    from test_gpu_mixed import reduced_bound

    monkeypatch.setenv("AMFLS_GB300_CSR_VECTOR", "1")
    prob = chain_csr()
    a = prob.to_dense()
    low = amfls.DeviceOperator(csr_tensor(prob)).reduced(values)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(prob.cols)
    y = rng.standard_normal(prob.rows)
    ax = low.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    aty = low.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()
    Lr = int(np.diff(prob.row_offsets).max())
    Lc = int(np.bincount(prob.column_indices, minlength=prob.cols).max())
    assert np.all(np.abs(ax - a @ x) <= reduced_bound(np.abs(a), x, Lr, values))
    assert np.all(np.abs(aty - a.T @ y) <= reduced_bound(np.abs(a.T), y, Lc, values))


@pytest.mark.parametrize("lam,tol", [(0.0, 1e-8), (1e-4, 1e-10)])
def test_vector_products_in_a_solve(amfls, monkeypatch, lam, tol):
    """The fused products with their epilogues (subtraction of the previous
    basis vector, norms, dots) inside AMFLS: the oracle's status, stop reason
    and depth, and the parity tests' checks on x."""
    from amfls_solver_gb300 import problems
    from test_gpu_parity import check_solution

    monkeypatch.setenv("AMFLS_GB300_CSR_VECTOR", "1")
    p = problems.scaled_uniform_csr(6000, 1500, per_row=10, decades=6.0, seed=11)
    ref = orc.solve_amfls(p, regularization=lam, tolerance=tol, seed=3)
    r = amfls.run_amfls(csr_tensor(p), torch.from_numpy(p.b).cuda(), regularization=lam,
                        tolerance=tol, seed=3)
    assert (r.status, r.stop_reason) == (ref["status"], ref["stop_reason"])
    assert r.depth == ref["counters"][9]
    check_solution(p, r.solution.cpu().numpy(), ref["solution"], lam, tol, r.status == 0)

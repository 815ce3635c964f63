"""GPU tests of the reduced-basis sweeps (options.reduced_basis; no
counterpart in the reference, whose sweeps are FP64 BLAS calls).

Width-one levels keep an FP32 copy of the right basis V and run their first
reorthogonalisation pass on it: c = V~^T fl32(r) with FP32 products summed in
FP32 over runs of 16 rows per lane and in FP64 above that, then
r <- r - fl64(V~ fl32(c)).  The recurrence, the operator products, the DGKS
second pass, the projected solve and the certified validation stay FP64, and a
level whose coefficients exceed 1e-3 ||r|| redoes the pass in FP64.  The
option serves the restart cycles of the mixed form, whose corrections need a
few digits each.

* The projection itself: each coefficient must lie within
  20 u32 ||v_j|| ||r|| of the FP64 sweep's on the same basis (two FP32
  roundings of the inputs and a 16-term FP32 sum, with slack).
* Restarted mixed solves: the certified FP64 validation decides success, so
  a success must pass the same host float64 checks as the FP64 drop-in's
  (backward error at most tol, x within 1e-4 relative of the reference's x on
  the 20000 x 5000 workload, the spread the reference's own x has against an
  exact least-squares solve); on a ridge problem x must agree with the
  restarted solve that sweeps in FP64 to what the energy-norm tolerance
  determines.
"""
import numpy as np
import pytest
import torch

from conftest import golden_options, load_replay

pytestmark = pytest.mark.gpu

U32 = 2.0 ** -24


@pytest.fixture(scope="module")
def amfls():
    import amfls_solver_gb300 as m

    m.load_library()
    return m


def _csr(prob):
    return torch.sparse_csr_tensor(torch.from_numpy(prob.row_offsets),
                                   torch.from_numpy(prob.column_indices),
                                   torch.from_numpy(prob.values),
                                   size=(prob.rows, prob.cols)).cuda()


def _backward_error(prob, x):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    a = sp.csr_matrix((prob.values, prob.column_indices, prob.row_offsets),
                      shape=(prob.rows, prob.cols))
    norm_a = spl.svds(a, k=1, return_singular_vectors=False, tol=1e-10)[0]
    r = a @ x - prob.b
    compat = np.linalg.norm(r) / (norm_a * np.linalg.norm(x) + np.linalg.norm(prob.b))
    ls = np.linalg.norm(a.T @ r) / (norm_a * np.linalg.norm(r))
    return min(compat, ls)


@pytest.mark.parametrize("n,k", [(5000, 37), (200_000, 64), (140_001, 96)])
def test_reduced_projection_matches_fp64_sweep(amfls, n, k):
    import ctypes
    from amfls_solver_gb300 import _native

    lib = _native.load()
    sec = (ctypes.c_double * 2)()
    err = ctypes.c_double(-1.0)
    stream = torch.cuda.current_stream().cuda_stream
    _native.check(lib.amfls_gpu_probe_reorthogonalization_reduced(
        n, k, 3, ctypes.c_void_p(stream), sec, ctypes.byref(err)))
    # the probe's basis pattern: V[row, col] = ((7 row + 13 col) mod 17 - 8) 1e-3
    rows = np.arange(n, dtype=np.int64)[:, None]
    cols = np.arange(k, dtype=np.int64)[None, :]
    v = (((rows * 7 + cols * 13) % 17) - 8) * 1e-3
    colnorm = np.sqrt((v * v).sum(axis=0)).max()
    assert 0.0 <= err.value <= 20 * U32 * colnorm
    assert sec[0] > 0.0 and sec[1] > 0.0


def test_plain_solve_reports_no_reduced_levels(amfls):
    from amfls_solver_gb300 import problems

    prob = problems.scaled_uniform_csr(3000, 800, per_row=10, decades=3.0, noise=1e-10, seed=3)
    r = amfls.solve_amfls(amfls.DeviceOperator(_csr(prob)), torch.from_numpy(prob.b).cuda(),
                          tolerance=1e-10)
    assert r.reduced_basis_levels == 0 and r.reduced_basis_fallbacks == 0


@pytest.mark.parametrize("cycle", [1000, 2000])
def test_restarted_mixed_solve_with_reduced_basis(amfls, cycle):
    """Residual correction in FP64 around restart cycles of `cycle` levels
    (inner solves on the FP64 operator, reduced-basis sweeps, an inner
    tolerance no cycle reaches): certified at the workload's tolerance, and x
    within the reference's spread of the reference's x."""
    data, prob = load_replay("replay_csr_20000x5000")
    opts = golden_options(data)
    op = amfls.DeviceOperator(_csr(prob))
    b = torch.from_numpy(prob.b).cuda()
    r = amfls.run_amfls_mixed(op, b, values="fp64", reduced_basis=True, inner_tolerance=1e-14,
                              maximum_refinements=40, maximum_depth=cycle,
                              regularization=opts["regularization"], tolerance=opts["tolerance"])
    assert r.status == 0 and r.backward_error_upper_bound <= opts["tolerance"]
    assert r.reduced_basis_levels > 0
    x, xr = r.solution.cpu().numpy(), data["solution"]
    assert _backward_error(prob, x) <= opts["tolerance"] * (1 + 1e-3)
    assert np.linalg.norm(x - xr) <= 1e-4 * np.linalg.norm(xr)


def test_restarted_ridge_solve_with_and_without_reduced_basis(amfls):
    """A power-law CSR ridge problem (the shape of the 2,000,000 x 500,000
    workload at 1/10 scale): restart cycles of 500 levels with FP32 and with
    FP64 sweeps both certify the 1e-10 relative energy error, and their x
    agree to 1e-10 cond(M) relative (cond(M) <= ||A|| / sqrt(lambda))."""
    from amfls_solver_gb300 import problems

    prob = problems.power_law_csr(200_000, 50_000, decades=8.0, noise=1e-6, seed=5)
    op = amfls.DeviceOperator(_csr(prob))
    b = torch.from_numpy(prob.b).cuda()
    reg, tol = 1e-4, 1e-10
    runs = {}
    for rb in (False, True):
        r = amfls.run_amfls_mixed(op, b, values="fp64", reduced_basis=rb, inner_tolerance=1e-14,
                                  maximum_refinements=60, maximum_depth=500,
                                  regularization=reg, tolerance=tol)
        assert r.status == 0 and r.relative_energy_error_upper_bound <= tol
        assert (r.reduced_basis_levels > 0) == rb
        runs[rb] = r.solution.cpu().numpy()
    norm_a = op.validation_error_model()[0]
    cond = norm_a / np.sqrt(reg)
    assert np.linalg.norm(runs[True] - runs[False]) <= 4 * tol * cond * np.linalg.norm(runs[False])

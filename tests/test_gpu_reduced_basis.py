"""GPU tests of the reduced-basis sweeps (options.reduced_basis; no
counterpart in the reference, whose sweeps are FP64 BLAS calls).

Width-one levels keep an FP32 or FP16 copy (FP16 holding 2^8 v) of the
right basis V and run their first reorthogonalisation pass on it:
c = V~^T fl32(r) with FP32 products summed in FP32 over runs of 16 rows per
lane and in FP64 above that, then r <- r - fl64(V~ fl32(c)).  The recurrence, the operator products, the DGKS
second pass, the projected solve and the certified validation stay FP64, and a
level whose coefficients exceed 1e-3 ||r|| redoes the pass in FP64.  The
option serves the restart cycles of the mixed form, whose corrections need a
few digits each.

* The projection itself: each coefficient must lie within
  20 u ||v_j|| ||r|| of the FP64 sweep's on the same basis (u the copy's unit
  roundoff, 2^-24 or 2^-11; roundings of the inputs and a 16-term FP32 sum,
  with slack).
* Restarted mixed solves on a ridge problem: the certified FP64 validation
  decides success, and x must agree with the restarted solve that sweeps in
  FP64 to what the energy-norm tolerance determines.  (Restart cycles suit
  regularised problems: on the unregularised 20000 x 5000 workload, condition
  1e6, forty cycles of 1000 or 2000 levels stay far from its 1e-8 tolerance,
  which the unrestarted solve reaches in 3786 levels.)
"""
import numpy as np
import pytest
import torch


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


@pytest.mark.parametrize("storage", [1, 2])
@pytest.mark.parametrize("n,k", [(5000, 37), (200_000, 64), (140_001, 96)])
def test_reduced_projection_matches_fp64_sweep(amfls, n, k, storage):
    import ctypes
    from amfls_solver_gb300 import _native

    lib = _native.load()
    sec = (ctypes.c_double * 2)()
    err = ctypes.c_double(-1.0)
    stream = torch.cuda.current_stream().cuda_stream
    _native.check(lib.amfls_gpu_probe_reorthogonalization_reduced(
        n, k, 3, storage, ctypes.c_void_p(stream), sec, ctypes.byref(err)))
    # the probe's basis pattern: V[row, col] = ((7 row + 13 col) mod 17 - 8) 1e-3
    rows = np.arange(n, dtype=np.int64)[:, None]
    cols = np.arange(k, dtype=np.int64)[None, :]
    v = (((rows * 7 + cols * 13) % 17) - 8) * 1e-3
    colnorm = np.sqrt((v * v).sum(axis=0)).max()
    u = U32 if storage == 1 else 2.0 ** -11  # the copy's unit roundoff (FP32, FP16)
    assert 0.0 <= err.value <= 20 * u * colnorm
    assert sec[0] > 0.0 and sec[1] > 0.0


def test_plain_solve_reports_no_reduced_levels(amfls):
    from amfls_solver_gb300 import problems

    prob = problems.scaled_uniform_csr(3000, 800, per_row=10, decades=3.0, noise=1e-10, seed=3)
    r = amfls.solve_amfls(amfls.DeviceOperator(_csr(prob)), torch.from_numpy(prob.b).cuda(),
                          tolerance=1e-10)
    assert r.reduced_basis_levels == 0 and r.reduced_basis_fallbacks == 0


def test_restarted_ridge_solve_with_and_without_reduced_basis(amfls):
    """A power-law CSR ridge problem (the shape of the 2,000,000 x 500,000
    workload at 1/10 scale): restart cycles of 1000 levels with FP32 and with
    FP64 sweeps both certify the 1e-10 relative energy error, and their x
    agree to 1e-10 cond(M) relative (cond(M) <= ||A|| / sqrt(lambda)); cycles
    of 500 levels, whose certificate alternates large and small decreases,
    also certify (the stopping rule looks two cycles back)."""
    from amfls_solver_gb300 import problems

    prob = problems.power_law_csr(200_000, 50_000, decades=8.0, noise=1e-6, seed=5)
    op = amfls.DeviceOperator(_csr(prob))
    b = torch.from_numpy(prob.b).cuda()
    reg, tol = 1e-4, 1e-10
    runs = {}
    for rb, cycle in ((False, 1000), (True, 1000), (True, 500), ("fp16", 1000)):
        r = amfls.run_amfls_mixed(op, b, values="fp64", reduced_basis=rb, inner_tolerance=1e-14,
                                  maximum_refinements=80, maximum_depth=cycle,
                                  regularization=reg, tolerance=tol)
        assert r.status == 0 and r.relative_energy_error_upper_bound <= tol
        assert (r.reduced_basis_levels > 0) == bool(rb)
        assert r.reduced_basis_fallbacks <= r.reduced_basis_levels // 100
        runs[rb, cycle] = r.solution.cpu().numpy()
    norm_a = op.validation_error_model()[0]
    cond = norm_a / np.sqrt(reg)
    ref = runs[False, 1000]
    for key in ((True, 1000), (True, 500), ("fp16", 1000)):
        assert np.linalg.norm(runs[key] - ref) <= 4 * tol * cond * np.linalg.norm(ref)


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_mixed_form_against_the_reference_on_a_tall_ridge_problem(amfls, storage):
    """The chosen form against the reference's own solve of a 60000 x 15000
    portable CSR ridge problem (lambda = 1e-4, tol 1e-10; the reference
    certified it in 2560 levels): restart cycles of 1000 levels with
    reduced-basis sweeps certify the tolerance, and x agrees with the
    reference's x to 2.5 tol in the energy norm ||v||_H^2 = ||A v||^2 +
    lambda ||v||^2 (both x lie within tol of the exact solution there) and
    to 2 tol ||M|| / sqrt(lambda) relative in the 2-norm."""
    import scipy.sparse as sp
    from conftest import golden_options, load_replay

    data, prob = load_replay("replay_csr_ridge_60000x15000")
    opts = golden_options(data)
    reg, tol = opts["regularization"], opts["tolerance"]
    op = amfls.DeviceOperator(_csr(prob))
    r = amfls.run_amfls_mixed(op, torch.from_numpy(prob.b).cuda(), values="fp64",
                              reduced_basis=storage, inner_tolerance=1e-14, maximum_refinements=60,
                              maximum_depth=1000, regularization=reg, tolerance=tol)
    assert r.status == 0 and r.relative_energy_error_upper_bound <= tol
    assert r.reduced_basis_levels > 0
    a = sp.csr_matrix((prob.values, prob.column_indices, prob.row_offsets),
                      shape=(prob.rows, prob.cols))
    hnorm = lambda v: np.sqrt(np.linalg.norm(a @ v) ** 2 + reg * np.linalg.norm(v) ** 2)
    x, xr = r.solution.cpu().numpy(), data["solution"]
    assert hnorm(x - xr) <= 2.5 * tol * hnorm(xr)
    norm_m = np.sqrt(op.validation_error_model()[0] ** 2 + reg)
    rel = np.linalg.norm(x - xr) / np.linalg.norm(xr)
    print(f"\nmixed form vs reference: {r.depth} levels ({int(r.trace_float.shape[0])} cycles), "
          f"x relative difference {rel:.2e}, energy norm {hnorm(x - xr) / hnorm(xr):.2e}")
    assert rel <= 2 * tol * norm_m / np.sqrt(reg)


def test_reduced_basis_through_a_widening_solve(amfls):
    """A solve that widens (the reference's forced schedule on a 2000 x 500
    ridge problem, replayed) starts at width one on the FP32 copy of the
    basis and continues on the block path, which projects on the FP64 basis:
    the replayed decisions, the reference's status and a certified result
    with x within 2.5 tol of the reference's in the energy norm."""
    import scipy.sparse as sp
    from conftest import golden_options, load_replay

    data, prob = load_replay("replay_csr_ridge_forced")
    opts = golden_options(data)
    reg, tol = opts["regularization"], opts["tolerance"]
    op = amfls.DeviceOperator(_csr(prob))
    r, decisions, overrun = amfls.solve_amfls_replay(
        op, torch.from_numpy(prob.b).cuda(), [int(v) for v in data["replay"]], reduced_basis=True,
        **opts)
    assert overrun == 0
    assert r.auxiliary_width > 0  # the solve widened
    assert (r.status, r.stop_reason) == (int(data["status"]), int(data["stop_reason"]))
    if r.status == 0:
        assert r.relative_energy_error_upper_bound <= tol
    a = sp.csr_matrix((prob.values, prob.column_indices, prob.row_offsets),
                      shape=(prob.rows, prob.cols))
    hnorm = lambda v: np.sqrt(np.linalg.norm(a @ v) ** 2 + reg * np.linalg.norm(v) ** 2)
    x, xr = r.solution.cpu().numpy(), data["solution"]
    assert hnorm(x - xr) <= 2.5 * tol * hnorm(xr)

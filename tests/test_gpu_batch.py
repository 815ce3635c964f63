"""GPU tests of batched solves (no counterpart in the reference): problems
solved concurrently by several workers must come out as solved one at a
time -- same status and stop reason, certified bounds within tolerance,
and solutions that agree to the accuracy the problems determine."""
import numpy as np
import pytest
import torch

from test_gpu_parity import csr_tensor

pytestmark = pytest.mark.gpu


def test_batch_matches_one_at_a_time():
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import problems

    batch = problems.uneven_csr_batch(10, seed=5, m_range=(2000, 20000), n_range=(500, 5000),
                                      cond_range=(1e3, 1e5))
    mats = [(csr_tensor(p), torch.from_numpy(p.b).cuda()) for p, _, _ in batch]
    regs = [r for _, r, _ in batch]
    tol = batch[0][2]
    results, seconds, wall = amfls.run_amfls_batch(mats, workers=4, regularization=regs,
                                                   tolerance=tol)
    assert len(results) == 10 and np.all(seconds > 0) and wall > 0
    for (mat, b), reg, r in zip(mats, regs, results):
        one = amfls.run_amfls(mat, b, regularization=reg, tolerance=tol)
        assert (r.status, r.stop_reason) == (one.status, one.stop_reason)
        if r.status == 0:
            assert r.relative_energy_error_upper_bound <= tol
            hn = lambda v: float(torch.linalg.norm(v))
            assert hn(r.solution - one.solution) <= 10 * tol * 1e5 * hn(one.solution)


def test_batch_matches_oracle():
    """Batched CSR solves against the oracle (the CPU restatement pinned to
    the reference): CSR operators never widen under the reference's cost
    model, so each problem's status, stop reason, depth and basis rank must
    equal the oracle's solve of it, and the certified bound must meet tol."""
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import problems
    from oracle import amfls_oracle as orc

    batch = problems.uneven_csr_batch(6, seed=9, m_range=(2000, 8000), n_range=(500, 2000),
                                      cond_range=(1e3, 1e5))
    mats = [(csr_tensor(p), torch.from_numpy(p.b).cuda()) for p, _, _ in batch]
    regs = [r for _, r, _ in batch]
    tol = batch[0][2]
    results, _, _ = amfls.run_amfls_batch(mats, workers=3, regularization=regs, tolerance=tol)
    for (p, reg, _), r in zip(batch, results):
        ref = orc.solve_amfls(p, regularization=reg, tolerance=tol)
        assert (r.status, r.stop_reason) == (ref["status"], ref["stop_reason"])
        assert (r.depth, r.basis_rank) == (int(ref["counters"][9]), int(ref["counters"][11]))
        if r.status == 0:
            assert r.relative_energy_error_upper_bound <= tol


def test_batch_reports_bad_problems_without_stopping_the_others():
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import problems

    p = problems.scaled_uniform_csr(3000, 500, seed=2)
    good = (csr_tensor(p), torch.from_numpy(p.b).cuda())
    with pytest.raises(RuntimeError, match="problem 1"):
        amfls.run_amfls_batch([good, good], workers=2, tolerance=[1e-8, 2.0])


def test_batch_rejects_a_shared_operator():
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import problems

    p = problems.scaled_uniform_csr(3000, 500, seed=2)
    op = amfls.DeviceOperator(csr_tensor(p))
    b = torch.from_numpy(p.b).cuda()
    with pytest.raises(RuntimeError, match="its own operator"):
        amfls.run_amfls_batch([(op, b), (op, b)], workers=2)

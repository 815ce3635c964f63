"""GPU tests of the learned width controller (no counterpart in the
reference): the CUDA forward pass and gradient against the numpy oracle
(oracle/width_mlp.py, itself pinned by finite differences), deterministic
GPU training, the controlled solve without a policy equal to the
reference's controller, and a trained policy on held-out problems, whose
gain over the heuristic is measured and printed (the FP64 certificate still
decides termination, so every solve must certify as the heuristic's does)."""
import numpy as np
import pytest
import torch

from oracle import width_mlp
from test_gpu_parity import csr_tensor

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    import amfls_solver_gb300 as m
    from amfls_solver_gb300 import learned

    m.load_library()
    return m, learned


def test_policy_kernels_match_the_oracle(mods):
    _, learned = mods
    rng = np.random.default_rng(3)
    p = learned.initial_params(7)
    assert p.shape == (width_mlp.P,) and np.all(np.isfinite(p))
    x = rng.standard_normal((300, width_mlp.I))
    y = rng.standard_normal(300)
    out = learned.forward(p, x)
    ref, _ = width_mlp.forward(p, x)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-13)
    loss, g = learned.gradient(p, x, y)
    rloss, rg = width_mlp.loss_and_grad(p, x, y)
    assert np.isclose(loss, rloss, rtol=1e-12)
    np.testing.assert_allclose(g, rg, rtol=1e-10, atol=1e-14)


def test_policy_training_is_deterministic_and_fits(mods):
    _, learned = mods
    rng = np.random.default_rng(5)
    x = rng.standard_normal((400, width_mlp.I))
    y = np.tanh(x[:, 0] - 0.5 * x[:, -1]) + 0.1 * x[:, 3]
    a = learned.WidthPolicy.train(x, y, epochs=800, learning_rate=3e-3, seed=1)
    b = learned.WidthPolicy.train(x, y, epochs=800, learning_rate=3e-3, seed=1)
    assert np.array_equal(a.params, b.params)
    first, last = a.losses
    assert last < 0.05 * first
    np.testing.assert_allclose(a.scores(x[:5, :-1])[:, 1],
                               width_mlp.forward(a.params, np.c_[x[:5, :-1], np.ones(5)])[0],
                               rtol=1e-12, atol=1e-13)


def test_uncontrolled_solve_is_the_reference_controller(mods):
    amfls, learned = mods
    from conftest import golden_options, load_golden

    data, prob = load_golden("solve_powerlaw_ridge")
    mat, b = csr_tensor(prob), torch.from_numpy(prob.b).cuda()
    opts = golden_options(data)
    plain = amfls.run_amfls(mat, b, **opts)
    ctl, log = learned.solve_controlled(mat, b, **opts)
    assert (ctl.status, ctl.stop_reason, ctl.depth, ctl.basis_rank, ctl.auxiliary_width) == \
        (plain.status, plain.stop_reason, plain.depth, plain.basis_rank, plain.auxiliary_width)
    assert torch.equal(ctl.solution, plain.solution)
    if len(log):
        assert np.array_equal(log[:, 11], log[:, 12])  # every action is the heuristic's


def test_trained_policy_on_held_out_problems(mods):
    amfls, learned = mods
    from amfls_solver_gb300 import problems

    opts = dict(tolerance=1e-10, maximum_auxiliary_width=64)
    logs = []
    for i, m in enumerate([4000, 6000, 8000]):
        prob = problems.banded_random_csr(m, m // 4, decades=9.0, seed=200 + i)
        op = amfls.DeviceOperator(csr_tensor(prob))
        b = torch.from_numpy(prob.b).cuda()
        for reg in (0.0, 1e-6):
            for es in (1, 2):
                r, log = learned.solve_controlled(op, b, exploration=0.4, exploration_seed=es + 7 * i,
                                                  regularization=reg, **opts)
                logs.append(log)
    data = learned.dataset(logs)
    policy = learned.WidthPolicy.train(data.inputs, data.targets, epochs=2000)
    assert policy.losses[1] < policy.losses[0]
    work = {"heuristic": 0, "learned": 0}
    for i, m in enumerate([10000, 12000]):
        prob = problems.banded_random_csr(m, m // 4, decades=9.0, seed=900 + i)
        op = amfls.DeviceOperator(csr_tensor(prob))
        b = torch.from_numpy(prob.b).cuda()
        for reg in (0.0, 1e-6):
            h, _ = learned.solve_controlled(op, b, regularization=reg, **opts)
            lr, log = learned.solve_controlled(op, b, policy=policy, regularization=reg, **opts)
            assert lr.status == h.status  # the certificate judges both the same way
            if lr.status == 0:
                assert (lr.backward_error_upper_bound if reg == 0.0
                        else lr.relative_energy_error_upper_bound) <= 1e-10
            work["heuristic"] += h.a_columns + h.at_columns
            work["learned"] += lr.a_columns + lr.at_columns
    print(f"\noperator columns on held-out problems: heuristic {work['heuristic']}, "
          f"learned {work['learned']} (gain {1 - work['learned'] / work['heuristic']:+.1%})")

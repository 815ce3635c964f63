"""Host-side pieces of the learned width controller; CPU only.

  * the parameter layout: the native library's parameter count, inputs and
    decision-log columns agree with the numpy restatement of the network
    (oracle/width_mlp.py), which the finite-difference test pins;
  * seeded initial parameters (computed on the host by the library): the
    same vector for the same seed, Glorot-uniform weights inside their
    bounds sqrt(6 / (fan_in + fan_out)), zero biases;
  * dataset(): only decision rows with a measured rate are kept, the inputs
    are the 11 features plus the action bit, and the targets are
    asinh(rate / scale) with the median |rate| as the default scale.
No compute call is made here.
"""
import numpy as np
import pytest

from amfls_solver_gb300 import _native
from amfls_solver_gb300.build import LIB
from oracle import width_mlp


@pytest.fixture(scope="module")
def learned():
    if not LIB.exists():
        from amfls_solver_gb300 import build
        build.build()
    from amfls_solver_gb300 import learned as m
    return m


def test_layout_matches_the_restated_network():
    assert _native.POLICY_PARAMS == width_mlp.P
    assert _native.POLICY_INPUTS == width_mlp.I == _native.POLICY_FEATURES + 1


def test_initial_params_are_seeded_glorot(learned):
    p = learned.initial_params(3)
    assert p.shape == (width_mlp.P,)
    assert np.array_equal(p, learned.initial_params(3))
    assert not np.array_equal(p, learned.initial_params(4))
    w = width_mlp.unpack(p)
    I, H = width_mlp.I, width_mlp.H
    for name, bound in (("W1", np.sqrt(6.0 / (I + H))), ("W2", np.sqrt(6.0 / (H + H))),
                        ("w3", np.sqrt(6.0 / (H + 1)))):
        assert np.all(np.abs(w[name]) < bound), name
        assert np.abs(w[name]).max() > 0.8 * bound, name  # the whole range is used
    for name in ("b1", "b2", "b3"):
        assert np.all(w[name] == 0.0), name


def test_dataset_keeps_measured_rows(learned):
    cols = _native.DECISION_COLUMNS
    rng = np.random.default_rng(1)
    log_a = rng.standard_normal((5, cols))
    log_b = rng.standard_normal((4, cols))
    for log in (log_a, log_b):
        log[:, 11] = rng.integers(0, 2, log.shape[0])   # the action taken
        log[:, 14] = [1, 0, 1, 1, 0][:log.shape[0]]     # measured or not
    data = learned.dataset([log_a, log_b])
    kept = np.concatenate([log_a[log_a[:, 14] > 0], log_b[log_b[:, 14] > 0]])
    assert data.inputs.shape == (kept.shape[0], _native.POLICY_INPUTS)
    assert np.array_equal(data.inputs[:, :_native.POLICY_FEATURES],
                          kept[:, :_native.POLICY_FEATURES])
    assert np.array_equal(data.inputs[:, -1], kept[:, 11])
    assert data.scale == float(np.median(np.abs(kept[:, 13])))
    assert np.allclose(data.targets, np.arcsinh(kept[:, 13] / data.scale))
    fixed = learned.dataset([log_a], scale=2.0)
    assert fixed.scale == 2.0
    with pytest.raises(ValueError):
        learned.dataset([np.zeros((3, cols))])

"""The oracle in schedule-replay mode against the reference's widening solves.

Each tests/golden/replay_*.npz fixture holds a reference run's width-decision
bits (recorded at the reference's decision sites, amfls.cpp:323-354) and the
outputs of the reference replaying them.  The oracle's controller
(oracle/amfls_oracle.py, a restatement of amfls.cpp:57-661) replaying the
same bits must take the same decisions at the same sites and reproduce the
reference's counters, trace and solution: bit for bit on x86-64, the machine
that made the fixtures (long double and libm may differ in the last bits
elsewhere, hence the 1e-9 bound on x).
"""
import numpy as np
import pytest

from conftest import GOLDEN, REPLAY_FIXTURES, golden_options, load_replay
from oracle import amfls_oracle as orc


# the full-size dense ridge fixture takes the oracle minutes (the reference
# about two); the GPU replay test compares with the reference's outputs
# there directly
ORACLE_REPLAYS = [n for n in REPLAY_FIXTURES if n != "replay_dense_ridge_100000x2000"]


@pytest.mark.parametrize("name", ORACLE_REPLAYS)
def test_oracle_replays_reference_widening(name, gelsy_ranks):
    data, prob = load_replay(name)
    opts = golden_options(data)
    r = orc.solve_amfls(prob, replay=[int(v) for v in data["replay"]], **opts)
    assert r["replay_overrun"] == 0
    np.testing.assert_array_equal(r["decisions"], data["decisions"])
    assert (r["status"], r["stop_reason"]) == (int(data["status"]), int(data["stop_reason"]))
    np.testing.assert_array_equal(r["counters"], data["counters"])
    np.testing.assert_array_equal(r["trace_int"], data["trace_int"])
    np.testing.assert_array_equal(r["trace_float"][:, :8], data["trace_float"][:, :8])
    xr = data["solution"]
    assert np.linalg.norm(r["solution"] - xr) <= 1e-9 * np.linalg.norm(xr)
    # full column rank at every dgelsy projected solve (lambda = 0): the
    # GPU's QR recurrence gives the same solution there
    assert all(rank == shape[1] for shape, rank in gelsy_ranks), gelsy_ranks
    assert gelsy_ranks or opts["regularization"] > 0.0


def test_replay_fixtures_widen():
    """The widening fixtures exercise the widening sites: Gaussian seeds were
    injected (counter 34), both decision kinds were taken, and the
    reference's own runs of the 20000 x 5000 CSR and 100000 x 2000 dense
    workloads take no widening decision."""
    widened = 0
    for name in REPLAY_FIXTURES:
        data = np.load(GOLDEN / f"{name}.npz")  # outputs only: no regeneration
        c = data["counters"]
        if "widening" in name or "forced" in name:
            assert c[34] > 0 and c[10] > 0 and data["decisions"].sum() == c[34]
            widened += 1
        else:
            assert c[34] == 0 and c[10] == 0
    assert widened >= 4

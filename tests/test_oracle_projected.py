"""The GPU's projected ridge solve against the reference's, on the T of every
evaluation of the ridge fixtures; CPU only.

For lambda > 0 the reference solves the projected problem
min ||T y - g||^2 + lambda ||y||^2 through the SVD of T and the filter
sigma / (sigma^2 + lambda) (krylov_workspace.cpp:833-925, restated in the
oracle's Workspace.evaluate).  The GPU reduces [T; sqrt(lambda) I] by
orthogonal rotations instead (the damped recurrence of its width-one
projected solve, a Householder QR for block levels).  Both are backward
stable for the same full-rank problem; recorded here, at every evaluation
of the reference's ridge fixtures, the two solutions agree to within 1e-12
in the projected energy norm sqrt(||T y||^2 + lambda ||y||^2), so the
choice of method does not move the iterates beyond rounding.
"""
import numpy as np
import pytest

from conftest import SOLVE_FIXTURES, golden_options, load_golden, load_replay
from oracle import amfls_oracle as orc

RIDGE_SOLVES = [n for n in SOLVE_FIXTURES if "ridge" in n or "basis_cap" in n]
RIDGE_REPLAYS = ["replay_csr_ridge_forced"]  # the two larger ridge replays take the oracle minutes


@pytest.fixture
def projected_pairs(monkeypatch):
    gaps = []
    evaluate = orc.Workspace.evaluate

    def recording(self, tolerance, epoch, auxiliary_width):
        out = evaluate(self, tolerance, epoch, auxiliary_width)
        if self.reg > 0.0 and self.k > 0:
            t, g, lam = self.projected_operator(), np.asarray(self.g), self.reg
            u, s, vt = np.linalg.svd(t, full_matrices=False)
            y_filter = vt.T @ ((s / (s * s + lam)) * (u.T @ g))
            k = t.shape[1]
            y_qr = np.linalg.lstsq(np.vstack([t, np.sqrt(lam) * np.eye(k)]),
                                   np.concatenate([g, np.zeros(k)]), rcond=None)[0]
            energy = lambda y: np.sqrt(np.linalg.norm(t @ y) ** 2 + lam * np.linalg.norm(y) ** 2)
            gaps.append(energy(y_filter - y_qr) / energy(y_filter))
        return out

    monkeypatch.setattr(orc.Workspace, "evaluate", recording)
    return gaps


@pytest.mark.parametrize("name", RIDGE_SOLVES + RIDGE_REPLAYS)
def test_damped_qr_matches_the_svd_filter(name, projected_pairs):
    if name.startswith("replay_"):
        data, prob = load_replay(name)
        opts = golden_options(data)
        orc.solve_amfls(prob, replay=[int(v) for v in data["replay"]], **opts)
    else:
        data, prob = load_golden(name)
        opts = golden_options(data)
        assert opts["regularization"] > 0.0
        if opts.pop("algorithm", "amfls") == "fixed_rbgk":
            orc.solve_fixed_rbgk(prob, **opts)
        else:
            orc.solve_amfls(prob, **opts)
    assert projected_pairs, "no ridge evaluation recorded"
    assert max(projected_pairs) <= 1e-12, projected_pairs

"""The CPU model of the reduced-basis sweeps (oracle/reduced_sweeps.py): the
two facts the mixed-precision form is built around, at sizes that run in
seconds.

1. One solve with reduced sweeps on an ill-conditioned problem (4000 x 1000
   CSR, column scales over 6 decades, lambda = 0): V stays orthogonal to
   about the reduced precision, but the left basis U, reorthogonalised only
   against its previous vector, loses orthogonality by orders of magnitude
   more, and the backward error after 600 levels is far above the
   FP64-swept solve's.  This is why the reduced sweeps run only inside
   restart cycles.
2. FP64 residual correction around restart cycles of 100 levels on a
   regularised problem (20000 x 5000 CSR, lambda = 1e-2): cycles swept on an
   FP32 or FP16 copy of the basis track the FP64-swept cycles' energy errors
   to within 1% at every cycle, down to below 1e-9.
"""
import numpy as np
import pytest
import scipy.linalg as sl
import scipy.sparse as sp

from amfls_solver_gb300 import problems
from oracle import reduced_sweeps as rs


def csr_matrix(p):
    return sp.csr_matrix((p.values, p.column_indices, p.row_offsets), shape=(p.rows, p.cols))


@pytest.fixture(scope="module")
def one_shot():
    p = problems.scaled_uniform_csr(4000, 1000, per_row=10, decades=6.0, noise=1e-8, seed=3)
    a = csr_matrix(p)
    out = {}
    for storage in ("fp64", "fp32"):
        gk = rs.GolubKahan(a, 600, storage)
        x = gk.solve(p.b, 600)
        r = p.b - a @ x
        backward = np.linalg.norm(a.T @ r) / np.linalg.norm(r)
        out[storage] = (rs.orthogonality_loss(gk.V), rs.orthogonality_loss(np.stack(gk.U, 1)),
                        backward, gk)
    return out


def test_one_shot_reduced_sweeps_lose_left_orthogonality(one_shot):
    v64, u64, be64, _ = one_shot["fp64"]
    v32, u32, be32, gk = one_shot["fp32"]
    assert v64 < 1e-12 and u64 < 1e-9
    assert v32 < 1e-6                  # V: about the FP32 level
    assert u32 > 1e-4 and u32 > 1e3 * v32  # U: amplified
    assert be32 > 10 * be64            # and the solve stalls
    assert gk.reduced_passes == 599


@pytest.fixture(scope="module")
def ridge():
    lam = 1e-2
    p = problems.scaled_uniform_csr(20000, 5000, per_row=10, decades=3.0, noise=1e-6, seed=5)
    a = csr_matrix(p)
    m = sp.vstack([a, np.sqrt(lam) * sp.identity(p.cols)]).tocsr()
    c = np.concatenate([p.b, np.zeros(p.cols)])
    normal = (a.T @ a).toarray() + lam * np.eye(p.cols)
    x_exact = sl.cho_solve(sl.cho_factor(normal), a.T @ p.b)
    return m, c, x_exact


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_restart_cycles_on_a_reduced_copy_track_fp64(ridge, storage):
    m, c, x_exact = ridge
    _, e64, _, _ = rs.restart_cycles(m, c, 100, 8, "fp64", x_exact)
    _, e, passes, fallbacks = rs.restart_cycles(m, c, 100, 8, storage, x_exact)
    assert passes == 8 * 99
    assert fallbacks == 0
    assert all(abs(a - b) <= 0.01 * b for a, b in zip(e, e64)), (e, e64)
    assert all(b < a for a, b in zip(e, e[1:]))
    assert e[-1] < 1e-9


def test_model_rejects_unknown_storage():
    with pytest.raises(ValueError):
        rs.GolubKahan(sp.identity(3).tocsr(), 2, "bf16")

"""CPU model of the reduced-basis sweeps of the mixed-precision form -- test
infrastructure only (nothing in the product imports it).

The reduced-basis sweeps have no counterpart in the reference; this module
restates, in numpy, the width-one Golub-Kahan recurrence of the reference's
workspace (krylov_workspace.cpp:589-831: right residual A^T u - beta v_prev
reorthogonalised against the whole right basis V with a DGKS second pass
(:82-310), left residual A v - alpha u reorthogonalised against the previous
left vector only, T's entries alpha + left coefficient and beta, g = U^T b,
the projected least-squares solve of :833-909) with the first right pass
optionally run the way the GPU's reduced sweeps run it:

    c = V~^T fl32(r)          (V~ the FP32 copy of V, or the FP16 copy of
                               2^8 V scaled back by 2^-8; products of the
                               rounded operands summed in FP64 here, in FP32
                               runs folded into FP64 on the GPU)
    if ||c|| > 1e-3 ||r||:    redo the pass in FP64 (counted as a fallback)
    else:                     r <- r - fl64(fl32(V~ fl32(c)))

and the DGKS second pass always in FP64.  `restart_cycles` adds the FP64
residual correction around restart cycles of L levels (each inner solve
returns its latest iterate at the depth limit).

It exists to show, on the CPU and at sizes that run in seconds, the two
facts the mixed form is designed around: a single solve with reduced sweeps
keeps V orthogonal to the reduced precision, but the one-sided scheme lets
the left basis U lose orthogonality by orders of magnitude more, so the
solve stalls; restart cycles on a regularised problem, where each cycle
needs only a few digits, track FP64-swept cycles to rounding.
"""
from __future__ import annotations

import numpy as np

REDUCED_COEFF_BOUND = 1e-3
STORAGES = ("fp64", "fp32", "fp16")


def _copy(v, storage):
    if storage == "fp32":
        return v.astype(np.float32)
    return (v * 256.0).astype(np.float32).astype(np.float16)


class GolubKahan:
    """Width-one levels on an operator M (scipy sparse), right basis swept
    in FP64 or on a reduced copy (`storage` "fp64", "fp32" or "fp16")."""

    def __init__(self, M, levels, storage="fp64"):
        if storage not in STORAGES:
            raise ValueError(f"storage must be one of {STORAGES}")
        self.M = M.tocsr()
        self.MT = M.T.tocsr()
        self.n = M.shape[1]
        self.storage = storage
        self.scale = 1.0 / 256.0 if storage == "fp16" else 1.0
        self.V = np.zeros((self.n, levels))
        self.W = None if storage == "fp64" else np.zeros(
            (self.n, levels), dtype=np.float32 if storage == "fp32" else np.float16)
        self.k = 0
        self.reduced_passes = 0
        self.fallbacks = 0
        self.U = []

    def _pass_fp64(self, r):
        vk = self.V[:, :self.k]
        return r - vk @ (vk.T @ r)

    def _pass_reduced(self, r):
        wk = self.W[:, :self.k]
        self.reduced_passes += 1
        c = (wk.astype(np.float64).T @ r.astype(np.float32).astype(np.float64)) * self.scale
        if not np.linalg.norm(c) <= REDUCED_COEFF_BOUND * np.linalg.norm(r):
            self.fallbacks += 1
            return self._pass_fp64(r)
        y = wk.astype(np.float32) @ c.astype(np.float32)  # FP32 sums
        return r - y.astype(np.float64) * self.scale

    def solve(self, rhs, levels):
        """`levels` width-one levels from u_1 = rhs / ||rhs||; returns the
        projected least-squares iterate x = V y."""
        beta = np.linalg.norm(rhs)
        u = rhs / beta
        self.U = [u]
        g = [u @ rhs]
        t = np.zeros((levels + 1, levels))
        beta_prev = 0.0
        for j in range(levels):
            r = self.MT @ u
            if j > 0:
                r = r - beta_prev * self.V[:, j - 1]
            if self.k > 0:
                before = np.linalg.norm(r)
                r = self._pass_fp64(r) if self.W is None else self._pass_reduced(r)
                if np.linalg.norm(r) < np.sqrt(0.5) * before:
                    r = self._pass_fp64(r)
            alpha = np.linalg.norm(r)
            v = r / alpha
            self.V[:, self.k] = v
            if self.W is not None:
                self.W[:, self.k] = _copy(v, self.storage)
            self.k += 1
            y = self.M @ v - alpha * u
            before = np.linalg.norm(y)
            coef = u @ y
            y = y - coef * u
            if np.linalg.norm(y) < np.sqrt(0.5) * before:
                extra = u @ y
                y = y - extra * u
                coef += extra
            beta_prev = np.linalg.norm(y)
            u = y / beta_prev
            self.U.append(u)
            g.append(u @ rhs)
            t[j, j] = alpha + coef
            t[j + 1, j] = beta_prev
        coeffs = np.linalg.lstsq(t, np.asarray(g), rcond=None)[0]
        return self.V[:, :levels] @ coeffs


def orthogonality_loss(q):
    """max |Q^T Q - I|."""
    q = np.asarray(q)
    return float(np.abs(q.T @ q - np.eye(q.shape[1])).max())


def restart_cycles(M, c, levels, cycles, storage="fp64", x_exact=None):
    """FP64 residual correction x <- x - d, d the latest iterate of a cycle of
    `levels` levels on min ||M d - (M x - c)||.  Returns x, the relative
    energy error ||M (x - x*)|| / ||M x*|| after each cycle (when x_exact is
    given), and the reduced passes and fallbacks of all cycles."""
    x = np.zeros(M.shape[1])
    errors, passes, fallbacks = [], 0, 0
    ref = None if x_exact is None else np.linalg.norm(M @ x_exact)
    for _ in range(cycles):
        gk = GolubKahan(M, levels, storage)
        x = x - gk.solve(M @ x - c, levels)
        passes += gk.reduced_passes
        fallbacks += gk.fallbacks
        if ref is not None:
            errors.append(float(np.linalg.norm(M @ (x - x_exact)) / ref))
    return x, errors, passes, fallbacks

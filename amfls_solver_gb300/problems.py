"""Seeded synthetic least-squares problems with the shapes of the AMFLS workloads.

No public dataset is involved: every matrix is drawn from a numpy
``Generator`` seeded by the caller, so a (family, sizes, seed) triple names a
problem exactly.  CSR matrices are returned as numpy arrays
(``row_offsets`` int64, ``column_indices`` int64 sorted within each row,
``values`` float64), the layout ``torch.sparse_csr_tensor`` and the reference's
``SparseCsrOperator`` both accept (sparse_csr_operator.hpp:13-21).

Families
--------
``scaled_uniform_csr``  fixed nonzeros per row at distinct uniform columns,
    N(0,1) values with column j scaled by 10^(-decades*j/n); b = A x + noise.
    At m=20000, n=5000, 10 per row, 6 decades, noise 1e-8 this is the
    CPU-runnable 20000x5000 CSR workload.
``power_law_csr``  row lengths L = min(L_max, ceil(x_m U^-2)), U ~ U(0,1]
    (tail exponent 1.5); with x_m = 0.04688 the mean is 20 and nnz is about
    20 m.  At m=2,000,000, n=500,000, 8 decades, noise 1e-6 this is the
    2Mx500k CSR workload.
``banded_random_csr``  a band of ``band`` columns centred on floor(i n / m)
    plus ``off_band`` distinct uniform columns, 10^(-decades*j/n) scaling
    (the 4Mx1M learned-width family).
``scaled_dense``  G diag(d) with G i.i.d. N(0,1), d geometric from 1 to
    10^-decades, b ~ N(0,1) (the 100000x2000 dense workload).
``portable_dense`` / ``portable_csr``  the same shapes from integer draws
    and power-of-two scalings only: bit-identical on every platform (the
    families above call libm, whose last bits differ between machines).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CsrProblem:
    rows: int
    cols: int
    row_offsets: np.ndarray
    column_indices: np.ndarray
    values: np.ndarray
    b: np.ndarray
    x_true: np.ndarray | None = None

    @property
    def nnz(self) -> int:
        return int(self.values.shape[0])

    def to_dense(self) -> np.ndarray:
        a = np.zeros((self.rows, self.cols))
        row_ids = np.repeat(np.arange(self.rows), np.diff(self.row_offsets))
        a[row_ids, self.column_indices] = self.values
        return a

    def matvec(self, x: np.ndarray) -> np.ndarray:
        row_ids = np.repeat(np.arange(self.rows), np.diff(self.row_offsets))
        return np.bincount(row_ids, weights=self.values * x[self.column_indices],
                           minlength=self.rows)


@dataclass
class DenseProblem:
    matrix: np.ndarray  # shape (rows, cols); contiguity tells the layout
    b: np.ndarray

    @property
    def rows(self) -> int:
        return int(self.matrix.shape[0])

    @property
    def cols(self) -> int:
        return int(self.matrix.shape[1])

    def to_dense(self) -> np.ndarray:
        return np.asarray(self.matrix)

    def matvec(self, x: np.ndarray) -> np.ndarray:
        return self.matrix @ x


def _distinct_columns(rng: np.random.Generator, lengths: np.ndarray, n: int) -> np.ndarray:
    """Uniform column indices, distinct within each row, sorted within each row."""
    lengths = np.minimum(lengths.astype(np.int64), n)
    total = int(lengths.sum())
    row_ids = np.repeat(np.arange(lengths.shape[0], dtype=np.int64), lengths)
    cols = rng.integers(0, n, size=total, dtype=np.int64)
    while True:
        key = row_ids * n + cols
        order = np.argsort(key, kind="stable")
        key_sorted = key[order]
        dup = np.zeros(total, dtype=bool)
        dup[1:] = key_sorted[1:] == key_sorted[:-1]
        if not dup.any():
            return key_sorted - row_ids * n  # rows stay in order; columns sorted
        redo = order[dup]
        cols[redo] = rng.integers(0, n, size=redo.shape[0], dtype=np.int64)


def _finish_csr(rng, m, n, lengths, cols, decades, noise):
    offsets = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    values = rng.standard_normal(cols.shape[0])
    values *= 10.0 ** (-decades * cols.astype(np.float64) / n)
    prob = CsrProblem(m, n, offsets, cols, values, np.zeros(m))
    x_true = rng.standard_normal(n)
    b = prob.matvec(x_true)
    if noise:
        b = b + noise * rng.standard_normal(m)
    prob.b = b
    prob.x_true = x_true
    return prob


def scaled_uniform_csr(m: int, n: int, per_row: int = 10, decades: float = 6.0,
                       noise: float = 1e-8, seed: int = 0) -> CsrProblem:
    rng = np.random.default_rng(seed)
    lengths = np.full(m, min(per_row, n), dtype=np.int64)
    cols = _distinct_columns(rng, lengths, n)
    return _finish_csr(rng, m, n, lengths, cols, decades, noise)


def power_law_csr(m: int, n: int, x_m: float = 0.04688, max_row: int = 2000,
                  decades: float = 8.0, noise: float = 1e-6, seed: int = 0) -> CsrProblem:
    rng = np.random.default_rng(seed)
    u = 1.0 - rng.random(m)  # (0, 1]
    lengths = np.minimum(max_row, np.ceil(x_m * u ** -2.0)).astype(np.int64)
    lengths = np.minimum(np.maximum(lengths, 1), n)
    cols = _distinct_columns(rng, lengths, n)
    return _finish_csr(rng, m, n, lengths, cols, decades, noise)


def banded_random_csr(m: int, n: int, band: int = 8, off_band: int = 8,
                      decades: float = 9.0, noise: float = 0.0, seed: int = 0) -> CsrProblem:
    rng = np.random.default_rng(seed)
    centre = (np.arange(m, dtype=np.int64) * n) // m
    start = np.clip(centre - band // 2, 0, max(0, n - band))
    band_cols = start[:, None] + np.arange(band, dtype=np.int64)[None, :]
    extra = _distinct_columns(rng, np.full(m, off_band + band, dtype=np.int64), n)
    extra = extra.reshape(m, off_band + band)
    merged = []
    for i in range(0, m, 65536):  # keep the per-chunk work bounded
        b_c = band_cols[i:i + 65536]
        e_c = extra[i:i + 65536]
        keep = ~(e_c[:, :, None] == b_c[:, None, :]).any(axis=2)
        # take the first off_band extra columns that miss the band
        rank = np.cumsum(keep, axis=1)
        sel = keep & (rank <= off_band)
        rows_sel = np.where(sel.sum(axis=1) == off_band)[0]
        if rows_sel.shape[0] != b_c.shape[0]:
            raise RuntimeError("band overlap exhausted the off-band candidates")
        chosen = e_c[sel].reshape(-1, off_band)
        merged.append(np.sort(np.concatenate([b_c, chosen], axis=1), axis=1))
    cols = np.concatenate(merged, axis=0).reshape(-1)
    lengths = np.full(m, band + off_band, dtype=np.int64)
    return _finish_csr(rng, m, n, lengths, cols, decades, noise)


def scaled_dense(m: int, n: int, decades: float = 6.0, seed: int = 0,
                 column_major: bool = True) -> DenseProblem:
    rng = np.random.default_rng(seed)
    d = 10.0 ** (-decades * np.arange(n) / max(1, n - 1))
    if column_major:
        g = np.asfortranarray(rng.standard_normal((n, m)).T)
    else:
        g = rng.standard_normal((m, n))
    g *= d[None, :]
    b = rng.standard_normal(m)
    return DenseProblem(g, b)


def portable_dense(m: int, n: int, octaves: int = 20, seed: int = 0,
                   column_major: bool = True) -> DenseProblem:
    """G diag(d) built from integer draws only: G_ij = k_ij 2^-20 with k_ij
    uniform in [-2^20, 2^20], d_j = 2^-floor(octaves j / (n - 1)) (condition
    about 2^octaves), b_i = k_i 2^-20.  Integer streams of a seeded numpy
    Generator and exact power-of-two scalings involve no libm call, so the
    arrays are the same bytes on every platform (the generators above use
    exp / log / pow, whose last bits differ between x86-64 and AArch64)."""
    rng = np.random.default_rng(seed)
    lim = 1 << 20
    shape = (n, m) if column_major else (m, n)
    g = np.ldexp(rng.integers(-lim, lim, size=shape, endpoint=True).astype(np.float64), -20)
    if column_major:
        g = np.asfortranarray(g.T)
    d = np.ldexp(1.0, -((octaves * np.arange(n)) // max(1, n - 1)))
    g *= d[None, :]
    b = np.ldexp(rng.integers(-lim, lim, size=m, endpoint=True).astype(np.float64), -20)
    return DenseProblem(g, b)


def portable_csr(m: int, n: int, per_row: int = 10, octaves: int = 20, noise_bits: int = 27,
                 seed: int = 0) -> CsrProblem:
    """CSR counterpart of portable_dense: per_row distinct uniform columns per
    row, values k 2^-20 scaled by 2^-floor(octaves j / n), b = A x_true plus
    integer noise of 2^-noise_bits units, x_true_j = k_j 2^-20.  The same
    bytes on every platform (b's sums are IEEE additions in a fixed order)."""
    rng = np.random.default_rng(seed)
    lim = 1 << 20
    lengths = np.full(m, min(per_row, n), dtype=np.int64)
    cols = _distinct_columns(rng, lengths, n)
    offsets = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    values = np.ldexp(rng.integers(-lim, lim, size=cols.shape[0], endpoint=True)
                      .astype(np.float64), -20)
    values *= np.ldexp(1.0, -((octaves * cols) // n))
    prob = CsrProblem(m, n, offsets, cols, values, np.zeros(m))
    x_true = np.ldexp(rng.integers(-lim, lim, size=n, endpoint=True).astype(np.float64), -20)
    row_ids = np.repeat(np.arange(m), lengths)
    b = np.zeros(m)
    np.add.at(b, row_ids, values * x_true[cols])  # sequential per element: fixed order
    b += np.ldexp(rng.integers(-lim, lim, size=m, endpoint=True).astype(np.float64),
                  -20 - noise_bits)
    prob.b = b
    prob.x_true = x_true
    return prob


def uneven_csr_batch(count: int = 256, seed: int = 0, m_range=(2_000, 200_000),
                     n_range=(500, 50_000), per_row=(5, 40), cond_range=(1e3, 1e8),
                     reg_range=(1e-8, 1e-2), tolerance: float = 1e-9, noise: float = 1e-8):
    """Independent CSR least-squares problems of uneven size: m and n
    log-uniform (n <= 2 m), 5..40 nonzeros per row (uniform per row), N(0,1)
    values with geometric column scaling to a log-uniform condition, lambda
    log-uniform; b = A x_true + noise.  Returns [(problem, lambda, tol)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        m = int(np.exp(rng.uniform(np.log(m_range[0]), np.log(m_range[1]))))
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        n = max(1, min(n, 2 * m))
        decades = float(rng.uniform(np.log10(cond_range[0]), np.log10(cond_range[1])))
        reg = float(np.exp(rng.uniform(np.log(reg_range[0]), np.log(reg_range[1]))))
        prng = np.random.default_rng([seed, i])
        lengths = prng.integers(per_row[0], per_row[1] + 1, size=m)
        cols = _distinct_columns(prng, lengths, n)
        prob = _finish_csr(prng, m, n, np.minimum(lengths, n), cols, decades, noise)
        out.append((prob, reg, tolerance))
    return out


# The named workloads (full sizes).  Each entry gives the generator, its
# keyword arguments and the solver options.
WORKLOADS = {
    "csr_20000x5000": dict(
        family="scaled_uniform_csr",
        kwargs=dict(m=20000, n=5000, per_row=10, decades=6.0, noise=1e-8),
        options=dict(regularization=0.0, tolerance=1e-8)),
    "dense_100000x2000": dict(
        family="scaled_dense",
        kwargs=dict(m=100000, n=2000, decades=6.0),
        options=dict(regularization=1e-6, tolerance=1e-10)),
    "csr_2000000x500000": dict(
        family="power_law_csr",
        kwargs=dict(m=2_000_000, n=500_000, decades=8.0, noise=1e-6),
        options=dict(regularization=1e-4, tolerance=1e-10)),
    "csr_4000000x1000000": dict(
        family="banded_random_csr",
        kwargs=dict(m=4_000_000, n=1_000_000, decades=9.0),
        options=dict(regularization=0.0, tolerance=1e-10, maximum_auxiliary_width=64)),
}

FAMILIES = {
    "portable_dense": portable_dense,
    "portable_csr": portable_csr,
    "scaled_uniform_csr": scaled_uniform_csr,
    "power_law_csr": power_law_csr,
    "banded_random_csr": banded_random_csr,
    "scaled_dense": scaled_dense,
}


def make(name: str, seed: int = 0, **overrides):
    spec = WORKLOADS[name]
    kwargs = dict(spec["kwargs"])
    kwargs.update(overrides)
    return FAMILIES[spec["family"]](seed=seed, **kwargs), dict(spec["options"])

"""The seeded workload generators against the shapes they promise.

The bench and the GPU tests name problems by (family, sizes, seed); these
checks hold the generators to the structure those names stand for, at sizes
that run in seconds:
  * CSR layout: int64 offsets from 0 to nnz, columns distinct and sorted
    within each row, values scaled by 10^(-decades j / n) by column;
  * the power-law row lengths of the 2,000,000 x 500,000 workload:
    L = min(2000, ceil(x_m U^-2)), mean about 20, P(L = 1) = 1 - sqrt(x_m);
  * the band of the 4,000,000 x 1,000,000 family: every row holds its band
    of 8 columns centred on floor(i n / m) plus 8 distinct off-band columns;
  * the uneven batch: sizes, nonzeros per row and lambda inside their ranges;
  * the portable families: the same bytes on every run (pinned digests).
"""
import hashlib

import numpy as np
import pytest

from amfls_solver_gb300 import problems


def check_csr_layout(p):
    off, col = p.row_offsets, p.column_indices
    assert off.dtype == np.int64 and col.dtype == np.int64 and p.values.dtype == np.float64
    assert off[0] == 0 and off[-1] == p.nnz and np.all(np.diff(off) >= 0)
    assert col.min() >= 0 and col.max() < p.cols
    row_ids = np.repeat(np.arange(p.rows), np.diff(off))
    same_row = row_ids[1:] == row_ids[:-1]
    assert np.all(col[1:][same_row] > col[:-1][same_row])  # distinct and sorted
    assert p.b.shape == (p.rows,)


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def test_scaled_uniform_csr():
    p = problems.scaled_uniform_csr(3000, 700, per_row=10, decades=6.0, noise=0.0, seed=2)
    check_csr_layout(p)
    assert np.all(np.diff(p.row_offsets) == 10)
    # N(0,1) values under the column scale: |v| / scale is a half-normal sample
    scale = 10.0 ** (-6.0 * p.column_indices / 700)
    z = np.abs(p.values) / scale
    assert 0.75 < np.mean(z) < 0.85  # E|N(0,1)| = 0.798
    assert np.allclose(p.matvec(p.x_true), p.b, rtol=0, atol=1e-12)  # noise 0: b = A x_true
    q = problems.scaled_uniform_csr(3000, 700, per_row=10, decades=6.0, noise=0.0, seed=2)
    assert np.array_equal(p.values, q.values) and np.array_equal(p.b, q.b)


def test_power_law_row_lengths():
    m, n = 200_000, 50_000
    p = problems.power_law_csr(m, n, seed=5)
    check_csr_layout(p)
    lengths = np.diff(p.row_offsets)
    assert lengths.min() == 1 and lengths.max() <= 2000
    # P(ceil(x_m U^-2) = 1) = P(U >= sqrt(x_m)) = 1 - sqrt(0.04688) = 0.7835
    assert abs(np.mean(lengths == 1) - (1 - np.sqrt(0.04688))) < 0.006
    # mean 20 (the heavy tail leaves a spread of about 0.4 at this m)
    assert 18.5 < lengths.mean() < 21.5
    assert np.any(lengths == 2000)  # the truncation is reached


def test_banded_rows_hold_their_band():
    m, n, band, off_band = 20_000, 5_000, 8, 8
    p = problems.banded_random_csr(m, n, band=band, off_band=off_band, seed=1)
    check_csr_layout(p)
    assert np.all(np.diff(p.row_offsets) == band + off_band)
    cols = p.column_indices.reshape(m, band + off_band)
    centre = (np.arange(m) * n) // m
    start = np.clip(centre - band // 2, 0, n - band)
    for k in range(band):
        assert np.all((cols == (start + k)[:, None]).any(axis=1))
    in_band = (cols >= start[:, None]) & (cols < (start + band)[:, None])
    assert np.all(in_band.sum(axis=1) == band)  # the off-band columns miss the band


def test_uneven_batch_ranges():
    batch = problems.uneven_csr_batch(count=6, seed=4, m_range=(2_000, 20_000),
                                      n_range=(500, 5_000))
    assert len(batch) == 6
    for prob, reg, tol in batch:
        check_csr_layout(prob)
        assert 2_000 <= prob.rows <= 20_000 and 1 <= prob.cols <= min(5_000, 2 * prob.rows)
        lengths = np.diff(prob.row_offsets)
        assert lengths.min() >= min(5, prob.cols) and lengths.max() <= min(40, prob.cols)
        assert 1e-8 <= reg <= 1e-2 and tol == 1e-9
    again = problems.uneven_csr_batch(count=6, seed=4, m_range=(2_000, 20_000),
                                      n_range=(500, 5_000))
    assert all(np.array_equal(a[0].values, b[0].values) and a[1] == b[1]
               for a, b in zip(batch, again))


def test_portable_families_are_pinned():
    p = problems.portable_csr(2000, 500, seed=3)
    check_csr_layout(p)
    assert digest(p.row_offsets, p.column_indices, p.values, p.b, p.x_true) == "2d448dd1c1db2b0b"
    d = problems.portable_dense(300, 40, seed=1)
    assert d.matrix.flags.f_contiguous
    assert digest(np.asarray(d.matrix, order="F"), d.b) == "147bf7b76626c2a6"
    r = problems.portable_dense(300, 40, seed=1, column_major=False)
    assert r.matrix.flags.c_contiguous
    assert digest(r.matrix, r.b) == "b597baefcc1888f8"


def test_make_applies_overrides_and_returns_the_options():
    p, opts = problems.make("csr_20000x5000", seed=7, m=500, n=120)
    assert (p.rows, p.cols) == (500, 120)
    assert opts == {"regularization": 0.0, "tolerance": 1e-8}
    _, opts3 = problems.make("csr_2000000x500000", seed=7, m=400, n=100)
    assert opts3 == {"regularization": 1e-4, "tolerance": 1e-10}
    with pytest.raises(KeyError):
        problems.make("no_such_workload")

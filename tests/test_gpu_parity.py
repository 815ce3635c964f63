"""GPU parity: the CUDA path against the reference's fixtures and the oracle.

Tolerances:
  * operator products: |y - y_ref| <= gamma_{2L+2} (|A| |x|)_i elementwise
    (L = row length), the reference's own rounding model for one product;
  * norm model: upper/lower bounds within 1e-13 relative, rounding steps exact;
  * end-to-end CSR solves: identical status, stop reason, depth, basis rank,
    search counters and per-checkpoint outcomes.  x itself is determined only
    to about cond(A) * tol by a backward-error stopping test (the reference's
    own x differs from a dense lstsq by 1e-4 on the 20000x5000 problem), so
    the checks on x are the ones the problem fixes: the backward error (or,
    for lambda > 0, the relative energy error against the exact ridge
    solution from a dense solve) recomputed on the host is at most tol, and
    ||x - x_ref|| <= 4 cond(A) tol ||x_ref|| (lambda = 0) or
    ||x - x_ref||_H <= 2.5 tol ||x_ref||_H (lambda > 0).
"""
import numpy as np
import pytest
import torch

from conftest import SOLVE_FIXTURES, golden_options, load_golden
from oracle import amfls_oracle as orc

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


@pytest.fixture(scope="module")
def amfls():
    import amfls_solver_gb300 as m

    m.load_library()
    return m


def csr_tensor(prob, dev="cuda"):
    return torch.sparse_csr_tensor(torch.from_numpy(prob.row_offsets),
                                   torch.from_numpy(prob.column_indices),
                                   torch.from_numpy(prob.values),
                                   size=(prob.rows, prob.cols), dtype=torch.float64).to(dev)


def product_bound(prob, x, transpose):
    """gamma_{2L+2} (|A| |x|) with L the longest row (or column)."""
    absp = type(prob)(prob.rows, prob.cols, prob.row_offsets, prob.column_indices,
                      np.abs(prob.values), prob.b)
    op = orc.Operator(absp)
    ax = np.abs(x)
    out = op.apply_transpose(ax) if transpose else op.apply(ax)
    lens = np.diff(prob.row_offsets)
    L = lens.max() if not transpose else np.bincount(prob.column_indices,
                                                     minlength=prob.cols).max()
    k = 2 * L + 2
    return out[:, 0] * (k * EPS / 2) / (1 - k * EPS / 2) + 1e-300


def check_solution(prob, x, xr, reg, tol, success):
    """Host float64 checks of what the problem determines (see module docstring)."""
    a = prob.to_dense()
    s = np.linalg.svd(a, compute_uv=False)
    norm_a = s[0]
    b = prob.b
    if reg == 0.0:
        if success and np.any(b):
            r = a @ x - b
            compat = np.linalg.norm(r) / (norm_a * np.linalg.norm(x) + np.linalg.norm(b))
            ls = np.linalg.norm(a.T @ r) / (norm_a * np.linalg.norm(r)) if np.any(r) else 0.0
            assert min(compat, ls) <= tol * (1 + 1e-3)
        smin = s[s > s[0] * 1e-12][-1]
        cond = norm_a / smin
        if s[-1] > s[0] * 1e-12:  # full column rank: x is unique up to cond * tol
            assert np.linalg.norm(x - xr) <= 4 * cond * tol * np.linalg.norm(xr) + 1e-300
    else:
        aug = np.vstack([a, np.sqrt(reg) * np.eye(a.shape[1])])
        xl = np.linalg.lstsq(aug, np.concatenate([b, np.zeros(a.shape[1])]), rcond=None)[0]
        hnorm = lambda v: np.sqrt(np.linalg.norm(a @ v) ** 2 + reg * np.linalg.norm(v) ** 2)
        if success:
            assert hnorm(x - xl) <= tol * hnorm(x) * (1 + 1e-3)
        assert hnorm(x - xr) <= 2.5 * tol * hnorm(xr) + 1e-300


@pytest.mark.parametrize("name", ["csr_products", "csr_ragged"])
def test_csr_products_match_reference(amfls, name):
    data, prob = load_golden(name)
    op = amfls.DeviceOperator(csr_tensor(prob))
    x = data["x"][:, 0] if data["x"].ndim == 2 else data["x"]
    y = data["y"][:, 0] if data["y"].ndim == 2 else data["y"]
    ax = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    aty = op.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()
    assert np.all(np.abs(ax - data["ax1"]) <= 2 * product_bound(prob, x, False))
    assert np.all(np.abs(aty - data["aty1"]) <= 2 * product_bound(prob, y, True))
    if "ax3" in data:
        X = torch.from_numpy(np.ascontiguousarray(data["x"])).cuda()
        Y = torch.from_numpy(np.ascontiguousarray(data["y"])).cuda()
        AX = op.apply(X).cpu().numpy()
        ATY = op.apply(Y, transpose=True).cpu().numpy()
        for c in range(X.shape[1]):
            assert np.all(np.abs(AX[:, c] - data["ax3"][:, c]) <=
                          2 * product_bound(prob, data["x"][:, c], False))
            assert np.all(np.abs(ATY[:, c] - data["aty3"][:, c]) <=
                          2 * product_bound(prob, data["y"][:, c], True))
    up, lo, sa, st = op.validation_error_model()
    np.testing.assert_allclose([up, lo], data["model"], rtol=1e-13)
    assert [sa, st] == list(data["steps"])


def skewed_csr(seed=7, m=6000, n=6000):
    """Rows of length 0..3 mixed with a few rows longer than one 2048-element
    tile (split into slices) and a column present in every row (a transpose
    row of m entries)."""
    from amfls_solver_gb300 import problems

    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 4, m)
    lens[rng.choice(m, 6, replace=False)] = [300, 2047, 2048, 2049, 4500, n]
    rows = []
    for i, ln in enumerate(lens):
        c = rng.choice(np.arange(1, n), min(int(ln), n - 1), replace=False)
        rows.append(np.sort(np.concatenate([[0], c]) if i % 3 else c))
    off = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int64)
    col = np.concatenate(rows).astype(np.int64)
    val = rng.standard_normal(col.size)
    return problems.CsrProblem(m, n, off, col, val, np.zeros(m))


@pytest.mark.parametrize("chains", ["0", "1"])
def test_csr_tiled_products_long_and_empty_rows(amfls, monkeypatch, chains):
    """Tiled products (row blocks or chain groups, slices of long rows, empty
    rows) against the oracle's sequential products within gamma_{2L+2}
    |A||x|, for 1..11 columns, and bit-identical on a repeat."""
    monkeypatch.setenv("AMFLS_GB300_CSR_CHAINS", chains)
    prob = skewed_csr()
    op = amfls.DeviceOperator(csr_tensor(prob))
    ref = orc.Operator(prob)
    rng = np.random.default_rng(3)
    for s in (1, 2, 3, 5, 8, 11):
        x = rng.standard_normal((prob.cols, s))
        y = rng.standard_normal((prob.rows, s))
        ax = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        aty = op.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()
        ax_ref = ref.apply(np.asfortranarray(x))
        aty_ref = ref.apply_transpose(np.asfortranarray(y))
        for c in range(s):
            assert np.all(np.abs(ax[:, c] - ax_ref[:, c]) <= 2 * product_bound(prob, x[:, c], False))
            assert np.all(np.abs(aty[:, c] - aty_ref[:, c]) <=
                          2 * product_bound(prob, y[:, c], True))
        again = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        assert np.array_equal(ax, again)
    lens = np.diff(prob.row_offsets)
    assert np.all(ax[lens == 0] == 0.0)


def chain_csr(seed=11, m=5000, n=700):
    """Every row length from 0 to 300 (most rows short) in shuffled order, so
    single-column products see chain groups from windows of short rows, chain
    groups of rows sorted by length up to 64, and whole long rows; columns
    hold about 100-170 entries each (whole rows on the transpose side)."""
    from amfls_solver_gb300 import problems

    rng = np.random.default_rng(seed)
    lens = np.concatenate([np.arange(301), rng.integers(0, 5, 3500),
                           rng.integers(5, 65, m - 301 - 3500)])
    rng.shuffle(lens)
    rows = [np.sort(rng.choice(n, int(ln), replace=False)) for ln in lens]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    col = np.concatenate(rows).astype(np.int64)
    val = rng.standard_normal(col.size)
    return problems.CsrProblem(m, n, off, col, val, np.zeros(m))


@pytest.mark.parametrize("chains", ["0", "1"])
def test_csr_single_column_chains_bit_exact(amfls, monkeypatch, chains):
    """Single-column products sum every row (and column) of up to 64
    nonzeros as one FMA chain in storage order from 0, as the reference's
    SparseCsrOperator::apply / apply_transpose do -- in chain groups and in
    row blocks -- so those entries are bit-identical to the oracle's; longer
    ones are within gamma_{2L+2}."""
    monkeypatch.setenv("AMFLS_GB300_CSR_CHAINS", chains)
    prob = chain_csr()
    op = amfls.DeviceOperator(csr_tensor(prob))
    ref = orc.Operator(prob)
    rng = np.random.default_rng(5)
    x = rng.standard_normal((prob.cols, 1))
    y = rng.standard_normal((prob.rows, 1))
    ax = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()[:, 0]
    aty = op.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()[:, 0]
    ax_ref = ref.apply(np.asfortranarray(x))[:, 0]
    aty_ref = ref.apply_transpose(np.asfortranarray(y))[:, 0]
    lens = np.diff(prob.row_offsets)
    clens = np.bincount(prob.column_indices, minlength=prob.cols)
    assert (lens > 64).any() and (lens <= 64).sum() > 4000
    assert np.array_equal(ax[lens <= 64], ax_ref[lens <= 64])
    assert np.array_equal(aty[clens <= 64], aty_ref[clens <= 64])
    assert np.all(np.abs(ax - ax_ref) <= 2 * product_bound(prob, x[:, 0], False))
    assert np.all(np.abs(aty - aty_ref) <= 2 * product_bound(prob, y[:, 0], True))


@pytest.mark.parametrize("name", ["dense_model_rm", "dense_model_cm"])
def test_dense_model_matches_reference(amfls, name):
    data, prob = load_golden(name)
    mat = torch.from_numpy(np.ascontiguousarray(prob.matrix)).cuda()
    op = amfls.DeviceOperator(mat)
    up, lo, sa, st = op.validation_error_model()
    np.testing.assert_allclose([up, lo], data["model"], rtol=1e-13)
    assert [sa, st] == list(data["steps"])
    x = np.random.default_rng(1).standard_normal(prob.cols)
    y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = prob.matrix @ x
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(prob.matrix) @ np.abs(x))
    yy = np.random.default_rng(2).standard_normal(prob.rows)
    t = op.apply(torch.from_numpy(yy).cuda(), transpose=True).cpu().numpy()
    assert np.max(np.abs(t - prob.matrix.T @ yy)) <= 1e-12 * np.max(
        np.abs(prob.matrix.T) @ np.abs(yy))


@pytest.mark.parametrize("layout", ["row", "col"])
@pytest.mark.parametrize("s", [1, 2, 3, 8, 11])
def test_dense_block_products(amfls, layout, s):
    """Block products read A once per eight columns; each column must equal a
    plain float64 product to rounding (|error| <= gamma_{n+2} |A| |x|)."""
    rng = np.random.default_rng(s)
    m, n = 3001, 517
    a = rng.standard_normal((m, n))
    t = torch.from_numpy(a).cuda() if layout == "row" else \
        torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    op = amfls.DeviceOperator(t)
    x = rng.standard_normal((n, s))
    y = rng.standard_normal((m, s))
    ax = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    aty = op.apply(torch.from_numpy(y).cuda(), transpose=True).cpu().numpy()
    for got, ref, bound, k in [(ax, a @ x, np.abs(a) @ np.abs(x), n),
                               (aty, a.T @ y, np.abs(a.T) @ np.abs(y), m)]:
        g = (k + 2) * EPS
        assert got.shape == ref.shape
        assert np.all(np.abs(got - ref) <= 2 * g * bound)


CSR_SOLVES = [n for n in SOLVE_FIXTURES if "dense" not in n and "fixed" not in n]


@pytest.mark.parametrize("chains", ["auto", "1"])
@pytest.mark.parametrize("name", CSR_SOLVES)
def test_csr_solve_matches_reference(amfls, monkeypatch, name, chains):
    """chains="1" builds chain groups for the short-row sides of these small
    matrices too (by default only sides of 2^21 nonzeros or more get them)."""
    if chains != "auto":
        monkeypatch.setenv("AMFLS_GB300_CSR_CHAINS", chains)
    data, prob = load_golden(name)
    opts = golden_options(data)
    r = amfls.run_amfls(csr_tensor(prob), torch.from_numpy(prob.b).cuda(), **opts)
    c = data["counters"]
    assert (r.status, r.stop_reason) == (int(data["status"]), int(data["stop_reason"]))
    assert (r.depth, r.basis_rank, r.auxiliary_width, r.iterations) == (c[9], c[11], c[10], c[8])
    assert (r.search_a_columns, r.search_at_columns) == (c[4], c[5])
    assert r.trace_int.shape[0] == data["trace_int"].shape[0]
    np.testing.assert_array_equal(r.trace_int[:, :3].numpy(), data["trace_int"][:, :3])
    x, xr = r.solution.cpu().numpy(), data["solution"]
    reg, tol = opts["regularization"], opts["tolerance"]
    check_solution(prob, x, xr, reg, tol, r.status == 0)
    # the certified bound is finite exactly when the reference's is (near
    # convergence both sit at their rounding floors, so values are not compared)
    for idx, name_ in [(10, "backward_error_upper_bound"),
                       (13, "relative_energy_error_upper_bound")]:
        assert np.isfinite(getattr(r, name_)) == np.isfinite(data["metrics"][idx]), name_
    if r.status == 0:
        cert = r.relative_energy_error_upper_bound if reg > 0 else r.backward_error_upper_bound
        assert cert <= tol


BLOCK_SOLVES = [n for n in SOLVE_FIXTURES if "dense" in n or "fixed" in n]


def _matrix_tensor(prob):
    """Dense problems keep their layout: a Fortran-ordered matrix becomes a
    column-major CUDA view (the transpose of a contiguous tensor)."""
    if hasattr(prob, "matrix"):
        mat = prob.matrix
        if mat.flags.c_contiguous:
            return torch.from_numpy(mat).cuda()
        return torch.from_numpy(np.ascontiguousarray(mat.T)).cuda().t()
    return csr_tensor(prob)


@pytest.mark.parametrize("name", BLOCK_SOLVES)
def test_block_and_dense_solves_match_reference(amfls, name):
    """Fixed-width RBGK (block levels from the first level) and dense AMFLS.

    Fixed RBGK's widths do not depend on timings, so its counters must match
    exactly.  Dense AMFLS's width controller weighs measured seconds (the
    dense cost model is flat), so its counters are compared only when the
    GPU took the same widening decisions."""
    data, prob = load_golden(name)
    opts = golden_options(data)
    algorithm = opts.pop("algorithm", "amfls")
    mat = _matrix_tensor(prob)
    b = torch.from_numpy(prob.b).cuda()
    fn = amfls.run_fixed_rbgk if algorithm == "fixed_rbgk" else amfls.run_amfls
    r = fn(mat, b, **opts)
    c = data["counters"]
    assert (r.status, r.stop_reason) == (int(data["status"]), int(data["stop_reason"]))
    if algorithm == "fixed_rbgk" or r.auxiliary_width == c[10]:
        assert (r.depth, r.basis_rank, r.auxiliary_width, r.iterations) == (c[9], c[11], c[10], c[8])
        assert (r.search_a_columns, r.search_at_columns) == (c[4], c[5])
        np.testing.assert_array_equal(r.trace_int[:, :3].numpy(), data["trace_int"][:, :3])
    x, xr = r.solution.cpu().numpy(), data["solution"]
    check_solution(prob, x, xr, opts["regularization"], opts["tolerance"], r.status == 0)
    if r.status == 0:
        reg = opts["regularization"]
        cert = r.relative_energy_error_upper_bound if reg > 0 else r.backward_error_upper_bound
        assert cert <= opts["tolerance"]


@pytest.mark.parametrize("width,lam,tol", [(4, 0.0, 1e-8), (8, 1e-4, 1e-10), (3, 1e-6, 1e-9)])
def test_medium_fixed_rbgk_against_oracle(amfls, width, lam, tol):
    from amfls_solver_gb300 import problems

    p = problems.scaled_uniform_csr(5000, 1200, per_row=8, decades=5.0, seed=21 + width)
    ref = orc.solve_fixed_rbgk(p, auxiliary_width=width, regularization=lam, tolerance=tol,
                               seed=5, maximum_depth=400)
    r = amfls.run_fixed_rbgk(csr_tensor(p), torch.from_numpy(p.b).cuda(), auxiliary_width=width,
                             regularization=lam, tolerance=tol, seed=5, maximum_depth=400)
    assert (r.status, r.stop_reason) == (ref["status"], ref["stop_reason"])
    assert (r.depth, r.basis_rank) == (ref["counters"][9], ref["counters"][11])
    assert (r.search_a_columns, r.search_at_columns) == (ref["counters"][4], ref["counters"][5])
    check_solution(p, r.solution.cpu().numpy(), ref["solution"], lam, tol, r.status == 0)


def test_medium_dense_against_oracle(amfls):
    from amfls_solver_gb300 import problems

    p = problems.scaled_dense(4000, 300, decades=6.0, seed=7)
    ref = orc.solve_amfls(p, regularization=1e-6, tolerance=1e-10, seed=1)
    r = amfls.run_amfls(_matrix_tensor(p), torch.from_numpy(p.b).cuda(), regularization=1e-6,
                        tolerance=1e-10, seed=1)
    assert (r.status, r.stop_reason) == (ref["status"], ref["stop_reason"])
    check_solution(p, r.solution.cpu().numpy(), ref["solution"], 1e-6, 1e-10, r.status == 0)


@pytest.mark.parametrize("lam,tol", [(0.0, 1e-8), (1e-4, 1e-10)])
def test_medium_csr_against_oracle(amfls, lam, tol):
    from amfls_solver_gb300 import problems

    p = problems.scaled_uniform_csr(6000, 1500, per_row=10, decades=6.0, seed=11)
    ref = orc.solve_amfls(p, regularization=lam, tolerance=tol, seed=3)
    r = amfls.run_amfls(csr_tensor(p), torch.from_numpy(p.b).cuda(), regularization=lam,
                        tolerance=tol, seed=3)
    assert (r.status, r.stop_reason) == (ref["status"], ref["stop_reason"])
    assert r.depth == ref["counters"][9]
    x, xr = r.solution.cpu().numpy(), ref["solution"]
    check_solution(p, x, xr, lam, tol, r.status == 0)
    # independent check of the returned solution's residuals in float64
    res = p.matvec(x) - p.b
    np.testing.assert_allclose(np.linalg.norm(res), r.residual_norm, rtol=1e-8)


def test_torch_op_schema_and_tuple(amfls):
    from amfls_solver_gb300 import problems

    p = problems.scaled_uniform_csr(300, 80, per_row=5, seed=2)
    out = torch.ops.amfls.run_amfls(csr_tensor(p), torch.from_numpy(p.b).cuda(), 0.0, 1e-8, 1e-6)
    assert isinstance(out, (tuple, list)) and len(out) == 8
    sol, metrics, counters, timings, tf, ti, status, reason = out
    assert sol.is_cuda and sol.shape == (80,) and sol.dtype == torch.float64
    assert metrics.shape == (21,) and counters.shape == (36,) and timings.shape == (9,)
    assert tf.shape[1] == 29 and ti.shape == (tf.shape[0], 4)
    assert isinstance(status, int) and isinstance(reason, int)


def test_invalid_csr_is_rejected_with_message(amfls):
    rows = torch.tensor([0, 2, 3], dtype=torch.int64)
    dup = torch.sparse_csr_tensor(rows, torch.tensor([1, 1, 0]), torch.tensor([1.0, 2.0, 3.0],
                                  dtype=torch.float64), size=(2, 3)).cuda()
    with pytest.raises(RuntimeError, match="duplicate"):
        amfls.DeviceOperator(dup)
    nan = torch.sparse_csr_tensor(rows, torch.tensor([0, 1, 2]),
                                  torch.tensor([1.0, float("nan"), 3.0], dtype=torch.float64),
                                  size=(2, 3)).cuda()
    with pytest.raises(RuntimeError, match="finite"):
        amfls.DeviceOperator(nan)
    b = torch.ones(2, dtype=torch.float64, device="cuda")
    ok = torch.sparse_csr_tensor(rows, torch.tensor([0, 1, 2]),
                                 torch.tensor([1.0, 2.0, 3.0], dtype=torch.float64),
                                 size=(2, 3)).cuda()
    with pytest.raises(RuntimeError, match="tolerance"):
        amfls.run_amfls(ok, b, tolerance=2.0)
    with pytest.raises(ValueError, match="CUDA"):
        amfls.run_amfls(ok.cpu(), b.cpu())

"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run (where the reference sources exist):
    make -C oracle ref && python tests/golden/make_golden.py

Each fixture holds the exact inputs and the reference's outputs, produced by
oracle/_ref/libamfls_ref.so (the reference's AMFLS sources compiled where they
lie, see oracle/Makefile).  Fixtures are small (sizes the oracle and a GPU
finish in well under a second) and self-contained, so tests on a machine
without the reference read them as plain data.

Only deterministic runs are stored: CSR operators never widen under the
reference's default cost model, and fixed-width RBGK has no width controller.
AMFLS widening on dense operators depends on measured seconds and is not
reproducible across machines, so the plain dense AMFLS fixtures use cases
whose outcome does not depend on timing (basis-limited ridge,
maximum_epochs=0 with auxiliary width 0, or a depth cap of one level).

Widening solves are stored as schedule-replay fixtures (``replay``): the
reference build records the candidate bit of every width decision
(oracle/ref_hooks.hpp wraps amfls.cpp:323-354); the fixture keeps that list,
and the reference run *replaying* it (which reproduces the recorded run
exactly, checked here) gives the stored outputs.  A solver that takes the
same bits follows the same widening path whatever its own timings.  Large
inputs (the 20000 x 5000 CSR workload, 16384 x 512 dense matrices) are not
stored: the fixture names the seeded generator in amfls_solver_gb300.problems
and the SHA-256 of the generated arrays, so a test regenerates them and
checks that it has the same bytes.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from amfls_solver_gb300 import problems  # noqa: E402
from oracle import ref  # noqa: E402

OUT = Path(__file__).resolve().parent


def save(name, **arrays):
    np.savez_compressed(OUT / f"{name}.npz", **arrays)
    print("wrote", name)


def csr_arrays(p):
    return dict(kind=np.int64(0), rows=np.int64(p.rows), cols=np.int64(p.cols),
                row_offsets=p.row_offsets, column_indices=p.column_indices,
                values=p.values, b=p.b)


def dense_arrays(p):
    kind = 1 if p.matrix.flags.c_contiguous else 2
    return dict(kind=np.int64(kind), rows=np.int64(p.rows), cols=np.int64(p.cols),
                matrix=np.array(p.matrix), b=p.b)


ALGORITHM_CODES = {"amfls": 0, "fixed_rbgk": 1, "lsqr": 2, "lsmr": 3}


def solve_fixture(name, p, arrays, **opts):
    """int_options: maximum_epochs, maximum_depth (maximum_iterations for
    LSQR / LSMR), maximum_auxiliary_width, maximum_basis_size, seed, stream,
    auxiliary_width, algorithm code."""
    r = ref.solve(p, **opts)
    options = np.array([opts.get("regularization", 0.0), opts.get("tolerance", 1e-8),
                        opts.get("failure_probability", 1e-6)])
    ints = np.array([opts.get("maximum_epochs", 0),
                     opts.get("maximum_iterations", opts.get("maximum_depth", 0)),
                     opts.get("maximum_auxiliary_width", 0),
                     opts.get("maximum_basis_size", 0), opts.get("seed", 0),
                     opts.get("stream", 0), opts.get("auxiliary_width", 4),
                     ALGORITHM_CODES[opts.get("algorithm", "amfls")]],
                    dtype=np.int64)
    save(name, **arrays, options=options, int_options=ints, solution=r["solution"],
         metrics=r["metrics"], counters=r["counters"], trace_float=r["trace_float"],
         trace_int=r["trace_int"], status=np.int64(r["status"]),
         stop_reason=np.int64(r["stop_reason"]))
    c = r["counters"]
    print(f"   status {r['status']}/{r['stop_reason']} depth {c[9]} aux {c[10]} "
          f"basis {c[11]} evals {len(r['trace_int'])} disp {c[35]}")


def problem_digest(p):
    """SHA-256 of a generated problem's arrays (CSR or dense) and b."""
    import hashlib
    h = hashlib.sha256()
    if hasattr(p, "row_offsets"):
        parts = (p.row_offsets, p.column_indices, p.values, p.b)
    else:
        parts = (np.asfortranarray(p.matrix) if not p.matrix.flags.c_contiguous
                 else p.matrix, p.b)
    for a in parts:
        h.update(np.ascontiguousarray(a).tobytes(order="A"))
    return h.hexdigest()


def replay_fixture(name, generator, store=False, **opts):
    """A solve on a regenerated problem: `generator` = (family, kwargs) of
    amfls_solver_gb300.problems (kwargs include the seed).  The reference runs
    once with its own timing-driven controller; its decision bits are then
    replayed by the reference (or `opts["replay"]` is replayed directly), and
    that replayed run must reproduce itself exactly before it is stored.
    store=True keeps the CSR arrays in the fixture (for generators that call
    libm, whose results differ in the last bits between platforms); the
    portable_* families regenerate bit for bit anywhere."""
    import json
    family, kwargs = generator
    p = problems.FAMILIES[family](**kwargs)
    replay = opts.pop("replay", None)
    if replay is None:
        first = ref.solve(p, **opts)
        replay = [int(v) for v in first["decisions"]]
    r = ref.solve(p, replay=replay, **opts)
    again = ref.solve(p, replay=replay, **opts)
    if not (np.array_equal(r["counters"][:35], again["counters"][:35]) and
            np.array_equal(r["solution"], again["solution"]) and r["replay_overrun"] == 0):
        raise RuntimeError(f"{name}: the replayed reference run is not reproducible")
    options = np.array([opts.get("regularization", 0.0), opts.get("tolerance", 1e-8),
                        opts.get("failure_probability", 1e-6)])
    ints = np.array([opts.get("maximum_epochs", 0), opts.get("maximum_depth", 0),
                     opts.get("maximum_auxiliary_width", 0), opts.get("maximum_basis_size", 0),
                     opts.get("seed", 0), opts.get("stream", 0), 4, 0], dtype=np.int64)
    stored = {}
    if store:
        stored = dict(rows=np.int64(p.rows), cols=np.int64(p.cols), row_offsets=p.row_offsets,
                      column_indices=p.column_indices.astype(np.int32), values=p.values, b=p.b)
    save(name, generator=np.array(json.dumps({"family": family, "kwargs": kwargs})),
         digest=np.array(problem_digest(p)), options=options, int_options=ints,
         replay=np.array(replay, dtype=np.int32), decisions=r["decisions"],
         solution=r["solution"], metrics=r["metrics"], counters=r["counters"],
         trace_float=r["trace_float"], trace_int=r["trace_int"],
         status=np.int64(r["status"]), stop_reason=np.int64(r["stop_reason"]), **stored)
    c = r["counters"]
    print(f"   status {r['status']}/{r['stop_reason']} depth {c[9]} aux {c[10]} basis {c[11]} "
          f"widenings {c[34]} decisions {''.join(map(str, r['decisions']))}")


def customs():
    """CSR problems of the solve fixtures solved through a custom
    MatrixOperator (the reference driver's forwarding operator: products and
    validation model of the CSR matrix, no extended-precision validation
    products), the counterpart of a callback operator."""
    c1 = problems.scaled_uniform_csr(2000, 500, seed=1)
    c2 = problems.power_law_csr(3000, 800, decades=4.0, noise=1e-6, seed=4)
    c3 = problems.scaled_uniform_csr(600, 1500, per_row=12, decades=3.0, noise=1e-3, seed=9)
    c4 = problems.scaled_uniform_csr(1500, 200, per_row=6, decades=2.0, noise=1.0, seed=21)
    solve_fixture("custom_csr_ls", c1, csr_arrays(c1), custom=True, regularization=0.0,
                  tolerance=1e-8, seed=7)
    solve_fixture("custom_csr_ridge", c1, csr_arrays(c1), custom=True, regularization=1e-4,
                  tolerance=1e-10, seed=7)
    solve_fixture("custom_powerlaw_ridge", c2, csr_arrays(c2), custom=True, regularization=1e-4,
                  tolerance=1e-10)
    solve_fixture("custom_csr_wide", c3, csr_arrays(c3), custom=True, regularization=0.0,
                  tolerance=1e-8)
    solve_fixture("custom_csr_inconsistent", c4, csr_arrays(c4), custom=True,
                  regularization=0.0, tolerance=1e-13)


def replays():
    """The 20000 x 5000 CSR workload (bench seed; arrays stored) and widening
    solves on portable problems."""
    replay_fixture("replay_csr_20000x5000",
                   ("scaled_uniform_csr", dict(m=20000, n=5000, per_row=10, decades=6.0,
                                               noise=1e-8, seed=20251203)),
                   store=True, regularization=0.0, tolerance=1e-8)
    # dense column-major operators on which the reference's own cost gate
    # widens (its decisions vary from run to run with the measured seconds;
    # the fixture keeps the run it recorded)
    replay_fixture("replay_dense_widening_16384x512",
                   ("portable_dense", dict(m=16384, n=512, octaves=20, seed=7)),
                   regularization=0.0, tolerance=1e-10, seed=3)
    replay_fixture("replay_dense_widening_8192x400",
                   ("portable_dense", dict(m=8192, n=400, octaves=20, seed=7)),
                   regularization=0.0, tolerance=1e-10, seed=3)
    replay_fixture("replay_dense_widening_2500x200",
                   ("portable_dense", dict(m=2500, n=200, octaves=20, seed=1)),
                   regularization=0.0, tolerance=1e-10, seed=3)
    # forced widening schedules on CSR operators (the reference's cost model never
    # widens there): ridge widened at every decision site, least squares at three
    replay_fixture("replay_csr_ridge_forced",
                   ("portable_csr", dict(m=2000, n=500, seed=1)),
                   regularization=1e-4, tolerance=1e-10, seed=7, replay=[1] * 64)
    replay_fixture("replay_csr_ls_forced",
                   ("portable_csr", dict(m=2000, n=500, seed=1)),
                   regularization=0.0, tolerance=1e-8, seed=7, replay=[0, 1, 1, 0, 1] + [0] * 64)
    # a tall ridge problem for the mixed form's comparison with the reference
    # (the 2,000,000 x 500,000 problem is out of the reference's reach)
    replay_fixture("replay_csr_ridge_60000x15000",
                   ("portable_csr", dict(m=60000, n=15000, per_row=10, octaves=20, seed=3)),
                   regularization=1e-4, tolerance=1e-10)


def full_size():
    """The 100000 x 2000 dense ridge configuration at full size, on the
    portable generator (the same bytes on every platform; condition about
    2^20, a uniform right-hand side, lambda = 1e-6, tol 1e-10).  The
    reference needs about two minutes per run for it, so it has its own
    argument."""
    replay_fixture("replay_dense_ridge_100000x2000",
                   ("portable_dense", dict(m=100000, n=2000, octaves=20, seed=20251203)),
                   regularization=1e-6, tolerance=1e-10)


def main():
    # ---- kernels: CSR products, validation model, Gaussian, norm intervals
    p = problems.scaled_uniform_csr(300, 120, per_row=7, decades=3.0, seed=11)
    rng = np.random.default_rng(5)
    x = np.asfortranarray(rng.standard_normal((120, 3)))
    y = np.asfortranarray(rng.standard_normal((300, 3)))
    model, steps = ref.validation_model(p)
    save("csr_products", **csr_arrays(p), x=x, y=y,
         ax1=ref.apply(p, x[:, 0]), aty1=ref.apply(p, y[:, 0], transpose=True),
         ax3=ref.apply(p, x), aty3=ref.apply(p, y, transpose=True),
         model=model, steps=steps)
    # ragged rows: empty rows, one heavy row, an empty column
    m, n = 64, 40
    lengths = rng.integers(0, 6, size=m)
    lengths[3] = 0
    lengths[10] = 39
    cols = problems._distinct_columns(rng, lengths, n - 1)  # last column empty
    off = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(lengths, out=off[1:])
    q = problems.CsrProblem(m, n, off, cols, rng.standard_normal(cols.shape[0]), np.zeros(m))
    xr = rng.standard_normal(n)
    yr = rng.standard_normal(m)
    model, steps = ref.validation_model(q)
    save("csr_ragged", **csr_arrays(q), x=xr, y=yr, ax1=ref.apply(q, xr),
         aty1=ref.apply(q, yr, transpose=True), model=model, steps=steps)

    for tag, dp in (("rm", problems.scaled_dense(50, 17, decades=4.0, seed=3, column_major=False)),
                    ("cm", problems.scaled_dense(50, 17, decades=4.0, seed=3, column_major=True))):
        model, steps = ref.validation_model(dp)
        save(f"dense_model_{tag}", **dense_arrays(dp), model=model, steps=steps)

    gauss = []
    params = [(37, 5, 12345, 7, 3), (16, 2, 0, 0, 0), (9, 3, 2**64 - 1, 2**63 + 5, 17)]
    for rows, cols_, seed, stream, first in params:
        gauss.append(ref.gaussian_matrix(rows, cols_, seed, stream, first))
    save("gaussian", params=np.array(params, dtype=np.uint64),
         g0=gauss[0], g1=gauss[1], g2=gauss[2])

    vecs = [rng.standard_normal(1000),
            np.concatenate([rng.standard_normal(10) * 1e-310, [0.0, 5e-324]]),
            np.zeros(17), rng.standard_normal(33) * 1e300, np.array([3.0, -4.0])]
    bounds = np.array([ref.norm_interval(v) for v in vecs])
    save("norm_interval", **{f"v{i}": v for i, v in enumerate(vecs)}, bounds=bounds)

    # ---- end-to-end solves
    c1 = problems.scaled_uniform_csr(2000, 500, seed=1)
    solve_fixture("solve_csr_ls", c1, csr_arrays(c1), regularization=0.0, tolerance=1e-8, seed=7)
    solve_fixture("solve_csr_ridge", c1, csr_arrays(c1), regularization=1e-4, tolerance=1e-10,
                  seed=7)
    c2 = problems.power_law_csr(3000, 800, decades=4.0, noise=1e-6, seed=4)
    solve_fixture("solve_powerlaw_ridge", c2, csr_arrays(c2), regularization=1e-4,
                  tolerance=1e-10)
    c3 = problems.scaled_uniform_csr(600, 1500, per_row=12, decades=3.0, noise=1e-3, seed=9)
    solve_fixture("solve_csr_wide", c3, csr_arrays(c3), regularization=0.0, tolerance=1e-8)
    # inconsistent, tight tolerance: exercises the extended-precision refinement
    c4 = problems.scaled_uniform_csr(1500, 200, per_row=6, decades=2.0, noise=1.0, seed=21)
    solve_fixture("solve_csr_inconsistent", c4, csr_arrays(c4), regularization=0.0,
                  tolerance=1e-13)
    solve_fixture("solve_csr_depth_cap", c1, csr_arrays(c1), regularization=0.0, tolerance=1e-8,
                  maximum_depth=40)
    solve_fixture("solve_csr_basis_cap", c1, csr_arrays(c1), regularization=1e-4,
                  tolerance=1e-12, maximum_basis_size=30)
    z = problems.scaled_uniform_csr(200, 50, seed=2)
    z.b = np.zeros(200)
    solve_fixture("solve_csr_zero_rhs", z, csr_arrays(z), regularization=0.0, tolerance=1e-8)
    # rank deficient: every column appears twice with proportional values
    half = problems.scaled_uniform_csr(400, 60, per_row=5, decades=1.0, noise=0.0, seed=13)
    dup_cols = np.stack([half.column_indices, half.column_indices + 60], axis=1).reshape(-1)
    dup_vals = np.stack([half.values, 2.0 * half.values], axis=1).reshape(-1)
    rd = problems.CsrProblem(400, 120, half.row_offsets * 2, dup_cols, dup_vals,
                             half.b.copy())
    solve_fixture("solve_csr_rank_deficient", rd, csr_arrays(rd), regularization=0.0,
                  tolerance=1e-8)

    d1 = problems.scaled_dense(600, 80, decades=6.0, seed=2, column_major=False)
    solve_fixture("solve_dense_rm_ridge_basis", d1, dense_arrays(d1), regularization=1e-6,
                  tolerance=1e-12, maximum_epochs=1, maximum_auxiliary_width=1)
    d2 = problems.scaled_dense(600, 80, decades=3.0, seed=5, column_major=True)
    solve_fixture("solve_dense_cm_depth1", d2, dense_arrays(d2), regularization=0.0,
                  tolerance=1e-10, maximum_depth=1)
    solve_fixture("solve_fixed_rbgk_dense", d2, dense_arrays(d2), algorithm="fixed_rbgk",
                  regularization=0.0, tolerance=1e-10, auxiliary_width=3, maximum_depth=40,
                  seed=11, stream=2)
    solve_fixture("solve_fixed_rbgk_csr_ridge", c1, csr_arrays(c1), algorithm="fixed_rbgk",
                  regularization=1e-4, tolerance=1e-10, auxiliary_width=7, maximum_depth=60,
                  seed=3)



def baselines():
    """Scalar LSQR and LSMR (src/algorithms/lsqr/lsqr.cpp, src/algorithms/lsmr/lsmr.cpp):
    well-conditioned least squares and ridge problems that certify, the
    ill-conditioned CSR problem up to the default iteration limit, an
    iteration cap, a dense column-major operator and a zero right-hand side."""
    c1 = problems.scaled_uniform_csr(2000, 500, seed=1)
    d2 = problems.scaled_dense(600, 80, decades=3.0, seed=5, column_major=True)
    z = problems.scaled_uniform_csr(200, 50, seed=2)
    z.b = np.zeros(200)
    w = problems.scaled_uniform_csr(2000, 500, decades=1.0, noise=1e-3, seed=3)
    for alg in ("lsqr", "lsmr"):
        solve_fixture(f"baseline_{alg}_wellcond_ls", w, csr_arrays(w), algorithm=alg,
                      regularization=0.0, tolerance=1e-8)
        solve_fixture(f"baseline_{alg}_wellcond_ridge", w, csr_arrays(w), algorithm=alg,
                      regularization=1e-2, tolerance=1e-10)
        solve_fixture(f"baseline_{alg}_csr_ls", c1, csr_arrays(c1), algorithm=alg,
                      regularization=0.0, tolerance=1e-8)
        solve_fixture(f"baseline_{alg}_csr_ridge", c1, csr_arrays(c1), algorithm=alg,
                      regularization=1e-4, tolerance=1e-10)
        solve_fixture(f"baseline_{alg}_csr_cap", c1, csr_arrays(c1), algorithm=alg,
                      regularization=0.0, tolerance=1e-12, maximum_iterations=25)
        solve_fixture(f"baseline_{alg}_dense_cm", d2, dense_arrays(d2), algorithm=alg,
                      regularization=1e-6, tolerance=1e-10)
        solve_fixture(f"baseline_{alg}_zero_rhs", z, csr_arrays(z), algorithm=alg,
                      regularization=0.0, tolerance=1e-8)


if __name__ == "__main__":
    # no argument: every fixture; "baselines": only the LSQR / LSMR ones;
    # "replays": only the schedule-replay fixtures; "customs": only the
    # custom-operator ones; "full": only the full-size dense ridge solve
    if sys.argv[1:] == ["baselines"]:
        baselines()
    elif sys.argv[1:] == ["full"]:
        full_size()
    elif sys.argv[1:] == ["replays"]:
        replays()
    elif sys.argv[1:] == ["customs"]:
        customs()
    else:
        main()
        baselines()
        replays()
        customs()
        full_size()

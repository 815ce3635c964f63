import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    """Fixture arrays plus the problem object they describe."""
    from amfls_solver_gb300 import problems

    data = dict(np.load(GOLDEN / f"{name}.npz"))
    kind = int(data["kind"])
    if kind == 0:
        prob = problems.CsrProblem(int(data["rows"]), int(data["cols"]), data["row_offsets"],
                                   data["column_indices"], data["values"], data["b"])
    else:
        mat = data["matrix"]
        mat = np.ascontiguousarray(mat) if kind == 1 else np.asfortranarray(mat)
        prob = problems.DenseProblem(mat, data["b"])
    return data, prob


def golden_options(data):
    o, i = data["options"], data["int_options"]
    if int(i[7]) in (2, 3):  # LSQR / LSMR: regularization, tolerance, maximum_iterations
        return dict(algorithm="lsqr" if int(i[7]) == 2 else "lsmr",
                    regularization=float(o[0]), tolerance=float(o[1]),
                    maximum_iterations=int(i[1]))
    opts = dict(regularization=float(o[0]), tolerance=float(o[1]),
                failure_probability=float(o[2]), seed=int(i[4]), stream=int(i[5]))
    if int(i[7]) == 1:
        opts.update(algorithm="fixed_rbgk", auxiliary_width=int(i[6]),
                    maximum_depth=int(i[1]), maximum_basis_size=int(i[3]))
    else:
        opts.update(maximum_epochs=int(i[0]), maximum_depth=int(i[1]),
                    maximum_auxiliary_width=int(i[2]), maximum_basis_size=int(i[3]))
    return opts


def load_replay(name):
    """A schedule-replay fixture and its problem: the arrays stored in the
    fixture, or else the problem rebuilt from the seeded generator it names
    (the portable families, bit-identical on every platform).  The SHA-256
    of the arrays must equal the fixture's, so the solve runs on the very
    bytes the reference solved."""
    import hashlib
    import json
    from amfls_solver_gb300 import problems

    data = dict(np.load(GOLDEN / f"{name}.npz"))
    if "row_offsets" in data:  # stored arrays (the generator calls libm)
        prob = problems.CsrProblem(int(data["rows"]), int(data["cols"]), data["row_offsets"],
                                   data["column_indices"].astype(np.int64), data["values"],
                                   data["b"])
    else:
        spec = json.loads(str(data["generator"]))
        prob = problems.FAMILIES[spec["family"]](**spec["kwargs"])
    h = hashlib.sha256()
    if hasattr(prob, "row_offsets"):
        parts = (prob.row_offsets, prob.column_indices, prob.values, prob.b)
    else:
        parts = (prob.matrix, prob.b)
    for a in parts:
        h.update(np.ascontiguousarray(a).tobytes(order="A"))
    assert h.hexdigest() == str(data["digest"]), f"{name}: regenerated problem differs"
    return data, prob


SOLVE_FIXTURES = sorted(p.stem for p in GOLDEN.glob("solve_*.npz"))
REPLAY_FIXTURES = sorted(p.stem for p in GOLDEN.glob("replay_*.npz"))
CUSTOM_FIXTURES = sorted(p.stem for p in GOLDEN.glob("custom_*.npz"))
BASELINE_FIXTURES = sorted(p.stem for p in GOLDEN.glob("baseline_*.npz"))


@pytest.fixture(scope="session")
def golden():
    return load_golden


@pytest.fixture
def gelsy_ranks(monkeypatch):
    """Records (shape of T, rank dgelsy found) for every projected solve the
    oracle makes with dgelsy (krylov_workspace.cpp:833-909, lambda = 0).  The
    GPU replaces dgelsy by a QR recurrence on T, the same least-squares
    solution whenever dgelsy finds full column rank; the fixtures' solves must
    all be in that case for their parity to cover the projected solve."""
    import scipy.linalg
    from oracle import amfls_oracle as orc

    calls = []

    class Recording:
        def __getattr__(self, name):
            return getattr(scipy.linalg, name)

        def lstsq(self, a, b, **kw):
            out = scipy.linalg.lstsq(a, b, **kw)
            if kw.get("lapack_driver") == "gelsy":
                calls.append((a.shape, int(out[2])))
            return out

    monkeypatch.setattr(orc, "sla", Recording())
    return calls

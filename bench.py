"""Time-to-tolerance benchmark of the GB300 AMFLS solver.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--c3 0|1] [--dense 0|1] [--spmm 0|1]
                    [--baselines 0|1] [--learned 0|1] [--batched COUNT]
                    [--cpu-sample 0|1]

A step is one complete AMFLS solve, to tolerance, of a seeded synthetic
problem.  The headline workload is the 20000 x 5000 CSR problem (10 nonzeros
per row at distinct uniform columns, N(0,1) values with column j scaled by
10^(-6 j / n), b = A x_true + 1e-8 noise; lambda = 0, tol = 1e-8, initial
width one): the configuration both arms solve completely within the run.
Prints one JSON line (rank 0).

value     mean device time of one solve with A and b already in HBM (CUDA
          events around the C-ABI solve on the launching stream; the
          operator is built once);
e2e       the same solve through the public API run_amfls on pinned host
          tensors: host->device copies of the CSR arrays and b, operator
          construction (transpose, task tables, certified norm model), solve,
          device->host copy of the solution;
roofline  the dominant kernels of the solve, the width-one
          reorthogonalisation sweeps (c = V^T r and r -= V c over the basis V),
          timed live with CUDA events on their stream at the solve's mean basis
          size; algorithmic bytes 8 n k + 8 n (+ 8 n for the update);
c3        time-to-tol on the 2,000,000 x 500,000 power-law CSR problem
          (lambda = 1e-4, tol = 1e-10; the metric's target workload): plain
          FP64 and the chosen form (FP64 residual correction around restart
          cycles with reduced-basis sweeps), status, depth, certificate, time
          split, speed-up, x against plain FP64's, and the roofline of each
          form's dominant sweeps;
dense     the 100000 x 2000 column-major dense operator (lambda = 1e-6,
          tol = 1e-10): plain FP64 and the mixed form;
spmm      CSR SpMM / SpMM^T GB/s (s = 1 and 8) on the 2M x 500k matrix;
baselines AMFLS against scalar LSQR / LSMR on the headline problem;
learned   the learned width controller against the heuristic: trained on
          exploration solves of the reference's dense study family, compared
          by time-to-tol on held-out instances;
batched   problems/s, p50 / p99 of batched solves of the uneven CSR workload
          (a bounded sample, described in the line);
cpu_baseline  one complete oracle solve (the CPU restatement of the
          reference, pinned bit for bit to the reference's own run of this
          problem) of the headline workload on this host's cores.
--impl reference times complete oracle solves of the headline workload on
the host cores, one per step (the reference itself cannot be built on the
GPU host: its sources are not shipped there), with the same config.
Multi-GPU: replicas only (each rank solves its own copy; no collective on the
data path); value is the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = ("time-to-tol (s) mixed+batched+learned vs plain FP64 AMFLS on GB300; "
          "SpMM HBM GB/s")
SEED = 20251203
C3_CYCLE = 2000  # restart-cycle length of the chosen form on the 2M x 500k problem
C3_STORAGE = "fp16"  # precision of the chosen form's copy of the basis ("fp32" or "fp16")
C3_STORAGE_CODE = {"fp32": 1, "fp16": 2}[C3_STORAGE]
# DRAM bytes of one V^T r + r - V c pair measured by ncu (--set full) on the
# warp-task sweeps at n = 5000, k = 1900: 76.875 + 1.307 MB and 76.860 + 1.436 MB
SWEEP_CAPTURE = {"n": 5000, "k": 1900, "bytes": (76.875 + 1.307 + 76.860 + 1.436) * 1e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="csr_20000x5000")
    ap.add_argument("--cpu-sample", type=int, default=1, help="0 skips the cpu_baseline leg")
    ap.add_argument("--c3", type=int, default=1,
                    help="0 skips the time-to-tol leg on the 2M x 500k CSR problem")
    ap.add_argument("--dense", type=int, default=1,
                    help="0 skips the 100000 x 2000 dense leg (plain and mixed)")
    ap.add_argument("--spmm", type=int, default=1,
                    help="0 skips the CSR SpMM GB/s measurement on the 2M x 500k matrix")
    ap.add_argument("--baselines", type=int, default=1,
                    help="0 skips the AMFLS vs LSQR / LSMR leg")
    ap.add_argument("--learned", type=int, default=1,
                    help="0 skips the learned-controller leg on the dense study family")
    ap.add_argument("--batched", type=int, default=48,
                    help="problems in the batched leg's sample (0 skips it)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.is_file():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True,
                    timeout=5).stdout.strip()
                if out:
                    self.samples.append([c.strip() for c in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


# ------------------------------------------------------------ workloads ----

def make_workload(name):
    from amfls_solver_gb300 import problems
    return problems.make(name, seed=SEED)


def bench_config(name, prob, opts):
    """The config object both arms print (identical keys and values)."""
    nnz = prob.nnz if hasattr(prob, "row_offsets") else prob.rows * prob.cols
    return {"workload": name, "rows": prob.rows, "cols": prob.cols, "nnz": nnz, "seed": SEED,
            **opts,
            "l2": "inputs larger than L2 or not, every solve rebuilds its basis from "
                  "scratch; the CSR arrays and the basis are re-read every level",
            "parallelism": "replicas"}


def csr_device(prob, dev):
    import torch
    return torch.sparse_csr_tensor(torch.from_numpy(prob.row_offsets),
                                   torch.from_numpy(prob.column_indices),
                                   torch.from_numpy(prob.values),
                                   size=(prob.rows, prob.cols)).to(dev)


def native_options(opts):
    from amfls_solver_gb300 import _native
    o = _native.default_options()
    for k, v in opts.items():
        setattr(o, k, v)
    return o


def certificate(r, reg):
    return r.relative_energy_error_upper_bound if reg > 0 else r.backward_error_upper_bound


# ------------------------------------------------------------ CPU legs ----

def oracle_solve_seconds(prob, opts):
    """One complete oracle solve (operator construction included) on the
    host's cores: (seconds, result dict)."""
    from oracle import amfls_oracle as orc
    t0 = time.perf_counter()
    r = orc.solve_amfls(prob, **opts)
    return time.perf_counter() - t0, r


def host_threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_baseline(prob, opts, name):
    t, r = oracle_solve_seconds(prob, opts)
    c = r["counters"]
    return {"value": t, "unit": "s", "cores": host_threads(), "kind": "port",
            "sample": (f"one complete oracle solve of {name} (operator construction and "
                       f"solve, numpy/scipy BLAS on {host_threads()} host threads): status "
                       f"{r['status']}/{r['stop_reason']}, depth {int(c[9])}"),
            "status": [int(r["status"]), int(r["stop_reason"])], "depth": int(c[9])}


# ------------------------------------------------------------ GPU legs ----

def reorth_roofline(lib, n, k, stream, peak, peak_kind):
    """The width-one reorthogonalisation sweeps timed live on `stream` at
    basis size k (amfls_gpu_probe_reorthogonalization: the solver's own
    kernels on its panel layout, CUDA events around each kind)."""
    import ctypes
    from amfls_solver_gb300 import _native
    secs = (ctypes.c_double * 2)()
    _native.check(lib.amfls_gpu_probe_reorthogonalization(n, k, 50, ctypes.c_void_p(stream),
                                                          secs))
    vt, vc = secs[0], secs[1]
    bytes_vt = 8.0 * n * k + 8.0 * n * ((k + 31) // 32)  # V once, r once per panel
    bytes_vc = 8.0 * n * k + 16.0 * n                    # V once, r in and out
    achieved = (bytes_vt + bytes_vc) / (vt + vc) / 1e9
    return {"kernel": "vt_r_kernel (c = V^T r) + v_c_kernel (r -= V c)", "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": peak_kind, "traffic": None, "basis_rows": n, "basis_cols": k,
            "launch_us": {"vt_r": vt * 1e6, "v_c": vc * 1e6},
            "algorithmic_bytes": {"vt_r": bytes_vt, "v_c": bytes_vc}}


def reduced_reorth_roofline(lib, n, k, stream, peak, peak_kind, storage):
    """The reduced-basis sweeps (an FP32 (storage 1) or FP16 (2) copy of V:
    c = V~^T r~, r -= fl64(V~ c~)) timed live on `stream` at basis size k
    (amfls_gpu_probe_reorthogonalization_reduced)."""
    import ctypes
    from amfls_solver_gb300 import _native
    secs = (ctypes.c_double * 2)()
    err = ctypes.c_double()
    _native.check(lib.amfls_gpu_probe_reorthogonalization_reduced(
        n, k, 50, storage, ctypes.c_void_p(stream), secs, ctypes.byref(err)))
    vt, vc = secs[0], secs[1]
    e = 4.0 if storage == 1 else 2.0                    # bytes per element of V~
    bytes_vt = e * n * k + 4.0 * n * ((k + 31) // 32)  # V~ once, r~ once per panel
    bytes_vc = e * n * k + 16.0 * n                    # V~ once, r in and out
    achieved = (bytes_vt + bytes_vc) / (vt + vc) / 1e9
    return {"kernel": ("vt_r32_kernel (c = V~^T r~) + v_c32_kernel (r -= fl64(V~ c~)), "
                       f"{'FP32' if storage == 1 else 'FP16'} copy of V"),
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
            "basis_rows": n, "basis_cols": k, "launch_us": {"vt_r32": vt * 1e6, "v_c32": vc * 1e6},
            "algorithmic_bytes": {"vt_r32": bytes_vt, "v_c32": bytes_vc},
            "max_coefficient_error_rel_r": err.value}


def spmm_measurement(dev, stream, peak):
    """CSR SpMM / SpMM^T HBM GB/s on the 2,000,000 x 500,000 power-law matrix,
    s = 1 and s = 8, through the C ABI on preallocated column-major device
    blocks (CUDA events on the stream).  Algorithmic bytes:
    nnz (8 + 4) + (rows + 1) 4 + s (m + n) 8."""
    import ctypes
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import _native

    prob, _ = make_workload("csr_2000000x500000")
    op = amfls.DeviceOperator(csr_device(prob, dev))
    lib = _native.load()
    m, n, nnz = prob.rows, prob.cols, prob.nnz
    choice, tuned = op.tile_schedule()
    out = {"workload": "csr_2000000x500000", "rows": m, "cols": n, "nnz": nnz, "peak_gbs": peak,
           "unit": "GB/s", "tiling": choice, "autotuner_us": tuned}
    for cols in (1, 8):
        x = torch.randn(cols * n, dtype=torch.float64, device=dev)
        y = torch.randn(cols * m, dtype=torch.float64, device=dev)
        res = {}
        for name, fn, src, dst, rows_out in (
                ("apply", lib.amfls_gpu_operator_apply, x, y, m),
                ("apply_transpose", lib.amfls_gpu_operator_apply_transpose, y, x, n)):
            def call():
                _native.check(fn(op.handle, ctypes.c_void_p(src.data_ptr()), cols,
                                 ctypes.c_void_p(dst.data_ptr()),
                                 ctypes.c_void_p(stream.cuda_stream)))
            for _ in range(5):
                call()
            reps = 30
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                call()
            e1.record(stream)
            e1.synchronize()
            t = e0.elapsed_time(e1) * 1e-3 / reps
            nbytes = nnz * 12 + (rows_out + 1) * 4 + cols * (m + n) * 8
            res[name] = {"us": t * 1e6, "achieved": nbytes / t / 1e9,
                         "frac": nbytes / t / 1e9 / peak, "algorithmic_bytes": nbytes}
        out[f"s{cols}"] = res
    return out


def timed_solve(fn):
    """Host wall time of one synchronous solve (after a device sync)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def c3_measurement(dev):
    """Time-to-tol on the 2,000,000 x 500,000 power-law CSR problem (the
    metric's target workload), plain FP64 drop-in and the chosen form, one
    solve each (host wall clock around the synchronous C-ABI solve, operator
    and b resident)."""
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import binding

    try:
        t0 = time.perf_counter()
        prob, opts = make_workload("csr_2000000x500000")
        gen = time.perf_counter() - t0
        op = amfls.DeviceOperator(csr_device(prob, dev))
        b = torch.from_numpy(prob.b).to(dev)
        reg = opts["regularization"]
        out = {"workload": "csr_2000000x500000", "rows": prob.rows, "cols": prob.cols,
               "nnz": prob.nnz, **opts, "generation_s": gen}

        def describe(r, t):
            return {"s": t, "status": r.status, "stop_reason": r.stop_reason, "depth": r.depth,
                    "basis_rank": r.basis_rank, "auxiliary_width": r.auxiliary_width,
                    "certificate": certificate(r, reg), "a_columns": r.a_columns,
                    "at_columns": r.at_columns,
                    "split_s": {"a": r.a_seconds, "at": r.at_seconds,
                                "orthogonalization": r.orthogonalization_seconds,
                                "projected_solve": r.projected_solve_seconds,
                                "validation": r.validation_seconds}}

        plain, t_plain = timed_solve(
            lambda: binding._decode(binding._solve_raw("amfls", op, b, native_options(opts))))
        out["fp64"] = describe(plain, t_plain)
        x_plain = plain.solution.clone()
        del plain
        torch.cuda.empty_cache()
        # the chosen form: FP64 residual correction around restart cycles of
        # C3_CYCLE levels whose first reorthogonalisation pass runs on a
        # C3_STORAGE copy of the basis (products, recurrence and validation
        # in FP64)
        mixed, t_mixed = timed_solve(lambda: amfls.run_amfls_mixed(
            op, b, values="fp64", reduced_basis=C3_STORAGE, inner_tolerance=1e-14,
            maximum_refinements=40, maximum_depth=C3_CYCLE, **opts))
        d = describe(mixed, t_mixed)
        xm = mixed.solution
        d.update({"form": (f"FP64 residual correction, restart cycles of {C3_CYCLE} levels, "
                           f"reduced-basis sweeps ({C3_STORAGE.upper()} copy of V, FP64 "
                           "subtraction), FP64 operator products"),
                  "cycles": int(mixed.trace_float.shape[0]),
                  "cycle_certificates": [float(v) for v in mixed.trace_float[:, 17]],
                  "reduced_basis_levels": mixed.reduced_basis_levels,
                  "reduced_basis_fallbacks": mixed.reduced_basis_fallbacks,
                  "x_rel_diff_vs_fp64": float(torch.linalg.norm(xm - x_plain) /
                                              torch.linalg.norm(x_plain)),
                  "speedup_vs_fp64": t_plain / t_mixed})
        out["mixed"] = d
        return out, x_plain
    except Exception as e:  # reported, not fatal to the bench line
        return {"error": f"{type(e).__name__}: {e}"}, None


def dense_measurement(dev):
    """The 100000 x 2000 dense operator: plain FP64 (status and time) and the
    mixed form (FP32 inner solves refined in FP64)."""
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import binding

    try:
        prob, opts = make_workload("dense_100000x2000")
        buf = np.ascontiguousarray(prob.matrix.T)
        mat = torch.from_numpy(buf).to(dev).t()
        op = amfls.DeviceOperator(mat)
        b = torch.from_numpy(prob.b).to(dev)
        reg = opts["regularization"]
        run = lambda: binding._decode(binding._solve_raw("amfls", op, b, native_options(opts)))
        run()
        plain, t_plain = timed_solve(run)
        low = op.reduced("fp32")
        mixed, t_mixed = timed_solve(lambda: amfls.run_amfls_mixed(
            op, b, reduced=low, inner_tolerance=1e-7, maximum_refinements=6, **opts))
        return {"workload": "dense_100000x2000", **opts,
                "fp64": {"s": t_plain, "status": plain.status, "stop_reason": plain.stop_reason,
                         "depth": plain.depth, "certificate": certificate(plain, reg)},
                "mixed_fp32": {"s": t_mixed, "status": mixed.status, "levels": mixed.depth,
                               "steps": int(mixed.trace_float.shape[0]),
                               "certificate": certificate(mixed, reg)}}
    except Exception as e:
        return {"error": f"{type(e).__name__}: {e}"}


def baselines_measurement(dev, op, b, prob, opts):
    """AMFLS against the scalar LSQR and LSMR baselines (the reference's own
    comparison) on the headline problem at its tolerance: host wall clock
    around each synchronous C-ABI solve on one prebuilt operator, after one
    warm-up each."""
    import ctypes
    from amfls_solver_gb300 import binding, _native

    try:
        reg, tol = opts["regularization"], opts["tolerance"]
        ob = _native.BaselineOptions()
        _native.load().amfls_gpu_default_baseline_options(ctypes.byref(ob))
        ob.regularization, ob.tolerance = reg, tol
        out = {"tolerance": tol, "regularization": reg,
               "maximum_iterations": min(prob.rows, prob.cols)}
        for name, options in (("amfls", native_options(opts)), ("lsqr", ob), ("lsmr", ob)):
            run = lambda: binding._decode(binding._solve_raw(name, op, b, options))
            run()
            r, t = timed_solve(run)
            out[name] = {"s": t, "status": r.status, "stop_reason": r.stop_reason,
                         "iterations": r.depth, "certificate": certificate(r, reg)}
        return out
    except Exception as e:
        return {"error": f"{type(e).__name__}: {e}"}


def dense_family(seeds):
    """The reference's tall dense study cases (16384 x 512, tol 1e-10; the
    spectral-coverage and ordinary suites, tests/golden/experiment_cases.json)
    at the given instance seeds, as (case, seed, matrix, b, options)."""
    from amfls_solver_gb300 import experiments as ex

    cases = json.loads((ROOT / "tests" / "golden" / "experiment_cases.json").read_text())
    for suite in cases["suites"]:
        if suite["suite"] not in ("large_dense_spectral_coverage_v1", "large_dense_ordinary_v2"):
            continue
        for case in suite["cases"]:
            for seed in seeds:
                p = ex.make_problem(case, seed)
                yield (case["name"], seed, p["matrix"].cuda(), p["b"].cuda(),
                       dict(regularization=p["regularization"], tolerance=suite["tolerance"],
                            maximum_epochs=suite["maximum_epochs"],
                            maximum_depth=suite["maximum_depth"],
                            maximum_auxiliary_width=suite["maximum_auxiliary_width"],
                            maximum_basis_size=suite["maximum_basis_size"],
                            seed=seed + suite["algorithm_seed_offset"]))


def learned_measurement(dev):
    """The learned width controller against the heuristic: trained on the
    plain controller's counterfactual traces of the dense study family
    (instance seeds 201, 202), compared on held-out instances (seeds 101,
    102) by time-to-tol."""
    from amfls_solver_gb300 import learned

    try:
        t0 = time.perf_counter()
        train = [(m, b, o) for _, _, m, b, o in dense_family((201, 202))]
        data = learned.counterfactual_dataset(train, max_sites=8)
        policy = learned.WidthPolicy.train(data.inputs, data.targets, epochs=2000)
        t_train = time.perf_counter() - t0
        held = list(dense_family((101, 102)))
        rows = learned.compare_controllers([(m, b, o) for _, _, m, b, o in held], policy)
        per = []
        for (name, seed, _, _, _), (h, th, lr, tl) in zip(held, rows):
            per.append({"case": name, "seed": seed, "heuristic_s": th, "learned_s": tl,
                        "status": [h.status, lr.status],
                        "auxiliary_width": [h.auxiliary_width, lr.auxiliary_width],
                        "operator_columns": [h.a_columns + h.at_columns,
                                             lr.a_columns + lr.at_columns]})
        th = sum(r["heuristic_s"] for r in per)
        tl = sum(r["learned_s"] for r in per)
        return {"family": "reference dense study, tall cases (16384 x 512), tol 1e-10",
                "training": {"problems": len(train), "pairs": int(data.inputs.shape[0]),
                             "loss": list(policy.losses), "seconds": t_train},
                "held_out": per, "heuristic_s": th, "learned_s": tl, "gain": 1.0 - tl / th}
    except Exception as e:  # reported, not fatal to the bench line
        return {"error": f"{type(e).__name__}: {e}"}


def batched_measurement(dev, count):
    """Batched solves of a bounded sample of the uneven CSR workload."""
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import problems

    try:
        batch = problems.uneven_csr_batch(count, seed=SEED, m_range=(2_000, 50_000),
                                          n_range=(500, 12_500))
        mats = [(amfls.DeviceOperator(csr_device(p, dev)), torch.from_numpy(p.b).to(dev))
                for p, _, _ in batch]
        regs = [r for _, r, _ in batch]
        out = {"sample": (f"{count} problems of the uneven workload's distribution with m in "
                          f"[2e3, 5e4] and n in [500, 1.25e4] (the full ranges reach 2e5 x 5e4);"
                          f" 5-40 nonzeros per row, condition 1e3-1e8, lambda 1e-8-1e-2, "
                          f"tol 1e-9"),
               "nnz": int(sum(p.nnz for p, _, _ in batch))}
        for workers in (16, 1):
            res, secs, wall = amfls.run_amfls_batch(mats, workers=workers, regularization=regs,
                                                    tolerance=1e-9)
            st = [r.status for r in res]
            out[f"workers_{workers}"] = {
                "problems_per_s": count / wall, "wall_s": wall,
                "p50_s": float(np.percentile(secs, 50)), "p99_s": float(np.percentile(secs, 99)),
                "certified": st.count(0), "levels": int(sum(r.depth for r in res))}
        # FP64 FMA floor of the batch: basis sweeps (one V^T r and one r - V c
        # per level: n k FMAs each at basis size k) and the two products per
        # level, at two FP64 lanes per SM clock
        fmas = sum(p.cols * r.basis_rank ** 2 + 2.0 * p.nnz * r.depth
                   for (p, _, _), r in zip(batch, res))
        props = torch.cuda.get_device_properties(dev)
        rate = 2.0 * props.multi_processor_count * 2.07e9
        out["fp64_fma_floor_s"] = fmas / rate
        out["fp64_fma_floor_note"] = ("sum over problems of n k^2 + 2 nnz depth FMAs at "
                                      f"{rate / 1e12:.2f} T FMA/s (2 FP64 lanes per SM clock)")
        return out
    except Exception as e:
        return {"error": f"{type(e).__name__}: {e}"}


# --------------------------------------------------------------- arms ----

def base_line(args, world, value, config):
    return {"metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded numpy generator)", "config": config}


def run_reference(args, world, rank):
    """Complete oracle solves of the headline workload on the host cores, one
    per step (W untimed, K timed).  Under torchrun only rank 0 runs."""
    if rank != 0:
        return
    prob, opts = make_workload(args.workload)
    times, last = [], None
    for i in range(args.warmup + args.steps):
        t, last = oracle_solve_seconds(prob, opts)
        if i >= args.warmup:
            times.append(t)
    v = statistics.mean(times)
    c = last["counters"]
    line = base_line(args, args.gpus, v, bench_config(args.workload, prob, opts))
    line.update({
        "impl": "reference",
        "status": [int(last["status"]), int(last["stop_reason"])], "depth": int(c[9]),
        "cpu_baseline": {"value": v, "unit": "s", "cores": host_threads(), "kind": "port",
                         "sample": (f"complete oracle solves of {args.workload} (the CPU "
                                    f"restatement of the reference, pinned bit for bit to the "
                                    f"reference's own run of this problem), one per step, "
                                    f"numpy/scipy BLAS on {host_threads()} host threads")},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_s": times})
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import ctypes
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import _native

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    amfls.load_library()
    prob, opts = make_workload(args.workload)
    if not hasattr(prob, "row_offsets"):
        raise SystemExit("the headline workload must be a CSR problem")
    host = dict(crow=torch.from_numpy(prob.row_offsets).pin_memory(),
                col=torch.from_numpy(prob.column_indices).pin_memory(),
                val=torch.from_numpy(prob.values).pin_memory())
    b_host = torch.from_numpy(prob.b).pin_memory()
    a_dev = torch.sparse_csr_tensor(host["crow"], host["col"], host["val"],
                                    size=(prob.rows, prob.cols)).to(dev)
    b_dev = b_host.to(dev)
    op = amfls.DeviceOperator(a_dev)
    o = native_options(opts)
    lib = _native.load()
    stream = torch.cuda.current_stream(dev)
    x = torch.empty(prob.cols, dtype=torch.float64, device=dev)
    res = _native.Result()

    def solve_device():
        _native.check(lib.amfls_gpu_solve_amfls(op.handle, b_dev.data_ptr(), ctypes.byref(o),
                                                x.data_ptr(), ctypes.byref(res), None, None, 0,
                                                stream.cuda_stream))

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        solve_device()
    torch.cuda.synchronize()
    times = []
    launches = 0
    with ClockSampler(local) as clocks:
        barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solve_device()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
            launches += int(res.kernel_launches)
        torch.cuda.synchronize()
        barrier()
    t_step = statistics.mean(times)
    depth, status = res.depth, [res.status, res.stop_reason]
    cert = res.metrics[10]  # backward-error bound (lambda = 0)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([t_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())

    # end-to-end through the public API with host buffers
    e2e_times = []
    h2d = sum(t.numel() * t.element_size() for t in host.values()) + b_host.numel() * 8
    d2h = prob.cols * 8
    for i in range(max(1, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a = torch.sparse_csr_tensor(host["crow"].to(dev, non_blocking=True),
                                    host["col"].to(dev, non_blocking=True),
                                    host["val"].to(dev, non_blocking=True),
                                    size=(prob.rows, prob.cols))
        bb = b_host.to(dev, non_blocking=True)
        r = amfls.run_amfls(a, bb, **opts)
        sol = r.solution.cpu()
        dt = time.perf_counter() - t0
        if i > 0:
            e2e_times.append(dt)
        del a, bb, sol
    e2e = statistics.mean(e2e_times)

    peak, peak_kind = measured_peaks()
    roof = reorth_roofline(lib, prob.cols, max(32, depth // 2), stream.cuda_stream, peak,
                           peak_kind)
    roof["note"] = ("kernels at the solve's mean basis size (depth / 2 columns); the "
                    "operator products of this problem are latency-bound single-column "
                    "SpMVs (spmm carries the HBM-bound ones)")
    if prob.cols == SWEEP_CAPTURE["n"]:
        # DRAM bytes of the pair from one ncu capture of the same kernels at
        # n = 5000, k = 1900 (the only traffic figure a live run cannot read),
        # scaled to this basis size
        k = roof["basis_cols"]
        roof["traffic"] = SWEEP_CAPTURE["bytes"] * k / SWEEP_CAPTURE["k"]
        roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                  "sweep_vt_kernel + sweep_vc_kernel at n = 5000, k = 1900, "
                                  "scaled by k")

    legs = {}
    if rank == 0:
        if args.baselines:
            legs["baselines"] = baselines_measurement(dev, op, b_dev, prob, opts)
        if args.spmm:
            legs["spmm"] = spmm_measurement(dev, stream, peak)
        if args.dense:
            legs["dense"] = dense_measurement(dev)
        if args.learned:
            legs["learned"] = learned_measurement(dev)
        if args.batched > 0:
            legs["batched"] = batched_measurement(dev, args.batched)
        if args.c3:
            c3, _ = c3_measurement(dev)
            if "fp64" in c3 and "depth" in c3["fp64"]:
                c3["roofline"] = reorth_roofline(lib, c3["cols"], max(32, c3["fp64"]["depth"] // 2),
                                                 stream.cuda_stream, peak, peak_kind)
            if "mixed" in c3:
                c3["mixed"]["roofline"] = reduced_reorth_roofline(
                    lib, c3["cols"], C3_CYCLE // 2, stream.cuda_stream, peak, peak_kind,
                    C3_STORAGE_CODE)
                c3["mixed"]["roofline"]["note"] = "at the mean basis size of a restart cycle"
            legs["c3"] = c3
    if rank != 0:
        return
    cpu = cpu_baseline(prob, opts, args.workload) if args.cpu_sample and world == 1 else None
    line = base_line(args, world, t_step, bench_config(args.workload, prob, opts))
    line.update({"status": status, "depth": depth, "certificate": cert, "step_s": times,
                 "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h},
                 "roofline": roof, **legs, "cpu_baseline": cpu, "clocks": clocks.summary(),
                 "gpu_launches": launches})
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()

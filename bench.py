"""Time-to-tolerance benchmark of the GB300 AMFLS solver.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

A step is one complete AMFLS solve to tolerance of a seeded synthetic
problem with the workload's shape.  Prints one JSON line (rank 0).  The
default workload is the 100000 x 2000 column-major dense operator
G diag(d) (d geometric from 1 to 1e-6, b ~ N(0,1), lambda = 1e-6,
tol = 1e-10); --workload csr_20000x5000 runs the 20000 x 5000 CSR problem.

value     mean device time of one solve with the operator and b already in
          HBM (CUDA events around the C-ABI solve call, operator built once);
e2e       the same solve through the public API run_amfls on host tensors:
          host->device copy of the CSR arrays / dense matrix and b, operator
          construction, solve, device->host copy of the solution;
spmm      CSR SpMM and SpMM^T GB/s (s = 1 and 8) on the 2,000,000 x 500,000
          power-law matrix, the metric's second half;
mixed     time-to-tol of the mixed-precision form (FP32 inner solves refined
          in FP64, certified by the FP64 validation) next to plain FP64 on
          the 20000 x 5000 CSR problem, and the mixed form on the headline
          workload;
baselines AMFLS against the scalar LSQR and LSMR baselines on the 20000 x 5000
          CSR problem at its tolerance (seconds, status, iterations,
          certificate), the reference's own comparison;
batched   problems/s, p50 and p99 per-problem time of batched solves on a
          bounded sample of the uneven 256-problem CSR workload (sizes as
          described in the line), 16 workers against 1;
roofline  the dominant kernel timed live with CUDA events on its stream over
          repeated launches (algorithmic bytes per launch / mean duration);
          for the dense operator the FP64 issue rate, not HBM, is the bound,
          so the line also carries its FP64 rate against a cuBLAS DGEMM
          measured in the same run;
cpu_baseline  the oracle (the CPU restatement of the reference) on this host,
          timed on bounded depth-capped samples and extrapolated to the GPU's
          depth with a fitted t(D) = a D + b D^2 (per-level cost grows with
          the basis); the sample is described in the line.
--impl reference times the same CPU restatement the same way (the reference
itself cannot be built on this host: its sources are not shipped here).
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="dense_100000x2000")
    ap.add_argument("--cpu-sample", type=int, default=1, help="0 skips the cpu_baseline leg")
    ap.add_argument("--spmm", type=int, default=1,
                    help="0 skips the CSR SpMM GB/s measurement on the 2M x 500k matrix")
    ap.add_argument("--mixed", type=int, default=1, help="0 skips the mixed-precision leg")
    ap.add_argument("--baselines", type=int, default=1,
                    help="0 skips the AMFLS vs LSQR / LSMR leg on the 20000 x 5000 CSR problem")
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
    prob, opts = problems.make(name, seed=20251203)
    return prob, opts


# oracle levels per depth-capped CPU sample (the larger of the two samples)
CPU_SAMPLE_LEVELS = {"dense_100000x2000": 240, "csr_20000x5000": 768}


def algorithmic_bytes(prob):
    """Bytes one single-column product moves at minimum (int32 indices and
    row offsets in HBM; the mean of A v and A^T u for CSR)."""
    if hasattr(prob, "row_offsets"):
        nnz = prob.nnz
        return nnz * (8 + 4) + (0.5 * (prob.rows + prob.cols) + 1) * 4 + (prob.rows + prob.cols) * 8
    m, n = prob.rows, prob.cols
    return 8 * m * n + 8 * (m + n)


# ------------------------------------------------------------ CPU legs ----

def cpu_estimate(prob, opts, gpu_depth, budget_levels):
    """Oracle time-to-tol estimate: operator construction timed once, then
    three depth-capped solves on the built operator, fitted exactly by
    t(D) = c + a D + b D^2 (b >= 0; otherwise the line through the two
    deepest samples) and evaluated at the GPU's depth."""
    from oracle import amfls_oracle as orc
    t0 = time.perf_counter()
    op = orc.Operator(prob)
    t_op = time.perf_counter() - t0
    d3 = max(6, min(budget_levels, gpu_depth))
    ds = [max(2, d3 // 3), max(4, (2 * d3) // 3), d3]
    ts = []
    for d in ds:
        t0 = time.perf_counter()
        orc.solve_amfls_operator(op, prob.b, maximum_depth=d, **opts)
        ts.append(time.perf_counter() - t0)
    x = np.array(ds, dtype=np.float64)
    c, a, b = np.linalg.solve(np.stack([np.ones(3), x, x * x], axis=1), np.array(ts))
    if b < 0.0 or a < 0.0:
        a = (ts[2] - ts[1]) / (x[2] - x[1])
        c, b = ts[2] - a * x[2], 0.0
    k = float(gpu_depth)
    solve = c + a * k + b * k * k if gpu_depth > d3 else ts[2]
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": t_op + solve, "unit": "s", "cores": threads, "kind": "port",
            "sample": (f"oracle (CPU restatement; dense products through the host BLAS) on "
                       f"{threads} host threads: operator construction {t_op:.2f} s, solves "
                       f"capped at depth {ds[0]}, {ds[1]}, {ds[2]} ({ts[0]:.2f}, {ts[1]:.2f}, "
                       f"{ts[2]:.2f} s) fitted by c + a D + b D^2 and evaluated at the "
                       f"GPU's depth {gpu_depth}")}


def fp64_dgemm_tflops(dev, stream):
    """cuBLAS DGEMM rate on this GPU (best of 3), the FP64 denominator."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    best = 0.0
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        torch.matmul(a, b)
        e1.record(stream)
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


# DRAM bytes (read + write) per launch of the dominant kernel from one ncu
# capture of the same workload (profiles/dense_block_product_100000x2000_full.md:
# mean of the A v and A^T u launches), or None when no capture covers it
TRAFFIC = {"dense_100000x2000": 0.5 * ((1.600079e9 + 7.885824e6) + (1.604726e9 + 3.578112e6))}


SPMM_WORKLOAD = "csr_2000000x500000"


def spmm_measurement(dev, stream, peak):
    """CSR SpMM / SpMM^T HBM GB/s on the 2,000,000 x 500,000 power-law matrix
    (40.2M nonzeros), s = 1 and s = 8 columns, through the C ABI on
    preallocated column-major device blocks (CUDA events on the stream).
    Algorithmic bytes: nnz (8 + 4) + (rows + 1) 4 + s (m + n) 8."""
    import ctypes
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import _native, problems

    prob, _ = problems.make(SPMM_WORKLOAD, seed=20251203)
    a = torch.sparse_csr_tensor(torch.from_numpy(prob.row_offsets),
                                torch.from_numpy(prob.column_indices),
                                torch.from_numpy(prob.values),
                                size=(prob.rows, prob.cols)).to(dev)
    op = amfls.DeviceOperator(a)
    lib = _native.load()
    m, n, nnz = prob.rows, prob.cols, prob.nnz
    out = {"workload": SPMM_WORKLOAD, "rows": m, "cols": n, "nnz": nnz, "peak_gbs": peak,
           "unit": "GB/s"}
    for cols in (1, 8):
        x = torch.randn(cols * n, dtype=torch.float64, device=dev)
        y = torch.randn(cols * m, dtype=torch.float64, device=dev)
        res = {}
        for name, fn, src, dst, rows_out in (
                ("apply", lib.amfls_gpu_operator_apply, x, y, m),
                ("apply_transpose", lib.amfls_gpu_operator_apply_transpose, y, x, n)):
            def call():
                _native.check(fn(op.handle, ctypes.c_void_p(src.data_ptr()), cols,
                                 ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(stream.cuda_stream)))
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


def baselines_measurement(dev):
    """AMFLS against the scalar LSQR and LSMR baselines (the reference's own
    comparison) on the 20000 x 5000 CSR problem at its tolerance: host wall
    clock around each synchronous C-ABI solve on one prebuilt operator, after
    one warm-up each, with status, iterations and certificate.  An error is
    reported in the object rather than raised."""
    import ctypes
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import binding, _native

    try:
        prob, opts = make_workload("csr_20000x5000")
        a = torch.sparse_csr_tensor(torch.from_numpy(prob.row_offsets),
                                    torch.from_numpy(prob.column_indices),
                                    torch.from_numpy(prob.values),
                                    size=(prob.rows, prob.cols)).to(dev)
        op = amfls.DeviceOperator(a)
        b = torch.from_numpy(prob.b).to(dev)
        reg, tol = opts["regularization"], opts["tolerance"]
        o = _native.default_options()
        for k, v in opts.items():
            setattr(o, k, v)
        ob = _native.BaselineOptions()
        _native.load().amfls_gpu_default_baseline_options(ctypes.byref(ob))
        ob.regularization, ob.tolerance = reg, tol
        out = {"workload": "csr_20000x5000", "tolerance": tol, "regularization": reg,
               "maximum_iterations": min(prob.rows, prob.cols)}
        for name, options in (("amfls", o), ("lsqr", ob), ("lsmr", ob)):
            def run():
                return binding._decode(binding._solve_raw(name, op, b, options))
            run()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = run()
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            out[name] = {"s": t, "status": r.status, "stop_reason": r.stop_reason,
                         "iterations": r.depth,
                         "certificate": r.relative_energy_error_upper_bound if reg > 0
                         else r.backward_error_upper_bound}
        return out
    except Exception as e:  # reported, not fatal to the bench line
        return {"error": f"{type(e).__name__}: {e}"}


def mixed_measurement(dev, headline_op, headline_b, headline_opts):
    """Plain FP64 vs mixed FP32 time-to-tol (host wall clock around the
    synchronous C-ABI solves, after one warm-up each)."""
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import binding, _native

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    def cert(r, reg):
        return r.relative_energy_error_upper_bound if reg > 0 else r.backward_error_upper_bound

    out = {}
    prob, opts = make_workload("csr_20000x5000")
    a = torch.sparse_csr_tensor(torch.from_numpy(prob.row_offsets),
                                torch.from_numpy(prob.column_indices),
                                torch.from_numpy(prob.values), size=(prob.rows, prob.cols)).to(dev)
    op = amfls.DeviceOperator(a)
    b = torch.from_numpy(prob.b).to(dev)
    o = _native.default_options()
    for k, v in opts.items():
        setattr(o, k, v)
    plain, t_plain = timed(lambda: binding._decode(binding._solve_raw("amfls", op, b, o)))
    low = op.reduced("fp32")
    mixed, t_mixed = timed(lambda: amfls.run_amfls_mixed(op, b, reduced=low, inner_tolerance=1e-7,
                                                         maximum_refinements=6, **opts))
    out["csr_20000x5000"] = {
        "tolerance": opts["tolerance"],
        "fp64": {"s": t_plain, "status": plain.status, "depth": plain.depth,
                 "certificate": cert(plain, 0.0)},
        "mixed_fp32": {"s": t_mixed, "status": mixed.status, "levels": mixed.depth,
                       "steps": int(mixed.trace_float.shape[0]), "inner_tolerance": 1e-7,
                       "certificate": cert(mixed, 0.0),
                       "x_rel_diff_vs_fp64": float(torch.linalg.norm(mixed.solution - plain.solution)
                                                   / torch.linalg.norm(plain.solution))},
        "speedup": t_plain / t_mixed}
    reg = headline_opts.get("regularization", 0.0)
    hlow = headline_op.reduced("fp32")
    hm, t_hm = timed(lambda: amfls.run_amfls_mixed(headline_op, headline_b, reduced=hlow,
                                                   inner_tolerance=1e-7, maximum_refinements=6,
                                                   **headline_opts))
    out["headline"] = {"s": t_hm, "status": hm.status, "levels": hm.depth,
                       "steps": int(hm.trace_float.shape[0]), "certificate": cert(hm, reg)}
    return out


def batched_measurement(dev, count):
    """Batched solves of a bounded sample of the uneven CSR workload."""
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import problems

    batch = problems.uneven_csr_batch(count, seed=20251203, m_range=(2_000, 50_000),
                                      n_range=(500, 12_500))
    mats = [(amfls.DeviceOperator(torch.sparse_csr_tensor(
        torch.from_numpy(p.row_offsets), torch.from_numpy(p.column_indices),
        torch.from_numpy(p.values), size=(p.rows, p.cols)).to(dev)),
        torch.from_numpy(p.b).to(dev)) for p, _, _ in batch]
    regs = [r for _, r, _ in batch]
    out = {"sample": (f"{count} problems of the uneven workload's distribution with m in "
                      f"[2e3, 5e4] and n in [500, 1.25e4] (the full ranges reach 2e5 x 5e4); "
                      f"5-40 nonzeros per row, condition 1e3-1e8, lambda 1e-8-1e-2, tol 1e-9"),
           "nnz": int(sum(p.nnz for p, _, _ in batch))}
    for workers in (16, 1):
        res, secs, wall = amfls.run_amfls_batch(mats, workers=workers, regularization=regs,
                                                tolerance=1e-9)
        st = [r.status for r in res]
        out[f"workers_{workers}"] = {
            "problems_per_s": count / wall, "wall_s": wall,
            "p50_s": float(np.percentile(secs, 50)), "p99_s": float(np.percentile(secs, 99)),
            "certified": st.count(0), "levels": int(sum(r.depth for r in res))}
    return out


# --------------------------------------------------------------- arms ----

# depth of the full solve on each workload (bench seed 20251203)
# (the dense workload never meets its tolerance before the basis fills the
# 2000 columns, on the reference and on this solver alike)
KNOWN_DEPTH = {"csr_20000x5000": 3797, "dense_100000x2000": 2000}

def run_reference(args, world, rank):
    if rank != 0:
        return
    prob, opts = make_workload(args.workload)
    # depth the solve reaches on this workload (same counters on both arms:
    # CSR levels never widen), measured by full solves
    depth_hint = int(os.environ.get("AMFLS_BENCH_DEPTH_HINT", "0")) or \
        KNOWN_DEPTH.get(args.workload, 4096)
    vals = []
    for i in range(args.warmup + args.steps):
        est = cpu_estimate(prob, opts, depth_hint, CPU_SAMPLE_LEVELS.get(args.workload, 512))
        if i >= args.warmup:
            vals.append(est)
    v = statistics.mean(e["value"] for e in vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": {"workload": args.workload},
            "cpu_baseline": dict(vals[-1], value=v),
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import _native
    import ctypes

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    amfls.load_library()
    prob, opts = make_workload(args.workload)
    is_csr = hasattr(prob, "row_offsets")
    if is_csr:
        host = dict(crow=torch.from_numpy(prob.row_offsets), col=torch.from_numpy(prob.column_indices),
                    val=torch.from_numpy(prob.values))
        for k in host:
            host[k] = host[k].pin_memory()
        mat_dev = torch.sparse_csr_tensor(host["crow"], host["col"], host["val"],
                                          size=(prob.rows, prob.cols)).to(dev)
    else:
        # column-major workloads travel as the row-major buffer of A^T and
        # are used on the device as the transposed (column-major) view
        col_major = not prob.matrix.flags.c_contiguous
        buf = np.ascontiguousarray(prob.matrix.T if col_major else prob.matrix)
        host = dict(mat=torch.from_numpy(buf).pin_memory())
        as_matrix = (lambda t: t.t()) if col_major else (lambda t: t)
        mat_dev = as_matrix(host["mat"].to(dev))
    b_host = torch.from_numpy(prob.b).pin_memory()
    b_dev = b_host.to(dev)
    op = amfls.DeviceOperator(mat_dev)
    o = _native.default_options()
    for k, v in opts.items():
        setattr(o, k, v)
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
    depth = res.depth
    status = (res.status, res.stop_reason)
    # timed region (inputs larger than L2 or not, every solve rebuilds its
    # basis from scratch; the matrix is re-read every level)
    times = []
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
        torch.cuda.synchronize()
        barrier()
    t_step = statistics.mean(times)
    launches = int(res.kernel_launches)  # per solve, counted by the library
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([t_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())

    # end-to-end through the public API with host buffers
    e2e_times = []
    h2d = sum(t.numel() * t.element_size() for t in host.values()) + b_host.numel() * 8
    d2h = prob.cols * 8 + (21 + 36 + 9) * 8
    for i in range(max(1, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if is_csr:
            a = torch.sparse_csr_tensor(host["crow"].to(dev, non_blocking=True),
                                        host["col"].to(dev, non_blocking=True),
                                        host["val"].to(dev, non_blocking=True),
                                        size=(prob.rows, prob.cols))
        else:
            a = as_matrix(host["mat"].to(dev, non_blocking=True))
        bb = b_host.to(dev, non_blocking=True)
        r = amfls.run_amfls(a, bb, **{k: v for k, v in opts.items()})
        sol = r.solution.cpu()
        dt = time.perf_counter() - t0
        if i > 0:
            e2e_times.append(dt)
        del a, bb, sol
    e2e = statistics.mean(e2e_times)

    # dominant-kernel roofline: the operator products (A v and A^T u
    # alternate in every level), timed live on the launching stream
    vec = torch.randn(prob.cols, dtype=torch.float64, device=dev)
    uvec = torch.randn(prob.rows, dtype=torch.float64, device=dev)

    def timed(fn, reps=40):
        for _ in range(5):
            fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / reps

    kt_a = timed(lambda: op.apply(vec))
    kt_at = timed(lambda: op.apply(uvec, transpose=True))
    kt = 0.5 * (kt_a + kt_at)
    peak, peak_kind = measured_peaks()
    nbytes = algorithmic_bytes(prob)
    achieved = nbytes / kt / 1e9
    roof = {"kernel": ("tile_product_kernel<double,1,256,fused> (A v, A^T u)" if is_csr else
                       "dot_block_kernel<1> (A^T u) / across_block_kernel<1> (A v)"),
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": TRAFFIC.get(args.workload),
            "launch_us": {"apply": kt_a * 1e6, "apply_transpose": kt_at * 1e6},
            "algorithmic_bytes": nbytes}
    if not is_csr:
        flops = 2.0 * prob.rows * prob.cols
        roof["fp64"] = {"achieved_tflops": flops / kt / 1e12,
                        "dgemm_tflops": fp64_dgemm_tflops(dev, stream),
                        "note": "FP64 issue-bound: 2 flops per 8-byte element against "
                                "the FP64 ridge; dgemm_tflops is cuBLAS DGEMM 4096^3 "
                                "measured in this run"}
        roof["fp64"]["frac"] = roof["fp64"]["achieved_tflops"] / roof["fp64"]["dgemm_tflops"]

    spmm = spmm_measurement(dev, stream, peak) if args.spmm else None
    mixed = mixed_measurement(dev, op, b_dev, opts) if args.mixed and rank == 0 else None
    baselines = baselines_measurement(dev) if args.baselines and rank == 0 else None
    batched = batched_measurement(dev, args.batched) if args.batched > 0 and rank == 0 else None

    if rank != 0:
        return
    cpu = None
    if args.cpu_sample and world == 1:
        levels = int(os.environ.get("AMFLS_BENCH_CPU_LEVELS", "0")) or \
            CPU_SAMPLE_LEVELS.get(args.workload, 512)
        cpu = cpu_estimate(prob, opts, depth, levels)
    line = {"metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded numpy generator)",
            "config": {"workload": args.workload, "rows": prob.rows, "cols": prob.cols,
                       "nnz": prob.nnz if is_csr else prob.rows * prob.cols, **opts,
                       "l2": "inputs larger than L2: every product re-reads the matrix "
                             "(CSR arrays or the 1.6 GB dense matrix) and every level "
                             "sweeps the basis; each solve rebuilds the basis from scratch",
                       "depth": depth, "status": list(status), "parallelism": "replicas"},
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": roof, "spmm": spmm, "mixed": mixed, "baselines": baselines, "batched": batched,
            "cpu_baseline": cpu, "clocks": clocks.summary(),
            "gpu_launches": launches * args.steps}
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

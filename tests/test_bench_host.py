"""Host-side parts of bench.py; CPU only.

  * the clock record: median SM clock under load, the maximum, and the
    throttle reasons that were active in any sample (a run that saw a
    hardware or thermal slowdown is rejected on that record);
  * the reference arm (--impl reference): one JSON line with the same
    metric, unit, direction and config keys as the GPU arm, impl
    "reference", a cpu_baseline describing the run and an e2e object with
    no host-device traffic, from complete oracle solves of the headline
    workload (one timed solve here, about 20 s on 8 cores).
"""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def row(sm, mx, *reasons):
    flags = ["Active" if r else "Not Active" for r in reasons]
    return ["0", str(sm), str(mx), "900.0", "0x0", *flags]


def test_clock_summary():
    s = bench.ClockSampler()
    assert s.summary()["reasons"] == ["unsampled"]
    s.samples = [row(2070, 2070, 0, 0, 0, 0), row(1980, 2070, 0, 0, 0, 1),
                 row(2055, 2070, 0, 0, 0, 0), row("[N/A]", "[N/A]", 0, 0, 0, 0)]
    out = s.summary()
    assert out["sm_mhz"] == 2055.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"] and out["samples"] == 4
    s.samples.append(row(1500, 2070, 1, 0, 1, 0))
    assert bench.ClockSampler.summary(s)["reasons"] == ["hw_slowdown", "sw_power_cap",
                                                        "sw_thermal_slowdown"]


def test_reference_arm_prints_the_contract_line():
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         env=env, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["unit"] == "s" and line["higher_is_better"] is False
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 0
    assert line["status"] == [0, 8] and line["depth"] == 3786  # the reference's own outcome
    cfg = line["config"]
    assert (cfg["workload"], cfg["rows"], cfg["cols"], cfg["nnz"], cfg["seed"]) == \
        ("csr_20000x5000", 20000, 5000, 200000, bench.SEED)
    assert line["cpu_baseline"]["value"] == line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert len(line["step_s"]) == 1


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun only rank 0 runs the reference arm; the others exit 0
    without work and print nothing."""
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--gpus", "2", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, env=env, cwd=ROOT, timeout=120)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""

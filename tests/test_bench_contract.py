"""Host-side checks of bench.py's output contract (no GPU): the seeded workload, the
roofline entry per kernel class, and the reference arm's JSON line."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_workload_is_seeded_and_in_range():
    b1, c1 = bench.workload(256, 2026)
    b2, c2 = bench.workload(256, 2026)
    assert (b1 == b2).all() and (c1 == c2).all()
    assert b1.min() >= 0.30 and b1.max() <= 0.60
    assert set(c1.tolist()) <= set(bench.CHIS)


def test_roofline_per_class():
    peaks = {"bf16_tflops": 1949.5, "hbm_gbs": 6782.4}
    # (launches, total ms, work): 1e12 flop per tc launch in 10 ms; 2e9 bytes per split launch in 2 ms
    prof = {"tc": (10, 100.0, 1e13), "split": (5, 10.0, 1e10), "chol": (3, 1.0, 1e6)}
    r = bench.roofline(prof, "tc", 1, None, peaks)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert abs(r["achieved"] - 100.0) < 1e-9
    assert abs(r["mma_achieved"] - 600.0) < 1e-9          # six BF16 plane products per 2mnk
    assert abs(r["frac"] - 100.0 / 1949.5) < 1e-12
    r = bench.roofline(prof, "split", 1, None, peaks)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert abs(r["achieved"] - 1000.0) < 1e-9
    assert abs(r["frac"] - 1000.0 / 6782.4) < 1e-12
    r = bench.roofline(prof, "chol", 1, None, peaks)
    assert r["bound"] == "latency" and r["achieved"] is None
    assert bench.roofline({"tc": (0, 0.0, 0.0)}, "tc", 1, None, peaks) is None


def test_reference_arm_prints_one_json_line():
    """`bench.py --impl reference` times the oracle on the host and prints the reference
    arm's line: impl, cpu_baseline and an e2e entry with zero transfer bytes."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--cpu-budget", "2", "--instances", "16"],
                         capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.strip().splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "config", "impl",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["metric"] == bench.METRIC

"""bench.py's reference arm on the CPU (the oracle port of the reference's
gather matvec, all host cores): one JSON line with the contract's keys, the
same metric and workload naming as the GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line(tmp_path):
    env = dict(os.environ, DOCI_BENCH_CACHE=str(tmp_path))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--L", "12",
                        "--N", "6", "--seed", "5", "--steps", "2", "--warmup", "1", "--cpu-seconds", "0.5"],
                       capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2
    assert d["config"]["workload"] == "DOCI sigma L=12 N=6 D=924 seed=5"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["metric"].startswith("sigma Gdet/s")


def test_reference_arm_prepares_once_and_finishes(tmp_path):
    """At 40 timed steps after 5 warm-ups the arm must end within its budget:
    the sample (rows, diagonal) is prepared for the calibration run and the
    sized sample only, never per step; L=20 keeps the sample cheap."""
    import time
    env = dict(os.environ, DOCI_BENCH_CACHE=str(tmp_path))
    t0 = time.perf_counter()
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--L", "20",
                        "--N", "10", "--seed", "3", "--steps", "40", "--warmup", "5", "--cpu-seconds", "0.2"],
                       capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    wall = time.perf_counter() - t0
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][0])
    assert d["sample_preparations"] <= 2
    assert d["steps"] == 40 and d["warmup"] == 5
    # 45 steps of at most 0.2 s of matvec each, plus setup
    assert wall < 120, wall

"""The bench's reference arm on the CPU: `bench.py --impl reference` prints
one JSON line with the keys of the measurement contract, the same metric and
workload name as the GPU arm (both come from `workload_name`), and an e2e
figure with no host-device traffic (the arm runs on the host cores)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    sys.path.insert(0, ROOT)
    import bench
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--rows", "96", "--cols", "128",
           "--cpu-rows", "8", "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "px/s"
    assert line["steps"] == 2 and line["warmup"] == 1 and line["higher_is_better"] is True
    assert line["config"]["workload"] == bench.workload_name(96, 128, "MLE")
    assert line["value"] > 0 and line["ms_per_step"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "px/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}

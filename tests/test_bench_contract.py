"""The benchmark's reference arm on the CPU: one JSON line with the keys the
benchmark contract names (metric, value, unit, config, cpu_baseline with the
core count and the kind of baseline, e2e with zero host/device bytes), on the
same workload name and metric as the GPU arm, within a small time budget."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    proc = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1",
                           "--n", "129", "--cpu-seconds", "1"], cwd=ROOT, capture_output=True, text=True,
                          timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [l for l in proc.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, proc.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "config", "cpu_baseline", "e2e", "impl", "dtype", "data", "scaling", "vs_baseline"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "GLUP/s" and d["higher_is_better"]
    assert d["steps"] == 2 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    sys.path.insert(0, ROOT)
    import bench
    assert d["metric"] == bench.METRIC
    assert d["config"]["workload"] == bench.workload_name(129)

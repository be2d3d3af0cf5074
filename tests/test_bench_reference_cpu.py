"""bench.py's reference arm runs on the host cores alone: the oracle (the
reference algorithm restated: dense forward-mode Jacobian and LU) on a
bounded sample of the default workload, reported with the GPU arm's metric,
unit and configuration."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                          "--cpu-seconds", "2", "--ref-step-seconds", "0.5"], cwd=ROOT, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    import bench

    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1 and d["higher_is_better"] is True
    assert d["config"]["workload"] == bench.DEFAULT_WORKLOAD and d["config"]["steps_on_outputs"] is True
    assert d["e2e"]["unit"] == d["unit"] and d["e2e"]["value"] == d["value"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "extrapolated" in cb
    assert d["cpu_structured"]["value"] > 0

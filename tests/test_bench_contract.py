"""bench.py's reference arm on the host (no GPU): the JSON line the contract
asks for, on the smallest workload, with the warm-up and step counts it was
given and the same config dict the GPU arm prints."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "vortex20", "--steps", "2", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["warmup"] == 3 and 1 <= d["steps"] <= 2 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["kind"] in ("port", "reference")
    sys.path.insert(0, ROOT)
    import bench
    K, Np = d["config"]["K"], d["config"]["Np"]
    assert d["config"] == bench.workload_config("vortex20", K, Np)
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT

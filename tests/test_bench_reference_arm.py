"""bench.py's reference arm on CPU: it times the oracle on the host cores (the reference's CPU
baker restated; the Rust reference cannot be built here), prints one JSON line with the same
metric string as the GPU arm so the two compare directly, names the bounded sample it timed, and
reports no host-device copies. CPU only (a one-step run of the small-room workload)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_shared_metric():
    oracle_lib = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
    if not os.path.exists(oracle_lib):
        pytest.skip("oracle not built (run __graft_entry__.build())")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "small_room", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["unit"] == "rays/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"] == "small_room" and line["config"]["timed_sample"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}

"""bench.py's reference arm on the host (no GPU): one JSON line with the
contract's keys, the oracle's port timed on a bounded sample; the other
workloads' reference arms say where their CPU figure is instead of running
the GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench(*args):
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    r = bench("--impl", "reference", "--nb", "20000", "--nq", "100", "--ref-queries", "20",
              "--steps", "2", "--warmup", "1")
    assert r["impl"] == "reference" and r["value"] > 0 and r["unit"] == "queries/s"
    assert r["higher_is_better"] is True and r["steps"] == 2 and r["warmup"] == 1
    assert r["config"]["nb"] == 20000 and "workload" in r["config"]
    cb = r["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == r["value"]
    assert r["e2e"] == {"value": r["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


@pytest.mark.parametrize("workload", ["kmeans1", "kmeans3", "hkm4", "knn_batch", "gmm"])
def test_reference_arm_other_workloads(workload):
    r = bench("--impl", "reference", "--workload", workload)
    assert r["impl"] == "reference" and "cpu_baseline" in r["unavailable"]

"""CPU: bench.py's reference arm prints one JSON line that keeps the bench
contract (metric, value, unit, impl, e2e, cpu_baseline with cores and CPU
model), on a small seeded genome so that it finishes in seconds."""

import json
import subprocess
import sys

from conftest import REPO


def test_reference_arm_prints_the_contract_line():
    cmd = [sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1",
           "--warmup", "3", "--genome-len", "200000", "--coverage", "5",
           "--reference-sample", "12"]
    out = subprocess.run(cmd, capture_output=True, text=True, check=True, timeout=600,
                         cwd=REPO).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    sys.path.insert(0, str(REPO))
    import bench
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["impl"] == "reference" and line["n_gpus"] == 1
    assert line["steps"] == 1 and line["warmup"] == 3
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["data"] == "synthetic" and "workload" in line["config"]
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["kind"] == "port"
    assert cpu["cores"] >= 1 and cpu["cpu_model"] and cpu["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # both arms describe the workload with the same config object
    import argparse
    args = argparse.Namespace(seed=2, genome_len=200000, coverage=5.0)
    assert line["config"] == json.loads(json.dumps(bench.bench_config(bench.make_workload(args))))

"""CPU checks of bench.py's contract: the reference arm's JSON line (it runs the
reference's CPU simplifier, or the oracle port where that is not built, on the
host cores, no GPU) and the traffic table's kernel groups."""
import json
import os
import subprocess
import sys

from parafrost_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--batch-n", "24"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["metric"] == "inprocessing clauses/s (BVE+SUB)" and line["unit"] == "clauses/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["config"]["workload"] == "batched"
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_traffic_table_names_profiler_groups():
    import bench
    L = _lib.lib()
    groups = {L.pfg_profile_name(i).decode() for i in range(L.pfg_profile_count())}
    assert bench.TRAFFIC
    for (workload, group), per_launch in bench.TRAFFIC.items():
        assert workload in ("batched",) or workload in bench.WORKLOADS
        assert group in groups, group
        assert per_launch > 0

"""The benchmark's reference arm (the reference's own CPU kernel, compiled
from its source into oracle/_ref, or where that source is absent the
oracle's C restatement of it, on the host cores) runs without a GPU and
prints one JSON line with the same metric as the GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "fcc_cu_32k",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["unit"] == "Gatom*pixel/s" and line["higher_is_better"] is True
    import oracle
    kind = "reference" if oracle.ref_lib() is not None else "port"
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == kind
    assert line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["config"]["workload"] == "fcc_cu_32k"

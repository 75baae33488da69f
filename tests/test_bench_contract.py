"""bench.py's reference arm prints the benchmark's JSON line, on the CPU.

`python bench.py --impl reference` times the oracle's single-threaded CG +
Jacobi on the 128^3 benchmark system: whole 536-iteration solves, with the
same metric, unit and `config` as the GPU arm, so the two lines compare
directly.  One step, no warm-up (about half a minute of CPU)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench

    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "ms"
    assert line["higher_is_better"] is False and line["n_gpus"] == 1
    assert line["steps"] == 1 and line["warmup"] == 0
    assert line["config"] == bench.config(1)  # the GPU arm prints the same dict
    assert line["result"]["iterations"] == 536 and line["result"]["reason"] == 2
    assert line["value"] > 0 and line["ms_per_step"] == line["value"]
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["kind"] == "port" and cpu["cores"] == 1
    assert cpu["os_cpu_count"] >= 1 and cpu["cpu_model"]
    assert "536-iteration" in cpu["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "ms", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}

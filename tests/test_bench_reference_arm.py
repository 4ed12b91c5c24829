"""`bench.py --impl reference` on the CPU: one JSON line in the benchmark's
contract (the headline metric, unit and workload, a cpu_baseline describing the
run, an e2e with no host transfers), and the only repository library the process
maps is the oracle's: the reference arm never loads the GPU library, so its
figure owes nothing to the code it is compared with."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line_and_libraries():
    sys.path.insert(0, ROOT)
    import bench
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.METRIC
    assert line["config"]["workload"] == bench.HEADLINE_WORKLOAD
    # fewer than three warm-up steps are raised to three (the timing rule)
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 3
    assert line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.METRIC, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["native_libraries"] == ["oracle/_build/libgpe_oracle.so"]

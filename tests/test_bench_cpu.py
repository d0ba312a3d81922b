"""The bench's reference arm runs on the CPU alone (the oracle's counter and the restated reference
preprocessing): its JSON line keeps the contract's keys."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line_on_cpu():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "rmat16",
                          "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600, env=env,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GTEPS" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 3
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert cb["single_core"]["cores"] == 1 and cb["single_core"]["gteps"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    rp = line["reference_preprocess"]
    assert rp["cores"] == 1 and rp["kind"] == "port" and 0 < rp["pairs"] <= rp["of_pairs"] and rp["seconds"] > 0
    assert "reference_kernel_sm103a" in line  # timed on a GPU host, else the reason it was not

"""The one-line JSON contract of bench.py, on the arm that runs without a GPU:
`--impl reference` (the reference's shaders compiled for the CPU, else the
oracle port) on a small mosaic. It prints one line with the metric, unit and
direction of the GPU arm, its CPU baseline record and an end-to-end object with
no host-device bytes, and its process maps no library of this package."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUN = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--size", "256x192", "--steps", "1", "--warmup", "1"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    if e.code not in (None, 0):
        raise
maps = open("/proc/self/maps").read()
print("MAPS_PRODUCT", int("libvkdt_cuda" in maps))
"""


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "-c", RUN], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    if "unavailable" in d:
        assert d["impl"] == "reference"
        return
    assert d["impl"] == "reference" and d["unit"] == "MP/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert "workload" in d["config"] and d["config"]["wd"] == 256 and d["config"]["ht"] == 192
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # the reference arm never maps the product library
    assert "MAPS_PRODUCT 0" in r.stdout, r.stdout

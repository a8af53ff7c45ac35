"""bench.py --impl reference (CPU only): the JSON line of the reference arm, which
times the FP64 CPU oracle on the full configuration (K steps after W warm-ups)
through the oracle's own case builder, without loading the GPU library."""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

# runs the reference arm in this process, then reports which of the project's
# shared libraries the process mapped
PROBE = r"""
import sys
sys.argv = ["bench.py", "--impl", "reference", "--config", "1", "--steps", "1", "--warmup", "3"]
import runpy
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPPED", "libpgdg_gpu" in maps, "liboracle" in maps)
"""


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "-c", PROBE], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["steps"] == 1 and d["warmup"] == 3
    assert d["value"] > 0 and d["unit"] == "cell-stage/s" and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]
    # the triple point's full configuration fits any host: the same grid as the GPU arm
    assert d["config"]["same_config"] is True and d["config"]["grid"] == [112, 48]
    # the oracle only: the GPU library is never loaded on this arm
    mapped = [l for l in r.stdout.splitlines() if l.startswith("MAPPED")]
    assert mapped == ["MAPPED False True"], r.stdout[-500:]

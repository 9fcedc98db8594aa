"""The benchmark's CPU arm (`bench.py --impl reference`), on the host only.

The arm times the C restatement of the correlator node on the host cores and
must never build or map the GPU library: its number is the CPU path's own.
This runs it on the small 2-station configuration, one step, in a fresh
process, and checks its JSON line and that process's memory map.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RUNNER = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--config", "c1", "--steps", "1", "--warmup", "0",
            "--cpu-sample-us", "31250"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPPED_GPU_LIBRARY", int("libsfxc_gpu" in maps))
"""


def test_reference_arm_line_and_no_gpu_library():
    env = dict(os.environ, WORLD_SIZE="1", RANK="0")
    r = subprocess.run([sys.executable, "-c", _RUNNER], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "MAPPED_GPU_LIBRARY 0"
    line = json.loads([ln for ln in lines if ln.startswith("{")][-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "Gsamples/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1
    base = line["cpu_baseline"]
    assert base["kind"] == "port" and base["value"] == line["value"]
    assert 1 <= base["cores"] <= base["nproc"]
    assert "lower bound" in base["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"].startswith("2 stations")

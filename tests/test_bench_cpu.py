"""bench.py's CPU legs, without a GPU: the reference arm (the float64 CPU
port of Simulation.step) runs on the host cores, prints the contract's
JSON line, and never loads the engine's library (it must time the
reference's path only)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import sys
sys.argv = ["bench.py", "--impl", "reference", "--size", "32", "--steps", "2", "--warmup", "1"]
sys.path.insert(0, ".")
import bench
bench.main()
maps = open("/proc/self/maps").read()
print("ENGINE_LIBRARY_MAPPED=%d" % ("libflowlab_gb300" in maps))
"""


def test_reference_arm_runs_without_the_engine_library():
    out = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    line = json.loads(next(x for x in lines if x.startswith("{")))
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["cores"] == 1 and line["cpu_baseline"]["host_cores"] >= 1
    assert lines[-1] == "ENGINE_LIBRARY_MAPPED=0"

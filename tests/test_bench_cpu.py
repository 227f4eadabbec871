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


def test_algorithmic_bytes_per_cell():
    """The per-cell byte counts behind the bench's roofline figures: a
    V(3,3) finest level 65 B down (three sweep pairs of 18 and 11 for the
    residual and restriction) and 64 up, MacCormack velocity 60 and dye 78
    per step over two launches, the defect pass 21, the end-of-step scan 8
    plus 13 on the residual diagnostic's steps."""
    sys.path.insert(0, ROOT)
    import bench
    from flowlab_gb300 import configs

    prm = configs.plume_params()
    b = bench.phase_bytes_per_cell(prm, 1024)
    assert b["mg_fine"] == (3 * 18 + 11 + 10 + 3 * 18) / 2 == 64.5
    assert b["advect_velocity"] == 30 and b["advect_dye"] == 39
    assert b["defect64"] == 21 and b["project"] == 21 and b["divergence"] == 12
    assert b["cfl"] == 8 + 13
    # levels 512^2..64^2 above the 32^2 tail, per launch averaged
    mid = sum((n / 1024) ** 2 for n in (512, 256, 128, 64))
    assert abs(b["mg_pre"] - 65 * mid / 4) < 1e-12 and abs(b["mg_post"] - 64 * mid / 4) < 1e-12
    prm.residual_every = 0
    assert bench.phase_bytes_per_cell(prm, 1024)["cfl"] == 8

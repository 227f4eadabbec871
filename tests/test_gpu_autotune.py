"""The autotuner on the GPU: its red-black tile depth leaves results
unchanged, and a tuned multigrid still reaches the tolerance."""
import numpy as np
import pytest

from flowlab_gb300 import autotune, configs, native
from flowlab_gb300.native import f32, ptr

pytestmark = pytest.mark.gpu


def run(scene, prm, steps):
    g, f, patch = scene
    e = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        if patch is not None:
            e.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        e.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
               ptr(f32(f.dye)))
        e.call("fl_step_auto", steps, None)
        u = np.empty(e.ufaces, np.float32)
        v = np.empty(e.vfaces, np.float32)
        e.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        return u, v, e.stats()
    finally:
        e.close()


def test_rb_tile_depth_does_not_change_results():
    scene = configs.karman(96, 64)
    base = configs.karman_params()
    ref = run(scene, base, 6)
    for q in (1, 2, 3):
        got = run(scene, autotune.with_params(base, rb_pairs=q), 6)
        assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])


def test_tuned_multigrid_reaches_tolerance(tmp_path):
    scene = configs.plume(64)
    base = configs.plume_params(tol=1e-6, max_cycles=30)
    space = {"mg_coarsest": (4, 8), "mg_coarse_sweeps": (8, 32)}
    best, table = autotune.tune_multigrid(scene, base, steps=3, warmup=2, space=space)
    assert best is not None and len(table) == 4
    _, _, st = run(scene, autotune.with_params(base, **best), 4)
    assert 0 <= st["rel_residual"] <= 1e-6


def test_omega_tuning_picks_the_smallest_residual():
    scene = configs.karman(64, 64)
    best, table = autotune.tune_red_black(scene, configs.karman_params(), omegas=(1.0, 1.5, 1.9), pairs=(4,),
                                          steps=2, warmup=1)
    res = dict(table["omega"])
    assert all(np.isfinite(r) and r >= 0 for r in res.values())
    assert best["omega"] == min(res, key=lambda w: (res[w], w))

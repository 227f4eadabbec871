"""The turbulence-grid configuration: a 16 x 16 lattice of solid squares
behind a u = 1 inflow, pressure solved to a relative residual of 1e-8 by the
float64 defect-correction loop around the float32 multigrid V(3,3). Checked
against the float32 oracle (identical), the float64 oracle on a subwindow
(stated tolerance) and for the residual target itself."""
import numpy as np
import pytest

from flowlab_gb300 import configs, native
from flowlab_gb300.native import f32, ptr
from tests.scene_setups import oracle_params

pytestmark = pytest.mark.gpu


def engine_for(g, f, prm):
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
             ptr(f32(f.dye)))
    return eng


def read(eng, p_dtype=native.FL_F32):
    u = np.empty(eng.ufaces, np.float32)
    v = np.empty(eng.vfaces, np.float32)
    p = np.empty(eng.cells, np.float64 if p_dtype == native.FL_F64 else np.float32)
    d = np.empty(eng.dye_len, np.float32)
    eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
    eng.call("fl_read_pressure", p_dtype, ptr(p))
    eng.call("fl_read_dye", native.FL_F32, ptr(d))
    return u, v, p, d


def test_every_step_reaches_1e_8():
    g, f, _ = configs.turbulence(256)
    eng = engine_for(g, f, configs.turbulence_params())
    try:
        for _ in range(5):
            eng.call("fl_step_auto", 1, None)
            st = eng.stats()
            assert 0 <= st["rel_residual"] <= 1e-8, st
            assert 0 < st["cycles"] < 40
    finally:
        eng.close()


def test_matches_float32_oracle(o32):
    g, f, _ = configs.turbulence(128)
    prm = configs.turbulence_params()
    eng = engine_for(g, f, prm)
    try:
        eng.call("fl_step_auto", 4, None)
        u, v, p, d = read(eng)
        st = eng.stats()
    finally:
        eng.close()
    sim = o32.simulation(g.nx, g.ny, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    for _ in range(4):
        sim.step()
    eu, ev, ep, ed = sim.get_fields()
    for name, a, b in (("u", eu, u), ("v", ev, v), ("dye", ed, d)):
        assert int((np.asarray(a, np.float32) != b).sum()) == 0, name
    assert abs(st["rel_residual"] - sim.info()["rel_res"]) <= 1e-6 * sim.info()["rel_res"]


def test_error_against_float64_oracle_on_subwindow(o64):
    """Per-field error against the float64 oracle on the central subwindow
    of 1/8 of the side (256^2 at 2048^2), after 3 steps at 512^2.
    Tolerance: 1e-4 of the field's peak for u, v and p (float32 advection
    against float64 advection, the solve itself converged to 1e-8)."""
    n = 512
    g, f, _ = configs.turbulence(n)
    prm = configs.turbulence_params()
    eng = engine_for(g, f, prm)
    try:
        eng.call("fl_step_auto", 3, None)
        u, v, p, _ = read(eng, native.FL_F64)
    finally:
        eng.close()
    sim = o64.simulation(g.nx, g.ny, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    for _ in range(3):
        sim.step()
    eu, ev, _, _ = sim.get_fields()
    ep = sim.get_p64()
    w = n // 8
    j0 = i0 = n // 2 - w // 2
    win = lambda a, nx: a.reshape(-1, nx)[j0:j0 + w, i0:i0 + w]
    for name, a, b, nx in (("u", eu, u, n + 1), ("v", ev, v, n), ("p", ep, p, n)):
        wa, wb = win(np.asarray(a, np.float64), nx), win(np.asarray(b, np.float64), nx)
        err = np.abs(wa - wb).max() / max(1e-30, np.abs(a).max())
        assert err < 1e-4, "%s: subwindow error %.3g of peak" % (name, err)

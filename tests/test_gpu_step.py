"""The fused step (GpuStep seam, C ABI fl_upload_fields / fl_step /
fl_step_auto) against the oracle's Simulation (simulation.ts:467-587) on the
benchmark configurations at test sizes, plus the reference's whole-step
invariants (src/core/simulation.test.ts, src/scenes/emitters.test.ts)."""
import ctypes

import numpy as np
import pytest

from flowlab_gb300 import configs, native, scenes as sc
from flowlab_gb300.native import f32, ptr
from tests.scene_setups import oracle_params

pytestmark = pytest.mark.gpu


def run_engine(g, f, patch, prm, steps, auto=True):
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        if patch is not None:
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        iters = ctypes.c_int()
        eng.call("fl_step_auto", steps, ctypes.byref(iters))
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        p = np.empty(eng.cells, np.float32)
        d = np.empty(eng.dye_len, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        eng.call("fl_read_pressure", native.FL_F32, ptr(p))
        eng.call("fl_read_dye", native.FL_F32, ptr(d))
        st = eng.stats()
    finally:
        eng.close()
    return u, v, p, d, st


def run_oracle(o, g, f, patch, prm, steps):
    sim = o.simulation(g.nx, g.ny, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    if patch is not None:
        sim.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
    for _ in range(steps):
        sim.step()
    u, v, p, d = sim.get_fields()
    return u, v, p, d, sim.info()


def mismatch(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return int((a != b).sum())


def test_plume_steps_match_float32_oracle(o32, o64):
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-4, max_cycles=12, mixed=0)
    steps = 12
    u, v, p, d, st = run_engine(g, f, patch, prm, steps)
    eu, ev, ep, ed, info = run_oracle(o32, g, f, patch, prm, steps)
    assert abs(st["time"] - info["time"]) <= 1e-12 * max(1.0, info["time"])
    for name, a, b in (("u", eu, u), ("v", ev, v), ("p", ep, p), ("dye", ed, d)):
        assert mismatch(a, b) == 0, "%s: %d values differ from the float32 oracle" % (name, mismatch(a, b))
    # float64 trajectory drift: reported, loosely bounded
    fu, fv, fp, fd, _ = run_oracle(o64, g, f, patch, prm, steps)
    for name, a, b in (("u", fu, u), ("v", fv, v), ("dye", fd, d)):
        diff = np.abs(a - b).max()
        assert diff < 1e-3 * max(1.0, np.abs(a).max()), "%s drift %.3g" % (name, diff)


def test_karman_steps_match_float32_oracle(o32):
    g, f, patch = configs.karman(64, 48)
    prm = configs.karman_params()
    steps = 10
    u, v, p, d, st = run_engine(g, f, patch, prm, steps)
    eu, ev, ep, ed, info = run_oracle(o32, g, f, patch, prm, steps)
    for name, a, b in (("u", eu, u), ("v", ev, v), ("p", ep, p), ("dye", ed, d)):
        assert mismatch(a, b) == 0, "%s: %d values differ from the float32 oracle" % (name, mismatch(a, b))
    # simulation.test.ts:22-39 — the outlet never takes inflow
    U = u.reshape(g.ny, g.nx + 1)
    assert (U[:, g.nx - 1] >= 0).all() and (U[:, g.nx] >= 0).all()


def test_host_dt_step_matches_device_dt_step():
    """fl_step with the caller's dt equals fl_step_auto when the caller passes
    the dt the device would compute."""
    g, f, patch = configs.plume(48)
    prm = configs.plume_params(tol=1e-4, max_cycles=8)
    ua, va, pa, da, st = run_engine(g, f, patch, prm, 1)
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        s0 = eng.stats()
        keep = (ctypes.c_double * 3)(*[np.exp(-d * np.float64(np.float32(s0["dt"]))) if d > 0 else 1.0
                                       for d in prm.dye_decay])
        eng.call("fl_step", prm.scheme, s0["dt"], s0["scale"], s0["grad_scale"], keep, None)
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
    finally:
        eng.close()
    assert mismatch(ua, u) == 0 and mismatch(va, v) == 0


def test_uniform_through_flow_is_steady():
    # emitters.test.ts:160-183 — u.fill(1) with an Air outlet is an exact
    # steady solution; 20 steps leave it bit-for-bit unchanged.
    g = sc.Grid(48, 32, 1 / 32)
    spec = sc.SceneSpec(labels=sc.open_right(), seed=sc.uniform_flow(1.0))
    f, _ = sc.reset_fields(g, g, spec)
    prm = native.default_params(scheme=native.FL_MACCORMACK, solver=native.FL_SOLVER_MG, tol=1e-6, mg_max_cycles=5)
    u, v, p, d, _ = run_engine(g, f, None, prm, 20)
    assert np.array_equal(u, f32(f.u)) and np.array_equal(v, f32(f.v))


def test_dye_decay_exponential_in_time():
    # simulation.test.ts:69-82 — zero velocity, dye 1 decays as exp(-2 t)
    g = sc.Grid(16, 16, 1 / 16)
    f = sc.create_fields(g)
    f.dye[:256] = 1.0
    prm = native.default_params(dye_decay=(2.0, 0.0, 0.0), solver=native.FL_SOLVER_MG)
    u, v, p, d, st = run_engine(g, f, None, prm, 30)
    assert abs(d[0] - np.exp(-2 * st["time"])) < 1e-5
    assert d[300] == 0


@pytest.mark.parametrize("mixed", [1, 2])
def test_plume_mixed_steps_match_float32_oracle(o32, mixed):
    """The plume with the defect-correction solve to 1e-6 (float64 or
    double-float pressure), identical to the oracle's float32-fields step with
    the same refined pressure."""
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-6, max_cycles=30, mixed=mixed)
    steps = 8
    u, v, p, d, st = run_engine(g, f, patch, prm, steps)
    eu, ev, ep, ed, info = run_oracle(o32, g, f, patch, prm, steps)
    for name, a, b in (("u", eu, u), ("v", ev, v), ("p", ep, p), ("dye", ed, d)):
        assert mismatch(a, b) == 0, "%s: %d values differ from the float32 oracle" % (name, mismatch(a, b))
    assert 0 <= st["rel_residual"] <= 1e-6 and abs(st["rel_residual"] - info["rel_res"]) <= 1e-9 * info["rel_res"] + 1e-15


def test_plume_reaches_relative_residual_target():
    g, f, patch = configs.plume(256)
    prm = configs.plume_params(tol=1e-6, max_cycles=40, mixed=1)
    u, v, p, d, st = run_engine(g, f, patch, prm, 5)
    assert 0 <= st["rel_residual"] <= 1e-6, st
    assert np.isfinite(u).all() and np.isfinite(d).all()


def run_steps(g, f, patch, prm, steps, eager):
    """fl_step_auto one step at a time; with `eager` the phases are profiled,
    which keeps the step off the CUDA-graph path."""
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        if patch is not None:
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        if eager:
            eng.profile(True)
        cyc = []
        for _ in range(steps):
            eng.call("fl_step_auto", 1, None)
            st = eng.stats()
            cyc.append((st["cycles"], st["rel_residual"], st["div_rms"]))
        prof = eng.profile() if eager else None
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        p = np.empty(eng.cells, np.float32)
        d = np.empty(eng.dye_len, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        eng.call("fl_read_pressure", native.FL_F32, ptr(p))
        eng.call("fl_read_dye", native.FL_F32, ptr(d))
    finally:
        eng.close()
    return (u, v, p, d), cyc, prof


@pytest.mark.parametrize("case", ["plume_mixed", "plume_float32", "karman_rb"])
def test_graph_steps_equal_eager_steps(case):
    """The whole-step CUDA graph (device-side V-cycle loop) performs exactly
    the eager path's kernels: identical fields and identical cycle counts and
    residuals, step by step."""
    if case == "karman_rb":
        g, f, patch = configs.karman(96, 64)
        prm = configs.karman_params()
    else:
        g, f, patch = configs.plume(96)
        prm = configs.plume_params(tol=1e-6 if case == "plume_mixed" else 1e-4, max_cycles=20,
                                   mixed=int(case == "plume_mixed"))
    a, ca, _ = run_steps(g, f, patch, prm, 6, eager=False)
    b, cb, prof = run_steps(g, f, patch, prm, 6, eager=True)
    for name, x, y in zip(("u", "v", "p", "dye"), a, b):
        assert mismatch(x, y) == 0, "%s: %d values differ between graph and eager steps" % (name, mismatch(x, y))
    # cycle counts identical; the residual norms are sums accumulated with
    # atomics in block order, so they agree to rounding, not bit for bit
    assert [c[0] for c in ca] == [c[0] for c in cb]
    for x, y in zip(ca, cb):
        assert np.allclose(x[1:], y[1:], rtol=1e-12, atol=0)
    assert sum(prof[n][1] for n in prof) > 0


def test_graph_rebuilt_after_parameter_change(o32):
    """Buoyancy, confinement and dye-patch changes rebuild the step graph: a
    run that changes them mid-way equals the oracle doing the same."""
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-4, max_cycles=12, mixed=0)
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    sim = o32.simulation(g.nx, g.ny, 1, **oracle_params(prm))
    try:
        eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
        sim.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
        eng.call("fl_step_auto", 3, None)
        for _ in range(3):
            sim.step()
        eng.call("fl_set_buoyancy", 2.0, 0.0)
        eng.call("fl_set_confinement", 0.0)
        prm2 = configs.plume_params(tol=1e-4, max_cycles=12, mixed=0)
        prm2.beta, prm2.alpha, prm2.confinement = 2.0, 0.0, 0.0
        sim2_params = oracle_params(prm2)
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        p = np.empty(eng.cells, np.float32)
        d = np.empty(eng.dye_len, np.float32)
        eng.call("fl_step_auto", 3, None)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        eng.call("fl_read_pressure", native.FL_F32, ptr(p))
        eng.call("fl_read_dye", native.FL_F32, ptr(d))
    finally:
        eng.close()
    su, sv, sp, sd = sim.get_fields()
    sim2 = o32.simulation(g.nx, g.ny, 1, **sim2_params)
    sim2.set_fields(su, sv, sp, f.label, sd)
    sim2.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
    for _ in range(3):
        sim2.step()
    eu, ev, ep, ed = sim2.get_fields()
    for name, x, y in (("u", eu, u), ("v", ev, v), ("p", ep, p), ("dye", ed, d)):
        assert mismatch(x, y) == 0, "%s: %d values differ from the float32 oracle" % (name, mismatch(x, y))


def test_engines_with_different_coarse_tails_coexist():
    """The coarse tail's shared-memory limit is per device and function:
    creating an engine with a smaller tail must not break a larger one."""
    g, f, patch = configs.plume(64)
    big = native.Engine(g.nx, g.ny, g.h, params=configs.plume_params(tol=1e-4, max_cycles=8, mixed=0))
    small = native.Engine(24, 16, 1 / 16, params=native.default_params(solver=native.FL_SOLVER_MG, mg_coarsest=2))
    try:
        big.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        big.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        big.call("fl_step_auto", 2, None)
        assert big.stats()["cycles"] > 0
    finally:
        small.close()
        big.close()


def refined_plume(n=64, dye_scale=2):
    g = sc.Grid(n, n, 1.0 / n)
    dg = sc.dye_grid(g, dye_scale)
    w = n * g.h
    spec = sc.SceneSpec(seed=sc.draught(), dye_source=sc.gaussian_sources([(0.35 * w, 0.1), (0.65 * w, 0.1)]))
    f, patch = sc.reset_fields(g, dg, spec)
    return g, dg, f, patch


def test_refined_dye_grid_steps_match_float32_oracle(o32):
    """dyeScale 2 (simulation.ts:262-277): dye on a grid twice as fine,
    buoyancy sampling it, decay and the inlet on it."""
    g, dg, f, patch = refined_plume()
    prm = configs.plume_params(tol=1e-4, max_cycles=12, mixed=0)
    eng = native.Engine(g.nx, g.ny, g.h, dye_scale=2, params=prm)
    try:
        eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        eng.call("fl_step_auto", 6, None)
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        d = np.empty(eng.dye_len, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        eng.call("fl_read_dye", native.FL_F32, ptr(d))
    finally:
        eng.close()
    sim = o32.simulation(g.nx, g.ny, 2, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    sim.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
    for _ in range(6):
        sim.step()
    eu, ev, _, ed = sim.get_fields()
    assert d.size == 3 * dg.nx * dg.ny
    for name, a, b in (("u", eu, u), ("v", ev, v), ("dye", ed, d)):
        assert mismatch(a, b) == 0, "%s: %d values differ from the float32 oracle" % (name, mismatch(a, b))


def test_label_edit_mid_run_matches_float32_oracle(o32):
    """setLabels + commitLabels between steps (stepGpu.ts:323-330,
    boundaries.ts:45-64): a disc turns solid after 3 steps."""
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-4, max_cycles=12, mixed=0)
    new_label = f.label.copy()
    sc.solid_disk(0.5, 0.5, 0.12)(g, new_label)
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        eng.call("fl_step_auto", 3, None)
        eng.call("fl_set_labels", ptr(new_label))
        eng.call("fl_step_auto", 3, None)
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        p = np.empty(eng.cells, np.float32)
        d = np.empty(eng.dye_len, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        eng.call("fl_read_pressure", native.FL_F32, ptr(p))
        eng.call("fl_read_dye", native.FL_F32, ptr(d))
    finally:
        eng.close()
    sim = o32.simulation(g.nx, g.ny, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    sim.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
    for _ in range(3):
        sim.step()
    su, sv, sp, sd = sim.get_fields()
    cp, cu, cv, cd = o32.commit_labels(g.nx, g.ny, sp, su, sv, new_label, sd, g.nx * g.ny)
    sim.set_fields(cu, cv, cp, new_label, cd)
    for _ in range(3):
        sim.step()
    eu, ev, ep, ed = sim.get_fields()
    for name, a, b in (("u", eu, u), ("v", ev, v), ("p", ep, p), ("dye", ed, d)):
        assert mismatch(a, b) == 0, "%s: %d values differ from the float32 oracle" % (name, mismatch(a, b))
    lab = new_label.reshape(g.ny, g.nx)
    assert (p.reshape(g.ny, g.nx)[lab == 2] == 0).all()


def test_stir_step_matches_oracle(o32):
    """A one-shot stir taken by the next step (simulation.ts:468-472, 504):
    exp() differs in the last bits between libraries, so the bar is 1e-5 of
    the peak after two steps (the second without the stir)."""
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-4, max_cycles=12, mixed=0)
    st = (0.4, 0.3, 0.08, 0.6, -0.2)
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        eng.call("fl_set_stir", ptr(np.asarray(st, np.float64)))
        eng.call("fl_step_auto", 2, None)
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
    finally:
        eng.close()
    sim = o32.simulation(g.nx, g.ny, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    sim.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
    sim.set_stir(st)
    for _ in range(2):
        sim.step()
    eu, ev, _, _ = sim.get_fields()
    base = run_oracle(o32, g, f, patch, prm, 2)
    assert np.abs(np.asarray(base[0]) - eu).max() > 1e-3  # the stir mattered
    for a, b in ((eu, u), (ev, v)):
        assert np.abs(np.asarray(a, np.float64) - b).max() <= 1e-5 * np.abs(a).max()


def test_step_host_follows_label_and_parameter_changes():
    """fl_step_host when the obstacles move between calls (a changed label
    upload: the compare on the third stream raises the flag and the gated
    multigrid rebuild runs before the solve reads the codes) and after
    fl_set_params changes the V-cycle depth (every graph, the host step's
    own included, rebuilt) gives the same fields and cycle counts as
    fl_upload_fields + fl_step_auto + fl_read_* on a second engine."""
    g, f, patch = configs.plume(96)
    prm = configs.plume_params(tol=1e-6, max_cycles=20, mixed=1)
    prm2 = configs.plume_params(tol=1e-6, max_cycles=20, mixed=1)
    prm2.mg_coarsest = 4
    labels = [np.ascontiguousarray(f.label)]
    moved = labels[0].copy().reshape(g.ny, g.nx)
    moved[40:52, 30:44] = 2  # a solid block appears
    labels.append(np.ascontiguousarray(moved.ravel()))
    moved2 = labels[0].copy().reshape(g.ny, g.nx)
    moved2[44:56, 50:62] = 2  # and moves
    labels.append(np.ascontiguousarray(moved2.ravel()))
    engs = [native.Engine(g.nx, g.ny, g.h, params=prm) for _ in range(2)]
    try:
        for eng in engs:
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        a, b = engs
        state = [f32(f.u).copy(), f32(f.v).copy(), f32(f.p).copy(), f32(f.dye).copy()]
        out_b = [np.empty_like(x) for x in state]
        schedule = [0, 0, 1, 1, 2, 2, 2, 0]
        for step, which in enumerate(schedule):
            if step == 5:
                for eng in engs:
                    eng.set_params(prm2)
            label = labels[which]
            a.call("fl_upload_fields", native.FL_F32, ptr(state[0]), ptr(state[1]), ptr(state[2]), ptr(label),
                   ptr(state[3]))
            ia = ctypes.c_int()
            a.call("fl_step_auto", 1, ctypes.byref(ia))
            out_a = [np.empty_like(x) for x in state]
            a.call("fl_read_velocity", native.FL_F32, ptr(out_a[0]), ptr(out_a[1]))
            a.call("fl_read_pressure", native.FL_F32, ptr(out_a[2]))
            a.call("fl_read_dye", native.FL_F32, ptr(out_a[3]))
            ib = ctypes.c_int()
            b.call("fl_step_host", native.FL_F32, ptr(state[0]), ptr(state[1]), ptr(state[2]), ptr(label),
                   ptr(state[3]), ptr(out_b[0]), ptr(out_b[1]), ptr(out_b[2]), ptr(out_b[3]), ctypes.byref(ib))
            for name, x, y in zip(("u", "v", "p", "dye"), out_a, out_b):
                assert mismatch(x, y) == 0, "step %d %s: %d values differ" % (step, name, mismatch(x, y))
            assert ia.value == ib.value
            state = [x.copy() for x in out_a]
    finally:
        for eng in engs:
            eng.close()


@pytest.mark.parametrize("mixed", [0, 1])
def test_extrapolated_warm_start_matches_float32_oracle(o32, mixed):
    """The second-order warm start 2 p(n) - p(n-1) (no reference
    counterpart) on the float32 and the float64 pressure."""
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-6 if mixed else 1e-4, max_cycles=20, mixed=mixed)
    prm.warm_extrapolate = 1
    u, v, p, d, st = run_engine(g, f, patch, prm, 8)
    eu, ev, ep, ed, info = run_oracle(o32, g, f, patch, prm, 8)
    for name, a, b in (("u", eu, u), ("v", ev, v), ("dye", ed, d)):
        assert mismatch(a, b) == 0, "%s: %d values differ from the float32 oracle" % (name, mismatch(a, b))
    if not mixed:
        assert mismatch(ep, p) == 0


@pytest.mark.parametrize("case", ["plume_mixed", "plume_float32", "karman_rb"])
def test_step_host_equals_upload_step_and_reads(case):
    """fl_step_host (the GpuStep.step seam with host buffers: upload, step,
    readback, copies overlapped with the step on a second stream) gives the
    same fields and cycle counts as fl_upload_fields + fl_step_auto +
    fl_read_*, step after step, with and without the upload."""
    if case == "karman_rb":
        g, f, patch = configs.karman(96, 64)
        prm = configs.karman_params()
    else:
        g, f, patch = configs.plume(96)
        prm = configs.plume_params(tol=1e-6 if case == "plume_mixed" else 1e-4, max_cycles=20,
                                   mixed=int(case == "plume_mixed"))
    engs = [native.Engine(g.nx, g.ny, g.h, params=prm) for _ in range(2)]
    try:
        for eng in engs:
            if patch is not None:
                eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        a, b = engs
        state = [f32(f.u).copy(), f32(f.v).copy(), f32(f.p).copy(), f32(f.dye).copy()]
        label = np.ascontiguousarray(f.label)
        out_b = [np.empty_like(x) for x in state]
        for step in range(6):
            upload = step % 3 != 2  # every third step continues on the device
            if upload:
                a.call("fl_upload_fields", native.FL_F32, ptr(state[0]), ptr(state[1]), ptr(state[2]), ptr(label),
                       ptr(state[3]))
            ia = ctypes.c_int()
            a.call("fl_step_auto", 1, ctypes.byref(ia))
            out_a = [np.empty_like(x) for x in state]
            a.call("fl_read_velocity", native.FL_F32, ptr(out_a[0]), ptr(out_a[1]))
            a.call("fl_read_pressure", native.FL_F32, ptr(out_a[2]))
            a.call("fl_read_dye", native.FL_F32, ptr(out_a[3]))
            ib = ctypes.c_int()
            if upload:
                b.call("fl_step_host", native.FL_F32, ptr(state[0]), ptr(state[1]), ptr(state[2]), ptr(label),
                       ptr(state[3]), ptr(out_b[0]), ptr(out_b[1]), ptr(out_b[2]), ptr(out_b[3]), ctypes.byref(ib))
            else:
                b.call("fl_step_host", native.FL_F32, None, None, None, None, None, ptr(out_b[0]), ptr(out_b[1]),
                       ptr(out_b[2]), ptr(out_b[3]), ctypes.byref(ib))
            for name, x, y in zip(("u", "v", "p", "dye"), out_a, out_b):
                assert mismatch(x, y) == 0, "step %d %s: %d values differ" % (step, name, mismatch(x, y))
            assert ia.value == ib.value
            state = [x.copy() for x in out_a]
    finally:
        for eng in engs:
            eng.close()


@pytest.mark.parametrize("mixed", [0, 1])
def test_tail_side_does_not_change_results(mixed):
    """The levels inside the single-CTA tail (mg_tail_side) against their own
    launches: identical fields and cycle counts for every split, on the
    256^2 plume (levels 256..8) and on a 64^2 scene the tail solves whole."""
    for n in (256, 64):
        g, f, patch = configs.plume(n)
        outs = []
        for side in (8, 16, 32, 64):
            prm = configs.plume_params(tol=1e-6 if mixed else 1e-4, max_cycles=20, mixed=mixed)
            prm.mg_tail_side = side
            outs.append(run_engine(g, f, patch, prm, 3))
        for side, o in zip((16, 32, 64), outs[1:]):
            for a, b, name in zip(outs[0][:4], o[:4], ("u", "v", "p", "dye")):
                assert np.array_equal(a, b), (n, side, name, mismatch(a, b))
            assert o[4]["cycles"] == outs[0][4]["cycles"]


def test_upload_rebuilds_the_multigrid_only_for_changed_labels():
    """fl_upload_fields rebuilds the multigrid labels and stencil codes (an IF
    node of the upload graph) only when the uploaded labels differ from the
    current ones: an engine re-uploaded with new labels (a solid block added)
    steps exactly like a fresh engine given them, and re-uploading the same
    labels again changes nothing."""
    g, f, patch = configs.plume(128)
    prm = configs.plume_params(tol=1e-6, max_cycles=30, mixed=1)
    label2 = f.label.copy().reshape(g.ny, g.nx)
    label2[60:70, 40:56] = 2
    label2 = np.ascontiguousarray(label2.reshape(-1))

    def upload(eng, label):
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(label),
                 ptr(f32(f.dye)))

    def read(eng):
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        return u, v, eng.stats()["cycles"]

    outs = []
    for first in (None, f.label, label2):
        eng = native.Engine(g.nx, g.ny, g.h, params=prm)
        try:
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
            if first is not None:
                upload(eng, first)
                eng.call("fl_step_auto", 2, None)
            upload(eng, label2)
            eng.call("fl_step_auto", 3, None)
            outs.append(read(eng))
        finally:
            eng.close()
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0]) and np.array_equal(o[1], outs[0][1]) and o[2] == outs[0][2]

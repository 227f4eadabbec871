"""The seam-level surface of the C ABI and its Python mirror, on the GPU:

  * the residual diagnostic (fl_params.residual_every, simulation.ts:193-206,
    539-540): the post-step divergence of the projected velocity, on the
    graph path and the eager path, every step and every third step, is
    identical to the float32 oracle's, with its FLUID-cell RMS and max;
  * fl_step's per-call advection scheme (simulation.ts:36-38) and
    fl_step_host with float64 host buffers (grid.ts:53-54);
  * flowlab_gb300/engine.py (GpuAdvector, GpuPressureSolver,
    GpuMultigridSolver, GpuStepper under Simulation) against the oracle;
  * the solver ladder of the reference's ARCHITECTURE.md:98-134 on one
    shared pressure problem (the vortex street's first solve at 128^2):
    cpu-sor -> cpu-rbsor (ordering), cpu-rbsor float64 -> float32
    (precision), cpu-rbsor float32 -> gpu-rbsor (plumbing), cpu-mg ->
    cpu-rbsor converged (algorithm), cpu-mg float32 -> gpu-mg (plumbing),
    gpu-mg -> cpu-mg float64 (precision), each with its own bar.
"""
import ctypes

import numpy as np
import pytest

from flowlab_gb300 import configs, engine, native
from flowlab_gb300 import scenes as sc
from flowlab_gb300.native import f32, ptr
from tests.scene_setups import oracle_params

pytestmark = pytest.mark.gpu


def upload(eng, f, patch=None):
    if patch is not None:
        eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
    eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
             ptr(f32(f.dye)))


def read_all(eng):
    u = np.empty(eng.ufaces, np.float32)
    v = np.empty(eng.vfaces, np.float32)
    p = np.empty(eng.cells, np.float32)
    d = np.empty(eng.dye_len, np.float32)
    eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
    eng.call("fl_read_pressure", native.FL_F32, ptr(p))
    eng.call("fl_read_dye", native.FL_F32, ptr(d))
    return u, v, p, d


def fluid_stats(div, label):
    d = np.asarray(div, np.float64)[label == sc.FLUID]
    return float(np.sqrt(np.mean(d * d))), float(np.abs(d).max())


# ----------------------------------------------------- residual diagnostic

@pytest.mark.parametrize("every", [1, 3])
@pytest.mark.parametrize("graph", [True, False])
def test_post_step_divergence_matches_the_oracle(o32, every, graph):
    g, f, patch = configs.karman(96, 64)
    prm = configs.karman_params()
    prm.residual_every = every
    steps = 5
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        upload(eng, f, patch)
        if not graph:
            eng.profile(True)  # profiled steps run eagerly
        eng.call("fl_step_auto", steps, None)
        st = eng.stats()
        div = np.empty(eng.cells, np.float32)
        eng.call("fl_read_divergence", native.FL_F32, ptr(div))
        u, v, _, _ = read_all(eng)
    finally:
        eng.close()
    sim = o32.simulation(g.nx, g.ny, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    for _ in range(steps):
        sim.step()
    ref, ref_step = sim.get_div_post()
    ou, ov, _, _ = sim.get_fields()
    assert np.array_equal(ou, u) and np.array_equal(ov, v)
    # steps 0..4: computed on 0..4 (every 1) or on 0 and 3 (every 3)
    assert ref_step == (steps - 1 if every == 1 else 3) == st["post_div_step"]
    assert np.array_equal(ref, div), "%d cells differ" % int((ref != div).sum())
    rms, mx = fluid_stats(ref, f.label)
    assert st["post_div_max"] == np.float32(mx)
    assert abs(st["post_div_rms"] - rms) <= 1e-9 * rms


def test_residual_diagnostic_off_leaves_nothing():
    g, f, patch = configs.karman(64, 64)
    prm = configs.karman_params()
    prm.residual_every = 0
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        upload(eng, f, patch)
        eng.call("fl_step_auto", 2, None)
        st = eng.stats()
        div = np.ones(eng.cells, np.float32)
        eng.call("fl_read_divergence", native.FL_F32, ptr(div))
    finally:
        eng.close()
    assert st["post_div_step"] == -1 and st["post_div_rms"] == 0.0
    assert not div.any()


# ------------------------------------------------------ per-call scheme

def test_step_scheme_is_per_call():
    """fl_step(scheme) on an engine configured for MacCormack equals the same
    call on an engine configured for semi-Lagrangian; later fl_step_auto
    calls keep the scheme the seam passed last."""
    g, f, patch = configs.plume(48)
    mac = configs.plume_params(tol=1e-5, max_cycles=8)
    sl = configs.plume_params(tol=1e-5, max_cycles=8)
    sl.scheme = native.FL_SEMI_LAGRANGIAN
    engs = [native.Engine(g.nx, g.ny, g.h, params=p) for p in (mac, sl)]
    try:
        outs = []
        for eng in engs:
            upload(eng, f, patch)
            s0 = eng.stats()
            keep = (ctypes.c_double * 3)(*[np.exp(-d * np.float64(np.float32(s0["dt"]))) if d > 0 else 1.0
                                           for d in mac.dye_decay])
            eng.call("fl_step", native.FL_SEMI_LAGRANGIAN, s0["dt"], s0["scale"], s0["grad_scale"], keep, None)
            eng.call("fl_step_auto", 2, None)
            outs.append(read_all(eng))
        with pytest.raises(native.FlowlabError) as ei:
            engs[0].call("fl_step", 7, 0.01, 1.0, 1.0, None, None)
        assert ei.value.status == native.FL_EINVAL
    finally:
        for eng in engs:
            eng.close()
    for name, a, b in zip(("u", "v", "p", "dye"), *outs):
        assert np.array_equal(a, b), name


# ------------------------------------------------ float64 host buffers

def test_step_host_float64_equals_upload_step_read():
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-6, max_cycles=10)
    a = native.Engine(g.nx, g.ny, g.h, params=prm)
    b = native.Engine(g.nx, g.ny, g.h, params=prm)
    f64 = lambda x: np.ascontiguousarray(x, np.float64)
    try:
        for eng in (a, b):
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        state = [f64(f.u), f64(f.v), f64(f.p), f64(f.dye)]
        for step in range(3):
            upload_now = step != 1  # the middle step continues from the device state
            if upload_now:
                a.call("fl_upload_fields", native.FL_F64, *[ptr(x) for x in state[:3]], ptr(f.label), ptr(state[3]))
            a.call("fl_step_auto", 1, None)
            out_a = [np.empty_like(x) for x in state]
            a.call("fl_read_velocity", native.FL_F64, ptr(out_a[0]), ptr(out_a[1]))
            a.call("fl_read_pressure", native.FL_F64, ptr(out_a[2]))
            a.call("fl_read_dye", native.FL_F64, ptr(out_a[3]))
            out_b = [np.empty_like(x) for x in state]
            ins = [ptr(x) for x in state[:3]] + [ptr(f.label), ptr(state[3])] if upload_now else [None] * 5
            b.call("fl_step_host", native.FL_F64, *ins, *[ptr(x) for x in out_b], None)
            for name, x, y in zip(("u", "v", "p", "dye"), out_a, out_b):
                assert np.array_equal(x, y), "step %d %s" % (step, name)
            state = out_a
    finally:
        a.close()
        b.close()


# --------------------------------------------------- the Python seam mirror

def karman_spec(nx, ny):
    g = sc.Grid(nx, ny, 1.0 / ny)
    r = 0.1 * ny * g.h
    return g, sc.SceneSpec(
        labels=sc.all_labels(sc.open_right(), sc.solid_disk(0.25 * nx * g.h, 0.5 * ny * g.h, r)),
        seed=sc.chain_seeds(sc.uniform_flow(1.0), sc.lcg_noise(1e-3)),
        dye=lambda dg, dye: sc.add_dye_stripes(dg, dye))


def test_simulation_mirror_against_the_float64_oracle(o64):
    """engine.Simulation (simulation.ts:259-593 with the GpuStepper) on the
    vortex street: host CFL dt, per-call scheme, the residual read back on
    its cadence; 6 steps within 1e-4 of each field's peak of the float64
    oracle (float32 against float64 over a few steps)."""
    nx, ny = 128, 64
    g, spec = karman_spec(nx, ny)
    prm = configs.karman_params()
    sim = engine.Simulation(nx, ny, params=dict(scheme="macCormack", cflTarget=0.5, pressureIters=60, omega=1.9,
                                                tol=0.0, residualEvery=2), engine_params=prm)
    try:
        sim.reset(spec)
        f0 = sc.reset_fields(g, g, spec)[0]
        assert np.array_equal(sim.f.u, f0.u) and np.array_equal(sim.f.label, f0.label)
        ref = o64.simulation(nx, ny, 1, **dict(oracle_params(prm), residualEvery=2))
        ref.set_fields(f0.u, f0.v, f0.p, f0.label, f0.dye)
        for _ in range(6):
            sim.step()
            ref.step()
            assert sim.iters == 60
        u, v, p, dye = ref.get_fields()
        for name, a, b in (("u", u, sim.f.u), ("v", v, sim.f.v)):
            assert np.abs(a - b).max() <= 1e-4 * np.abs(a).max(), name
        dp = np.empty(nx * ny, np.float64)
        sim.stepper.read_pressure(dp)
        assert np.abs(p - dp).max() <= 1e-4 * np.abs(p).max()
        ddye = np.empty(dye.size, np.float64)
        sim.stepper.read_dye(ddye)
        assert np.abs(dye - ddye).max() <= 1e-4 * np.abs(dye).max()
        # the residual of step 4 (every second step), read back into sim.div
        rdiv, rstep = ref.get_div_post()
        assert rstep == 4 and sim.steps == 6
        assert np.abs(rdiv - sim.div).max() <= 1e-3 * np.abs(rdiv).max()
        dmax, drms = sim.divergence_stats(sim.max_face_speed())
        assert dmax > 0 and drms > 0
    finally:
        sim.stepper.destroy()


def test_advector_and_solver_mirrors_against_the_float32_oracle(o32):
    from tests import fixtures as fx

    h, dt, u, v, label, dye, dnx, dny, dh = fx.advect_fixture(1)
    ctx = engine.init_gpu()
    assert ctx is not None
    g = sc.Grid(fx.NX, fx.NY, h)
    adv = engine.GpuAdvector(ctx, g)
    try:
        uo, vo = np.empty_like(f32(u)), np.empty_like(f32(v))
        adv.velocity(g, "macCormack", u, v, uo, vo, label, np.float32(dt))
        nd = dnx * dny
        planes_in = [f32(dye)[c * nd:(c + 1) * nd] for c in range(3)]
        planes_out = [np.empty(nd, np.float32) for _ in range(3)]
        adv.dye(g, "macCormack", u, v, planes_in, planes_out, label, np.float32(dt))
    finally:
        adv.destroy()
    hf, dtf = float(np.float32(h)), float(np.float32(dt))
    eu, ev = o32.advect_velocity(fx.NX, fx.NY, hf, True, f32(u), f32(v), label, dtf)
    assert np.array_equal(eu, uo) and np.array_equal(ev, vo)
    eq = o32.advect_dye(fx.NX, fx.NY, hf, dnx, dny, float(np.float32(dh)), True, f32(u), f32(v), f32(dye), label,
                        dtf)
    assert np.array_equal(eq, np.concatenate(planes_out))


# ------------------------------------------------------- the solver ladder

@pytest.fixture(scope="module")
def karman_problem():
    """The vortex street's first pressure problem at 128^2 (div, label,
    scale), from one float64 oracle step."""
    from oracle import Oracle

    g, f, patch = configs.karman(128, 128)
    prm = configs.karman_params()
    sim = Oracle("f64").simulation(g.nx, g.ny, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    sim.step()
    return g, sim.get_div(), f.label, float(np.float32(sim.scale()))


def test_solver_ladder(o32, o64, karman_problem):
    g, div, label, scale = karman_problem
    n, nx, ny = g.nx * g.ny, g.nx, g.ny
    p0 = np.zeros(n)
    peak = lambda a: float(np.abs(a).max())
    ctx = engine.init_gpu()
    # converged references in float64: red-black (cpu-rbsor) and multigrid
    # (cpu-mg) to 1e-12; lexicographic SOR with its four sweep directions
    # (cpu-sor) converges slowest on this channel (at the optimal omega it
    # stalls near 2e-6; at 1.9 it reaches ~3e-8 in 20000 sweeps)
    rel = lambda p: o64.rms_remaining(nx, ny, p, div, label, scale) / o64.fluid_div_rms(div, label)
    w = engine.optimal_omega(nx, ny)
    p_rb, _ = o64.rb_solve(nx, ny, p0, div, label, scale, 20000, w, 1e-12)
    p_mg, _, rr = o64.mg_solve(nx, ny, p0, div, label, scale, 60, 1e-12)
    p_sor, _ = o64.sor_solve(nx, ny, p0, div, label, scale, 20000, 1.9, 1e-12)
    assert rr <= 1e-12 and rel(p_rb) <= 1e-12 and rel(p_sor) <= 1e-7
    # ordering: lexicographic and red-black converge to the same pressure
    assert np.abs(p_sor - p_rb).max() <= 1e-6 * peak(p_rb)
    # algorithm: multigrid and red-black converge to the same pressure
    assert np.abs(p_mg - p_rb).max() <= 1e-10 * peak(p_rb)

    # red-black on a fixed budget (the reference's GPU use): float64 ->
    # float32 (precision), float32 oracle -> gpu-rbsor (plumbing: identical)
    iters, omega = 60, 1.9
    rb64, _ = o64.rb_solve(nx, ny, p0, div, label, scale, iters, omega, 0.0)
    rb32, _ = o32.rb_solve(nx, ny, p0, f32(div), label, np.float32(scale), iters, omega, 0.0)
    assert np.abs(rb32 - rb64).max() <= 1e-5 * peak(rb64)
    gs = engine.GpuPressureSolver(ctx, g)
    try:
        p_gpu = np.zeros(n, np.float32)
        used = gs.solve(g, p_gpu, f32(div), label, np.float32(scale), iters, omega, 0.0)
    finally:
        gs.destroy()
    assert used == iters
    assert np.array_equal(p_gpu, rb32), "%d cells differ" % int((p_gpu != rb32).sum())

    # multigrid with the reference's V(2,2), 3 cycles: float32 oracle ->
    # gpu-mg (identical), gpu-mg -> float64 (precision)
    mg32, used32, _ = o32.mg_solve(nx, ny, p0, f32(div), label, np.float32(scale), 3, 0.0)
    mg64, _, _ = o64.mg_solve(nx, ny, p0, div, label, scale, 3, 0.0)
    gm = engine.GpuMultigridSolver(ctx, g, cycles=3)
    try:
        p_gmg = np.zeros(n, np.float32)
        used = gm.solve(g, p_gmg, f32(div), label, np.float32(scale), 0, 0.0, 0.0)
    finally:
        gm.destroy()
    assert used == used32 == 3
    assert np.array_equal(p_gmg, mg32), "%d cells differ" % int((p_gmg != mg32).sum())
    assert np.abs(p_gmg - mg64).max() <= 1e-5 * peak(mg64)

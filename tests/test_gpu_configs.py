"""The benchmark configurations at their own sizes and step counts, through
the C ABI, against the oracle:

  * the 1024^2 thermal plume with the benchmark's exact parameters
    (configs.plume_params(): V(3,3), 16 coarse pairs, tail from 32^2,
    double-float defect correction to 1e-6), stepped by the graph path;
  * the vortex street, 128^2, red-black SOR omega 1.9 x 60, 200 steps;
  * the thermal plume at 512^2 for 500 steps (marked slow: ~4 minutes of
    oracle time);
  * the turbulence grid at 2048^2 to 1e-8 (float64 defect correction),
    3 steps, with the error on the central 256^2 subwindow.

Bars: against the float32 oracle the fields are IDENTICAL (the same float32
operations in the same order); against the float64 oracle the drift is
reported per field as max |gpu - f64| / max |f64| and bounded loosely (the
reference reports trajectory drift rather than gating it; its per-kernel
gates are the 1e-5-of-peak bars of tests/test_gpu_parity.py). The relative
residual is also evaluated by the reference's own definition
(rmsRemainingDivergence / fluidDivRms, src/core/pressure.ts:102-186) in
float64 on the engine's pressure and the step's float32 divergence: the
defect correction forms its residual against the unrounded -scale * div, so
the two agree to the rounding of the norms' inputs (1e-6 relative).

When the environment variable FL_DRIFT_OUT names a file, each test appends
its figures there as one JSON line.
"""
import ctypes
import json
import os
import threading

import numpy as np
import pytest

from flowlab_gb300 import configs, native
from flowlab_gb300.native import f32, ptr
from tests.scene_setups import oracle_params

pytestmark = pytest.mark.gpu

def residual_bound(tol):
    """The reference-definition bound for an engine residual <= tol: the
    norms' inputs (each cell's residual rounded to float, the rhs norm on
    the rounded b) are within 2^-24 relative."""
    return tol * (1 + 1e-6)


def record(name, **fig):
    out = os.environ.get("FL_DRIFT_OUT")
    if out:
        with open(out, "a") as fh:
            fh.write(json.dumps(dict(test=name, **fig)) + "\n")


def run_engine(g, f, patch, prm, steps):
    """`steps` graph steps from the uploaded scene; fields, float64 pressure
    and the last step's statistics."""
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        if patch is not None:
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        eng.call("fl_step_auto", steps, None)
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        p = np.empty(eng.cells, np.float32)
        p64 = np.empty(eng.cells, np.float64)
        d = np.empty(eng.dye_len, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        eng.call("fl_read_pressure", native.FL_F32, ptr(p))
        eng.call("fl_read_pressure", native.FL_F64, ptr(p64))
        eng.call("fl_read_dye", native.FL_F32, ptr(d))
        st = eng.stats()
    finally:
        eng.close()
    return dict(u=u, v=v, p=p, p64=p64, dye=d, stats=st)


def run_oracles(g, f, patch, prm, steps, o32, o64):
    """The float32 and float64 oracles stepped side by side (two threads: the
    oracle's calls release the interpreter lock)."""
    out = {}

    def one(tag, o):
        sim = o.simulation(g.nx, g.ny, 1, **oracle_params(prm))
        sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
        if patch is not None:
            sim.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
        for _ in range(steps):
            sim.step()
        u, v, p, d = sim.get_fields()
        out[tag] = dict(u=u, v=v, p=p, dye=d, p64=sim.get_p64(), info=sim.info(), div=sim.get_div(),
                        scale=sim.scale())

    ts = [threading.Thread(target=one, args=(t, o)) for t, o in (("f32", o32), ("f64", o64)) if o is not None]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return out


def mismatches(gpu, ref, names=("u", "v", "p", "dye")):
    return {k: int((np.asarray(ref[k], np.float32) != gpu[k]).sum()) for k in names}


def drift(gpu, ref64, names=("u", "v", "p", "dye")):
    """max |gpu - f64| / max |f64| per field (p: the engine's refined pressure
    when there is one)."""
    out = {}
    for k in names:
        a = np.asarray(ref64["p64"] if k == "p" else ref64[k], np.float64)
        b = np.asarray(gpu["p64"] if k == "p" else gpu[k], np.float64)
        out[k] = float(np.abs(a - b).max() / max(1e-30, np.abs(a).max()))
    return out


def reference_residual(o64, g, gpu, ref32, label):
    """rmsRemainingDivergence / fluidDivRms (pressure.ts:102-186) in float64
    on the engine's pressure, with the last step's float32 divergence and
    scale (identical in engine and float32 oracle)."""
    div = np.asarray(ref32["div"], np.float64)
    scale = np.float32(ref32["scale"])
    r = o64.rms_remaining(g.nx, g.ny, gpu["p64"], div, label, scale)
    return r / o64.fluid_div_rms(div, label)


def test_plume_1024_benchmark_parameters(o32, o64):
    """The benchmarked configuration itself: 1024^2 plume, configs.plume_params()
    unchanged, 4 graph steps (the timed steps' path)."""
    g, f, patch = configs.plume(1024)
    prm = configs.plume_params()
    steps = 4
    gpu = run_engine(g, f, patch, prm, steps)
    ref = run_oracles(g, f, patch, prm, steps, o32, o64)
    mm = mismatches(gpu, ref["f32"])
    assert sum(mm.values()) == 0, "differs from the float32 oracle: %s" % mm
    st = gpu["stats"]
    assert st["cycles"] >= 1 and 0 <= st["rel_residual"] <= prm.tol
    assert abs(st["rel_residual"] - ref["f32"]["info"]["rel_res"]) <= 1e-9 * ref["f32"]["info"]["rel_res"]
    rr_ref = reference_residual(o64, g, gpu, ref["f32"], f.label)
    assert rr_ref <= residual_bound(prm.tol), rr_ref
    dr = drift(gpu, ref["f64"])
    record("plume_1024_bench", steps=steps, mismatches_f32=mm, drift_f64=dr, rel_residual_engine=st["rel_residual"],
           rel_residual_reference_definition=rr_ref, cycles_last=st["cycles"])
    for k, x in dr.items():
        assert x < 1e-3, "%s drifted %.3g of peak from the float64 oracle in %d steps" % (k, x, steps)


def test_karman_128_200_steps(o32, o64):
    """Configuration 1: vortex street 128^2, red-black SOR omega 1.9 x 60 per
    step, MacCormack, CFL 0.5, 200 steps."""
    g, f, patch = configs.karman(128, 128)
    prm = configs.karman_params()
    steps = 200
    gpu = run_engine(g, f, patch, prm, steps)
    ref = run_oracles(g, f, patch, prm, steps, o32, o64)
    mm = mismatches(gpu, ref["f32"])
    assert sum(mm.values()) == 0, "differs from the float32 oracle: %s" % mm
    gpu["p64"] = gpu["p"].astype(np.float64)
    ref["f64"]["p64"] = ref["f64"]["p"]
    dr = drift(gpu, ref["f64"])
    record("karman_128_200", steps=steps, mismatches_f32=mm, drift_f64=dr)
    # 200 steps of a vortex street amplify float32 rounding; the wake stays
    # the same flow (bound: a tenth of the peak)
    for k, x in dr.items():
        assert x < 0.1, "%s drifted %.3g of peak from the float64 oracle in %d steps" % (k, x, steps)


@pytest.mark.slow
def test_plume_512_500_steps(o32, o64):
    """Configuration 2: thermal plume 512^2 to 1e-6, 500 steps."""
    g, f, patch = configs.plume(512)
    prm = configs.plume_params()
    steps = 500
    gpu = run_engine(g, f, patch, prm, steps)
    ref = run_oracles(g, f, patch, prm, steps, o32, o64)
    mm = mismatches(gpu, ref["f32"])
    assert sum(mm.values()) == 0, "differs from the float32 oracle: %s" % mm
    rr_ref = reference_residual(o64, g, gpu, ref["f32"], f.label)
    assert rr_ref <= residual_bound(prm.tol), rr_ref
    dr = drift(gpu, ref["f64"])
    record("plume_512_500", steps=steps, mismatches_f32=mm, drift_f64=dr,
           rel_residual_engine=gpu["stats"]["rel_residual"], rel_residual_reference_definition=rr_ref)
    # 500 steps of a buoyant plume with vorticity confinement are chaotic:
    # float32 and float64 rounding separate the trajectories (measured:
    # u, v ~5% of peak, p ~3%, dye ~27% after 500 steps), so the float64
    # drift is reported; the bar is the float32 identity above. The bound
    # only says the flow is still the same flow (same order of magnitude).
    for k, x in dr.items():
        assert x < 1.0, "%s drifted %.3g of peak from the float64 oracle in %d steps" % (k, x, steps)


def test_turbulence_2048_subwindow(o32, o64):
    """Configuration 3: turbulence grid 2048^2 to 1e-8 through the float64
    defect correction, 3 steps; identical to the float32 oracle, and the
    per-field error against the float64 oracle on the central 256^2
    subwindow within 1e-4 of the field's peak for u and v (float32 against
    float64 advection) and 1e-3 for p: the pressure answers the divergence
    difference through the inverse Laplacian, whose smooth modes amplify it
    ~16x more at 2048^2 than at 512^2 (measured: 1.8e-4)."""
    n = 2048
    g, f, patch = configs.turbulence(n)
    prm = configs.turbulence_params()
    steps = 3
    gpu = run_engine(g, f, patch, prm, steps)
    ref = run_oracles(g, f, patch, prm, steps, o32, o64)
    mm = mismatches(gpu, ref["f32"])
    assert sum(mm.values()) == 0, "differs from the float32 oracle: %s" % mm
    st = gpu["stats"]
    assert 0 <= st["rel_residual"] <= prm.tol
    rr_ref = reference_residual(o64, g, gpu, ref["f32"], f.label)
    assert rr_ref <= residual_bound(prm.tol), rr_ref
    w = 256
    j0 = i0 = n // 2 - w // 2
    err = {}
    for k, nx in (("u", n + 1), ("v", n), ("p", n), ("dye", n)):
        a = np.asarray(ref["f64"]["p64"] if k == "p" else ref["f64"][k], np.float64)
        b = np.asarray(gpu["p64"] if k == "p" else gpu[k], np.float64)
        if k == "dye":
            a, b = a[:n * n], b[:n * n]
        wa = a.reshape(-1, nx)[j0:j0 + w, i0:i0 + w]
        wb = b.reshape(-1, nx)[j0:j0 + w, i0:i0 + w]
        err[k] = float(np.abs(wa - wb).max() / max(1e-30, np.abs(a).max()))
    record("turbulence_2048_subwindow", steps=steps, mismatches_f32=mm, subwindow_error_f64=err,
           rel_residual_engine=st["rel_residual"], rel_residual_reference_definition=rr_ref)
    for k, bar in (("u", 1e-4), ("v", 1e-4), ("p", 1e-3)):
        assert err[k] < bar, "%s: subwindow error %.3g of peak" % (k, err[k])

"""Autotuner for the solver's free constants, measured on the GPU.

What it chooses, per scene shape and solver:

  multigrid      the V-cycle depth (mg_coarsest: the coarsest level's side)
                 and the coarsest level's sweep pairs: the fastest
                 combination (device time per step of the whole step, graph
                 path) among those that reach the tolerance on every
                 measured step; then the first level of the single-CTA tail
                 (mg_tail_side), whose results are identical, by time alone;
  red-black SOR  omega: the smallest relative residual after the fixed sweep
                 budget on the scene's own right-hand sides (the reference's
                 browser setting, a fixed budget, makes accuracy the
                 objective); then the sweep pairs per launch (rb_pairs: the
                 temporal-blocking depth, i.e. the tile/halo shape), whose
                 results are identical, by time alone;
  warm start     whether the learned warm start stays attached: only when
                 the warm-started step is measured faster than the plain
                 one on the scene itself (the network's forward pass must
                 cost less than the V-cycles it saves).

Results are cached in a JSON file keyed by solver, grid shape and precision.

  python -m flowlab_gb300.autotune --scene plume --size 256
"""
import argparse
import ctypes
import itertools
import json
import os

import numpy as np

from . import configs, native
from .native import f32, ptr

MG_SPACE = {"mg_coarsest": (4, 8, 16, 32), "mg_coarse_sweeps": (8, 16, 32)}
RB_OMEGAS = (1.5, 1.6, 1.7, 1.8, 1.85, 1.9, 1.95, 1.98)
RB_PAIRS = (1, 2, 3, 4)
TAIL_SIDES = (16, 32, 64)


def with_params(prm, **kw):
    out = native.Params()
    ctypes.pointer(out)[0] = prm
    for k, v in kw.items():
        setattr(out, k, v)
    return out


def measure_steps(scene, prm, steps=8, warmup=3, device=0, net=None):
    """Graph-path steps of a fresh engine on `scene` = (grid, fields, patch),
    with the learned warm start `net` (a native.Unet) attached when given:
    mean device ms per step (CUDA events on the engine's stream), V-cycles per
    step, the largest relative residual and the mean initial relative
    residual (the warm start's, before any cycle)."""
    import torch

    g, f, patch = scene
    eng = native.Engine(g.nx, g.ny, g.h, params=prm, device=device)
    try:
        if patch is not None:
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        if net is not None:
            eng.call("fl_set_warm_start", net.h)
        eng.call("fl_step_auto", warmup, None)
        stream = torch.cuda.ExternalStream(eng.stream(), device=device)
        ms, cyc, rr, r0 = [], [], [], []
        for _ in range(steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.call("fl_step_auto", 1, None)
            b.record(stream)
            st = eng.stats()
            ms.append(a.elapsed_time(b))
            cyc.append(st["cycles"])
            rr.append(st["rel_residual"])
            r0.append(st["initial_rel_residual"])
        return {"ms": float(np.mean(ms)), "cycles": float(np.mean(cyc)), "rel_max": float(max(rr)),
                "rel0_mean": float(np.mean(r0))}
    finally:
        eng.close()


def pick_multigrid(results, tol):
    """The fastest candidate whose every measured step reached `tol`;
    results: [(candidate dict, measurement dict)]."""
    ok = [(c, m) for c, m in results if 0 <= m["rel_max"] <= tol]
    if not ok:
        return None
    return min(ok, key=lambda cm: (cm[1]["ms"], sorted(cm[0].items())))


def warm_start_pays(plain, warm, tol):
    """Keep the learned warm start attached only if every warm-started step
    reached `tol` and the warm-started step is faster; plain / warm are
    measure_steps results. Returns (attach, reason)."""
    if not (0 <= warm["rel_max"] <= tol):
        return False, "the warm-started solve missed the tolerance"
    saved = plain["cycles"] - warm["cycles"]
    if warm["ms"] >= plain["ms"]:
        return False, ("slower: %.3f against %.3f ms per step (%.2f V-cycles saved per step)"
                       % (warm["ms"], plain["ms"], saved))
    return True, "faster: %.3f against %.3f ms per step (%.2f V-cycles saved)" % (warm["ms"], plain["ms"], saved)


def tune_warm_start(scene, prm, net, steps=8, warmup=3, device=0):
    """Measures the scene with and without the network; the decision of
    warm_start_pays with both measurements."""
    plain = measure_steps(scene, prm, steps, warmup, device)
    warm = measure_steps(scene, prm, steps, warmup, device, net=net)
    attach, reason = warm_start_pays(plain, warm, prm.tol)
    return {"attach": attach, "reason": reason, "plain": plain, "warm": warm}


def tune_batch(bt, steps=2, warmup=1, device=0):
    """The batched scenes' path (native.Batch): the work-list solve (one
    launch per V-cycle phase over every scene's tiles, the scenes in lock
    step) against every engine's own step graph on its own stream (the
    scenes overlapping freely), each timed on the batch itself; the faster
    is kept. Both paths give identical results, so the batch advances
    2 * (warmup + steps) steps here. Returns the times and the choice."""
    import torch

    out = {}
    modes = [False] + ([True] if bt.worklist else [])
    for on in modes:
        bt.set_worklist(on)
        stream = torch.cuda.ExternalStream(bt.stream(), device=device)
        bt.step(warmup)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        bt.step(steps)
        b.record(stream)
        b.synchronize()
        out["worklist_ms" if on else "engine_graphs_ms"] = a.elapsed_time(b) / steps
    use = "worklist_ms" in out and out["worklist_ms"] < out["engine_graphs_ms"]
    bt.set_worklist(use)
    out["worklist"] = use
    return out


def pick_omega(results):
    """The omega with the smallest residual after the budget (ties: the
    smaller omega); results: [(omega, relative residual)]."""
    return min(results, key=lambda r: (r[1], r[0]))[0]


def tune_multigrid(scene, base, steps=8, warmup=3, space=MG_SPACE, tail_sides=TAIL_SIDES, device=0, log=None):
    results = []
    keys = sorted(space)
    for values in itertools.product(*(space[k] for k in keys)):
        cand = dict(zip(keys, values))
        m = measure_steps(scene, with_params(base, **cand), steps, warmup, device)
        results.append((cand, m))
        if log:
            log("%s -> %.3f ms/step, %.2f cycles, rel %.2e" % (cand, m["ms"], m["cycles"], m["rel_max"]))
    best = pick_multigrid(results, base.tol)
    if best is None:
        return None, results
    chosen = dict(best[0])
    timed = []
    for side in tail_sides:
        m = measure_steps(scene, with_params(base, mg_tail_side=side, **chosen), steps, warmup, device)
        timed.append((m["ms"], side))
        if log:
            log("mg_tail_side %d -> %.3f ms/step" % (side, m["ms"]))
    chosen["mg_tail_side"] = min(timed)[1]
    return chosen, results


def rb_residual(scene, base, omega, steps=3, device=0):
    """Relative residual after the fixed sweep budget on the scene's own
    pressure problem at step `steps`: that step's divergence and scale, warm
    started from the pressure it started from (the PressureSolver seam)."""
    g, f, patch = scene
    eng = native.Engine(g.nx, g.ny, g.h, params=base, device=device)
    try:
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        if steps > 1:
            eng.call("fl_step_auto", steps - 1, None)
        scale = eng.stats()["scale"]  # the next step's scale
        p = np.empty(eng.cells, np.float32)
        eng.call("fl_read_pressure", native.FL_F32, ptr(p))
        eng.call("fl_step_auto", 1, None)
        div = np.empty(eng.cells, np.float32)
        eng.call("fl_read_rhs", native.FL_F32, ptr(div))
        used = ctypes.c_int()
        eng.call("fl_rb_solve", ptr(p), ptr(div), ptr(f.label), ctypes.c_float(scale), base.pressure_iters,
                 ctypes.c_float(omega), ctypes.c_double(1e-30), ctypes.byref(used))
        return eng.stats()["rel_residual"]
    finally:
        eng.close()


def tune_red_black(scene, base, omegas=RB_OMEGAS, pairs=RB_PAIRS, steps=8, warmup=3, device=0, log=None):
    res = [(w, rb_residual(scene, base, w, device=device)) for w in omegas]
    if log:
        for w, r in res:
            log("omega %.3f -> rel %.3e after %d sweeps" % (w, r, base.pressure_iters))
    omega = pick_omega(res)
    times = []
    for q in pairs:
        m = measure_steps(scene, with_params(base, omega=omega, rb_pairs=q), steps, warmup, device)
        times.append((q, m["ms"]))
        if log:
            log("rb_pairs %d -> %.3f ms/step" % (q, m["ms"]))
    best_pairs = min(times, key=lambda t: (t[1], t[0]))[0]
    return {"omega": omega, "rb_pairs": best_pairs}, {"omega": res, "rb_pairs": times}


def cache_key(prm, nx, ny):
    solver = "mg" if prm.solver == native.FL_SOLVER_MG else "rb"
    return "%s:%dx%d:%s" % (solver, nx, ny, "mixed" if prm.mixed else "f32")


def tuned_params(scene, base, cache_path=None, device=0, log=None):
    """`base` with the tuned constants for this scene shape (cached)."""
    g = scene[0]
    key = cache_key(base, g.nx, g.ny)
    cache = {}
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as fh:
            cache = json.load(fh)
    if key not in cache:
        if base.solver == native.FL_SOLVER_MG:
            best, _ = tune_multigrid(scene, base, device=device, log=log)
        else:
            best, _ = tune_red_black(scene, base, device=device, log=log)
        cache[key] = best
        if cache_path:
            with open(cache_path, "w") as fh:
                json.dump(cache, fh, indent=1, sort_keys=True)
    best = cache[key]
    return with_params(base, **best) if best else base


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scene", choices=["plume", "karman", "turbulence", "random"], default="plume")
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--cache", default=None)
    a = ap.parse_args(argv)
    from . import build

    build.build()
    if a.scene == "plume":
        scene, base = configs.plume(a.size), configs.plume_params()
    elif a.scene == "karman":
        scene, base = configs.karman(a.size, a.size), configs.karman_params()
    elif a.scene == "turbulence":
        scene, base = configs.turbulence(a.size), configs.turbulence_params()
    else:
        scene, base = configs.random_scene(a.size, 1), configs.random_scene_params(mixed=1)
    prm = tuned_params(scene, base, a.cache, log=lambda m: print(m, flush=True))
    print(json.dumps({"scene": a.scene, "size": a.size, "mg_coarsest": prm.mg_coarsest,
                      "mg_coarse_sweeps": prm.mg_coarse_sweeps, "mg_tail_side": prm.mg_tail_side,
                      "omega": prm.omega, "rb_pairs": prm.rb_pairs}))


if __name__ == "__main__":
    main()

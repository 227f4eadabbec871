"""Host-side mirror of the reference's GPU seams, over the CUDA engine.

Same names, argument meanings and error behaviour as the reference's
TypeScript classes, so code written against them reads the same here:

  GpuAdvector          src/gpu/advectGpu.ts:54    (Advector, src/core/advector.ts:28-63)
  GpuPressureSolver    src/gpu/pressureGpu.ts:68  (PressureSolver, src/core/pressureSolver.ts:21-41)
  GpuMultigridSolver   src/gpu/multigridGpu.ts:59 (PressureSolver)
  GpuStepper           src/gpu/stepGpu.ts:89      (GpuStep, src/core/simulation.ts:35-84)
  Simulation           src/core/simulation.ts:259 driving a GpuStepper
  init_gpu             src/gpu/device.ts:32

Host arrays follow src/core/grid.ts's MAC layout; float64 or float32 arrays
are accepted (the reference's FieldArray union) and converted at the
boundary, as the reference's GPU path converts to f32 on upload. Every call
runs on the device; there is no CPU path behind these classes.
"""
import ctypes
import math

import numpy as np

from . import native
from .native import FlowlabError, f32, ptr
from .scenes import DYE_CHANNELS, FLUID, Fields, Grid, apply_dye_patch, commit_labels, create_fields, dye_grid

SCHEMES = {"semiLagrangian": native.FL_SEMI_LAGRANGIAN, "macCormack": native.FL_MACCORMACK}


class GpuContext:
    """device.ts:22-30. `lost` mirrors the device-lost flag every seam checks."""

    def __init__(self, device=0):
        self.device = device
        self.lost = False


def init_gpu(device=0):
    """device.ts:32-45 — a context, or None when no CUDA device is usable."""
    try:
        eng = native.Engine(2, 2, device=device)
        eng.close()
    except (RuntimeError, OSError):
        return None
    return GpuContext(device)


def _check_ctx(ctx):
    if ctx.lost:
        raise RuntimeError("GPU device lost")


def _planes(q, cells):
    """The reference's qIn: FieldArray[] (advector.ts:52-62), or one flat
    3-plane array: three contiguous float32 planes of `cells` each."""
    if isinstance(q, (list, tuple)):
        planes = [f32(np.asarray(c).ravel()) for c in q]
    else:
        a = np.asarray(q).ravel()
        planes = [f32(a[c * cells:(c + 1) * cells]) for c in range(DYE_CHANNELS)]
    assert len(planes) == DYE_CHANNELS and all(pl.size == cells for pl in planes)
    return planes


def _plane_ptrs(planes):
    return (ctypes.c_void_p * len(planes))(*[pl.ctypes.data for pl in planes])


def _store(dst, planes):
    if isinstance(dst, (list, tuple)):
        for d, pl in zip(dst, planes):
            d[:] = pl
    else:
        dst[:] = np.concatenate(planes)


class GpuAdvector:
    """advectGpu.ts:54 — the Advector seam on the device."""

    name = "gpu"

    def __init__(self, ctx, g, dg=None):
        self.ctx = ctx
        self.g = g
        self.dg = dg or g
        scale = self.dg.nx // g.nx
        self.eng = native.Engine(g.nx, g.ny, g.h, scale, device=ctx.device)
        self.busy = False

    def _guard(self, what):
        if self.busy:
            raise RuntimeError("GpuAdvector.%s() is not re-entrant" % what)
        _check_ctx(self.ctx)

    def velocity(self, g, scheme, u_in, v_in, u_out, v_out, label, dt):
        self._guard("velocity")
        uo = np.empty(self.eng.ufaces, np.float32)
        vo = np.empty(self.eng.vfaces, np.float32)
        a, b, lab = f32(u_in), f32(v_in), np.ascontiguousarray(label, np.uint8)
        self.eng.call("fl_advect_velocity", SCHEMES[scheme], ptr(a), ptr(b), ptr(uo), ptr(vo), ptr(lab), float(dt))
        u_out[:] = uo
        v_out[:] = vo

    def dye(self, g, scheme, u, v, q_in, q_out, label, dt, dg=None):
        self._guard("dye")
        n = self.eng.dnx * self.eng.dny
        q = _planes(q_in, n)
        qo = [np.empty(n, np.float32) for _ in range(DYE_CHANNELS)]
        a, b, lab = f32(u), f32(v), np.ascontiguousarray(label, np.uint8)
        self.eng.call("fl_advect_dye", SCHEMES[scheme], ptr(a), ptr(b), _plane_ptrs(q), _plane_ptrs(qo), ptr(lab),
                      float(dt))
        _store(q_out, qo)

    def destroy(self):
        self.eng.close()


class GpuPressureSolver:
    """pressureGpu.ts:68 — red-black SOR behind the PressureSolver seam.
    Unlike the WGSL solver it honours `tol` (checked every 12 sweeps, as the
    CPU twin pressureRedBlack.ts:342-347 does); tol <= 0 runs the budget."""

    name = "gpu-rbsor"

    def __init__(self, ctx, g):
        self.ctx = ctx
        self.eng = native.Engine(g.nx, g.ny, g.h, device=ctx.device)
        self.busy = False

    def solve(self, g, p, div, label, scale, iterations, omega, tol):
        if self.busy:
            raise RuntimeError("GpuPressureSolver.solve() is not re-entrant")
        _check_ctx(self.ctx)
        pp = f32(p).copy()
        used = ctypes.c_int(0)
        d, lab = f32(div), np.ascontiguousarray(label, np.uint8)
        self.eng.call("fl_rb_solve", ptr(pp), ptr(d), ptr(lab), float(scale), int(iterations), float(omega), float(tol),
                      ctypes.byref(used))
        p[:] = pp
        return used.value

    def destroy(self):
        self.eng.close()


class GpuMultigridSolver:
    """multigridGpu.ts:59 — the V-cycle behind the PressureSolver seam.
    `cycles` caps the V-cycles; the shape is the reference's V(2,2) with 8
    coarse sweep pairs and a 4-cell coarsest level unless given. `tol` is
    honoured (the CPU twin's test, pressureMultigrid.ts:313-317)."""

    name = "gpu-mg"

    def __init__(self, ctx, g, cycles=3, pre=2, post=2, coarse_sweeps=8, coarsest=4):
        self.ctx = ctx
        self.cycles = cycles
        prm = native.default_params(mg_pre=pre, mg_post=post, mg_coarse_sweeps=coarse_sweeps, mg_coarsest=coarsest,
                                    mg_max_cycles=cycles, solver=native.FL_SOLVER_MG)
        self.eng = native.Engine(g.nx, g.ny, g.h, params=prm, device=ctx.device)
        self.last_rel_residual = -1.0
        self.busy = False

    def solve(self, g, p, div, label, scale, iterations, omega, tol):
        if self.busy:
            raise RuntimeError("GpuMultigridSolver.solve() is not re-entrant")
        _check_ctx(self.ctx)
        pp = f32(p).copy()
        used = ctypes.c_int(0)
        rr = ctypes.c_double(-1)
        d, lab = f32(div), np.ascontiguousarray(label, np.uint8)
        self.eng.call("fl_mg_solve", ptr(pp), ptr(d), ptr(lab), float(scale), int(self.cycles), float(tol),
                      ctypes.byref(used), ctypes.byref(rr))
        p[:] = pp
        self.last_rel_residual = rr.value
        return used.value

    def destroy(self):
        self.eng.close()


class GpuStepper:
    """stepGpu.ts:89 — the whole step on the device, u, v, p and dye
    resident. step() returns after the device finished and f.u / f.v hold
    the step's velocity (the reference reads them back one frame late; here
    the readback is in order). f.p is NOT updated: the pressure lives on the
    device (simulation.ts:29-33); read_pressure() fetches it."""

    def __init__(self, ctx, g, dg=None, params=None):
        self.ctx = ctx
        self.g = g
        self.dg = dg or g
        self.params = params if params is not None else native.default_params()
        self.eng = native.Engine(g.nx, g.ny, g.h, self.dg.nx // g.nx, params=self.params, device=ctx.device)
        self.dirty = True
        self.busy = False
        self.patch = None

    def invalidate(self):
        self.dirty = True

    def set_dye_patch(self, patch):
        self.patch = patch
        if patch is None:
            self.eng.call("fl_set_dye_patch", 0, 0, 0, 0, None)
            return
        # stepGpu.ts:346-348
        if patch.data.size != (DYE_CHANNELS + 1) * patch.nx * patch.ny:
            raise ValueError("dye patch is not PATCH_PLANES planes of nx*ny")
        self._patch_data = f32(patch.data)
        self.eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(self._patch_data))

    def set_buoyancy(self, w, alpha=0.0):
        self.eng.call("fl_set_buoyancy", float(w), float(alpha))

    def set_confinement(self, eps):
        self.eng.call("fl_set_confinement", float(eps))

    def set_stir(self, stir):
        if stir is None:
            self.eng.call("fl_set_stir", None)
        else:
            arr = (ctypes.c_double * 5)(stir["x"], stir["y"], stir["r"], stir["dx"], stir["dy"])
            self.eng.call("fl_set_stir", arr)

    def set_labels(self, label):
        self._label = np.ascontiguousarray(label, np.uint8)
        self.eng.call("fl_set_labels", ptr(self._label))

    def upload(self, f):
        dtype = native.FL_F64 if f.u.dtype == np.float64 else native.FL_F32
        cast = (lambda a: np.ascontiguousarray(a, np.float64)) if dtype == native.FL_F64 else f32
        u, v, p, dye = cast(f.u), cast(f.v), cast(f.p), cast(f.dye)
        lab = np.ascontiguousarray(f.label, np.uint8)
        self.eng.call("fl_upload_fields", dtype, ptr(u), ptr(v), ptr(p), ptr(lab), ptr(dye))
        self.dirty = False

    def step(self, f, scheme, dt, scale, grad_scale, dye_keep, perf=None):
        if self.busy:
            raise RuntimeError("GpuStepper.step() is not re-entrant")
        _check_ctx(self.ctx)
        self.busy = True
        try:
            if self.dirty:
                self.upload(f)
            keep = (ctypes.c_double * 3)(*dye_keep)
            iters = ctypes.c_int(0)
            # the scheme is per step, as in the seam (simulation.ts:36-38)
            self.eng.call("fl_step", SCHEMES[scheme], float(dt), float(scale), float(grad_scale), keep,
                          ctypes.byref(iters))
            self.params.scheme = SCHEMES[scheme]
            self.read_velocity(f)
            return iters.value
        finally:
            self.busy = False

    def step_auto(self, f, n):
        """n steps with dt from the device's own CFL reduction; no host
        round trip between steps. Reads nothing back."""
        if self.dirty:
            self.upload(f)
        iters = ctypes.c_int(0)
        self.eng.call("fl_step_auto", int(n), ctypes.byref(iters))
        return iters.value

    def read_velocity(self, f):
        dtype = native.FL_F64 if f.u.dtype == np.float64 else native.FL_F32
        self.eng.call("fl_read_velocity", dtype, ptr(f.u), ptr(f.v))

    def read_dye(self, dye):
        """stepGpu.ts:372-391 — nothing to bring back while the host holds truth."""
        if self.dirty:
            return
        dtype = native.FL_F64 if dye.dtype == np.float64 else native.FL_F32
        self.eng.call("fl_read_dye", dtype, ptr(dye))

    def read_pressure(self, p):
        dtype = native.FL_F64 if p.dtype == np.float64 else native.FL_F32
        self.eng.call("fl_read_pressure", dtype, ptr(p))

    def read_divergence(self, div):
        """The post-step divergence of the last step that computed it."""
        dtype = native.FL_F64 if div.dtype == np.float64 else native.FL_F32
        self.eng.call("fl_read_divergence", dtype, ptr(div))

    def stats(self):
        return self.eng.stats()

    def destroy(self):
        self.eng.close()


def optimal_omega(nx, ny=None):
    """simulation.ts:218-221."""
    ny = nx if ny is None else ny
    rho = 0.5 * (math.cos(math.pi / nx) + math.cos(math.pi / ny))
    return 2 / (1 + math.sqrt(1 - rho * rho))


DEFAULT_PARAMS = dict(cflTarget=2.0, scheme="semiLagrangian", dtMax=1 / 30, pressureIters=100, tol=5e-3,
                      omega=0.0, rho=1.0, dyeDecay=0.0, buoyancy=0.0, residualEvery=1)


def dye_keep_for(decay, dt):
    """simulation.ts:243-247."""
    k = lambda d: math.exp(-d * dt) if d > 0 else 1.0
    if isinstance(decay, (int, float)):
        return (k(decay),) * 3
    return tuple(k(d) for d in decay)


class Simulation:
    """simulation.ts:259-593 with the fused GPU stepper installed: the host
    keeps the clock and the CFL dt (from f.u/f.v, which the stepper refreshes
    each step), the device does the step."""

    def __init__(self, nx, ny=None, params=None, dtype=np.float64, dye_scale=1, ctx=None, engine_params=None):
        ny = nx if ny is None else ny
        self.params = dict(DEFAULT_PARAMS, omega=optimal_omega(nx, ny))
        self.params.update(params or {})
        self.g = Grid(nx, ny, 1.0 / ny)
        self.dye_g = dye_grid(self.g, dye_scale)
        self.f = create_fields(self.g, self.dye_g, dtype)
        self.time = 0.0
        self.dt = 0.0
        self.iters = 0
        self.stir = None
        self.dye_patch = None
        self.ctx = ctx or init_gpu()
        if self.ctx is None:
            raise RuntimeError("no CUDA device: the flowlab_gb300 engine has no CPU path")
        prm = engine_params if engine_params is not None else native.default_params()
        # the residual diagnostic runs on the device, on the same cadence
        prm.residual_every = int(self.params["residualEvery"])
        self.stepper = GpuStepper(self.ctx, self.g, self.dye_g, prm)
        self._u_max = None
        # simulation.ts:324-326, 369: steps taken (never reset) and the
        # post-step divergence, refreshed every residualEvery steps
        self.steps = 0
        self.div = np.zeros(nx * ny, dtype)

    def reset(self, scene):
        """simulation.ts:388-416 — seeds in order, commitLabels, then the
        inlet applied once at t = 0."""
        g, f = self.g, self.f
        for a in (f.u, f.v, f.p, f.dye):
            a[:] = 0
        f.label[:] = FLUID
        if scene.labels:
            scene.labels(g, f.label)
        if scene.seed:
            scene.seed(g, f.u, f.v)
        if scene.dye:
            scene.dye(self.dye_g, f.dye)
        commit_labels(g, f)
        self.dye_patch = scene.dye_source(self.dye_g, g) if scene.dye_source else None
        if self.dye_patch is not None:
            apply_dye_patch(self.dye_g, f.dye, self.dye_patch)
        self.stepper.set_dye_patch(self.dye_patch)
        self.stepper.set_buoyancy(self.params.get("buoyancy", 0.0), self.params.get("alpha", 0.0))
        self.stepper.set_confinement(self.params.get("confinement", 0.0))
        self.time = 0.0
        self.dt = 0.0
        self._u_max = None
        self.stepper.invalidate()

    def commit_label_edits(self):
        """simulation.ts:436-439."""
        commit_labels(self.g, self.f)
        self.stepper.set_labels(self.f.label)

    def max_face_speed(self):
        """simulation.ts:451-459."""
        if self._u_max is None:
            self._u_max = float(max(np.abs(self.f.u).max(), np.abs(self.f.v).max()))
        return self._u_max

    def step(self):
        """simulation.ts:467-587, fused path."""
        p, g = self.params, self.g
        stir, self.stir = self.stir, None
        u_max = self.max_face_speed()
        dt = min(p["dtMax"], (p["cflTarget"] * g.h) / u_max) if u_max > 1e-9 else p["dtMax"]
        scale = (p["rho"] * g.h * g.h) / dt
        grad_scale = dt / (p["rho"] * g.h)
        self.stepper.set_stir(stir)
        keep = dye_keep_for(p["dyeDecay"], dt)
        self.iters = self.stepper.step(self.f, p["scheme"], dt, scale, grad_scale, keep)
        # simulation.ts:495-496: the residual on this step's cadence, computed
        # on the device from the projected velocity and read back
        if p["residualEvery"] > 0 and self.steps % p["residualEvery"] == 0:
            self.stepper.read_divergence(self.div)
        self._u_max = None
        self.dt = dt
        self.time += dt
        self.steps += 1

    def divergence_stats(self, max_speed):
        """viz/fieldView.ts:44-60 divergenceStats on the device's figures:
        (divMax, divRms as a fraction of maxSpeed/h) over FLUID cells."""
        st = self.stepper.stats()
        return st["post_div_max"], st["post_div_rms"] / ((max_speed or 1) / self.g.h)

    @property
    def cfl(self):
        return (self.max_face_speed() * self.dt) / self.g.h

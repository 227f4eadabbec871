"""Failure paths, injected on the host (no GPU fault is provoked):

  * a NaN in an uploaded velocity makes the step report FL_ENONFINITE —
    from fl_step_auto when it returns statistics, from fl_step_host, and
    from the next fl_synchronize after an asynchronous fl_step_auto — and
    the engine recovers on the next upload (the reference's GPU path has no
    such check; its device-loss errors are src/gpu/device.ts:58-71 and
    src/gpu/stepGpu.ts:402-403);
  * a cycle cap of 1 under a tolerance no cycle reaches leaves the solve
    unconverged and says so (cycles = 1, rel_residual > tol), as the
    reference's capped solve returns its cap (pressureMultigrid.ts:314-317);
  * the tensor-core convolutions' bounded waits: with the progress-wait
    limit at one poll the forward pass gives up and returns FL_ETIMEOUT;
    the kernels still drain their own copies and MMAs before freeing their
    tensor memory (the drain waits keep their default bound), so the
    context stays usable and the next forward pass with the default limit
    matches the one before.
"""
import ctypes

import numpy as np
import pytest

from flowlab_gb300 import configs, native
from flowlab_gb300.native import f32, ptr

pytestmark = pytest.mark.gpu


def upload(eng, f, u=None):
    eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u if u is None else u)), ptr(f32(f.v)), ptr(f32(f.p)),
             ptr(f.label), ptr(f32(f.dye)))


def status(fn):
    try:
        fn()
    except native.FlowlabError as err:
        return err.status
    return native.FL_OK


def test_nan_velocity_is_reported_and_the_engine_recovers():
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-6, max_cycles=10)
    bad = f32(f.u).copy()
    bad[bad.size // 2] = np.nan
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        iters = ctypes.c_int()
        upload(eng, f, bad)
        assert status(lambda: eng.call("fl_step_auto", 1, ctypes.byref(iters))) == native.FL_ENONFINITE
        assert b"non-finite" in eng.lib.fl_last_error(eng.handle)

        upload(eng, f, bad)
        eng.call("fl_step_auto", 1, None)  # asynchronous: reported by the next synchronising call
        assert status(lambda: eng.call("fl_synchronize")) == native.FL_ENONFINITE

        n = (eng.ufaces, eng.vfaces, eng.cells, eng.dye_len)
        outs = [np.empty(k, np.float32) for k in n]
        st = status(lambda: eng.call("fl_step_host", native.FL_F32, ptr(bad), ptr(f32(f.v)), ptr(f32(f.p)),
                                     ptr(f.label), ptr(f32(f.dye)), *[ptr(o) for o in outs], ctypes.byref(iters)))
        assert st == native.FL_ENONFINITE

        # recovery: clean fields step normally and match a fresh engine
        upload(eng, f)
        eng.call("fl_step_auto", 2, ctypes.byref(iters))
        u = np.empty(eng.ufaces, np.float32)
        v = np.empty(eng.vfaces, np.float32)
        eng.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
        assert np.isfinite(u).all() and np.isfinite(v).all()
    finally:
        eng.close()
    fresh = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        upload(fresh, f)
        fresh.call("fl_step_auto", 2, None)
        u2 = np.empty(fresh.ufaces, np.float32)
        v2 = np.empty(fresh.vfaces, np.float32)
        fresh.call("fl_read_velocity", native.FL_F32, ptr(u2), ptr(v2))
    finally:
        fresh.close()
    assert np.array_equal(u, u2) and np.array_equal(v, v2)


@pytest.mark.parametrize("mixed", [0, 2])
def test_cycle_cap_reports_an_unconverged_solve(mixed):
    g, f, patch = configs.plume(64)
    prm = configs.plume_params(tol=1e-12, max_cycles=1, mixed=mixed)
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        upload(eng, f)
        iters = ctypes.c_int()
        for _ in range(3):
            eng.call("fl_step_auto", 1, ctypes.byref(iters))
            st = eng.stats()
            assert iters.value == 1 and st["cycles"] == 1
            assert st["rel_residual"] > prm.tol, st
    finally:
        eng.close()


def test_tensor_core_wait_timeout_is_reported_and_recoverable():
    lib = native.load()
    from oracle import unet_oracle as U

    rng = np.random.default_rng(5)
    th = U.init_params(3)
    layout, _ = U.param_layout()
    _, wo, nw, bo, _ = layout[-1]
    th[wo:wo + nw] = rng.standard_normal(nw).astype(np.float32) * 0.2
    x = rng.standard_normal((1, 64, 128, 3)).astype(np.float32)
    x[..., 1] = 1.0
    net = native.Unet(64 * 128)
    try:
        lib.fl_unet_use_tensor_cores(1)
        net.set_params(th)
        before = net.forward(x)
        assert lib.fl_unet_set_wait_limit(1) == native.FL_OK
        try:
            st = status(lambda: net.forward(x))
        finally:
            assert lib.fl_unet_set_wait_limit(0) == native.FL_OK
        assert st == native.FL_ETIMEOUT
        after = net.forward(x)
        assert np.array_equal(before, after)
    finally:
        net.close()

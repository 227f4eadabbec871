"""The no-allocation velocity advection (fl_advect_velocity_noalloc) against the
allocating per-pass entry point (fl_advect_velocity), through the C ABI.

fl_advect_velocity_noalloc serves callers that cannot allocate device memory
where they advect (real-time threads that must not block in cudaMalloc,
memory owned by someone else's arena, a device-memory budget fixed up front):
it takes their device buffers and keeps its MacCormack scratch in a fixed
array of the library's own device memory. The test holds its device buffers
in torch tensors (the test may allocate; the entry point must not), runs two
calls in a row on different inputs, and requires the same output as the
existing entry point — bit for bit, the tolerance every other advection test
here uses — and the device's free memory unchanged across a call made after
the first. This file is named to run last, so a failure here cannot hide
another test's result.
"""
import ctypes

import numpy as np
import pytest

from flowlab_gb300 import native
from flowlab_gb300.native import f32, ptr
from tests import fixtures as fx

pytestmark = pytest.mark.gpu


def engine_advect(nx, ny, h, scheme, u, v, label, dt):
    eng = native.Engine(nx, ny, h)
    try:
        uo = np.empty(eng.ufaces, np.float32)
        vo = np.empty(eng.vfaces, np.float32)
        eng.call("fl_advect_velocity", scheme, ptr(f32(u)), ptr(f32(v)), ptr(uo), ptr(vo), ptr(label), np.float32(dt))
    finally:
        eng.close()
    return uo, vo


def noalloc_advect(lib, torch, nx, ny, h, scheme, u, v, label, dt, stream):
    dev = torch.device("cuda", 0)
    du = torch.from_numpy(f32(u)).to(dev)
    dv = torch.from_numpy(f32(v)).to(dev)
    dl = torch.from_numpy(np.ascontiguousarray(label, np.uint8)).to(dev)
    uo = torch.full_like(du, float("nan"))
    vo = torch.full_like(dv, float("nan"))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    st = lib.fl_advect_velocity_noalloc(scheme, nx, ny, float(h), float(np.float32(dt)), du.data_ptr(), dv.data_ptr(),
                                        uo.data_ptr(), vo.data_ptr(), dl.data_ptr(), ctypes.c_void_p(stream))
    assert st == native.FL_OK, lib.fl_last_error(None).decode()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info(dev)[0]
    return uo.cpu().numpy(), vo.cpu().numpy(), free0, free1


@pytest.mark.parametrize("scheme", [native.FL_SEMI_LAGRANGIAN, native.FL_MACCORMACK])
def test_noalloc_matches_allocating_entry_point_twice(scheme):
    torch = pytest.importorskip("torch")
    lib = native.load()
    stream = torch.cuda.current_stream().cuda_stream
    cases = []
    h, dt, u, v, label, _, _, _, _ = fx.advect_fixture(1)
    cases.append((fx.NX, fx.NY, h, u, v, label, dt))
    nx, ny = 256, 192
    h2, dt2, u2, v2, label2, _, _, _, _ = fx.advect_fixture(1, nx, ny)
    label2 = fx.scaled_block_labels(nx, ny)
    cases.append((nx, ny, h2, -0.7 * u2, 1.3 * v2, label2, 0.8 * dt2))
    for k, (nx, ny, h, u, v, label, dt) in enumerate(cases):  # two calls in a row, different inputs and sizes
        eu, ev = engine_advect(nx, ny, h, scheme, u, v, label, dt)
        gu, gv, free0, free1 = noalloc_advect(lib, torch, nx, ny, h, scheme, u, v, label, dt, stream)
        if k > 0:
            # the set-up (address look-up, kernel loading) is done: no device memory taken
            assert free1 == free0, "device free memory changed by %d bytes" % (free0 - free1)
        assert np.isfinite(gu).all() and np.isfinite(gv).all()
        assert np.array_equal(eu, gu), "u differs in %d faces" % int((eu != gu).sum())
        assert np.array_equal(ev, gv), "v differs in %d faces" % int((ev != gv).sum())


def test_noalloc_records_into_a_cuda_graph():
    """After its set-up call, the entry point can be recorded by stream
    capture (it makes no allocating or synchronising call, either of which
    would invalidate a global-mode capture); the recorded launch, replayed on
    new inputs written into the same buffers, matches the allocating entry
    point on those inputs."""
    torch = pytest.importorskip("torch")
    lib = native.load()
    nx, ny = 256, 192
    h, dt, u, v, _, _, _, _, _ = fx.advect_fixture(1, nx, ny)
    label = fx.scaled_block_labels(nx, ny)
    dev = torch.device("cuda", 0)
    du = torch.from_numpy(f32(u)).to(dev)
    dv = torch.from_numpy(f32(v)).to(dev)
    dl = torch.from_numpy(np.ascontiguousarray(label, np.uint8)).to(dev)
    uo = torch.full_like(du, float("nan"))
    vo = torch.full_like(dv, float("nan"))

    def call():
        s = torch.cuda.current_stream().cuda_stream
        return lib.fl_advect_velocity_noalloc(native.FL_MACCORMACK, nx, ny, float(h), float(np.float32(dt)),
                                              du.data_ptr(), dv.data_ptr(), uo.data_ptr(), vo.data_ptr(),
                                              dl.data_ptr(), ctypes.c_void_p(s))

    assert call() == native.FL_OK, lib.fl_last_error(None).decode()  # the set-up call
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        st = call()
    assert st == native.FL_OK, lib.fl_last_error(None).decode()
    u2, v2 = -0.7 * np.asarray(u, np.float32), 1.3 * np.asarray(v, np.float32)
    du.copy_(torch.from_numpy(f32(u2)))
    dv.copy_(torch.from_numpy(f32(v2)))
    uo.fill_(float("nan"))
    vo.fill_(float("nan"))
    graph.replay()
    torch.cuda.synchronize()
    eu, ev = engine_advect(nx, ny, h, native.FL_MACCORMACK, u2, v2, label, dt)
    gu, gv = uo.cpu().numpy(), vo.cpu().numpy()
    assert np.array_equal(eu, gu), "u differs in %d faces" % int((eu != gu).sum())
    assert np.array_equal(ev, gv), "v differs in %d faces" % int((ev != gv).sum())
    del graph


def test_noalloc_rejects_overlapping_outputs():
    torch = pytest.importorskip("torch")
    lib = native.load()
    nx, ny = 40, 32
    u = torch.zeros((nx + 1) * ny, device="cuda")
    v = torch.zeros(nx * (ny + 1), device="cuda")
    lab = torch.zeros(nx * ny, dtype=torch.uint8, device="cuda")
    vo = torch.zeros_like(v)
    st = lib.fl_advect_velocity_noalloc(native.FL_MACCORMACK, nx, ny, 1.0 / ny, 0.01, u.data_ptr(), v.data_ptr(),
                                        u.data_ptr(), vo.data_ptr(), lab.data_ptr(), None)
    assert st == native.FL_EINVAL
    assert b"overlap" in lib.fl_last_error(None)


def test_noalloc_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = native.load()
    x = torch.zeros(16, device="cuda")
    st = lib.fl_advect_velocity_noalloc(native.FL_MACCORMACK, 2048, 2048, 1.0 / 2048, 0.01, x.data_ptr(), x.data_ptr(),
                                        x.data_ptr(), x.data_ptr(), x.data_ptr(), None)
    assert st == native.FL_EINVAL
    assert b"at most" in lib.fl_last_error(None)

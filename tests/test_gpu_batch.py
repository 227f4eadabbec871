"""Batched scenes (fl_batch_*): every engine's step graph launched on its
own stream per step; each engine's result equals stepping it alone, bit for
bit."""
import numpy as np
import pytest

from flowlab_gb300 import batch, configs, native
from flowlab_gb300.native import f32, ptr

pytestmark = pytest.mark.gpu


def karman_engine():
    g, f, patch = configs.karman(96, 64)
    e = native.Engine(g.nx, g.ny, g.h, params=configs.karman_params())
    e.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
           ptr(f32(f.dye)))
    return e


def fields(e):
    u = np.empty(e.ufaces, np.float32)
    v = np.empty(e.vfaces, np.float32)
    p = np.empty(e.cells, np.float32)
    d = np.empty(e.dye_len, np.float32)
    e.call("fl_read_velocity", native.FL_F32, ptr(u), ptr(v))
    e.call("fl_read_pressure", native.FL_F32, ptr(p))
    e.call("fl_read_dye", native.FL_F32, ptr(d))
    return u, v, p, d


def test_batch_equals_engines_stepped_alone():
    sides = [64, 128, 64, 256]
    steps = 5
    alone = batch.make_engines(sides, seed=11) + [karman_engine()]
    together = batch.make_engines(sides, seed=11) + [karman_engine()]
    try:
        ref = []
        for e in alone:
            e.call("fl_step_auto", steps, None)
            ref.append((fields(e), e.stats()))
        b = native.Batch(together)
        try:
            b.step(steps)
        finally:
            b.close()
        for k, e in enumerate(together):
            got = fields(e)
            st = e.stats()
            for name, x, y in zip(("u", "v", "p", "dye"), ref[k][0], got):
                assert np.array_equal(x, y), "scene %d: %s differs" % (k, name)
            assert st["cycles"] == ref[k][1]["cycles"] and st["steps"] == ref[k][1]["steps"]
            assert abs(st["time"] - ref[k][1]["time"]) <= 1e-12
    finally:
        batch.close_all(alone + together)


def test_batch_then_single_steps_stay_ordered():
    """Steps through the batch, then through each engine, equal the same
    number of single steps."""
    a = batch.make_engines([64, 128], seed=3)
    c = batch.make_engines([64, 128], seed=3)
    try:
        for e in a:
            e.call("fl_step_auto", 4, None)
        b = native.Batch(c)
        b.step(2)
        b.close()
        for e in c:
            e.call("fl_step_auto", 2, None)
        for x, y in zip(a, c):
            for fx, fy in zip(fields(x), fields(y)):
                assert np.array_equal(fx, fy)
    finally:
        batch.close_all(a + c)


def test_engines_at_different_parities_step_together():
    """An engine one step ahead of the other (the other buffer parity) steps
    in the same batch; both equal the same steps taken alone."""
    a = batch.make_engines([64, 128], seed=5)
    c = batch.make_engines([64, 128], seed=5)
    try:
        a[0].call("fl_step_auto", 4, None)
        a[1].call("fl_step_auto", 3, None)
        c[0].call("fl_step_auto", 1, None)
        b = native.Batch(c)
        b.step(3)
        b.close()
        for x, y in zip(a, c):
            for fx, fy in zip(fields(x), fields(y)):
                assert np.array_equal(fx, fy)
            assert x.stats()["steps"] == y.stats()["steps"]
    finally:
        batch.close_all(a + c)


def test_engine_listed_twice_is_refused():
    es = batch.make_engines([64], seed=5)
    try:
        with pytest.raises(native.FlowlabError):
            native.Batch([es[0], es[0]])
    finally:
        batch.close_all(es)


def plume_engine(n=64):
    g, f, patch = configs.plume(n)
    e = native.Engine(g.nx, g.ny, g.h, params=configs.plume_params(max_cycles=20))
    e.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
    e.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
           ptr(f32(f.dye)))
    return e


def assert_same(alone, together, what):
    for k, (x, y) in enumerate(zip(alone, together)):
        for name, fx, fy in zip(("u", "v", "p", "dye"), fields(x), fields(y)):
            assert np.array_equal(fx, fy), "%s, scene %d: %s differs" % (what, k, name)
        sx, sy = x.stats(), y.stats()
        assert sx["cycles"] == sy["cycles"] and sx["steps"] == sy["steps"], (what, k, sx, sy)
        assert sx["rel_residual"] == sy["rel_residual"] or abs(sx["rel_residual"] - sy["rel_residual"]) <= \
            1e-9 * abs(sx["rel_residual"]), (what, k)


@pytest.mark.parametrize("mixed", [0, 1, 2])
def test_worklist_batch_equals_engines_stepped_alone(mixed):
    """All-multigrid batches run the work-list solve (one launch per V-cycle
    phase over every scene's tiles): uneven sides, 32^2 (tail only) to 256^2,
    in float32, with the float64 and with the double-float defect
    correction; a plume with its dye patch, buoyancy and confinement joins
    the double-float batch. Every scene equals the same scene stepped
    alone, bit for bit, cycle counts included."""
    sides = [64, 256, 32, 128, 64]
    steps = 4
    tol = 1e-4 if mixed == 0 else 1e-6  # float32 alone stalls above 1e-6 on these scenes
    alone = batch.make_engines(sides, seed=21, mixed=mixed, tol=tol)
    together = batch.make_engines(sides, seed=21, mixed=mixed, tol=tol)
    if mixed == 2:
        alone.append(plume_engine())
        together.append(plume_engine())
    try:
        for e in alone:
            e.call("fl_step_auto", steps, None)
        b = native.Batch(together)
        try:
            assert b.worklist
            b.step(steps)
        finally:
            b.close()
        assert_same(alone, together, "mixed %d" % mixed)
    finally:
        batch.close_all(alone + together)


def test_worklist_batch_follows_engine_changes():
    """Between work-list batch steps: one engine steps alone (its parity
    moves away from the others') and another changes its tolerance (its
    graphs are rebuilt); the batch rebuilds its own graphs and the results
    equal the same sequence without the batch."""
    sides = [64, 128, 64]
    alone = batch.make_engines(sides, seed=8)
    together = batch.make_engines(sides, seed=8)
    try:
        b = native.Batch(together)
        try:
            assert b.worklist
            b.step(2)
            together[0].call("fl_step_auto", 1, None)
            tighter = configs.random_scene_params(tol=1e-7, max_cycles=40, mixed=1)
            together[1].set_params(tighter)
            b.step(3)
        finally:
            b.close()
        for e in alone:
            e.call("fl_step_auto", 2, None)
        alone[0].call("fl_step_auto", 1, None)
        alone[1].set_params(configs.random_scene_params(tol=1e-7, max_cycles=40, mixed=1))
        for e in alone:
            e.call("fl_step_auto", 3, None)
        assert_same(alone, together, "after changes")
    finally:
        batch.close_all(alone + together)


def test_batch_with_a_red_black_scene_launches_engine_graphs():
    es = batch.make_engines([64], seed=2) + [karman_engine()]
    try:
        b = native.Batch(es)
        try:
            assert not b.worklist
            b.step(1)
        finally:
            b.close()
    finally:
        batch.close_all(es)


def test_switching_paths_keeps_results():
    """The same batch stepped through both paths in turn (work list, engine
    graphs, work list) equals the scenes stepped alone."""
    sides = [128, 64, 32]
    alone = batch.make_engines(sides, seed=13)
    together = batch.make_engines(sides, seed=13)
    try:
        for e in alone:
            e.call("fl_step_auto", 6, None)
        b = native.Batch(together)
        try:
            assert b.worklist
            b.step(2)
            b.set_worklist(False)
            assert not b.worklist
            b.step(2)
            b.set_worklist(True)
            assert b.worklist
            b.step(2)
        finally:
            b.close()
        assert_same(alone, together, "switching")
    finally:
        batch.close_all(alone + together)

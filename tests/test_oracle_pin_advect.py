"""Pins the oracle's advection, divergence, boundary and body-force passes
against the reference's own known-answer tests (src/core/advect.test.ts,
divergence.test.ts, boundaries.test.ts, buoyancy.test.ts, grid.test.ts),
run on the float64 restatement. No GPU."""
import math

import numpy as np

from flowlab_gb300 import scenes as sc

H = 0.5  # advect.test.ts:15


def faces(nx, ny):
    return np.zeros((nx + 1) * ny), np.zeros(nx * (ny + 1))


def test_every_face_written(o64):
    # advect.test.ts:25-46
    u, v = faces(4, 4)
    u[:] = 0.3
    v[:] = -0.2
    uo, vo = o64.advect_velocity(4, 4, H, False, u, v, np.zeros(16, np.uint8), 0.25 * H)
    assert np.isfinite(uo).all() and np.isfinite(vo).all()


def test_uniform_velocity_advects_to_itself(o64):
    # advect.test.ts:48-78
    nx = ny = 4
    u, v = faces(nx, ny)
    u[:] = 0.75
    v[:] = -0.25
    uo, vo = o64.advect_velocity(nx, ny, H, False, u, v, np.zeros(16, np.uint8), 0.3 * H)
    uu = uo.reshape(ny, nx + 1)[:, 1:nx]
    vv = vo.reshape(ny + 1, nx)[1:ny, :]
    assert np.abs(uu - 0.75).max() < 1e-12 and np.abs(vv + 0.25).max() < 1e-12


def test_rk2_ramp_closed_form(o64):
    # advect.test.ts:88-111
    nx, ny = 6, 4
    u, v = faces(nx, ny)
    u.reshape(ny, nx + 1)[:] = np.arange(nx + 1)
    dt = 0.5 * H
    r = dt / H
    factor = 1 - r + 0.5 * r * r
    uo, _ = o64.advect_velocity(nx, ny, H, False, u, v, np.zeros(nx * ny, np.uint8), dt)
    got = uo.reshape(ny, nx + 1)[:, 1:nx]
    want = np.arange(1, nx) * factor
    assert np.abs(got - want).max() < 1e-12
    assert (np.abs(got - np.arange(1, nx) * (1 - r)) > 1e-9).all()


def test_rk2_ramp_closed_form_v(o64):
    # advect.test.ts:113-137
    nx, ny = 4, 6
    u, v = faces(nx, ny)
    v.reshape(ny + 1, nx)[:] = np.arange(ny + 1)[:, None]
    dt = 0.5 * H
    factor = 1 - 0.5 + 0.5 * 0.25  # r = dt/h = 0.5
    _, vo = o64.advect_velocity(nx, ny, H, False, u, v, np.zeros(nx * ny, np.uint8), dt)
    got = vo.reshape(ny + 1, nx)[1:ny, :]
    assert np.abs(got - np.arange(1, ny)[:, None] * factor).max() < 1e-12


def test_normal_velocity_stays_zero_on_walls(o64):
    # advect.test.ts:139-168
    nx = ny = 6
    u, v = faces(nx, ny)
    u.reshape(ny, nx + 1)[:] = np.sin(math.pi * np.arange(nx + 1) / nx)
    v.reshape(ny + 1, nx)[:] = np.sin(math.pi * np.arange(ny + 1) / ny)[:, None]
    uo, vo = o64.advect_velocity(nx, ny, H, False, u, v, np.zeros(36, np.uint8), 0.4 * H)
    U, V = uo.reshape(ny, nx + 1), vo.reshape(ny + 1, nx)
    assert np.abs(U[:, 0]).max() < 1e-12 and np.abs(U[:, nx]).max() < 1e-12
    assert np.abs(V[0, :]).max() < 1e-12 and np.abs(V[ny, :]).max() < 1e-12


def rough_faces(nx, ny):
    """advect.test.ts:172-178."""
    u, v = faces(nx, ny)
    j, i = np.meshgrid(np.arange(ny), np.arange(nx + 1), indexing="ij")
    u.reshape(ny, nx + 1)[:] = np.sin(i * 1.7) * np.cos(j * 2.3)
    j, i = np.meshgrid(np.arange(ny + 1), np.arange(nx), indexing="ij")
    v.reshape(ny + 1, nx)[:] = np.cos(i * 1.1) * np.sin(j * 0.9)
    return u, v


def test_huge_timestep_stays_bounded(o64):
    # advect.test.ts:170-207 (semi-Lagrangian) and 459-490 (MacCormack limiter)
    nx = ny = 8
    u, v = rough_faces(nx, ny)
    for mac in (False, True):
        uo, vo = o64.advect_velocity(nx, ny, H, mac, u, v, np.zeros(64, np.uint8), 50 * H)
        assert np.isfinite(uo).all() and (np.abs(uo) <= np.abs(u).max() + 1e-12).all()
        assert np.isfinite(vo).all() and (np.abs(vo) <= np.abs(v).max() + 1e-12).all()


def test_scalar_stripe_translates_one_cell(o64):
    # advect.test.ts:267-287 (x) and 289-312 (y)
    n = 8
    u, v = faces(n, n)
    u[:] = 0.75
    q = np.zeros(3 * n * n)
    q[0:n * n].reshape(n, n)[:, 3] = 1
    out = o64.advect_dye(n, n, H, n, n, H, False, u, v, q, np.zeros(n * n, np.uint8), H / 0.75)
    want = np.zeros((n, n))
    want[:, 4] = 1
    assert np.abs(out[0:n * n].reshape(n, n) - want).max() < 1e-12
    u[:] = 0
    v[:] = 0.5
    q[:] = 0
    q[0:n * n].reshape(n, n)[3, :] = 1
    out = o64.advect_dye(n, n, H, n, n, H, False, u, v, q, np.zeros(n * n, np.uint8), H / 0.5)
    want = np.zeros((n, n))
    want[4, :] = 1
    assert np.abs(out[0:n * n].reshape(n, n) - want).max() < 1e-12


def test_scalar_no_new_extrema_and_uniform_untouched(o64):
    # advect.test.ts:314-361
    n = 16
    g = sc.Grid(n, n, H)
    u, v = faces(n, n)
    sc.add_vortex_pair(g, u, v)
    q = np.zeros(3 * n * n)
    q[0:n * n].reshape(n, n)[:, :8] = 1
    out = o64.advect_dye(n, n, H, n, n, H, False, u, v, q, np.zeros(n * n, np.uint8), 50 * H)
    assert np.isfinite(out).all() and out.min() >= -1e-12 and out.max() <= 1 + 1e-12
    q[:] = 0.7
    out = o64.advect_dye(n, n, H, n, n, H, False, u, v, q, np.zeros(n * n, np.uint8), 0.3 * H)
    assert np.abs(out - 0.7).max() < 1e-12


def test_scalar_rk2_ramp(o64):
    # advect.test.ts:366-395
    nx, ny = 8, 4
    u, v = faces(nx, ny)
    u.reshape(ny, nx + 1)[:] = np.arange(nx + 1)
    q = np.zeros(3 * nx * ny)
    q[0:nx * ny].reshape(ny, nx)[:] = np.arange(nx) + 0.5
    dt = 0.5 * H
    factor = 1 - 0.5 + 0.5 * 0.25  # r = dt/h = 0.5
    out = o64.advect_dye(nx, ny, H, nx, ny, H, False, u, v, q, np.zeros(nx * ny, np.uint8), dt)
    got = out[0:nx * ny].reshape(ny, nx)[:, 1:]
    assert np.abs(got - (np.arange(1, nx) + 0.5) * factor).max() < 1e-12


def test_maccormack_uniform_and_peak(o64):
    # advect.test.ts:432-457 and 492-525
    n = 6
    u, v = faces(n, n)
    u[:] = 0.75
    v[:] = -0.25
    uo, vo = o64.advect_velocity(n, n, H, True, u, v, np.zeros(36, np.uint8), 0.3 * H)
    assert np.abs(uo.reshape(n, n + 1)[:, 1:n] - 0.75).max() < 1e-12
    assert np.abs(vo.reshape(n + 1, n)[1:n, :] + 0.25).max() < 1e-12

    nx, ny = 64, 16
    u, v = faces(nx, ny)
    u[:] = 1.0
    sigma = 4 * H
    x = (np.arange(nx) + 0.5) * H - 8 * H
    y = (np.arange(ny) + 0.5) * H - 8 * H
    blob = np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / (2 * sigma * sigma)).ravel()
    lab = np.zeros(nx * ny, np.uint8)

    def run(mac):
        q = np.concatenate([blob, np.zeros(2 * nx * ny)])
        for _ in range(40):
            q = o64.advect_dye(nx, ny, H, nx, ny, H, mac, u, v, q, lab, 0.5 * H)
        return q[0:nx * ny].max()

    sl, mc = run(False), run(True)
    assert mc > sl + 0.05 and mc <= 1 + 1e-12


def test_divergence_closed_forms(o64):
    # divergence.test.ts:8-55
    nx, ny = 5, 4
    u, v = faces(nx, ny)
    u[:] = 0.4
    v[:] = -1.3
    assert np.abs(o64.divergence(nx, ny, H, u, v)).max() < 1e-12
    u.reshape(ny, nx + 1)[:] = np.arange(nx + 1) * H
    v[:] = 0
    assert np.abs(o64.divergence(nx, ny, H, u, v) - 1).max() < 1e-12
    u[:] = 0
    v.reshape(ny + 1, nx)[:] = (np.arange(ny + 1) * H)[:, None]
    assert np.abs(o64.divergence(nx, ny, H, u, v) - 1).max() < 1e-12


def test_commit_labels(o64):
    # boundaries.test.ts:8-59
    nx = ny = 5
    lab = np.zeros(25, np.uint8)
    lab[2 + 2 * 5] = sc.SOLID
    lab[0] = sc.AIR
    u, v = faces(nx, ny)
    u[:] = 1
    v[:] = 1
    p = np.ones(25)
    dye = np.ones(75)
    p2, u2, v2, d2 = o64.commit_labels(nx, ny, p, u, v, lab, dye, 25)
    U, V = u2.reshape(ny, nx + 1), v2.reshape(ny + 1, nx)
    assert U[2, 2] == 0 and U[2, 3] == 0 and U[2, 1] == 1 and U[2, 4] == 1
    assert V[2, 2] == 0 and V[3, 2] == 0 and V[1, 2] == 1
    assert U[:, 0].min() == 1 and U[:, nx].min() == 1  # prescribed boundary faces kept
    assert p2[0] == 0 and p2[12] == 0 and p2[1] == 1
    assert d2[12] == 0 and d2[25 + 12] == 0 and d2[0] == 1


def test_outflow(o64):
    # boundaries.test.ts:61-124
    nx, ny = 4, 3
    lab = np.zeros(12, np.uint8)
    lab.reshape(ny, nx)[:, nx - 1] = sc.AIR
    u, v = faces(nx, ny)
    U = u.reshape(ny, nx + 1)
    U[:, nx - 1] = [0.5, -0.25, 0.0]
    U[:, nx] = 9.0
    u2, v2 = o64.outflow(nx, ny, u, v, lab)
    U2 = u2.reshape(ny, nx + 1)
    assert list(U2[:, nx - 1]) == [0.5, 0.0, 0.0] and list(U2[:, nx]) == [0.5, 0.0, 0.0]
    u3, v3 = o64.outflow(nx, ny, u, v, np.zeros(12, np.uint8))  # closed box: no-op
    assert np.array_equal(u3, u) and np.array_equal(v3, v)


def test_buoyancy_faces_and_values(o64):
    # buoyancy.test.ts:82-109 — interior faces get exactly w*dt*heat; solid
    # and boundary faces untouched.
    nx = ny = 6
    lab = np.zeros(36, np.uint8)
    lab[2 + 3 * 6] = sc.SOLID
    heat = np.ones(36)
    v = np.zeros(nx * (ny + 1))
    v2 = o64.buoyancy(nx, ny, 1 / 6, nx, ny, 1 / 6, v, heat, np.zeros(36), lab, 1.0, 0.0, 0.1)
    V = v2.reshape(ny + 1, nx)
    assert (V[0] == 0).all() and (V[ny] == 0).all()
    assert V[3, 2] == 0 and V[4, 2] == 0
    assert V[1, 0] == 0.1 and V[5, 5] == 0.1


def test_buoyancy_finer_dye_grid(o64):
    # buoyancy.test.ts:124-142 — heat on a 2x dye grid stepping 0 -> 1 at the
    # face row samples 0.5 there.
    nx = ny = 8
    dnx = dny = 16
    heat = np.zeros(dnx * dny)
    heat.reshape(dny, dnx)[8:, :] = 1
    v = np.zeros(nx * (ny + 1))
    v2 = o64.buoyancy(nx, ny, 1 / 8, dnx, dny, 1 / 16, v, heat, np.zeros_like(heat), np.zeros(64, np.uint8), 1.0, 0.0, 1.0)
    assert np.abs(v2.reshape(ny + 1, nx)[4] - 0.5).max() < 1e-12


def test_buoyancy_alpha_term_is_linear(o64):
    """NEW soot term: v += -alpha*dt*s, additive to the heat term."""
    nx = ny = 8
    lab = np.zeros(64, np.uint8)
    heat = np.linspace(0, 1, 64)
    smoke = np.linspace(1, 0, 64)
    v = np.zeros(nx * (ny + 1))
    vb = o64.buoyancy(nx, ny, 1 / 8, nx, ny, 1 / 8, v, heat, smoke, lab, 1.0, 0.0, 0.1)
    va = o64.buoyancy(nx, ny, 1 / 8, nx, ny, 1 / 8, v, heat, smoke, lab, 0.0, 0.05, 0.1)
    vab = o64.buoyancy(nx, ny, 1 / 8, nx, ny, 1 / 8, v, heat, smoke, lab, 1.0, 0.05, 0.1)
    assert np.abs(vab - (vb + va)).max() < 1e-15
    assert (va <= 0).all() and va.min() < 0


def test_grid_samplers(o64):
    # grid.test.ts:57-93 via a zero-velocity advection (identity at centres)
    n = 4
    q = np.zeros(3 * n * n)
    q[:n * n] = np.arange(n * n, dtype=float)
    u, v = faces(n, n)
    out = o64.advect_dye(n, n, H, n, n, H, True, u, v, q, np.zeros(n * n, np.uint8), 0.1)
    assert np.array_equal(out, q)


def test_vorticity_of_solid_rotation(o64):
    """vorticity.ts:24-42: u = -y, v = x gives curl 2 everywhere."""
    nx = ny = 8
    h = 1 / 8
    u, v = faces(nx, ny)
    u.reshape(ny, nx + 1)[:] = -((np.arange(ny) + 0.5) * h)[:, None]
    v.reshape(ny + 1, nx)[:] = (np.arange(nx) + 0.5) * h
    w = o64.vorticity(nx, ny, h, u, v)
    assert np.abs(w - 2).max() < 1e-12

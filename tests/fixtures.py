"""The reference's own GPU-vs-CPU fixtures (src/gpu/*.gputest.ts), rebuilt in
numpy so the CUDA engine is diffed against the oracle on the same inputs."""
import math

import numpy as np

from flowlab_gb300.scenes import AIR, SOLID, js_lcg_uniform

NX, NY = 40, 32  # redBlack.gputest.ts:30-31


def block_labels(nx=NX, ny=NY, block=((10, 16), (12, 20))):
    """Air outlet column at i = nx-1 and a solid block
    (redBlack.gputest.ts:38-44)."""
    label = np.zeros(nx * ny, np.uint8)
    lab = label.reshape(ny, nx)
    lab[:, nx - 1] = AIR
    (i0, i1), (j0, j1) = block
    lab[j0:j1, i0:i1] = SOLID
    return label


def pressure_fixture(nx=NX, ny=NY):
    """redBlack.gputest.ts:38-52 / multigrid.gputest.ts:43-57."""
    return block_labels(nx, ny), js_lcg_uniform(nx * ny, 12345)


def scaled_block_labels(nx, ny):
    """pressureMultigrid.test.ts:34-42's boundary fixture at any size."""
    label = np.zeros(nx * ny, np.uint8)
    lab = label.reshape(ny, nx)
    lab[:, nx - 1] = AIR
    lab[ny >> 2:ny >> 1, nx >> 2:(nx * 3) >> 3] = SOLID
    return label


def advect_fixture(dye_scale=1, nx=NX, ny=NY):
    """advect.gputest.ts:45-86: shear + swirl, solid block, Air column, sharp
    dye on the (possibly refined) dye grid. Returns (h, dt, u, v, label, dye,
    dnx, dny, dh)."""
    h = 1.0 / ny
    dt = (1.5 * h) / 1.2
    u = np.zeros((nx + 1) * ny)
    v = np.zeros(nx * (ny + 1))
    j, i = np.meshgrid(np.arange(ny), np.arange(nx + 1), indexing="ij")
    u.reshape(ny, nx + 1)[:] = 1.2 * np.sin(3 * (j + 0.5) * h) + 0.4 * np.cos(5 * i * h)
    j, i = np.meshgrid(np.arange(ny + 1), np.arange(nx), indexing="ij")
    v.reshape(ny + 1, nx)[:] = -0.9 * np.sin(4 * (i + 0.5) * h) + 0.3 * np.cos(2 * j * h)
    label = block_labels(nx, ny)
    s = dye_scale
    dnx, dny = nx * s, ny * s
    dh = 1.0 / (ny * s)
    jj, ii = np.meshgrid(np.arange(dny), np.arange(dnx), indexing="ij")
    x = (ii + 0.5) * dh
    y = (jj + 0.5) * dh
    d0 = np.where(x < 0.5 * nx * h, 1.0, 0.0)
    d1 = np.where((np.floor(x / h) + np.floor(y / h)) % 7 < 3, 0.8, 0.1)
    d2 = np.where(y > (ny / 3) * h, 0.5, 0.0)
    dye = np.concatenate([d0.ravel(), d1.ravel(), d2.ravel()])
    return h, dt, u, v, label, dye, dnx, dny, dh


def project_fixture(nx=NX, ny=NY, seed=98765):
    """project.gputest.ts:56-87: pseudo-random u, v, p, dye without the
    solid-face invariant, same label layout."""
    label = block_labels(nx, ny)
    vals = js_lcg_uniform((nx + 1) * ny + nx * (ny + 1) + nx * ny + 3 * nx * ny, seed)
    o = 0
    u = vals[o:o + (nx + 1) * ny]; o += (nx + 1) * ny
    v = vals[o:o + nx * (ny + 1)]; o += nx * (ny + 1)
    p = vals[o:o + nx * ny]; o += nx * ny
    dye = 0.25 + 0.5 * np.abs(vals[o:o + 3 * nx * ny])
    return label, u.copy(), v.copy(), p.copy(), dye.copy()


def patch_fixture(ny=NY, cols=3):
    """project.gputest.ts:114-122: values varying in both directions, coverage
    0 on every fifth row and 0.4 on every seventh."""
    cells = cols * ny
    data = np.zeros(4 * cells, np.float32)
    for j in range(ny):
        for i in range(cols):
            k = i + j * cols
            if j % 5 == 0:
                continue
            data[0 * cells + k] = 0.1 * i + 0.01 * j
            data[1 * cells + k] = 1 - 0.02 * j
            data[2 * cells + k] = 0.5
            data[3 * cells + k] = 0.4 if j % 7 == 0 else 1.0
    return data


def max_rel(expected, got):
    peak = float(np.abs(expected).max())
    return float(np.abs(np.asarray(expected, np.float64) - np.asarray(got, np.float64)).max()), peak

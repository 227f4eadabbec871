"""Scene setup for the projection step: MAC-grid fields, geometry, velocity
seeds and dye sources, in the reference's world coordinates.

Host-side numpy, float64, following the reference's scene helpers
(src/scenes/*.ts, src/core/grid.ts, src/core/dye.ts) operation for operation,
so the same scene rasterises to the same labels and seeds on every engine.
The domain is one unit tall (h = 1/ny, simulation.ts:365).

Field layout (grid.ts:1-36): p and label nx*ny (stride nx), u (nx+1)*ny
(stride nx+1), v nx*(ny+1) (stride nx); dye is 3 planes of dnx*dny laid end to
end. Everything is a flat 1-D array.
"""
from dataclasses import dataclass, field
import math

import numpy as np

FLUID, AIR, SOLID = 0, 1, 2  # grid.ts:41-45
DYE_CHANNELS = 3             # grid.ts:73
PATCH_PLANES = DYE_CHANNELS + 1  # dye.ts:127


@dataclass(frozen=True)
class Grid:
    """grid.ts:57-62."""

    nx: int
    ny: int
    h: float


def create_grid(nx, ny, h=None):
    return Grid(nx, ny, 1.0 / ny if h is None else h)


def dye_grid(g, dye_scale=1):
    """simulation.ts:366-367 — whole-number refinement of the velocity grid."""
    s = max(1, int(round(dye_scale)))
    return g if s == 1 else Grid(g.nx * s, g.ny * s, 1.0 / (g.ny * s))


@dataclass
class Fields:
    """grid.ts:84-116 — zero-initialised, so every cell starts Fluid."""

    p: np.ndarray
    u: np.ndarray
    v: np.ndarray
    label: np.ndarray
    dye: np.ndarray  # 3 planes end to end

    @property
    def dye_planes(self):
        n = self.dye.size // DYE_CHANNELS
        return [self.dye[c * n:(c + 1) * n] for c in range(DYE_CHANNELS)]


def create_fields(g, dg=None, dtype=np.float64):
    dg = dg or g
    return Fields(
        p=np.zeros(g.nx * g.ny, dtype),
        u=np.zeros((g.nx + 1) * g.ny, dtype),
        v=np.zeros(g.nx * (g.ny + 1), dtype),
        label=np.zeros(g.nx * g.ny, np.uint8),
        dye=np.zeros(DYE_CHANNELS * dg.nx * dg.ny, dtype),
    )


def idx_p(g, i, j):
    return i + j * g.nx


def idx_u(g, i, j):
    return i + j * (g.nx + 1)


def idx_v(g, i, j):
    return i + j * g.nx


# ------------------------------------------------------------- geometry

def all_labels(*seeds):
    """obstacles.ts:111-115."""
    def apply(g, label):
        for s in seeds:
            s(g, label)
    return apply


def solid_disk(cx, cy, r):
    """obstacles.ts:126-137 — rasterised by cell centre."""
    def apply(g, label):
        r2 = r * r
        j = np.arange(g.ny)
        i = np.arange(g.nx)
        y = (j + 0.5) * g.h
        x = (i + 0.5) * g.h
        d = (x[None, :] - cx) ** 2 + (y[:, None] - cy) ** 2
        lab = label.reshape(g.ny, g.nx)
        lab[d <= r2] = SOLID
    return apply


def solid_rect(x0, y0, x1, y1):
    """obstacles.ts:145-156 — corners in world units, by cell centre."""
    def apply(g, label):
        y = (np.arange(g.ny) + 0.5) * g.h
        x = (np.arange(g.nx) + 0.5) * g.h
        rows = (y >= y0) & (y <= y1)
        cols = (x >= x0) & (x <= x1)
        lab = label.reshape(g.ny, g.nx)
        lab[np.ix_(rows, cols)] = SOLID
    return apply


def open_right():
    """obstacles.ts:234-238 — the rightmost column becomes Air."""
    def apply(g, label):
        label.reshape(g.ny, g.nx)[:, g.nx - 1] = AIR
    return apply


def paint_solid(g, label, x0, y0, x1, y1, r):
    """obstacles.ts:178-218 — a solid capsule; only Fluid becomes Solid."""
    dx, dy = x1 - x0, y1 - y0
    len_sq = dx * dx + dy * dy
    r2 = r * r
    lo = lambda w: max(0, math.floor(w / g.h - 0.5))
    i0 = lo(min(x0, x1) - r)
    i1 = min(g.nx - 1, math.ceil((max(x0, x1) + r) / g.h - 0.5))
    j0 = lo(min(y0, y1) - r)
    j1 = min(g.ny - 1, math.ceil((max(y0, y1) + r) / g.h - 0.5))
    changed = False
    for j in range(j0, j1 + 1):
        y = (j + 0.5) * g.h
        for i in range(i0, i1 + 1):
            k = idx_p(g, i, j)
            if label[k] != FLUID:
                continue
            x = (i + 0.5) * g.h
            t = min(max(((x - x0) * dx + (y - y0) * dy) / len_sq, 0.0), 1.0) if len_sq > 0 else 0.0
            px = x0 + t * dx - x
            py = y0 + t * dy - y
            if px * px + py * py <= r2:
                label[k] = SOLID
                changed = True
    return changed


# ----------------------------------------------------------- velocity seeds

def add_curl_of_stream(g, u, v, psi, amp):
    """testFields.ts:40-54 — discrete curl of a stream function sampled at
    cell corners; divergence-free to machine precision. `psi(i, j)` takes
    integer index arrays (broadcast) and returns an array."""
    inv = amp / g.h
    J, I = np.meshgrid(np.arange(g.ny), np.arange(g.nx + 1), indexing="ij")
    u.reshape(g.ny, g.nx + 1)[:] += inv * (psi(I, J + 1) - psi(I, J))
    J, I = np.meshgrid(np.arange(g.ny + 1), np.arange(g.nx), indexing="ij")
    v.reshape(g.ny + 1, g.nx)[:] += -inv * (psi(I + 1, J) - psi(I, J))


def width_of(g):
    return g.nx * g.h


def add_rotational(g, u, v, amp=1.0):
    """testFields.ts:61-64."""
    w = width_of(g)
    add_curl_of_stream(g, u, v, lambda i, j: np.sin(math.pi * i * g.h / w) * np.sin(math.pi * j * g.h), amp)


def add_gradient(g, u, v, amp=1.0):
    """testFields.ts — pure gradient part on interior faces."""
    inv = amp / g.h
    w = width_of(g)
    phi = lambda i, j: np.cos(2 * math.pi * (i + 0.5) * g.h / w) * np.cos(2 * math.pi * (j + 0.5) * g.h)
    J, I = np.meshgrid(np.arange(g.ny), np.arange(1, g.nx), indexing="ij")
    u.reshape(g.ny, g.nx + 1)[:, 1:g.nx] += inv * (phi(I, J) - phi(I - 1, J))
    J, I = np.meshgrid(np.arange(1, g.ny), np.arange(g.nx), indexing="ij")
    v.reshape(g.ny + 1, g.nx)[1:g.ny, :] += inv * (phi(I, J) - phi(I, J - 1))


def add_vortex_pair(g, u, v, amp=1.0, sigma=0.08):
    """testFields.ts addVortexPair — counter-rotating Gaussian pair."""
    k = sigma / (math.sqrt(2) * math.exp(-0.5))
    cx = 0.5 * width_of(g)

    def psi(i, j):
        x = i * g.h
        y = j * g.h
        blob = lambda bx, by: np.exp(-((x - bx) ** 2 + (y - by) ** 2) / (sigma * sigma))
        return k * (blob(cx - 0.15, 0.3) - blob(cx + 0.15, 0.3))

    add_curl_of_stream(g, u, v, psi, amp)


def lcg(seed):
    """testFields.ts:401-408 — s = s*1664525 + 1013904223 (mod 2^32), /2^32."""
    s = [seed & 0xFFFFFFFF]

    def rand():
        s[0] = (s[0] * 1664525 + 1013904223) & 0xFFFFFFFF
        return s[0] / 4294967296.0

    return rand


def add_vortex_cluster(g, u, v, amp=1.0, count=14, sigma=0.05, seed=12345):
    """testFields.ts addVortexCluster — alternating-sign Gaussian vortices."""
    k = sigma / (math.sqrt(2) * math.exp(-0.5))
    margin = 3.5 * sigma
    span_x = width_of(g) - 2 * margin
    span_y = 1 - 2 * margin
    rand = lcg(seed)
    cx, cy, sign = [], [], []
    for n in range(count):
        cx.append(margin + rand() * span_x)
        cy.append(margin + rand() * span_y)
        sign.append(1.0 if n % 2 == 0 else -1.0)

    def psi(i, j):
        x = i * g.h
        y = j * g.h
        out = np.zeros(np.broadcast(x, y).shape)
        for n in range(count):
            dx = x - cx[n]
            dy = y - cy[n]
            out = out + sign[n] * np.exp(-(dx * dx + dy * dy) / (sigma * sigma))
        return k * out

    add_curl_of_stream(g, u, v, psi, amp)


def draught(amp=0.004):
    """plume.ts:401-421 — the one-time odd+even box-scale kick."""
    def seed(g, u, v):
        w = g.nx * g.h

        def psi(i, j):
            x = (i * g.h) / w
            across = np.sin(2 * math.pi * x) + 0.6 * np.sin(3 * math.pi * x)
            return np.sin(math.pi * j * g.h) * across

        add_curl_of_stream(g, u, v, psi, amp)
    return seed


def uniform_flow(speed):
    """karman.ts:90 — u.fill(speed)."""
    def seed(g, u, v):
        u[:] = speed
    return seed


def js_lcg_uniform(n, seed=12345):
    """The fixtures' generator (redBlack.gputest.ts:45-50,
    pressureMultigrid.test.ts:23-30): s = (s*1103515245 + 12345) & 0x7fffffff,
    value (s/0x7fffffff)*2 - 1. In JavaScript the product is a float64 that
    exceeds 2^53, so it is ROUNDED before `&` truncates it to 32 bits; this
    evaluates it the same way (Python floats are IEEE doubles) so the fixture
    values are the reference's, not those of an exact integer LCG."""
    out = np.empty(n)
    s = seed
    for k in range(n):
        s = (int(float(s) * 1103515245.0 + 12345.0) % 4294967296) & 0x7FFFFFFF
        out[k] = (s / 0x7FFFFFFF) * 2 - 1
    return out


def lcg_noise(amplitude, seed=12345):
    """Seeded uniform noise in [-amplitude, amplitude] added to every u face,
    then every v face, from js_lcg_uniform."""
    def apply(g, u, v):
        vals = js_lcg_uniform(u.size + v.size, seed)
        u += amplitude * vals[:u.size]
        v += amplitude * vals[u.size:]
    return apply


def chain_seeds(*seeds):
    def apply(g, u, v):
        for s in seeds:
            s(g, u, v)
    return apply


# ------------------------------------------------------------------- dye

def ramp(t):
    """emitters.ts:30-33 — clamped smoothstep."""
    c = min(max(t, 0.0), 1.0)
    return c * c * (3 - 2 * c)


@dataclass
class DyePatch:
    """dye.ts:118-124 — 3 value planes then 1 coverage plane, float32."""

    i0: int
    j0: int
    nx: int
    ny: int
    data: np.ndarray


def make_dye_patch(i0, j0, nx, ny, fill):
    """dye.ts:134-154. `fill(i, j, rgb)` gets global dye indices and returns
    coverage."""
    cells = nx * ny
    data = np.zeros(PATCH_PLANES * cells, np.float32)
    rgb = np.zeros(DYE_CHANNELS, np.float32)
    for j in range(ny):
        for i in range(nx):
            rgb[:] = 0
            cov = fill(i0 + i, j0 + j, rgb)
            k = i + j * nx
            for c in range(DYE_CHANNELS):
                data[c * cells + k] = rgb[c]
            data[DYE_CHANNELS * cells + k] = cov
    return DyePatch(i0, j0, nx, ny, data)


def apply_dye_patch(dg, dye, patch):
    """dye.ts:158-175 (host half)."""
    cells = patch.nx * patch.ny
    n = dg.nx * dg.ny
    for j in range(patch.ny):
        dj = patch.j0 + j
        if dj < 0 or dj >= dg.ny:
            continue
        for i in range(patch.nx):
            di = patch.i0 + i
            if di < 0 or di >= dg.nx:
                continue
            s = i + j * patch.nx
            cov = float(patch.data[DYE_CHANNELS * cells + s])
            if cov == 0:
                continue
            k = di + dj * dg.nx
            for c in range(DYE_CHANNELS):
                dye[c * n + k] += cov * (float(patch.data[c * cells + s]) - dye[c * n + k])


def in_dye_cells(cells, g, dg):
    """dye.ts:186-188."""
    return max(1, round((cells * g.h) / dg.h))


def hot_vent(centres=(0.5,), half_width=0.17, taper=0.06, height=0.03, heat=1.0, smoke=1.0):
    """plume.ts:328-368 — full-width patch, profile in the coverage plane."""
    def source(dg, g):
        width = g.nx * g.h
        depth = min(max(2, round(height / dg.h)), dg.ny)

        def fill(i, j, rgb):
            x = (i + 0.5) * dg.h
            y = (j + 0.5) * dg.h
            cover = 0.0
            for c in centres:
                d = abs(x - c * width)
                if d < half_width:
                    cover = max(cover, ramp((half_width - d) / taper))
            cover *= ramp((height - y) / height)
            if cover <= 0:
                return 0.0
            rgb[0] = heat
            rgb[1] = smoke
            return cover

        return make_dye_patch(0, 0, dg.nx, depth, fill)
    return source


def gaussian_sources(centres, sigma_cells=8.0, heat=1.0, smoke=1.0, reach=3.0):
    """Heat + smoke sources whose COVERAGE is a Gaussian of `sigma_cells`
    velocity cells about each centre (centres in world units), on one patch
    spanning every source's 3-sigma box. Channel 0 is heat, channel 1 smoke
    (plume.ts:249-251); the value planes are constant and the lerp of dye.ts
    blends them in by coverage, as hot_vent does."""
    def source(dg, g):
        sig = sigma_cells * g.h
        r = reach * sig
        xs0 = min(c[0] for c in centres) - r
        xs1 = max(c[0] for c in centres) + r
        ys0 = min(c[1] for c in centres) - r
        ys1 = max(c[1] for c in centres) + r
        i0 = max(0, int(math.floor(xs0 / dg.h)))
        i1 = min(dg.nx, int(math.ceil(xs1 / dg.h)))
        j0 = max(0, int(math.floor(ys0 / dg.h)))
        j1 = min(dg.ny, int(math.ceil(ys1 / dg.h)))
        nx, ny = i1 - i0, j1 - j0
        cells = nx * ny
        x = (np.arange(i0, i1) + 0.5) * dg.h
        y = (np.arange(j0, j1) + 0.5) * dg.h
        cov = np.zeros((ny, nx))
        for cx, cy in centres:
            d2 = (x[None, :] - cx) ** 2 + (y[:, None] - cy) ** 2
            cov = np.maximum(cov, np.exp(-d2 / (2 * sig * sig)))
        cov[cov < 1e-4] = 0.0
        data = np.zeros(PATCH_PLANES * cells, np.float32)
        on = (cov > 0).ravel()
        data[0 * cells:1 * cells][on] = heat
        data[1 * cells:2 * cells][on] = smoke
        data[3 * cells:4 * cells] = cov.ravel().astype(np.float32)
        return DyePatch(i0, j0, nx, ny, data)
    return source


def add_dye_stripes(dg, dye, period_cells=None, lines=30):
    """testFields.ts addDyeStripes/stripeAt/hueAt — horizontal bands."""
    if period_cells is None:
        period_cells = max(8, round(dg.ny / lines))
    n = dg.nx * dg.ny
    for j in range(dg.ny):
        band = 0.5 + 0.5 * math.cos((2 * math.pi * j) / period_cells)
        for c in range(DYE_CHANNELS):
            hue = 0.5 + 0.5 * math.cos(2 * math.pi * (j / dg.ny - c / DYE_CHANNELS))
            dye[c * n + j * dg.nx: c * n + (j + 1) * dg.nx] = band * band * hue


def add_dye_disk(g, dye_plane, r=0.15, cx=None, cy=0.5):
    """testFields.ts:84-100 — one-cell smoothstep edge."""
    if cx is None:
        cx = 0.5 * width_of(g)
    y = (np.arange(g.ny) + 0.5) * g.h
    x = (np.arange(g.nx) + 0.5) * g.h
    d = np.hypot(x[None, :] - cx, y[:, None] - cy)
    t = np.clip((r - d) / g.h + 0.5, 0, 1)
    dye_plane.reshape(g.ny, g.nx)[:] += t * t * (3 - 2 * t)


# ---------------------------------------------------------- scene specs

@dataclass
class SceneSpec:
    """simulation.ts:127-132."""

    labels: object = None
    seed: object = None
    dye: object = None
    dye_source: object = None
    params: dict = field(default_factory=dict)


def karman_channel(g, speed=1.0, diameter=0.14, cx=0.45):
    """karman.ts:80-96."""
    cy = 0.5 + 0.25 * g.h  # karman.ts:75-77
    return SceneSpec(labels=all_labels(open_right(), solid_disk(cx, cy, 0.5 * diameter)),
                     seed=uniform_flow(speed))


def reset_fields(g, dg, spec, dtype=np.float64):
    """simulation.ts:388-416 order: zero, labels, velocity seed, dye seed,
    commitLabels, then the dye source applied once at t = 0. Returns
    (fields, patch)."""
    f = create_fields(g, dg, np.float64)
    if spec.labels:
        spec.labels(g, f.label)
    if spec.seed:
        spec.seed(g, f.u, f.v)
    if spec.dye:
        spec.dye(dg, f.dye)
    commit_labels(g, f)
    patch = spec.dye_source(dg, g) if spec.dye_source else None
    if patch is not None:
        apply_dye_patch(dg, f.dye, patch)
    if dtype != np.float64:
        f = Fields(*(a.astype(dtype) if a.dtype != np.uint8 else a for a in (f.p, f.u, f.v, f.label, f.dye)))
    return f, patch


def commit_labels(g, f):
    """boundaries.ts:45-64 (host half): p = 0 off-fluid, dye cleared in Solid
    (indexed on the velocity grid, as the reference does), faces touching an
    in-domain solid zeroed."""
    lab = f.label
    nondfluid = lab != FLUID
    f.p[nondfluid] = 0
    solid = lab == SOLID
    n = f.dye.size // DYE_CHANNELS
    ks = np.nonzero(solid)[0]
    ks = ks[ks < n]
    for c in range(DYE_CHANNELS):
        f.dye[c * n + ks] = 0
    s2 = solid.reshape(g.ny, g.nx)
    uu = f.u.reshape(g.ny, g.nx + 1)
    left = np.zeros((g.ny, g.nx + 1), bool)
    left[:, 1:] |= s2      # cell (i-1, j) solid for face i
    left[:, :-1] |= s2     # cell (i, j) solid
    uu[left] = 0
    vv = f.v.reshape(g.ny + 1, g.nx)
    below = np.zeros((g.ny + 1, g.nx), bool)
    below[1:, :] |= s2
    below[:-1, :] |= s2
    vv[below] = 0

"""The benchmark configurations' scenes and engine parameters.

  karman(...)  vortex street: inflow u = 1 at the left wall, Air outlet
               column, cylinder of radius 0.1*ny cells at (0.25 nx, 0.5 ny),
               seeded 1e-3 noise, seeded horizontal dye stripes; MacCormack,
               CFL 0.5, red-black SOR omega 1.9 x 60 per step.
  plume(...)   thermal plume in a closed box: heat + smoke sources whose
               coverage is a Gaussian of sigma 8 cells at (0.35, 0.1) and
               (0.65, 0.1) of the box, the draught seed of src/scenes/plume.ts;
               buoyancy beta 1 (heat) and alpha 0.05 (smoke), confinement 0.3,
               MacCormack, multigrid V(3,3) to an 8x8 coarsest level inside a
               defect-correction loop whose pressure and residual are
               double-float pairs (float32 arithmetic throughout), solved to a
               relative residual of 1e-6 (float32 alone stalls near 3e-5 at
               1024^2).
  turbulence(...)  turbulence grid: inflow u = 1 at the left wall, Air outlet
               column, a 16 x 16 lattice of solid squares of side 24 cells (at
               2048^2; scaled with the grid) in the inlet's first ~40% of the
               width, seeded 1e-3 noise and dye stripes; MacCormack, CFL 0.5,
               multigrid V(3,3) to an 8x8 coarsest level inside the float64
               defect-correction loop, solved to a relative residual of 1e-8.
  random_scene(side, seed)  batched-scenes member: a closed box of the given
               side with 0-12 seeded solid discs (radius 2-10% of the side),
               a divergence-free velocity (curl of Gaussian-smoothed seeded
               noise, scaled to an RMS face speed of 0.5) and a dye blob;
               MacCormack, CFL 2, multigrid V(3,3) to 1e-6 (float32; with
               mixed=1 the float64 defect correction, which 1e-6 needs).
Scenes come from flowlab_gb300.scenes (float64 host arrays, the reference's
helpers); parameters are fl_params for the engine.
"""
from . import native, scenes as sc

# The plume fades its heat and keeps its smoke (src/scenes/catalog.ts:304).
PLUME_DECAY = (1.5, 0.1, 0.0)


def plume(n=1024, sigma_cells=8.0):
    g = sc.Grid(n, n, 1.0 / n)
    w = n * g.h
    spec = sc.SceneSpec(seed=sc.draught(), dye_source=sc.gaussian_sources(
        [(0.35 * w, 0.1), (0.65 * w, 0.1)], sigma_cells=sigma_cells))
    f, patch = sc.reset_fields(g, g, spec)
    return g, f, patch


# The coarsest level's sweep pairs: the autotuner (flowlab_gb300.autotune) on
# the 1024^2 plume with the 8x8 coarsest level measured 16 pairs fastest at the
# same V-cycle count as 32 (0.90 against 0.93 ms per step); 8 pairs needed
# more cycles.
PLUME_COARSE_SWEEPS = 16


# The plume's defect correction keeps its pressure as double-float pairs
# (mixed = 2): the configuration is float32 throughout, and the pairs'
# ~48-bit residual reaches 1e-6 with the same cycle counts as float64.
PLUME_MIXED = 2


def plume_params(tol=1e-6, max_cycles=20, mixed=PLUME_MIXED, coarse_sweeps=PLUME_COARSE_SWEEPS):
    return native.default_params(
        cfl_target=2.0, dt_max=1 / 30, scheme=native.FL_MACCORMACK, solver=native.FL_SOLVER_MG, tol=tol,
        mg_max_cycles=max_cycles, mg_pre=3, mg_post=3, mg_coarse_sweeps=coarse_sweeps, mg_coarsest=8,
        dye_decay=PLUME_DECAY, beta=1.0, alpha=0.05, confinement=0.3, mixed=mixed)


def karman(nx=128, ny=128, noise=1e-3):
    g = sc.Grid(nx, ny, 1.0 / ny)
    r = 0.1 * ny * g.h
    spec = sc.SceneSpec(
        labels=sc.all_labels(sc.open_right(), sc.solid_disk(0.25 * nx * g.h, 0.5 * ny * g.h, r)),
        seed=sc.chain_seeds(sc.uniform_flow(1.0), sc.lcg_noise(noise)),
        dye=lambda dg, dye: sc.add_dye_stripes(dg, dye))
    f, patch = sc.reset_fields(g, g, spec)
    return g, f, patch


def karman_params(iters=60, omega=1.9):
    return native.default_params(cfl_target=0.5, dt_max=1 / 30, scheme=native.FL_MACCORMACK,
                                 solver=native.FL_SOLVER_RBSOR, pressure_iters=iters, omega=omega, tol=0.0)


def turbulence_lattice(n, count=16, side_cells=24):
    """Square centres and side (cells) of the turbulence-grid lattice on an
    n x n grid: `count` rows spread evenly over the height, `count` columns
    at a pitch of twice the side starting 5% of the width from the inlet;
    the side is 24 cells at 2048^2 and scales with n (at least 2 cells)."""
    side = max(2, int(round(side_cells * n / 2048)))
    pitch_x, pitch_y = 2 * side, n / count
    x0 = 0.05 * n
    return [(x0 + (a + 0.5) * pitch_x, (b + 0.5) * pitch_y) for a in range(count) for b in range(count)], side


def turbulence(n=2048, count=16, noise=1e-3):
    g = sc.Grid(n, n, 1.0 / n)
    centres, side = turbulence_lattice(n, count)
    half = 0.5 * side * g.h
    rects = [sc.solid_rect(cx * g.h - half, cy * g.h - half, cx * g.h + half, cy * g.h + half) for cx, cy in centres]
    spec = sc.SceneSpec(
        labels=sc.all_labels(sc.open_right(), *rects),
        seed=sc.chain_seeds(sc.uniform_flow(1.0), sc.lcg_noise(noise)),
        dye=lambda dg, dye: sc.add_dye_stripes(dg, dye))
    f, patch = sc.reset_fields(g, g, spec)
    return g, f, patch


def turbulence_params(tol=1e-8, max_cycles=40, mixed=1, coarse_sweeps=32):
    return native.default_params(
        cfl_target=0.5, dt_max=1 / 30, scheme=native.FL_MACCORMACK, solver=native.FL_SOLVER_MG, tol=tol,
        mg_max_cycles=max_cycles, mg_pre=3, mg_post=3, mg_coarse_sweeps=coarse_sweeps, mg_coarsest=8, mixed=mixed)


def random_scene(side, seed):
    """A closed box of `side` cells with seeded discs, a smoothed-noise
    stream function and a dye blob (all from numpy's PCG64 seeded by `seed`)."""
    import numpy as np
    from scipy.ndimage import gaussian_filter
    from scipy.ndimage import label as connected

    rng = np.random.default_rng(seed)
    g = sc.Grid(side, side, 1.0 / side)
    # redraw the discs until the fluid is one connected region: a pocket
    # sealed off by discs and walls has no solution for a nonzero net
    # divergence, and the solve would stall there
    while True:
        discs = []
        for _ in range(int(rng.integers(0, 13))):
            r = float(rng.uniform(0.02, 0.10))
            discs.append(sc.solid_disk(float(rng.uniform(r, 1 - r)), float(rng.uniform(r, 1 - r)), r))
        lab = np.zeros(side * side, np.uint8)
        for d in discs:
            d(g, lab)
        if connected(lab.reshape(side, side) == 0)[1] <= 1:
            break
    psi = gaussian_filter(rng.standard_normal((side + 1, side + 1)), sigma=max(1.0, side / 16.0), mode="wrap")
    # zero on the box's boundary, so that no flow crosses the walls: with
    # flux through the walls the pure-Neumann pressure problem of a closed
    # box is incompatible wherever a disc touches a wall (no solution), and
    # the solve runs to its cycle cap
    window = np.sin(np.pi * np.arange(side + 1) / side)
    psi *= window[:, None] * window[None, :]

    def seed_velocity(g, u, v):
        sc.add_curl_of_stream(g, u, v, lambda i, j: psi[np.minimum(j, side), np.minimum(i, side)], 1.0)
        rms = np.sqrt(np.mean(np.concatenate([u, v]) ** 2))
        if rms > 0:
            u *= 0.5 / rms
            v *= 0.5 / rms

    cx, cy = (float(x) for x in rng.uniform(0.2, 0.8, 2))
    spec = sc.SceneSpec(labels=sc.all_labels(*discs) if discs else None, seed=seed_velocity,
                        dye=lambda dg, dye: sc.add_dye_disk(dg, dye[:dg.nx * dg.ny], r=0.1, cx=cx, cy=cy))
    f, patch = sc.reset_fields(g, g, spec)
    return g, f, patch


def random_scene_params(tol=1e-6, max_cycles=40, mixed=0):
    return native.default_params(
        cfl_target=2.0, dt_max=1 / 30, scheme=native.FL_MACCORMACK, solver=native.FL_SOLVER_MG, tol=tol,
        mg_max_cycles=max_cycles, mg_pre=3, mg_post=3, mg_coarse_sweeps=32, mg_coarsest=8, mixed=mixed)

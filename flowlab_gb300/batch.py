"""Batched uneven scenes: many independent closed-box scenes stepped together.

The batched-scene configuration holds `count` scenes whose sides are drawn
log-uniformly from 64..1024 (powers of two), each a `configs.random_scene`
(seeded discs, a divergence-free smoothed-noise velocity, a dye blob),
multigrid to 1e-6: float32 fields and smoothing, with the float64 residual
and correction (float32 alone stalls above 1e-6 on these scenes and runs
to the cycle cap). All scenes on a GPU advance together
(`fl_batch_step`): every engine's whole step, with its own device-side
V-cycle loop, is one graph launched on the engine's own stream, so small
scenes run beside large ones instead of one after another (up to
CUDA_DEVICE_MAX_CONNECTIONS hardware queues at once).

Across GPUs the scenes shard with no collective: `shard()` deals scenes to
ranks by their cost (cells), largest first, each to the least-loaded rank.
"""
import numpy as np

from . import configs, native
from .native import f32, ptr

SIDES = (64, 128, 256, 512, 1024)


def scene_sides(count=256, seed=2024):
    """Sides 2^U{6..10}, drawn with numpy's PCG64 seeded by `seed`."""
    rng = np.random.default_rng(seed)
    return [int(SIDES[k]) for k in rng.integers(0, len(SIDES), count)]


def shard(costs, world, rank):
    """Indices of the items rank `rank` of `world` owns: greedy assignment of
    items, largest cost first, to the currently least-loaded rank (ties to
    the lower rank). Every item goes to exactly one rank."""
    load = [0.0] * world
    owner = [0] * len(costs)
    for k in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += costs[k]
    return [k for k in range(len(costs)) if owner[k] == rank]


# The V-cycle cap of the batched scenes. Obstacle-rich scenes contract ~0.9
# per V-cycle in this multigrid (the float64 oracle alike); a few stall just
# above 1e-6 (measured: a cap of 100 left the same scenes there, 7.6e-6 at
# worst, and cost a third of the batch's rate).
BATCH_MAX_CYCLES = 40


def make_engines(sides, seed=2024, device=0, params=None, tol=1e-6, max_cycles=BATCH_MAX_CYCLES, mixed=1):
    """One engine per side, fields uploaded; scene k uses seed + k."""
    engines = []
    for k, n in enumerate(sides):
        g, f, patch = configs.random_scene(n, seed + k)
        prm = params or configs.random_scene_params(tol=tol, max_cycles=max_cycles, mixed=mixed)
        e = native.Engine(g.nx, g.ny, g.h, params=prm, device=device)
        e.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
               ptr(f32(f.dye)))
        engines.append(e)
    return engines


def close_all(engines):
    for e in engines:
        e.close()

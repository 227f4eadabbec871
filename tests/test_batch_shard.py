"""Sharding of the batched scenes across ranks (host logic, CPU): every
scene owned by exactly one rank, loads balanced; and the same plan computed
independently on two gloo ranks."""
import os

import pytest

from flowlab_gb300 import batch


def test_every_scene_has_one_owner_and_loads_balance():
    sides = batch.scene_sides(256, seed=2024)
    costs = [s * s for s in sides]
    for world in (1, 2, 3, 4, 8):
        owned = [batch.shard(costs, world, r) for r in range(world)]
        flat = sorted(k for o in owned for k in o)
        assert flat == list(range(len(sides)))
        loads = [sum(costs[k] for k in o) for o in owned]
        # greedy largest-first: no rank exceeds the mean by more than the largest item
        assert max(loads) - sum(loads) / world <= max(costs)


def test_sides_are_log_uniform_powers_of_two():
    sides = batch.scene_sides(2000, seed=1)
    assert set(sides) <= set(batch.SIDES)
    counts = [sides.count(s) for s in batch.SIDES]
    assert min(counts) > 300


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch

    sides = batch.scene_sides(64, seed=7)
    mine = batch.shard([s * s for s in sides], world, rank)
    t = torch.zeros(len(sides), dtype=torch.int64)
    t[mine] = 1
    dist.all_reduce(t)
    out.put((rank, t.tolist()))
    dist.destroy_process_group()


def test_two_gloo_ranks_cover_the_batch_once():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
    for _, counts in res:
        assert counts == [1] * 64


def _bench_rank_main(rank, world, port, out):
    """bench.py's own multi-rank plumbing on a gloo rank: dist_setup from the
    torchrun environment, the barrier, the max over ranks of the timed
    region and the batch workload's shard of the scenes."""
    import sys

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), LOCAL_RANK=str(rank),
                      WORLD_SIZE=str(world))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench

    w, r, local, pg = bench.dist_setup(world)
    bench.barrier(pg)
    slowest = bench.max_over_ranks(pg, 10.0 + rank)  # rank 1 is the slower one
    sides = batch.scene_sides(256, seed=2024)
    mine = batch.shard([s * s for s in sides], w, r)
    cells = float(sum(sides[k] ** 2 for k in mine))
    total = bench.max_over_ranks(pg, cells) + 0.0  # the larger share, seen by both ranks
    out.put((r, w, slowest, sorted(mine), cells, total))
    pg.destroy_process_group()


def test_bench_multi_rank_path_on_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 30500 + os.getpid() % 1000
    ps = [ctx.Process(target=_bench_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=180) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1] and all(x[1] == 2 for x in res)
    assert all(x[2] == 11.0 for x in res)  # the max over ranks of the timed region
    owned = res[0][3] + res[1][3]
    assert sorted(owned) == list(range(256))  # every scene on exactly one rank
    sides = batch.scene_sides(256, seed=2024)
    assert res[0][4] + res[1][4] == sum(s * s for s in sides)
    assert res[0][5] == res[1][5] == max(res[0][4], res[1][4])

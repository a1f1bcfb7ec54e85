"""Scene sharding for multi-GPU batching: host logic on CPU, including a
world_size-2 gloo run in which each rank derives its share independently."""

import os
import socket

import numpy as np
import pytest

from bevy_millions_ball_gb300.sharding import my_scenes, partition_by_size


def test_partition_covers_every_scene_once_and_balances():
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(1024), np.log(262144), 512)).astype(int)
    for ranks in (1, 2, 3, 8):
        parts = partition_by_size(sizes, ranks)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= int(sizes.max())  # LPT bound
    assert partition_by_size([], 4) == [[], [], [], []]
    with pytest.raises(ValueError):
        partition_by_size([1], 0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, sizes, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = my_scenes(sizes, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    load = sum(sizes[i] for i in mine)
    loads = [None] * world
    dist.all_gather_object(loads, load)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, gathered, loads))


def test_two_ranks_agree_on_disjoint_complete_shares():
    import torch.multiprocessing as mp

    sizes = [5000, 300, 120000, 7, 64000, 64000, 1, 99999, 2048, 4096]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    views = {r: g for r, g, _ in results}
    assert views[0] == views[1]  # every rank sees the same assignment
    shares = views[0]
    assert sorted(shares[0] + shares[1]) == list(range(len(sizes)))
    assert not set(shares[0]) & set(shares[1])
    loads = results[0][2]
    assert abs(loads[0] - loads[1]) <= max(sizes)

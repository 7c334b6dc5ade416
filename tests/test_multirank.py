"""Multi-rank paths on CPU with the gloo backend (world size 2): the
deterministic placement of independent trees agrees across ranks and covers
every tree once, and the bench's max / sum over ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from afivo_gb300 import placement
    import bench
    work = [float((7 * i) % 13 + 1) for i in range(40)]
    need = [int(w * 10) for w in work]
    mine = placement.shard(list(range(40)), work, rank, world, capacity=10 ** 6, need=need)
    got = [None] * world
    dist.all_gather_object(got, mine)
    mx = bench.max_over_ranks(float(rank + 1), world)
    sm = bench.sum_over_ranks(float(rank + 1), world)
    loads = [sum(work[i] for i in g) for g in got]
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got, mx, sm, loads))


def test_placement_and_reductions_gloo_world2():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, mx, sm, loads in out:
        assert mx == 2.0 and sm == 3.0
        flat = sorted(i for g in got for i in g)
        assert flat == list(range(40))            # every tree on exactly one rank
        assert max(loads) - min(loads) <= 13.0    # balanced within one item
    assert out[0][1] == out[1][1]                 # both ranks computed the same placement


def test_placement_respects_capacity():
    from afivo_gb300 import placement
    owner = placement.place([5, 4, 3, 2], 2, capacity=7, need=[5, 4, 3, 2])
    used = [0, 0]
    for i, o in enumerate(owner):
        used[o] += [5, 4, 3, 2][i]
    assert max(used) <= 7
    with pytest.raises(ValueError):
        placement.place([5, 5, 5], 2, capacity=6, need=[5, 5, 5])

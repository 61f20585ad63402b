"""Replica parallelism on CPU: two gloo ranks run the host logic of a
multi-GPU job (instance sharding, slowest-rank time, ordered gather) without
a GPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, count, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root), str(root / "itensorsgpu.jl_gb300")]
    import torch.distributed as dist
    from itg import replicas
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        assert replicas.world_rank() == (world, rank)
        mine = replicas.shard(count, world, rank)
        # per-instance "energies" stand in for the chains each rank advances
        local = [(-1.0 - 0.01 * i, i) for i in mine]
        allres = replicas.gather_in_order(local, count)
        slowest = replicas.max_over_ranks(0.5 + rank)
        q.put((rank, list(mine), allres, slowest))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("count", [256, 7])
def test_two_gloo_ranks_shard_and_gather(count):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world = 2
    procs = [ctx.Process(target=_worker, args=(r, world, port, count, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    owned = [i for _, mine, _, _ in out for i in mine]
    assert owned == list(range(count))                     # each instance once, in rank order
    assert abs(len(out[0][1]) - len(out[1][1])) <= 1
    for _, _, allres, slowest in out:
        assert [i for _, i in allres] == list(range(count))  # same ordered list on every rank
        assert slowest == 1.5                                 # the slowest rank's time


def test_shard_single_process_and_errors():
    from itg import replicas
    assert list(replicas.shard(5, 1, 0)) == [0, 1, 2, 3, 4]
    sizes = [len(replicas.shard(10, 4, r)) for r in range(4)]
    assert sizes == [3, 3, 2, 2]
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.gather_in_order([1, 2], 2) == [1, 2]

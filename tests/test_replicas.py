"""The multi-GPU path's host logic (replicas, no data exchange), on CPU:
sharding of independent lattices and the post-run reductions over a
world_size-2 gloo process group."""
import os
import socket

import pytest

from dlbc_gb300 import replicas


def test_shard_assigns_every_lattice_once_and_balances():
    sizes = [32 ** 3, 96 ** 3, 48 ** 3, 64 ** 3, 80 ** 3, 32 ** 3, 96 ** 3, 64 ** 3]
    for world in (1, 2, 3, 8, 11):
        parts = replicas.shard(sizes, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        # LPT: the most loaded rank exceeds the least by at most the largest item
        assert max(loads) - min(loads) <= max(sizes)
    assert replicas.shard([5, 5, 5, 5], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        replicas.shard([1], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mx = replicas.max_over_ranks(1.5 + rank, dist)
        got = replicas.gather_to_root({"rank": rank, "sims": replicas.shard([3, 1, 2, 2], world)[rank]}, dist)
        out.put((rank, mx, got))
    finally:
        dist.destroy_process_group()


def test_reductions_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, mx, got = q.get(timeout=120)
        res[rank] = (mx, got)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][0] == res[1][0] == 2.5
    assert res[1][1] is None
    # LPT over sizes [3, 1, 2, 2]: 3 -> rank 0, 2 -> rank 1, 2 -> rank 1, 1 -> rank 0
    assert res[0][1] == [{"rank": 0, "sims": [0, 1]}, {"rank": 1, "sims": [2, 3]}]


def test_without_process_group():
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.gather_to_root("x") == ["x"]

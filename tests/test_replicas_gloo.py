"""Multi-process replica path on CPU (gloo, world size 2): each rank gets its
own images, the only collective is the max-over-ranks time reduction."""
import os
import socket

import pytest

from akaze_gb300 import replicas


def test_shard_covers_every_item_once():
    items = list(range(17))
    parts = [replicas.shard(items, r, 4) for r in range(4)]
    assert sum(parts, []) == items
    assert max(map(len, parts)) - min(map(len, parts)) <= 1


def test_rank_seeds_are_disjoint():
    a, b = replicas.rank_seeds(0, 64), replicas.rank_seeds(1, 64)
    assert not set(a) & set(b)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        imgs = replicas.shard(list(range(10)), rank, world)
        elapsed = 1.0 + rank  # rank 1 is the slow one
        m = replicas.max_over_ranks(elapsed, dist)
        v = replicas.job_throughput(len(imgs), world, m)
        q.put((rank, imgs, m, v))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, i0, m0, v0), (r1, i1, m1, v1) = res
    assert i0 == [0, 1, 2, 3, 4] and i1 == [5, 6, 7, 8, 9]
    assert m0 == m1 == 2.0
    assert v0 == v1 == 5.0

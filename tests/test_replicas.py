"""Multi-GPU host logic (replicas) on CPU: world-size-2 gloo ranks.

The data path has no collective; these tests cover what the ranks share:
the image split, the max-over-ranks timing, the whole-job throughput and
the gather of per-rank results, plus a rank that fails before joining.
"""
import multiprocessing as mp
import os
import socket

import pytest

from partapp_gb300 import replicas


def test_image_range_partitions():
    for n in (0, 1, 5, 16, 17):
        for world in (1, 2, 3, 8):
            got = [replicas.image_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            for (a, b), (c, d) in zip(got, got[1:]):
                assert b == c
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.image_range(4, 2, 2)


def test_throughput():
    assert replicas.throughput(8, 1000.0) == pytest.approx(8.0)
    with pytest.raises(ValueError):
        replicas.throughput(1, 0.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, n_images, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        first, last = replicas.image_range(n_images, rank, world)
        ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
        ms_max = replicas.max_over_ranks(ms, dist)
        images = replicas.sum_over_ranks(last - first, dist)
        value = replicas.throughput(images, ms_max)
        got = replicas.gather_results(list(range(first, last)), dist)
        q.put((rank, ms_max, images, value, got))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, 7, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, *rest = q.get(timeout=120)
        res[rank] = rest
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ms_max, images, value, _ = res[r]
        assert ms_max == 150.0
        assert images == 7
        assert value == pytest.approx(7 / 0.15)
    assert res[0][3] == [[0, 1, 2, 3], [4, 5, 6]]
    assert res[1][3] is None


def _rank_fail(rank, world, port, q):
    import datetime

    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    if rank == 1:
        q.put((rank, "left"))
        return  # never joins the group
    try:
        dist.init_process_group("gloo", rank=rank, world_size=world,
                                timeout=datetime.timedelta(seconds=3))
        q.put((rank, "joined"))
    except Exception as e:  # the missing rank surfaces as a host-side error
        q.put((rank, type(e).__name__))


def test_missing_rank_is_a_host_error():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_fail, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
    assert got[1] == "left"
    assert got[0] != "joined"

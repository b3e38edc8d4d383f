"""The rank-sharded sampler (circuitsimulator_gb300/shard.py) on CPU ranks
(gloo, world size 2): the same answer as one process, in draw order, and a
failing rank is reported instead of hanging."""
import datetime
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from circuitsimulator_gb300 import shard


class FakeBackend:
    """Stands in for one GPU: the value of state i of stream `seed` is a fixed
    function of (seed, i), like the counter-based generator's states."""

    def __init__(self):
        self.seed, self.next = 0, 0

    def rng_position(self, seed, first):
        self.seed, self.next = seed, first

    def singleProjectorSample(self, P, L, exact, count, rng, seed):
        idx = np.arange(self.next, self.next + count)
        self.next += count
        return np.sin(idx * 0.37 + self.seed) ** 2 * 3.0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, mode, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    try:
        if mode == "fail" and rank == 1:
            raise SystemExit(3)  # a rank dies before the gather
        v = shard.sharded_multi_sampled_projector(FakeBackend(), None, None, False, 1.0, 37, 3, 11, rank, world)
        if rank == 0:
            q.put(("ok", v))
    except Exception as e:  # the surviving rank must see an error, not hang
        if rank == 0:
            q.put(("error", type(e).__name__))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(mode):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, mode, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
    alive = [p for p in procs if p.is_alive()]
    for p in alive:
        p.kill()
    assert not alive, "a rank hung"
    return q.get(timeout=5)


def test_shard_bounds_partition():
    for total in (1, 2, 7, 100):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_bounds(total, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == total
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))


def test_two_ranks_equal_one():
    one = shard.median_of_means(_single_values(37 * 3, 11), 37, 3)
    status, v = _run("ok")
    assert status == "ok"
    assert v == one


def _single_values(count, seed):
    b = FakeBackend()
    b.rng_position(seed, 0)
    return b.singleProjectorSample(None, None, False, count, 0, 0)


def test_failed_rank_is_reported():
    status, what = _run("fail")
    assert status == "error"

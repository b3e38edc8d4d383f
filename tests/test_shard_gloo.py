"""The rank-sharded estimators (circuitsimulator_gb300/shard.py) on CPU ranks
(gloo, world size 2 and 3): the same answer as one process, in draw order and
in row order, and a failing rank is reported instead of hanging.  The
reduction itself is the native one (csim_median_of_means), checked here
against the C library's own qsort with the reference's truncating comparator
(libcirc/innerprod.c:17-41)."""
import ctypes as C
import datetime
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from circuitsimulator_gb300 import backend, shard


class FakeBackend:
    """Stands in for one GPU: the value of state i of stream `seed` is a fixed
    function of (seed, i), like the counter-based generator's states; row i of
    an exact projector is a fixed function of i."""

    def __init__(self):
        self.seed, self.next = 0, 0

    def rng_position(self, seed, first):
        self.seed, self.next = seed, first

    def singleProjectorSample(self, P, L, exact, count, rng, seed):
        idx = np.arange(self.next, self.next + count)
        self.next += count
        # bin means spread by more than 1, where the truncating comparator matters
        return np.sin(idx * 0.37 + self.seed) ** 2 * 3.0 + (idx % 7) * 0.9

    def exactProjectorRows(self, P, L, exact, i0, i1):
        i = np.arange(i0, i1, dtype=np.float64)
        return np.cos(i * 0.91) * (1.0 + i % 5) * 1e-3, np.sin(i * 0.53) / (1.0 + i)

    def exactProjector(self, P, L, exact, norm):
        chi = (1 << ((P.nqubits + 1) // 2)) if exact else (1 << len(L))
        re, im = self.exactProjectorRows(P, L, exact, 0, chi)
        tr = ti = 0.0
        for a, b in zip(re, im):
            tr += float(a)
            ti += float(b)
        return float(np.sqrt(tr * tr + ti * ti))


class FakeProjector:
    def __init__(self, nstabs, nqubits):
        self.nstabs, self.nqubits = nstabs, nqubits


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
        if mode.startswith("fail") and rank == 1:
            raise SystemExit(3)  # a rank dies before the gather
        if mode.endswith("exact"):
            v = shard.sharded_exact_projector(FakeBackend(), FakeProjector(4, 21), None, True, 1.0, rank, world)
        else:
            v = shard.sharded_multi_sampled_projector(FakeBackend(), None, None, False, 1.0, 37, 5, 11, rank, world)
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


def _run(mode, world=2):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, mode, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
    alive = [p for p in procs if p.is_alive()]
    for p in alive:
        p.kill()
    assert not alive, "a rank hung"
    return q.get(timeout=5)


_CMP = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double))


def _libc_median_of_means(values, samples, bins):
    """The reference's reduction with the C library's qsort and its comparator
    (int)(a - b), called directly through ctypes."""
    libc = C.CDLL(None)
    means = []
    for b in range(bins):
        tot = 0.0
        for v in values[b * samples:(b + 1) * samples]:
            tot += float(v)
        means.append(tot / samples)
    if bins == 1:
        return means[0]
    arr = (C.c_double * bins)(*means)
    cmp = _CMP(lambda a, b: int(a[0] - b[0]))
    libc.qsort.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, _CMP]
    libc.qsort.restype = None
    libc.qsort(arr, bins, 8, cmp)
    s = list(arr)
    return s[(bins - 1) // 2] if bins % 2 == 1 else (s[bins // 2] + s[bins // 2 - 1]) / 2


def _single_values(count, seed):
    b = FakeBackend()
    b.rng_position(seed, 0)
    return b.singleProjectorSample(None, None, False, count, 0, 0)


def test_shard_bounds_partition():
    for total in (1, 2, 7, 100):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_bounds(total, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == total
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))


def test_row_bounds_partition_balances_pairs():
    for chi in (1, 2, 5, 64, 1000, 1 << 11):
        for world in (1, 2, 3, 8):
            spans = [shard.row_bounds(chi, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == chi
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            pairs = [sum(chi - i for i in range(lo, hi)) for lo, hi in spans]
            assert sum(pairs) == chi * (chi + 1) // 2
            if chi >= 64:
                assert max(pairs) - min(pairs) <= 2 * chi  # each boundary within one row of an even split


def test_native_median_is_the_libc_qsort_median():
    """Bin means spread by more than 1 (where (int)(a - b) calls unequal means
    equal and the order depends on the sort algorithm)."""
    means = [1.78, 1.18, 0.51, 1.51, 2.95]
    assert backend.median_of_means(means, 1, 5) == _libc_median_of_means(means, 1, 5)
    rs = np.random.RandomState(3)
    for bins in (2, 3, 4, 5, 7, 9, 16):
        for _ in range(20):
            v = rs.exponential(rs.choice([0.3, 1.5, 4.0]), size=3 * bins)
            assert backend.median_of_means(v, 3, bins) == _libc_median_of_means(v, 3, bins)


def test_two_ranks_equal_one():
    one = _libc_median_of_means(_single_values(37 * 5, 11), 37, 5)
    status, v = _run("ok")
    assert status == "ok"
    assert v == one


def test_three_ranks_exact_projector_equal_one():
    one = FakeBackend().exactProjector(FakeProjector(4, 21), None, True, 1.0)
    for world in (2, 3):
        status, v = _run("ok-exact", world)
        assert status == "ok"
        assert v == one


def test_failed_rank_is_reported():
    status, what = _run("fail")
    assert status == "error"


def test_failed_rank_is_reported_exact():
    status, what = _run("fail-exact")
    assert status == "error"

"""Many backend queries at once (csim_run_queries).

Batched mode shares launches between queries of different t, codes and
estimators, but every query draws from its own seed.  So each query must give
bit-identical numerator/denominator to the plain one-after-another mode, and
to itself when run alone.  The plain mode matches the reference backend
(tests/golden/e2e_cases.json.gz) within 1e-12 relative."""
import gzip
import json
import os

import numpy as np
import pytest

from circuitsimulator_gb300 import backend
from helpers import close, random_projector_rows

HERE = os.path.dirname(os.path.abspath(__file__))
pytestmark = pytest.mark.gpu


def e2e_cases():
    with gzip.open(os.path.join(HERE, "golden", "e2e_cases.json.gz"), "rt") as f:
        return json.load(f)


@pytest.fixture(scope="module")
def be():
    b = backend.Backend(0)
    yield b
    b.close()


def _key(r):
    return (r["status"], r["numerator"].hex(), r["denominator"].hex(), r["norm"].hex(), r["exact"], r["k"],
            r["noapprox"], r["pairs"])


def _cfg(t, **kw):
    cfg = dict(quiet=1, verbose=0, noapprox=0, samples=8, bins=1, t=t, k=0, exact=0, fidbound=1e-5, fidelity=0,
               rank=0, forceL=0, forceSample=1)
    cfg.update(kw)
    return cfg


def mixed_queries(seed=7, count=24):
    """Queries of several t, both decompositions, sampled and exact estimators,
    Philox and rand() draws."""
    rs = np.random.RandomState(seed)
    out = []
    for i in range(count):
        t = int(rs.choice([3, 6, 9, 12, 17, 24, 33, 40]))
        exact = int(t <= 12 and rs.randint(2))
        k = 0 if exact else int(min(t, rs.choice([2, 4, 6, 8])))
        noapprox = int(t <= 12 and rs.randint(4) == 0)
        cfg = _cfg(t, exact=exact, k=k, noapprox=noapprox, samples=int(rs.choice([4, 9, 16])),
                   bins=int(rs.choice([1, 2, 3])), forceSample=0 if noapprox else 1)
        ng = int(rs.randint(1, min(t, 8) + 1))
        g = random_projector_rows(rs, t, ng)
        h = (g[0][1:], g[1][1:], g[2][1:])  # H' drops the measured row, as probability.py's truncation does
        out.append({"cfg": cfg, "projs": [(*g, t), (*h, t)], "seed": 1000 + i,
                    "rng": backend.RNG_PHILOX if rs.randint(2) else backend.RNG_LIBC})
    return out


def test_e2e_cases_batched_equal_plain_and_reference(be):
    cases = e2e_cases()
    qs = [{"input": c["input"], "seed": c["seed"]} for c in cases]
    plain = be.run_queries(qs, batched=False)
    batched = be.run_queries(qs, batched=True)
    for c, p, b in zip(cases, plain, batched):
        assert _key(p) == _key(b), c["label"]
        num, den = float(c["ref"][-2]), float(c["ref"][-1])
        assert close(b["numerator"], num, 1e-12, 1e-12), (c["label"], b["numerator"], num)
        assert close(b["denominator"], den, 1e-12, 1e-12), (c["label"], b["denominator"], den)


def test_mixed_queries_batched_equal_plain(be):
    qs = mixed_queries()
    plain = be.run_queries(qs, batched=False)
    batched = be.run_queries(qs, batched=True)
    assert any(r["noapprox"] for r in batched) and any(not r["noapprox"] for r in batched)
    assert any(r["exact"] for r in batched) and any(not r["exact"] for r in batched)
    for i, (p, b) in enumerate(zip(plain, batched)):
        assert _key(p) == _key(b), (i, p, b)


def test_each_query_alone_equals_it_in_the_mix(be):
    qs = mixed_queries(seed=11, count=12)
    mix = be.run_queries(qs, batched=True)
    for i, q in enumerate(qs):
        alone = be.run_queries([q], batched=True)[0]
        assert _key(alone) == _key(mix[i]), i


def test_bad_query_fails_alone(be):
    qs = mixed_queries(seed=3, count=4)
    bad = dict(qs[1])
    bad["cfg"] = dict(bad["cfg"], bins=0, noapprox=0, forceSample=1)
    qs[1] = bad
    res = be.run_queries(qs, batched=True, check=False)
    assert res[1]["status"] == -1
    ok = be.run_queries([qs[0], qs[2], qs[3]], batched=True)
    assert [_key(r) for r in ok] == [_key(res[0]), _key(res[2]), _key(res[3])]


def test_empty_batch(be):
    assert be.run_queries([], batched=True) == []


def test_empty_numerator_projector_seeds_the_denominator(be):
    """G' empty, H' sampled: H' draws from the query's fresh seed in both modes
    (probability.c seeds rand() before either projector)."""
    rs = np.random.RandomState(5)
    qs = []
    for i, rng in enumerate((backend.RNG_LIBC, backend.RNG_PHILOX)):
        t = 9
        h = random_projector_rows(rs, t, 3)
        qs.append({"cfg": _cfg(t, exact=0, k=4, samples=6, bins=1), "projs": [([], [], [], t), (*h, t)],
                   "seed": 77 + i, "rng": rng})
    other = mixed_queries(seed=19, count=3)
    plain_first = be.run_queries(other + qs, batched=False)[-2:]
    plain_alone = be.run_queries(qs, batched=False)
    batched = be.run_queries(qs, batched=True)
    assert [_key(r) for r in plain_first] == [_key(r) for r in plain_alone] == [_key(r) for r in batched]


@pytest.mark.parametrize("kernel,slots", [(2, 0), (5, 0), (5, 1)])
def test_batched_pair_kernels_agree(kernel, slots):
    """The engine's block-prefix and direct-restriction launches
    (CSIM_OPT_PAIR_KERNEL 2 and 5) give bit-identical results, batched and
    plain.  With one constraint slot (CSIM_OPT_DIRECT_SLOTS 1) most states go
    on to the block-prefix kernel, so one direct bucket runs both kernels."""
    qs = mixed_queries(seed=29, count=16)
    ref_be = backend.Backend(0)
    ref_be.set_option(backend.OPT_AUTOTUNE, 0)
    ref_be.set_option(backend.OPT_PAIR_KERNEL, 2)
    b = backend.Backend(0)
    b.set_option(backend.OPT_AUTOTUNE, 0)
    b.set_option(backend.OPT_PAIR_KERNEL, kernel)
    b.set_option(backend.OPT_DIRECT_SLOTS, slots)
    try:
        ref = ref_be.run_queries(qs, batched=False)
        batched = b.run_queries(qs, batched=True)
        plain = b.run_queries(qs, batched=False)
    finally:
        ref_be.close()
        b.close()
    assert [_key(r) for r in batched] == [_key(r) for r in ref]
    assert [_key(r) for r in plain] == [_key(r) for r in ref]


def test_round_splitting_does_not_change_results():
    """Tiny rounds (many per query) give the same results as one big round."""
    qs = mixed_queries(seed=23, count=10)
    ref = backend.Backend(0).run_queries(qs, batched=True)
    srv = backend.Server(0, round_pairs=1 << 8, round_states=16)
    try:
        tickets = [srv.submit(q) for q in qs]
        res = [srv.wait(t, timeout=300) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    assert [_key(r) for r in res] == [_key(r) for r in ref]
    assert st["rounds"] > len(qs)
    assert st["completed"] == len(qs)


def test_server_mix_equals_alone_with_staggered_arrivals():
    """Queries submitted from several threads while others are on the GPU give
    the same results as each query run alone."""
    import threading
    import time

    qs = mixed_queries(seed=29, count=18)
    alone = []
    b = backend.Backend(0)
    for q in qs:
        alone.append(b.run_queries([q], batched=True)[0])
    b.close()
    srv = backend.Server(0, round_pairs=1 << 18)
    tickets = [None] * len(qs)
    try:
        def client(idx):
            for i in idx:
                tickets[i] = srv.submit(qs[i])
                time.sleep(0.002 * (i % 3))

        th = [threading.Thread(target=client, args=(list(range(j, len(qs), 3)),)) for j in range(3)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        res = [srv.wait(t, timeout=300) for t in tickets]
        for t in tickets:
            assert srv.release(t) == 0
        st = srv.stats()
    finally:
        srv.close()
    for i, (a, r) in enumerate(zip(alone, res)):
        assert _key(a) == _key(r), i
        assert r["latency_s"] > 0
    assert st["completed"] == len(qs) and st["failed"] == 0


def test_server_memory_budget_admits_in_turn():
    """A budget below two decompositions: queries wait for memory, unused
    decompositions are evicted, results are unchanged."""
    qs = [q for q in mixed_queries(seed=31, count=16) if q["cfg"]["t"] >= 17][:6]
    ref = backend.Backend(0).run_queries(qs, batched=True)
    srv = backend.Server(0, hbm_budget_bytes=1 << 16)
    try:
        tickets = [srv.submit(q) for q in qs]
        res = [srv.wait(t, timeout=300) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    assert [_key(r) for r in res] == [_key(r) for r in ref]
    assert st["resident_bytes"] <= (1 << 16) + (1 << 21)


def test_server_bad_query_fails_alone():
    qs = mixed_queries(seed=37, count=3)
    bad = dict(qs[1])
    bad["cfg"] = dict(bad["cfg"], t=70)
    srv = backend.Server(0)
    try:
        tickets = [srv.submit(q) for q in (qs[0], bad, qs[2])]
        res = [srv.wait(t, timeout=300) for t in tickets]
    finally:
        srv.close()
    assert res[1]["status"] == -1
    assert res[0]["status"] == 0 and res[2]["status"] == 0


def test_serving_daemon_equals_run_queries(be):
    """`gpubackend serve`: a stream of protocol inputs in one process gives,
    query by query, what csim_run_queries gives with the same seeds."""
    cases = e2e_cases()
    rc, out = backend.serve_backend([c["input"] for c in cases], seed=5000, timeout=300)
    assert rc == 0 and len(out) == len(cases)
    ref = be.run_queries([{"input": c["input"], "seed": 5000 + i} for i, c in enumerate(cases)], batched=True)
    for (st, num, den), r in zip(out, ref):
        assert st == 0
        assert (num, den) == (r["numerator"], r["denominator"])


def test_server_wait_timeout_and_shutdown_with_work_queued():
    """csim_wait returns PENDING on a timeout; destroying the server with work
    still queued completes every ticket (as failed) and returns."""
    qs = [q for q in mixed_queries(seed=41, count=24) if q["cfg"]["t"] >= 24][:4]
    heavy = []
    for q in qs:  # make them take a while: more samples
        h = dict(q)
        h["cfg"] = dict(q["cfg"], samples=4000, bins=1, noapprox=0, forceSample=1)
        heavy.append(h)
    srv = backend.Server(0, round_pairs=1 << 20)
    tickets = [srv.submit(q) for q in heavy]
    assert srv.wait(tickets[-1], timeout=0.0) is None
    srv.close()  # shuts down with work pending: must not hang

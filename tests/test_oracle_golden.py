"""The oracle restatement (oracle/csim_oracle.c) against the reference's own
known answers: the reference unit-test fixtures and vectors produced by the
reference's C code compiled from source (tests/golden/make_golden.py).
Everything here runs on the CPU."""
import numpy as np
import pytest

from golden.golden_io import state_from_json, states_from_json
from oracle_ffi import make_projector


def full_view(s):
    s = s.reshape(-1)[0]
    n = int(s["n"])
    return (n, int(s["k"]), int(s["Q"]), int(s["h"]), int(s["D1"]), int(s["D2"]),
            tuple(int(x) for x in s["G"][:n]), tuple(int(x) for x in s["Gbar"][:n]),
            tuple(int(x) for x in s["J"][:n]))


def test_rand_streams(oracle, golden_seeded):
    for rec in golden_seeded["rand_streams"]:
        r = oracle.rng(rec["seed"])
        assert [oracle.rand(r) for _ in range(len(rec["values"]))] == rec["values"]


def test_fixture_exponential_sum(oracle, golden_fixtures):
    for c in golden_fixtures["exponential_sum"]:
        s = state_from_json(c["in"])
        got = oracle.exponential_sum(s)
        assert list(got) == list(c["ref"])
        want = c["fixture"]
        assert got[0] == want[0] and got[1] == want[1] and got[2] % 8 == want[2] % 8
        assert full_view(s) == full_view(state_from_json(c["ref_state"]))


def test_fixture_shrink(oracle, golden_fixtures):
    for c in golden_fixtures["shrink"]:
        s = state_from_json(c["in"])
        st = oracle.shrink(s, int(c["xi"], 16), c["alpha"], 0)
        assert st == c["ref_status"] == c["fixture"]["status"]
        assert full_view(s) == full_view(state_from_json(c["ref_state"]))


def test_fixture_measure_pauli(oracle, golden_fixtures):
    for c in golden_fixtures["measure_pauli"]:
        s = state_from_json(c["in"])
        res = oracle.measure_pauli(s, c["m"], int(c["zeta"], 16), int(c["xi"], 16))
        assert res == c["ref_result"]
        assert abs(res - c["fixture"]["result"]) < 1e-4
        assert full_view(s) == full_view(state_from_json(c["ref_state"]))


def test_fixture_extend(oracle, golden_fixtures):
    for c in golden_fixtures["extend"]:
        s = state_from_json(c["in"])
        oracle.extend(s, int(c["xi"], 16))
        assert full_view(s) == full_view(state_from_json(c["ref_state"]))
        assert int(s["k"][0]) == c["fixture"]["k"]


def test_fixture_inner_product(oracle, golden_fixtures):
    for c in golden_fixtures["inner_product"]:
        got = oracle.inner_product(state_from_json(c["a"]), state_from_json(c["b"]))
        assert list(got) == list(c["ref"])


def test_random_states(oracle, golden_seeded):
    by_n = {}
    for rec in golden_seeded["random_states"]:
        by_n.setdefault(rec["n"], []).append(rec)
    for n, recs in by_n.items():
        r = oracle.rng(1000 + n)  # the stream the generator drew them from
        for rec in recs:
            s = oracle.random_state(n, r)
            assert full_view(s) == full_view(state_from_json(rec["state"]))
            rr = oracle.rng_replay(np.array(rec["words"], dtype=np.uint32))
            s2 = oracle.random_state(n, rr)
            assert full_view(s2) == full_view(s)
            assert rr.pos == len(rec["words"]) and not rr.overrun


def test_term_pairs(oracle, golden_seeded):
    for e in golden_seeded["term_pairs"]:
        t = e["t"]
        L = np.array([int(x, 16) for x in e["L"]], dtype=np.uint64)
        thetas = states_from_json(e["theta"])
        for a, th in enumerate(thetas):
            for jj, j in enumerate(e["j"]):
                assert list(oracle.inner_product(th[None], oracle.prep_l(j, t, L))) == list(e["prod_l"][a][jj])
            for jj, j in enumerate(e.get("jh", [])):
                assert list(oracle.inner_product(th[None], oracle.prep_h(j, t))) == list(e["prod_h"][a][jj])
        for jj, d in enumerate(e["phi_l"]):
            assert full_view(oracle.prep_l(e["j"][jj], t, L)) == full_view(state_from_json(d))
        for jj, d in enumerate(e.get("phi_h", [])):
            assert full_view(oracle.prep_h(e["jh"][jj], t)) == full_view(state_from_json(d))


def test_term_pairs_threaded_grid(oracle, golden_seeded):
    e = [x for x in golden_seeded["term_pairs"] if x["t"] == 24][0]
    L = np.array([int(x, 16) for x in e["L"]], dtype=np.uint64)
    thetas = states_from_json(e["theta"])
    j0, nj = min(e["j"]), max(e["j"]) - min(e["j"]) + 1
    eps, p, m = oracle.term_products(e["t"], 0, L, len(L), thetas, j0, nj, threads=4)
    for a in range(len(thetas)):
        for jj, j in enumerate(e["j"]):
            w = a * nj + (j - j0)
            assert [eps[w], p[w], m[w]] == list(e["prod_l"][a][jj])


def test_state_pairs(oracle, golden_seeded):
    for c in golden_seeded["state_pairs"]:
        got = oracle.inner_product(state_from_json(c["a"]), state_from_json(c["b"]))
        assert list(got) == list(c["ref"])


def test_estimators(oracle, golden_seeded):
    for e in golden_seeded["estimators"]:
        t, k, exact = e["t"], e["k"], e["exact"]
        pr = e["projector"]
        P = make_projector(pr["phase"], [int(x, 16) for x in pr["xs"]], [int(x, 16) for x in pr["zs"]], t)
        L = np.array([int(x, 16) for x in e["L"]], dtype=np.uint64)
        r = oracle.rng(e["seed"])
        singles = [oracle.single_projector_sample(P, L, k, exact, r) for _ in range(len(e["singles"]))]
        assert singles == e["singles"]
        r = oracle.rng(e["seed"])
        assert oracle.multi_sampled_projector(P, L, k, exact, e["norm"], e["samples"], e["bins"], r) == e["multi"]
        if e["exact_projector"] is not None:
            assert oracle.exact_projector(P, L, k, exact, e["norm"]) == e["exact_projector"]


def test_decompose(oracle, golden_seeded):
    for d in golden_seeded["decompose"]:
        e, k, norm, L = oracle.decompose(d["t"], d["fidbound"], d["rank"], d["fidelity"], d["forceL"], 0,
                                         d["k_in"], oracle.rng(1))
        assert (e, k, norm) == (d["exact"], d["k"], d["norm"])
        if d["L"] is not None:
            assert ["%x" % int(x) for x in L] == d["L"]
    assert oracle.assert_failures.value == 0

"""The front end (circuitsimulator_gb300.frontend) and the in-process
probability() / sampleQubits() (circuitsimulator_gb300.sample) against the
reference (tests/golden/frontend_cases.json.gz, written by make_frontend.py).

CPU: countY, projectors() and truncate() equal the reference's on its own
circuits and on seeded random ones, with fixed x/y strings and with seeded
numpy draws; the caller's measure dict ends up the same.
GPU: probability() and sampleQubits() equal the reference's with its C
backend on the same numpy seed and backend seed."""
import gzip
import json
import os

import numpy as np
import pytest

from circuitsimulator_gb300 import frontend
from helpers import close

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def cases():
    with gzip.open(os.path.join(HERE, "golden", "frontend_cases.json.gz"), "rt") as f:
        return json.load(f)


def _bits(mask, width):
    return "".join("1" if (mask >> i) & 1 else "0" for i in range(width))


def _as_json(P, width):
    ph, xs, zs = P[0], P[1], P[2]
    return {"phases": list(ph), "xs": [_bits(x, width) for x in xs], "zs": [_bits(z, width) for z in zs]}


def test_count_y_matches_reference(cases):
    for c in cases["count_y"]:
        t, ms, mts = frontend.count_y(c["circ"])
        assert (t, ms, mts) == (c["t"], c["Ms"], c["MTs"]), c["name"]


def test_projectors_and_truncate_match_reference(cases):
    assert len(cases["projectors"]) >= 20
    for c in cases["projectors"]:
        measure = {int(k): v for k, v in c["measure"].items()}
        rng = np.random.RandomState(c["seed"]) if c["seed"] is not None else np.random.RandomState(0)
        G, H, n, t = frontend.projectors(c["circ"], measure, rng=rng, x=c["x"], y=c["y"])
        assert (n, t) == (c["n"], c["t"]), c["name"]
        size = n + t
        assert _as_json(G, size) == c["G"], c["name"]
        assert _as_json(H, size) == c["H"], c["name"]
        Gp, u = frontend.truncate(n, G)
        Hp, v = frontend.truncate(n, H)
        assert (u, v) == (c["u"], c["v"]), c["name"]
        assert _as_json(Gp, t) == c["Gp"], c["name"]
        assert _as_json(Hp, t) == c["Hp"], c["name"]
        assert {str(k): int(x) for k, x in measure.items()} == c["measure_after"], c["name"]


def test_probability_sends_the_reference_protocol(cases):
    """The query probability() hands the backend is what the reference writes
    to its backend's stdin for the same circuit, measure, config and draws."""
    from circuitsimulator_gb300 import backend, sample

    checked = 0
    for c in cases["probability"]:
        measure = {int(k): v for k, v in c["measure"].items()}
        cfg = dict(c["config"], quiet=True, seed=1)
        gen = sample.probability_steps(c["circ"], measure, cfg, np.random.RandomState(c["seed"]))
        try:
            q = next(gen)
        except StopIteration:
            assert c["protocol"] is None, c["name"]
            continue
        except Exception:
            assert c["protocol"] is None, c["name"]
            continue
        ref_cfg, ref_projs = backend.parse_protocol(c["protocol"])
        assert q["cfg"] == ref_cfg, (c["name"], c["config"])
        for (ph, xs, zs, nq), (rph, rxs, rzs, rnq) in zip(q["projs"], ref_projs):
            assert (list(ph), list(xs), list(zs), nq) == (rph, rxs, rzs, rnq), c["name"]
        checked += 1
    assert checked >= 5


def test_bad_x_string_is_refused(cases):
    c = next(c for c in cases["projectors"] if c["x"] is not None and len(c["x"]) > 0)
    with pytest.raises(ValueError):
        frontend.projectors(c["circ"], {}, x=c["x"] + "0", y=c["y"])


@pytest.mark.gpu
def test_probability_matches_reference_backend(cases):
    from circuitsimulator_gb300 import sample

    for c in cases["probability"]:
        cfg = dict(c["config"], quiet=True, seed=c["backend_seed"])
        measure = {int(k): v for k, v in c["measure"].items()}
        want = c["value"]
        if isinstance(want, str):
            with pytest.raises(Exception):
                sample.probability(c["circ"], measure, cfg, rng=np.random.RandomState(c["seed"]))
            continue
        got = sample.probability(c["circ"], measure, cfg, rng=np.random.RandomState(c["seed"]))
        if want is None:
            assert got is None
        else:
            assert close(float(got), want, 1e-12, 1e-12), (c["name"], c["config"], got, want)


@pytest.mark.gpu
def test_sample_qubits_matches_reference_backend(cases):
    from circuitsimulator_gb300 import sample

    for c in cases["sample"]:
        cfg = dict(c["config"], quiet=True, seed=c["backend_seed"])
        out = sample.sampleQubits(c["circ"], dict(c["measure"]), list(c["sample"]), cfg,
                                  rng=np.random.RandomState(c["seed"]))
        assert out == c["output"], c["name"]


@pytest.mark.gpu
def test_sample_batch_equals_shots_alone(cases):
    from circuitsimulator_gb300 import sample

    c = next(c for c in cases["sample"] if c["name"] == "controlledT.circ")  # two queries per shot
    cfg = dict(c["config"], quiet=True, seed=c["backend_seed"])
    seeds = [11, 12, 13, 14, 15, 16]
    alone = [sample.sampleQubits(c["circ"], {}, [0, 1, 2], dict(cfg), rng=np.random.RandomState(s)) for s in seeds]
    for groups in (1, 2, 3):  # one call per step, or groups pipelined with the front ends
        stats = {}
        batch = sample.sample_qubits_batch(c["circ"], {}, [0, 1, 2], cfg, seeds, stats=stats, groups=groups)
        assert batch == alone, groups
        assert stats["steps"] >= 1 and max(stats["queries_per_step"]) >= 2
        assert stats["gpu_s"] > 0 and stats["host_s"] > 0

"""Probabilities against an FP64 state-vector simulation (tests/statevector.py)
for circuits of n <= 20 qubits.

CPU: the state vector reproduces the reference's HT-stack known answers
(circuits/HTstack.circ:1-22 comments, main.py:177-190); the c1 circuit,
regenerated from its seed, gives exactly the committed workload_c1.txt through
the front end; and the oracle's exact estimator (exactProjector on the exact
|H^t> decomposition) equals the state-vector probability to 1e-12 on small
seeded circuits.
GPU: probability() equals the state-vector value to 1e-12 with the exact
decomposition and no sampling (exactProjector), and lies within the method's
stated statistical error when it samples (L random states per projector,
sigma = sqrt((2^t-1)/(2^t+1)) mu / sqrt(L), libcirc/innerprod.py:35-41, with
Chebyshev's bound at the reference's default failure probability, 0.05 per
estimate)."""
import os
import sys

import numpy as np
import pytest

import statevector as sv
from circuitsimulator_gb300 import sample

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from circuits import compiled, random_circuit  # noqa: E402

REL = 1e-12
FAILPROB = 0.1  # Chebyshev, 0.05 for each of numerator and denominator (probability.py's default)

# circuits/HTstack.circ's comments: the probability of reading 0 after H (T H)^i
HT_COMMENTS = [0.5, 0.8536, 0.75, 0.5732, 0.9786, 0.4634, 0.9375, 0.6433, 0.6714, 0.9176]


def ht_circuit(nt):
    return "\n".join(["H"] + ["T", "H"] * nt) + "\n"


def seeded_case(n, t, nmeas, seed):
    """A seeded random circuit (compiled) and an outcome on qubits 0..nmeas-1
    drawn from its own distribution, so the probability is not tiny."""
    rs = np.random.RandomState(seed)
    circ = compiled(random_circuit(n, t, rs)[0])
    psi, _ = sv.run(circ)
    prob = np.abs(psi) ** 2
    i = int(rs.choice(len(prob), p=prob / prob.sum()))
    return circ, {q: (i >> q) & 1 for q in range(nmeas)}


def c1_case():
    """The c1 workload's circuit and outcome, regenerated exactly as
    make_workloads.py drew them (n = 10, t = 12, 3 measured qubits, seed 100,
    first attempt)."""
    rs = np.random.RandomState(100)
    circ, _ = random_circuit(10, 12, rs)
    outcome = rs.randint(2, size=3).tolist()
    return compiled(circ), {q: outcome[q] for q in range(3)}


def oracle_answer(oracle, q):
    """The backend's main (probability.c:146-216) on the oracle: decompose,
    the noapprox rule, then exactProjector or multiSampledProjector on G', H'."""
    from oracle_ffi import make_projector

    cfg = q["cfg"]
    e, k, norm, L = oracle.decompose(cfg["t"], cfg["fidbound"], cfg["rank"], cfg["fidelity"], cfg["forceL"],
                                     cfg["exact"], cfg["k"], oracle.rng(1))
    noapprox = cfg["noapprox"]
    if not noapprox and not cfg["forceSample"]:
        chi = 2 ** ((cfg["t"] + 1) // 2) if e else 2 ** k
        if cfg["samples"] * cfg["bins"] * 2 > chi - 1:
            noapprox = 1
    Ps = [make_projector(ph, xs, zs, nq) for (ph, xs, zs, nq) in q["projs"]]
    if noapprox:
        return tuple(oracle.exact_projector(P, L, k, e, norm) for P in Ps)
    r = oracle.rng(q["seed"])
    return tuple(oracle.multi_sampled_projector(P, L, k, e, norm, cfg["samples"], cfg["bins"], r) for P in Ps)


def oracle_probability(oracle, circ, measure, config, rs):
    gen = sample.probability_steps(circ, dict(measure), dict(config), rs)
    try:
        q = next(gen)
        gen.send(oracle_answer(oracle, q))
    except StopIteration as stop:
        return stop.value
    raise AssertionError("more than one backend query")


# ---------------------------------------------------------------- CPU
def test_state_vector_ht_stack_known_answers():
    for nt, want in enumerate(HT_COMMENTS):
        p = sv.probability(ht_circuit(nt), {0: 0})
        assert abs(p - sv.ht_stack(nt)) < 1e-14, nt
        assert abs(p - want) < 6e-5, (nt, p, want)


def test_state_vector_gates():
    """One qubit per gate rule: S|+> phases, CNOT copies, M-controlled lines act
    only where the measured qubit is 1."""
    assert abs(sv.probability("H\nS\nH\n", {0: 0}) - 0.5) < 1e-15
    assert abs(sv.probability("X_\nCX\n", {1: 1}) - 1.0) < 1e-15
    assert abs(sv.probability("H_\nCX\n", {0: 1, 1: 0})) < 1e-15
    # X on qubit 1 conditioned on measured qubit 0 (in state |+>): copies it
    assert abs(sv.probability("H_\nMX\n", {0: 1, 1: 1}) - 0.5) < 1e-15
    assert abs(sv.probability("H_\nMX\n", {0: 0, 1: 1})) < 1e-15


def test_c1_circuit_gives_the_committed_workload():
    """The regenerated c1 circuit, through the front end with the numpy seed
    make_workloads.py used, sends exactly workload_c1.txt to the backend."""
    from circuitsimulator_gb300 import backend

    circ, measure = c1_case()
    cfg = {"exact": True, "samples": 2000, "bins": 1, "forceSample": True, "quiet": True, "seed": 1}
    q = next(sample.probability_steps(circ, dict(measure), cfg, np.random.RandomState(100)))
    ref_cfg, ref_projs = backend.parse_protocol(open(os.path.join(HERE, "golden", "workload_c1.txt")).read())
    assert q["cfg"] == ref_cfg
    for a, b in zip(q["projs"], ref_projs):
        assert (list(a[0]), list(a[1]), list(a[2]), a[3]) == b


@pytest.mark.parametrize("n,t,nmeas,seed", [(3, 3, 1, 1), (4, 5, 2, 2), (5, 6, 2, 3), (6, 7, 3, 4), (7, 8, 3, 5),
                                             (8, 8, 2, 6)])
def test_oracle_exact_estimator_equals_state_vector(oracle, n, t, nmeas, seed):
    circ, measure = seeded_case(n, t, nmeas, seed)
    want = sv.probability(circ, measure)
    got = oracle_probability(oracle, circ, measure, {"exact": True, "noapprox": True, "quiet": True, "seed": 1},
                             np.random.RandomState(seed))
    assert abs(got - want) <= REL * want + 1e-15, (got, want)


# ---------------------------------------------------------------- GPU
GPU_CASES = [("c1",) + c1_case()] + [("n%d_t%d" % (n, t),) + seeded_case(n, t, m, s)
                                      for (n, t, m, s) in ((12, 10, 3, 11), (16, 14, 4, 12), (20, 16, 3, 13))]


@pytest.mark.gpu
@pytest.mark.parametrize("name,circ,measure", GPU_CASES, ids=[c[0] for c in GPU_CASES])
def test_gpu_exact_probability_equals_state_vector(name, circ, measure):
    want = sv.probability(circ, measure)
    got = sample.probability(circ, dict(measure), {"exact": True, "noapprox": True, "quiet": True, "seed": 3},
                             rng=np.random.RandomState(5))
    assert abs(got - want) <= REL * want + 1e-15, (got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("name,circ,measure", GPU_CASES, ids=[c[0] for c in GPU_CASES])
def test_gpu_sampled_probability_within_stated_error(name, circ, measure):
    """L = 2000 states per projector (the reference's default), forceSample, for
    three backend seeds: each estimate within the stated error of the exact
    probability."""
    want = sv.probability(circ, measure)
    t = sum(1 for ln in circ.splitlines() if "T" in ln)
    bound = sv.ratio_bound(t, 2000, FAILPROB)
    for seed in (1, 2, 3):
        got = sample.probability(circ, dict(measure), {"exact": True, "samples": 2000, "bins": 1,
                                                       "forceSample": True, "quiet": True, "seed": seed},
                                 rng=np.random.RandomState(7 + seed))
        assert abs(got - want) <= bound * want, (seed, got, want, bound)

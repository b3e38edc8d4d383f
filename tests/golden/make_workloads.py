"""Generates the benchmark workloads and end-to-end golden outputs.

Run where the reference checkout exists (its Python front end compiles the
circuits; its C backend, built by ``make -C oracle ref REF=<checkout>``, gives
the reference outputs):

    python tests/golden/make_workloads.py REFERENCE_ROOT [--c1-golden-only]

(or set CSIM_REFERENCE instead of passing REFERENCE_ROOT).  With
--c1-golden-only the committed workloads are kept and only workload_c1_ref.json
is recorded.

Outputs (committed):
  workload_c1.txt  stdin-protocol input of the c1 configuration: seeded random
                   Clifford+T circuit on n=10 qubits with exactly t=12 T/T^dagger
                   gates, probability of a fixed random 3-bit outcome on qubits
                   0..2; exact decomposition (chi = 2^6), L = 2000, forceSample.
  workload_c2.txt  c2: n=24, t=40, 8 measured qubits; k=16 code (fidelity bound
                   0.01), L = 4096.
  workload_c1_ref.json  the reference backend's output lines on workload_c1.txt
                   for fixed seeds (CSIM_REF_SEED): the whole c1 query, 2000
                   states per projector.
  e2e_cases.json.gz  small protocol inputs with the reference backend's output
                   lines for fixed seeds (CSIM_REF_SEED), used by the
                   end-to-end tests of gpubackend.

Gate mix (per drawn gate): H/S/X/Z with probability 0.55, CNOT on a random
ordered pair 0.30, T or T^dagger 0.15 (T^dagger = S S S T, Z = H X H... written
inline since the base gate set is H, X, S, T, CX).
"""
import gzip
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
_ARGS = [a for a in sys.argv[1:] if not a.startswith("--")]
REFROOT = _ARGS[0] if _ARGS else os.environ.get("CSIM_REFERENCE", "")
if not REFROOT or not os.path.isdir(os.path.join(REFROOT, "libcirc")):
    sys.exit("usage: make_workloads.py REFERENCE_ROOT (the reference checkout; or set CSIM_REFERENCE)")
REFBACKEND = os.path.join(ROOT, "oracle", "_ref", "refbackend")
sys.path.insert(0, HERE)
from circuits import random_circuit  # noqa: E402
sys.path.insert(0, REFROOT)


def protocol_input(circ, measure, config, seed):
    """The stdin text libcirc/probability.py writes for this query (config['file'])."""
    import libcirc.compile.compilecirc as compilecirc
    from libcirc.probability import probability

    np.random.seed(seed)  # the front end's random postselection (projectors.py:29-64)
    path = os.path.join(HERE, "_tmp_proto.txt")
    if os.path.exists(path):
        os.remove(path)
    cfg = dict(config)
    cfg["file"] = path
    cfg["quiet"] = True
    compiled = compilecirc.compileCircuit(raw=circ)
    probability(compiled, dict(measure), cfg)
    if not os.path.exists(path):
        return None
    text = open(path).read()
    os.remove(path)
    return text


def make_workload(name, n, t, nmeas, config, seed):
    rs = np.random.RandomState(seed)
    for attempt in range(200):
        circ, gates = random_circuit(n, t, rs)
        outcome = rs.randint(2, size=nmeas).tolist()
        measure = {q: outcome[q] for q in range(nmeas)}
        try:
            text = protocol_input(circ, measure, config, seed + attempt)
        except Exception:
            text = None
        if text is None:
            continue
        lines = text.split()
        if int(lines[5]) != t or int(lines[13]) == 0 or int(lines[13]) == 0:
            continue
        with open(os.path.join(HERE, name), "w") as f:
            f.write(text)
        meta = {"n": n, "t": t, "measured": nmeas, "outcome": outcome, "gates": gates, "seed": seed,
                "attempt": attempt, "config": config}
        print(name, meta)
        return meta
    raise RuntimeError("no usable circuit")


def run_ref(text, seed):
    env = dict(os.environ, CSIM_REF_SEED=str(seed))
    r = subprocess.run([REFBACKEND, "stdin"], input=text.encode(), stdout=subprocess.PIPE, env=env, check=True)
    return r.stdout.decode().splitlines()


def e2e_cases():
    import libcirc.compile.compilecirc as compilecirc  # noqa: F401

    cases = []
    ht = open(os.path.join(REFROOT, "circuits", "HTstack.circ")).read()
    # HTstack with the block comment holding T gates 5..9 in place; measured qubit 0 -> 0
    for (label, config, seed) in (
        ("HT4 exact terms, noapprox", {"exact": True, "noapprox": True}, 1),
        ("HT4 exact terms, sampled", {"exact": True, "samples": 40, "forceSample": True}, 2),
        ("HT4 L code k=2, sampled", {"exact": False, "k": 2, "samples": 30, "forceSample": True}, 3),
        ("HT4 L code k=2, bins=3", {"exact": False, "k": 2, "samples": 10, "bins": 3, "forceSample": True}, 4),
    ):
        text = protocol_input(ht, {0: 0}, config, seed)
        cases.append({"label": label, "input": text, "seed": 1000 + seed, "ref": run_ref(text, 1000 + seed)})
    rs = np.random.RandomState(77)
    for (n, t, nm, config, seed) in ((6, 6, 2, {"exact": True, "samples": 25, "forceSample": True}, 5),
                                     (6, 7, 2, {"exact": False, "k": 3, "samples": 20, "forceSample": True}, 6),
                                     (8, 9, 3, {"exact": True, "noapprox": True}, 7),
                                     (8, 10, 3, {"exact": False, "k": 4, "noapprox": True}, 8),
                                     (7, 8, 2, {"exact": False, "k": 3, "samples": 12, "bins": 2,
                                                "forceSample": True, "fidelity": True}, 9)):
        for attempt in range(100):
            circ, _ = random_circuit(n, t, rs)
            outcome = rs.randint(2, size=nm).tolist()
            try:
                text = protocol_input(circ, {q: outcome[q] for q in range(nm)}, config, seed * 100 + attempt)
            except Exception:
                text = None
            if text is None or int(text.split()[13]) == 0:
                continue
            cases.append({"label": "random n=%d t=%d %s" % (n, t, config), "input": text, "seed": 2000 + seed,
                          "ref": run_ref(text, 2000 + seed)})
            break
    with gzip.open(os.path.join(HERE, "e2e_cases.json.gz"), "wt") as f:
        json.dump(cases, f)
    print("e2e cases:", len(cases))


C1_SEEDS = (1, 4242)


def c1_golden():
    """The reference backend on the committed c1 workload, in full (exact
    decomposition chi = 2^6, 2000 states per projector, forceSample), for
    fixed seeds."""
    text = open(os.path.join(HERE, "workload_c1.txt")).read()
    out = []
    for seed in C1_SEEDS:
        lines = run_ref(text, seed)
        out.append({"seed": seed, "ref": lines})
        print("c1 seed", seed, lines[-2:])
    with open(os.path.join(HERE, "workload_c1_ref.json"), "w") as f:
        json.dump(out, f, indent=1)


def main():
    if "--c1-golden-only" in sys.argv:
        c1_golden()
        return
    metas = {}
    metas["c1"] = make_workload("workload_c1.txt", 10, 12, 3,
                                {"exact": True, "samples": 2000, "bins": 1, "forceSample": True}, 100)
    metas["c2"] = make_workload("workload_c2.txt", 24, 40, 8,
                                {"exact": False, "k": 16, "fidbound": 0.01, "samples": 4096, "bins": 1}, 200)
    with open(os.path.join(HERE, "workloads.json"), "w") as f:
        json.dump(metas, f, indent=1)
    e2e_cases()
    c1_golden()


if __name__ == "__main__":
    main()

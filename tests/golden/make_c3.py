"""Generates the batched-query workload: 256 independent probability queries.

Run here, where the reference checkout exists (its Python front end compiles
each circuit and writes the backend's stdin input):

    python tests/golden/make_c3.py [REFERENCE_ROOT]

Per query (seeded, numpy RandomState(300)):
  n ~ uniform[8, 32] qubits, t ~ uniform[8, 60] T/T^dagger gates, gate mix as in
  make_workloads.py; 1..4 measured qubits with a random outcome.
  Decomposition: exact (prepH, chi = 2^ceil(t/2)) when t <= 16, else |L> with k
  from the fidelity bound 0.02 (libcirc/probability.c:330), capped at 18, sent
  as k so chi stays within 2^4..2^18.
  Samples from the relative error 0.05 and failure probability 0.05 through the
  reference's own rule (libcirc/probability.py:150-167): L = 8000, bins = 1.
  forceSample is off, so the backend picks exactProjector where 2 L > chi - 1
  (libcirc/probability.c:162-174), as it would for these inputs.

Output (committed): workload_c3.json.gz, a list of {"input", "seed", "n", "t",
"measured"} records.
"""
import gzip
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_workloads as mw  # noqa: E402  (puts the reference on sys.path)

COUNT = 256
ERROR = 0.05
FAILPROB = 0.05
FIDBOUND = 0.02
KMAX = 18


def k_for(t):
    return min(KMAX, int(math.ceil(1 - 2 * t * math.log2(math.cos(math.pi / 8)) - math.log2(FIDBOUND))))


def main():
    rs = np.random.RandomState(300)
    out = []
    while len(out) < COUNT:
        n = int(rs.randint(8, 33))
        t = int(rs.randint(8, 61))
        nm = int(rs.randint(1, 5))
        if t <= 16:
            config = {"exact": True}
        else:
            config = {"exact": False, "k": k_for(t), "fidbound": FIDBOUND}
        config.update({"error": ERROR, "failprob": FAILPROB})
        for attempt in range(50):
            circ, _ = mw.random_circuit(n, t, rs)
            qubits = sorted(rs.choice(n, size=nm, replace=False).tolist())
            outcome = rs.randint(2, size=nm).tolist()
            seed = 300000 + 100 * len(out) + attempt
            try:
                text = mw.protocol_input(circ, {q: b for q, b in zip(qubits, outcome)}, dict(config), seed)
            except Exception:
                text = None
            if text is None or int(text.split()[5]) != t:
                continue
            out.append({"input": text, "seed": 5000 + len(out), "n": n, "t": t, "measured": nm})
            break
        print(len(out), n, t, flush=True)
    with gzip.open(os.path.join(HERE, "workload_c3.json.gz"), "wt") as f:
        json.dump(out, f)


if __name__ == "__main__":
    main()

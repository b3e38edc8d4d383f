"""Times the front end (projectors() + truncate() of G' and H') against the
reference's own Python on the same compiled circuits.

Run here, where the reference checkout exists:

    python tests/golden/time_frontend.py [REFERENCE_ROOT]

Circuits: seeded random Clifford+T (make_workloads.random_circuit, numpy seed 7)
at the c1, c2 and c4 shapes, compiled by the reference's compileCircuit, with
the first min(8, n) qubits measured as 0.  Prints the mean time per call of
each implementation (fresh numpy draws each call)."""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import make_workloads as mw  # noqa: E402  (puts the reference on sys.path)


def main():
    import libcirc.compile.compilecirc as cc
    import libcirc.compile.projectors as pj

    from circuitsimulator_gb300 import frontend

    for n, t in ((10, 12), (24, 40), (40, 64)):
        raw, _ = mw.random_circuit(n, t, np.random.RandomState(7))
        circ = cc.compileCircuit(raw=raw)
        meas = {q: 0 for q in range(min(8, n))}
        reps = 20
        t0 = time.perf_counter()
        for r in range(reps):
            G, H, nn, _ = frontend.projectors(circ, dict(meas), rng=np.random.RandomState(r))
            frontend.truncate(nn, G)
            frontend.truncate(nn, H)
        ours = (time.perf_counter() - t0) / reps
        reps_ref = 3
        t0 = time.perf_counter()
        for r in range(reps_ref):
            np.random.seed(r)
            G, H, nn, _ = pj.projectors(circ, dict(meas))
            pj.truncate(nn, G)
            pj.truncate(nn, H)
        ref = (time.perf_counter() - t0) / reps_ref
        print("n=%d t=%d (%d circuit lines): frontend %.2f ms, reference %.1f ms per projectors() + truncate()"
              % (n, t, len(circ.splitlines()), ours * 1e3, ref * 1e3), flush=True)


if __name__ == "__main__":
    main()

"""Generates the sampleQubits-chain workload: a seeded random Clifford+T
circuit with n = 32 qubits and t = 64 T/T^dagger gates (gate mix of
make_workloads.py), compiled by the reference's own compileCircuit.

    python tests/golden/make_c4.py [REFERENCE_ROOT]

Output (committed): workload_c4.json = {"n", "t", "seed", "circ" (compiled),
"sample" (the 16 sampled qubits), "config"}.  The chain samples 16 output
qubits with a k = 14 code (chi = 2^14) and L = 2048 states per conditional
probability.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_workloads as mw  # noqa: E402  (puts the reference on sys.path)


def main():
    import libcirc.compile.compilecirc as cc

    rs = np.random.RandomState(400)
    raw, gates = mw.random_circuit(32, 64, rs)
    circ = cc.compileCircuit(raw=raw)
    out = {"n": 32, "t": 64, "seed": 400, "gates": gates, "circ": circ, "sample": list(range(16)),
           "config": {"exact": False, "k": 14, "samples": 2048, "bins": 1, "forceSample": True, "quiet": True}}
    with open(os.path.join(HERE, "workload_c4.json"), "w") as f:
        json.dump(out, f)
    print(len(circ.splitlines()), "lines")


if __name__ == "__main__":
    main()

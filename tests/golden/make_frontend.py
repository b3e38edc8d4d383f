"""Generates the front-end and sampling fixtures from the reference.

Run here, where the reference checkout and its compiled backend exist:

    make -C oracle ref
    python tests/golden/make_frontend.py [REFERENCE_ROOT]

Outputs (committed) frontend_cases.json.gz:
  "projectors": compiled circuits (the reference's circuits/*.circ through its
      own compileCircuit, plus seeded random Clifford+T circuits), a measure
      dict, and either fixed x/y strings or a numpy seed.  Each case holds the
      reference's projectors() and truncate() outputs (phases, x and z rows as
      0/1 strings) and the measure dict after the call.
  "count_y": countY of each circuit.
  "probability": probability() of the reference with its C backend
      (oracle/_ref/refbackend, process id fixed by CSIM_REF_SEED) after
      np.random.seed(seed), and the stdin text it sends (config["file"]).
  "sample": sampleQubits() of the reference the same way.
"""
import gzip
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_workloads as mw  # noqa: E402  (puts the reference on sys.path)

REFBACKEND = mw.REFBACKEND
CIRCUITS = ["controlledT.circ", "toffoli.circ", "phaseEstimation.circ", "HTstack.circ"]


def bits(row):
    return "".join(str(int(v) % 2) for v in row)


def proj_json(P):
    ph, xs, zs = P[0], P[1], P[2]
    return {"phases": [int(p) for p in ph], "xs": [bits(x) for x in xs], "zs": [bits(z) for z in zs]}


def compiled_circuits():
    import libcirc.compile.compilecirc as cc

    out = []
    for name in CIRCUITS:
        out.append((name, cc.compileCircuit(fname=os.path.join(mw.REFROOT, "circuits", name))))
    rs = np.random.RandomState(900)
    for i, (n, t) in enumerate(((4, 3), (6, 5), (8, 9), (10, 12), (12, 16))):
        raw, _ = mw.random_circuit(n, t, rs)
        out.append(("random n=%d t=%d" % (n, t), cc.compileCircuit(raw=raw)))
    return out


def main():
    import libcirc.compile.gadgetize as gz
    import libcirc.compile.projectors as pj
    from libcirc.probability import probability
    from libcirc.sample import sampleQubits

    circs = compiled_circuits()
    rs = np.random.RandomState(901)
    cases, county = [], []
    for name, circ in circs:
        t, Ms, MTs = gz.countY(circ)
        county.append({"name": name, "circ": circ, "t": t, "Ms": list(Ms), "MTs": list(MTs)})
        n = len(circ.splitlines()[0])
        for rep in range(3):
            nm = int(rs.randint(1, min(3, n) + 1))
            qubits = [int(q) for q in rs.choice(n, size=nm, replace=False) if q not in Ms]
            measure = {q: int(rs.randint(2)) for q in qubits}
            if rep == 0:
                x = "".join(str(int(b)) for b in rs.randint(2, size=len(Ms)))
                tt = t + sum(1 for M in MTs if x[Ms.index(M)] == "1")
                y = "".join(str(int(b)) for b in rs.randint(2, size=tt))
                seed = None
            else:
                x = y = None
                seed = int(rs.randint(1 << 30))
                np.random.seed(seed)
            m_in = dict(measure)
            G, H, nn, tt = pj.projectors(circ, measure, x=x, y=y)
            Gp, u = pj.truncate(nn, G)
            Hp, v = pj.truncate(nn, H)
            cases.append({"name": name, "circ": circ, "measure": {str(k): v_ for k, v_ in m_in.items()},
                          "x": x, "y": y, "seed": seed, "n": nn, "t": tt,
                          "G": proj_json(G), "H": proj_json(H), "Gp": proj_json(Gp), "Hp": proj_json(Hp),
                          "u": int(u), "v": int(v),
                          "measure_after": {str(k): int(v_) for k, v_ in measure.items()}})
    # probability() and sampleQubits() with the reference backend
    os.environ["CSIM_REF_SEED"] = "4242"
    base = {"cpath": REFBACKEND, "mpirun": "", "quiet": True}
    probs, samples = [], []
    small = [c for c in circs if c[0] in ("controlledT.circ", "HTstack.circ") or c[0].startswith("random n=4")
             or c[0].startswith("random n=6") or c[0].startswith("random n=8")]
    for name, circ in small:
        n = len(circ.splitlines()[0])
        t = gz.countY(circ)[0]
        for cfg_extra in ({"exact": True, "samples": 60, "forceSample": True},
                          {"exact": False, "k": max(1, min(t, 4)), "samples": 50, "forceSample": True},
                          {"exact": True, "noapprox": True}):
            if t > 16 and cfg_extra.get("noapprox"):
                continue
            seed = int(rs.randint(1 << 30))
            measure = {0: int(rs.randint(2))}
            cfg = dict(base, **cfg_extra)
            # the stdin text the reference would send (config["file"]), same draws
            path = os.path.join(HERE, "_tmp_frontend_proto.txt")
            np.random.seed(seed)
            try:
                probability(circ, dict(measure), dict(cfg, file=path))
                proto = open(path).read() if os.path.exists(path) else None
            except Exception:
                proto = None
            if os.path.exists(path):
                os.remove(path)
            np.random.seed(seed)
            try:
                p = probability(circ, dict(measure), dict(cfg))
            except Exception as e:  # the reference fails on some inputs; keep the failure
                p = "error: %s" % type(e).__name__
            probs.append({"name": name, "circ": circ, "measure": {str(k): v_ for k, v_ in measure.items()},
                          "config": cfg_extra, "seed": seed, "backend_seed": 4242, "protocol": proto,
                          "value": p if isinstance(p, str) or p is None else float(p)})
        if n >= 3:
            seed = int(rs.randint(1 << 30))
            cfg = dict(base, exact=True, samples=40, forceSample=True)
            np.random.seed(seed)
            out = sampleQubits(circ, {}, [0, 1, 2], dict(cfg))
            samples.append({"name": name, "circ": circ, "sample": [0, 1, 2], "measure": {},
                            "config": {"exact": True, "samples": 40, "forceSample": True}, "seed": seed,
                            "backend_seed": 4242, "output": out})
        print(name, len(probs), len(samples), flush=True)
    with gzip.open(os.path.join(HERE, "frontend_cases.json.gz"), "wt") as f:
        json.dump({"projectors": cases, "count_y": county, "probability": probs, "sample": samples}, f)


if __name__ == "__main__":
    main()

"""Measures the roofline work unit of the pair kernel: packed 64-bit row
operations per (theta, term) pair of the elementary-update algorithm, on the
c2 workload (tests/golden/workload_c2.txt: t = 40, k = 16 code).

States are drawn and projected exactly as the reference does (oracle
restatement, srand(seed) stream); terms are sampled uniformly from the 2^16
codewords.  Every counted pair is also checked against the dense restatement
(orc_inner_product_exact), so the count belongs to a correct run.

    python oracle/rowops.py [nstates] [terms_per_state]

Prints one JSON line; the figure is copied into bench.py (ROWOPS_PER_PAIR_T40)
and profiles/rowops_c2.md.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from bench import parse_protocol  # noqa: E402
from oracle_ffi import Oracle, make_projector  # noqa: E402


def main():
    nstates = int(sys.argv[1]) if len(sys.argv) > 1 else 24
    nterms = int(sys.argv[2]) if len(sys.argv) > 2 else 400
    O = Oracle()
    cfg, projs = parse_protocol(open(os.path.join(ROOT, "tests", "golden", "workload_c2.txt")).read())
    t = cfg["t"]
    exact, k, norm, L = O.decompose(t, cfg["fidbound"], cfg["rank"], cfg["fidelity"], cfg["forceL"], cfg["exact"],
                                    cfg["k"], O.rng(1))
    rs = np.random.RandomState(3)
    r = O.rng(2024)
    ops, orth, pairs, per_proj = [], 0, 0, {}
    for pi, (ph, xs, zs, nq) in enumerate(projs):
        P = make_projector(ph, xs, zs, nq)
        got = 0
        while got < nstates // 2:
            s = O.random_state(t, r)
            if O.project(s, P) == 0:
                continue
            got += 1
            for j in rs.randint(0, 2 ** k, size=nterms):
                x = O.codeword(int(j), L)
                res, n_ops = O.pair_rowops(s, x)
                ref = O.inner_product(s, O.prep_l(int(j), t, L))
                assert tuple(res) == tuple(ref), (res, ref)
                ops.append(n_ops)
                orth += res[0] == 0
                pairs += 1
        per_proj[pi] = float(np.mean(ops[-(nstates // 2) * nterms:]))
    out = {"workload": "c2 (t=40, k=16)", "pairs": pairs, "rowops_per_pair": float(np.mean(ops)),
           "rowops_p50": float(np.median(ops)), "rowops_p95": float(np.percentile(ops, 95)),
           "orthogonal_fraction": orth / pairs, "per_projector": per_proj}
    print(json.dumps(out))


if __name__ == "__main__":
    main()

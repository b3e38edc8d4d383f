"""Measures the roofline work unit of the pair kernel: packed 64-bit row
operations per (theta, term) pair of the elementary-update algorithm, on the
c2 workload (tests/golden/workload_c2.txt: t = 40, k = 16 code).

States are drawn and projected exactly as the reference does (oracle
restatement, srand(seed) stream); terms are sampled uniformly from the 2^16
codewords.  Every counted pair is also checked against the dense restatement
(orc_inner_product_exact), so the count belongs to a correct run.

    python oracle/rowops.py [nstates] [terms_per_state]

The same pairs are also run through the direct-restriction path
(csim_pair_core.cuh's canon_theta and pair_direct, compiled for the host from
tests/native/tp_host_check.cpp), which counts the rows of J and constraint
masks it reads, copies or updates per pair (CSIM_COUNT_ROWS): the work unit of
the direct kernel.  Its (eps, p, m mod 8) are checked against the oracle too.

Prints one JSON line; the figures are copied into bench.py (ROWOPS_PER_PAIR_T40,
DIRECT_ROWS_PER_PAIR_T40) and profiles/rowops_c2.md.
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from bench import parse_protocol  # noqa: E402
from oracle_ffi import Oracle, make_projector  # noqa: E402


def direct_counter():
    """The host build of the pair core with its row counter."""
    src = os.path.join(ROOT, "tests", "native", "tp_host_check.cpp")
    so = os.path.join(ROOT, "tests", "native", "_build", "libtphost_rows.so")
    os.makedirs(os.path.dirname(so), exist_ok=True)
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-o", so])
    lib = C.CDLL(so)
    lib.tp_host_direct.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.tp_host_direct.restype = C.c_int
    lib.tp_host_rows_take.restype = C.c_int64
    return lib


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
    dlib = direct_counter()
    dlib.tp_host_rows_take()
    ops, orth, pairs, per_proj, drows = [], 0, 0, {}, []
    for pi, (ph, xs, zs, nq) in enumerate(projs):
        P = make_projector(ph, xs, zs, nq)
        got = 0
        while got < nstates // 2:
            s = O.random_state(t, r)
            if O.project(s, P) == 0:
                continue
            got += 1
            refs, xs = [], []
            for j in rs.randint(0, 2 ** k, size=nterms):
                x = O.codeword(int(j), L)
                res, n_ops = O.pair_rowops(s, x)
                ref = O.inner_product(s, O.prep_l(int(j), t, L))
                assert tuple(res) == tuple(ref), (res, ref)
                ops.append(n_ops)
                orth += res[0] == 0
                pairs += 1
                refs.append(ref)
                xs.append(x)
            xa = np.array(xs, dtype=np.uint64)
            e, p, m = (np.zeros(len(xs), dtype=np.int32) for _ in range(3))
            for i in range(len(xs)):  # one pair at a time, so each count is one pair's
                assert dlib.tp_host_direct(s.ctypes.data, 1, xa[i:].ctypes.data, 1, e[i:].ctypes.data,
                                           p[i:].ctypes.data, m[i:].ctypes.data) == 0
                drows.append(dlib.tp_host_rows_take())
            for i, ref in enumerate(refs):
                assert (e[i], p[i] if e[i] else 0, (m[i] - ref[2]) % 8 if e[i] else 0) == \
                    (ref[0], ref[1] if ref[0] else 0, 0), (i, e[i], p[i], m[i], ref)
        per_proj[pi] = float(np.mean(ops[-(nstates // 2) * nterms:]))
    out = {"workload": "c2 (t=40, k=16)", "pairs": pairs, "rowops_per_pair": float(np.mean(ops)),
           "rowops_p50": float(np.median(ops)), "rowops_p95": float(np.percentile(ops, 95)),
           "orthogonal_fraction": orth / pairs, "per_projector": per_proj,
           "direct_rows_per_pair": float(np.mean(drows)), "direct_rows_p50": float(np.median(drows)),
           "direct_rows_p95": float(np.percentile(drows, 95))}
    print(json.dumps(out))


if __name__ == "__main__":
    main()

"""Generates the golden vectors under tests/golden/ from the reference.

Run here (where the reference checkout and oracle/_ref exist):

    make -C oracle ref && python tests/golden/make_golden.py [REFERENCE_ROOT]

Two sources, both the reference's own:

1. The known-answer fixtures of the reference's C unit tests
   (tests/units/tests-c/*.txt, read exactly as tests/units/stabtests.c reads
   them: stride-n matrices, "value > 0" sets a bit).  Each case keeps the
   fixture's expected values AND the full output of the reference's own C code
   (oracle/_ref/libcsimref.so) on that input, which is checked here to agree
   with the fixture on every field the reference test compares.
2. Seeded vectors from the reference's C code compiled from source: rand()
   streams, random states with the exact rand() words they consumed,
   projected states and (eps, p, m) for state/term pairs at t = 6..64,
   estimator values and decompose() outputs.

The output files are committed; the tests never read the reference checkout.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from circuitsimulator_gb300.state import STATE_DTYPE, block_view  # noqa: E402
from golden.golden_io import save, state_to_json  # noqa: E402
from oracle_ffi import RefLib, make_projector  # noqa: E402

REFROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CSIM_REFERENCE", "")
if not REFROOT or not os.path.isdir(os.path.join(REFROOT, "libcirc")):
    sys.exit("usage: make_golden.py REFERENCE_ROOT (the reference checkout; or set CSIM_REFERENCE)")
FIX = os.path.join(REFROOT, "tests", "units", "tests-c")


# ----------------------------------------------------------------- fixture parsing
def _lines(name):
    with open(os.path.join(FIX, name)) as f:
        return [ln.rstrip("\n") for ln in f]


def _arr(line):
    return [float(v) for v in line.split(",") if v.strip() != ""]


def _vec_word(vals, n):
    w = 0
    for i in range(n):
        if int(vals[i]) % 2 == 1:  # BitVectorSet(vec, i, (unsigned)value): value % 2 == 1
            w |= 1 << i
    return w


def _mat_words(vals, n):
    rows = []
    for i in range(n):
        w = 0
        for j in range(n):
            if vals[i * n + j] > 0:
                w |= 1 << j
        rows.append(w)
    return rows


def _set_d(s, vals, n):
    for i in range(n):
        v = int(vals[i])
        v2 = int(v / 2)
        d1 = int(np.fmod(v2, 2)) & 1
        d2 = int(np.fmod(int((v2 - int(np.fmod(v2, 2))) / 2), 2)) & 1
        s["D1"] = np.uint64(int(s["D1"][0]) | (d1 << i))
        s["D2"] = np.uint64(int(s["D2"][0]) | (d2 << i))


def _alloc(n, k):
    s = np.zeros(1, dtype=STATE_DTYPE)
    s["n"] = n
    s["k"] = k
    for i in range(n):
        s["G"][0, i] = np.uint64(1 << i)
        s["Gbar"][0, i] = np.uint64(1 << i)
    return s


def _getd_list(s, count):
    return [2 * (2 * ((int(s["D2"][0]) >> i) & 1) + ((int(s["D1"][0]) >> i) & 1)) for i in range(count)]


def fixtures(R):
    out = {}

    # exponentialSumTests.txt: n, k, Q, D, J, eps, p, m  (stabtests.c:38-103)
    L = _lines("exponentialSumTests.txt")
    cases = []
    for c in range(len(L) // 8):
        b = L[c * 8:(c + 1) * 8]
        n, k = int(b[0]), int(b[1])
        s = _alloc(n, k)
        s["Q"] = int(b[2])
        d, j = _arr(b[3]), _arr(b[4])
        assert len(d) == n and len(j) == n * n
        _set_d(s, d, n)
        s["J"][0, :n] = np.array(_mat_words(j, n), dtype=np.uint64)
        want = (int(b[5]), int(b[6]), int(b[7]))
        work = s.copy()
        got = R.exponential_sum(work)
        assert got[0] == want[0] and got[1] == want[1] and got[2] % 8 == want[2] % 8, (c, got, want)
        cases.append({"in": state_to_json(s), "fixture": want, "ref": got, "ref_state": state_to_json(work)})
    out["exponential_sum"] = cases

    # shrinkTests.txt (stabtests.c:105-255)
    L = _lines("shrinkTests.txt")
    cases = []
    for c in range(len(L) // 18):
        b = L[c * 18:(c + 1) * 18]
        n, k = int(b[0]), int(b[1])
        s = _alloc(n, k)
        s["Q"] = int(b[2])
        alpha = int(b[3])
        s["h"] = np.uint64(_vec_word(_arr(b[4]), n))
        _set_d(s, _arr(b[5]), n)
        xi = _vec_word(_arr(b[6]), n)
        s["G"][0, :n] = np.array(_mat_words(_arr(b[7]), n), dtype=np.uint64)
        s["Gbar"][0, :n] = np.array(_mat_words(_arr(b[8]), n), dtype=np.uint64)
        s["J"][0, :n] = np.array(_mat_words(_arr(b[9]), n), dtype=np.uint64)
        fx = {
            "status": int(b[10]),
            "k": int(b[11]),
            "Q": int(b[12]),
            "h": "%x" % _vec_word(_arr(b[13]), n),
            "D": [int(v) for v in _arr(b[14])],
            "G": ["%x" % w for w in _mat_words(_arr(b[15]), n)],
            "Gbar": ["%x" % w for w in _mat_words(_arr(b[16]), n)],
            "J": ["%x" % w for w in _mat_words(_arr(b[17]), n)],
        }
        work = s.copy()
        st = R.shrink(work, xi, alpha, 0)
        w0 = work[0]
        assert st == fx["status"] and int(w0["k"]) == fx["k"] and int(w0["Q"]) == fx["Q"], c
        assert "%x" % int(w0["h"]) == fx["h"], c
        assert _getd_list(work, int(w0["k"])) == fx["D"][: int(w0["k"])], c
        assert ["%x" % int(x) for x in w0["G"][:n]] == fx["G"], c
        assert ["%x" % int(x) for x in w0["Gbar"][:n]] == fx["Gbar"], c
        cases.append({"in": state_to_json(s), "xi": "%x" % xi, "alpha": alpha, "fixture": fx, "ref_status": st,
                      "ref_state": state_to_json(work)})
    out["shrink"] = cases

    # measurePauliTests.txt (stabtests.c:401-580)
    L = _lines("measurePauliTests.txt")
    cases = []
    for c in range(len(L) // 19):
        b = L[c * 19:(c + 1) * 19]
        n, k = int(b[0]), int(b[1])
        s = _alloc(n, k)
        s["Q"] = int(b[2])
        m = int(b[3])
        s["h"] = np.uint64(_vec_word(_arr(b[4]), n))
        _set_d(s, _arr(b[5]), n)
        zeta = _vec_word(_arr(b[6]), n)
        xi = _vec_word(_arr(b[7]), n)
        s["G"][0, :n] = np.array(_mat_words(_arr(b[8]), n), dtype=np.uint64)
        s["Gbar"][0, :n] = np.array(_mat_words(_arr(b[9]), n), dtype=np.uint64)
        s["J"][0, :n] = np.array(_mat_words(_arr(b[10]), n), dtype=np.uint64)
        fx = {
            "result": float(b[11]),
            "k": int(b[12]),
            "Q": int(b[13]),
            "h": "%x" % _vec_word(_arr(b[14]), n),
            "D": [int(v) for v in _arr(b[15])],
            "G": ["%x" % w for w in _mat_words(_arr(b[16]), n)],
            "Gbar": ["%x" % w for w in _mat_words(_arr(b[17]), n)],
            "J": ["%x" % w for w in _mat_words(_arr(b[18]), n)],
        }
        work = s.copy()
        res = R.measure_pauli(work, m, zeta, xi)
        w0 = work[0]
        kk = int(w0["k"])
        assert res - fx["result"] < 0.0001 and kk == fx["k"] and int(w0["Q"]) == fx["Q"], c
        assert "%x" % int(w0["h"]) == fx["h"], c
        assert _getd_list(work, kk) == fx["D"][:kk], c
        km = (1 << kk) - 1
        assert [int(x) & km for x in w0["J"][:kk]] == [int(x, 16) & km for x in fx["J"][:kk]], c
        cases.append({"in": state_to_json(s), "m": m, "zeta": "%x" % zeta, "xi": "%x" % xi, "fixture": fx,
                      "ref_result": res, "ref_state": state_to_json(work)})
    out["measure_pauli"] = cases

    # extendTests.txt (no C driver in the reference; format n, k, xi, G, Gbar, outk, outG, outGbar)
    L = _lines("extendTests.txt")
    cases = []
    for c in range(len(L) // 8):
        b = L[c * 8:(c + 1) * 8]
        n, k = int(b[0]), int(b[1])
        s = _alloc(n, k)
        xi = _vec_word(_arr(b[2]), n)
        s["G"][0, :n] = np.array(_mat_words(_arr(b[3]), n), dtype=np.uint64)
        s["Gbar"][0, :n] = np.array(_mat_words(_arr(b[4]), n), dtype=np.uint64)
        fx = {"k": int(b[5]), "G": ["%x" % w for w in _mat_words(_arr(b[6]), n)],
              "Gbar": ["%x" % w for w in _mat_words(_arr(b[7]), n)]}
        work = s.copy()
        R.extend(work, xi)
        w0 = work[0]
        assert int(w0["k"]) == fx["k"], c
        assert ["%x" % int(x) for x in w0["G"][:n]] == fx["G"], c
        assert ["%x" % int(x) for x in w0["Gbar"][:n]] == fx["Gbar"], c
        cases.append({"in": state_to_json(s), "xi": "%x" % xi, "fixture": fx, "ref_state": state_to_json(work)})
    out["extend"] = cases

    # innerProductTests-backup.txt (stabtests.c:258-398; the full file is not shipped)
    L = _lines("innerProductTests-backup.txt")
    cases = []
    for c in range(len(L) // 19):
        b = L[c * 19:(c + 1) * 19]
        st = []
        for off in (0, 8):
            n, k = int(b[off]), int(b[off + 1])
            s = _alloc(n, k)
            s["Q"] = int(b[off + 2])
            s["h"] = np.uint64(_vec_word(_arr(b[off + 3]), n))
            _set_d(s, _arr(b[off + 4]), n)
            s["G"][0, :n] = np.array(_mat_words(_arr(b[off + 5]), n), dtype=np.uint64)
            s["Gbar"][0, :n] = np.array(_mat_words(_arr(b[off + 6]), n), dtype=np.uint64)
            s["J"][0, :n] = np.array(_mat_words(_arr(b[off + 7]), n), dtype=np.uint64)
            st.append(s)
        want = (int(b[16]), int(b[17]), int(b[18]))
        got = R.inner_product(st[0], st[1])
        assert (got[0] == 0 and want[0] == 0) or (got[0] == want[0] and got[1] == want[1]
                                                   and got[2] % 8 == want[2] % 8), (got, want)
        cases.append({"a": state_to_json(st[0]), "b": state_to_json(st[1]), "fixture": want, "ref": got})
    out["inner_product"] = cases
    return out


# ----------------------------------------------------------------- seeded vectors
def rand_word(rs, n):
    w = 0
    for c in range(n):
        if rs.randint(2):
            w |= 1 << c
    return w


def random_projector(rs, t, nstabs):
    ph = rs.randint(0, 4, size=nstabs).tolist()
    xs = [rand_word(rs, t) for _ in range(nstabs)]
    zs = [rand_word(rs, t) for _ in range(nstabs)]
    return ph, xs, zs


def seeded(R):
    out = {}
    # rand() streams (the libc generator the CSIM_RNG_LIBC sampler reproduces)
    out["rand_streams"] = []
    for seed in (0, 1, 2, 77, 123456789, 4000000000):
        R.srand(seed)
        out["rand_streams"].append({"seed": seed, "values": [R.rand() for _ in range(400)]})

    # random states + the rand() words each consumed (for replay on the GPU)
    recs = []
    for n in (1, 2, 3, 5, 8, 12, 24, 40, 63, 64):
        R.srand(1000 + n)
        for _ in range(6):
            st, words = R.record(lambda: R.random_state(n))
            recs.append({"n": n, "words": [int(w) for w in words], "state": state_to_json(st)})
    out["random_states"] = recs

    # projected states and (eps, p, m) against decomposition terms
    pairs = []
    rs = np.random.RandomState(2024)
    for (t, kl, ntheta, nj) in ((6, 4, 6, 16), (12, 6, 8, 24), (17, 8, 6, 24), (24, 10, 6, 24), (40, 16, 6, 20),
                                (57, 12, 4, 12), (64, 14, 4, 12)):
        R.srand(7 * t + 1)
        ph, xs, zs = random_projector(rs, t, max(1, t // 4))
        P = make_projector(ph, xs, zs, t)
        thetas, factors = [], []
        tries = 0
        while len(thetas) < ntheta and tries < 200:
            tries += 1
            th = R.random_state(t)
            pf = 1.0
            for r in range(len(ph)):
                m = 2 * ((ph[r] // 2) % 2) + (ph[r] % 2)
                res = R.measure_pauli(th, m, zs[r], xs[r])
                pf *= res
                if res == 0:
                    break
            if pf != 0:
                thetas.append(th)
                factors.append(pf)
        L = [rand_word(rs, t) for _ in range(kl)]
        jl = sorted(set(int(x) for x in rs.randint(0, 2 ** kl, size=nj)))
        prods = []
        for th in thetas:
            row = []
            for j in jl:
                row.append(R.inner_product(th, R.prep_l(j, t, L)))
            prods.append(row)
        entry = {"t": t, "projector": {"phase": ph, "xs": ["%x" % x for x in xs], "zs": ["%x" % z for z in zs]},
                 "theta": [state_to_json(th) for th in thetas], "projfactor": factors,
                 "L": ["%x" % x for x in L], "j": jl, "prod_l": prods,
                 "phi_l": [state_to_json(R.prep_l(j, t, L)) for j in jl[:4]]}
        if t <= 24:
            jh = sorted(set(int(x) for x in rs.randint(0, 2 ** ((t + 1) // 2), size=nj)))
            entry["jh"] = jh
            entry["prod_h"] = [[R.inner_product(th, R.prep_h(j, t)) for j in jh] for th in thetas]
            entry["phi_h"] = [state_to_json(R.prep_h(j, t)) for j in jh[:4]]
        pairs.append(entry)
    out["term_pairs"] = pairs

    # general state pairs (two random, possibly projected, states)
    gen = []
    for n in (1, 2, 3, 4, 7, 13, 31, 32, 33, 40, 64):
        R.srand(555 + n)
        for _ in range(8):
            a, b = R.random_state(n), R.random_state(n)
            if rs.randint(2):
                R.measure_pauli(a, rs.randint(4), rand_word(rs, n), rand_word(rs, n))
            gen.append({"a": state_to_json(a), "b": state_to_json(b), "ref": R.inner_product(a, b)})
    out["state_pairs"] = gen

    # estimators on the same draws (srand(seed) before each call)
    est = []
    for (t, kl, exact, samples, bins, seed) in ((5, 3, 1, 40, 1, 11), (8, 4, 0, 30, 1, 12), (12, 6, 1, 20, 1, 13),
                                                (12, 5, 0, 16, 3, 14), (10, 4, 0, 12, 4, 15), (20, 6, 0, 6, 1, 16)):
        ph, xs, zs = random_projector(rs, t, max(1, t // 3))
        P = make_projector(ph, xs, zs, t)
        L = [rand_word(rs, t) for _ in range(kl)]
        R.srand(seed)
        singles = [R.single_projector_sample(P, L, kl, exact) for _ in range(6)]
        R.srand(seed)
        v = R.multi_sampled_projector(P, L, kl, exact, 1.25, samples, bins)
        ex = R.exact_projector(P, L, kl, exact, 1.25) if (exact and t <= 12) or (not exact and kl <= 5) else None
        est.append({"t": t, "k": kl, "exact": exact, "samples": samples, "bins": bins, "seed": seed, "norm": 1.25,
                    "projector": {"phase": ph, "xs": ["%x" % x for x in xs], "zs": ["%x" % z for z in zs]},
                    "L": ["%x" % x for x in L], "singles": singles, "multi": v, "exact_projector": ex})
    out["estimators"] = est

    # decompose() from the unseeded (seed 1) stream, as the reference master calls it
    dec = []
    for (t, fid, rank, fidelity, forceL, k) in ((12, 1e-5, 0, 0, 0, 0), (40, 0.01, 0, 0, 1, 16),
                                                (40, 0.01, 1, 0, 0, 16), (20, 0.05, 1, 1, 0, 0),
                                                (24, 0.02, 0, 1, 1, 0), (9, 0.1, 0, 0, 0, 0), (64, 0.02, 1, 0, 1, 14)):
        R.srand(1)
        e, kk, norm, L = R.decompose(t, fid, rank, fidelity, forceL, 0, k)
        dec.append({"t": t, "fidbound": fid, "rank": rank, "fidelity": fidelity, "forceL": forceL, "k_in": k,
                    "exact": e, "k": kk, "norm": norm, "L": None if L is None else ["%x" % int(x) for x in L]})
    out["decompose"] = dec
    return out


def main():
    R = RefLib()
    fx = fixtures(R)
    print({k: len(v) for k, v in fx.items()})
    save("ref_fixtures.json.gz", fx)
    sd = seeded(R)
    print({k: len(v) for k, v in sd.items()})
    save("ref_seeded.json.gz", sd)


if __name__ == "__main__":
    main()

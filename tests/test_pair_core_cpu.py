"""The thread-per-pair kernel's pair routine (csim_pair_core.cuh), compiled
for the host, against the oracle: (eps, p, m) bit-exact, m unreduced, on
seeded projected states at t = 1..64 and on the reference's golden pairs."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from golden.golden_io import states_from_json
from helpers import phase_m, rand_word, random_projector_rows

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "tp_host_check.cpp")
SO = os.path.join(HERE, "native", "_build", "libtphost.so")
CORES = [os.path.join(os.path.dirname(HERE), "circuitsimulator_gb300", "csrc", f)
         for f in ("csim_pair_core.cuh", "csim_block_prefix.cuh")]


@pytest.fixture(scope="module", params=["32", "0"], ids=["wide_above_32", "always_wide"])
def tp(request):
    """The host build of the pair routine; "always_wide" runs the 64-bit code
    for every k, as a lane with a small k does in a warp that holds a larger one."""
    so = SO.replace(".so", "_w%s.so" % request.param)
    os.makedirs(os.path.dirname(so), exist_ok=True)
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(f) for f in [SRC] + CORES):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-DCSIM_TP_WIDE_FROM=" + request.param,
                               SRC, "-o", so])
    lib = C.CDLL(so)
    lib.tp_host_pairs.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.tp_host_pairs.restype = C.c_int
    lib.tp_host_block.argtypes = lib.tp_host_pairs.argtypes
    lib.tp_host_block.restype = C.c_int
    lib.tp_host_runs.argtypes = lib.tp_host_pairs.argtypes[:4] + [C.c_int] + lib.tp_host_pairs.argtypes[4:]
    lib.tp_host_runs.restype = C.c_int
    lib.tp_host_direct.argtypes = lib.tp_host_pairs.argtypes
    lib.tp_host_direct.restype = C.c_int

    def run(thetas, xs, block=False, run_len=0):
        thetas = np.ascontiguousarray(thetas)
        xs = np.ascontiguousarray(np.asarray(xs, dtype=np.uint64))
        n = len(thetas) * len(xs)
        e, p, m = (np.zeros(n, dtype=np.int32) for _ in range(3))
        if run_len == -1:
            err = lib.tp_host_direct(thetas.ctypes.data, len(thetas), xs.ctypes.data, len(xs), e.ctypes.data,
                                     p.ctypes.data, m.ctypes.data)
            return err, e, p, m
        if run_len:
            err = lib.tp_host_runs(thetas.ctypes.data, len(thetas), xs.ctypes.data, len(xs), run_len, e.ctypes.data,
                                   p.ctypes.data, m.ctypes.data)
            return err, e, p, m
        fn = lib.tp_host_block if block else lib.tp_host_pairs
        err = fn(thetas.ctypes.data, len(thetas), xs.ctypes.data, len(xs), e.ctypes.data, p.ctypes.data,
                 m.ctypes.data)
        return err, e, p, m

    return run


def _projected_thetas(oracle, rs, t, count=8):
    rows = random_projector_rows(rs, t, max(1, t // 3))
    r = oracle.rng(t)
    thetas = []
    for _ in range(5 * count):
        s = oracle.random_state(t, r)
        pf = 1.0
        for q in range(len(rows[0])):
            res = oracle.measure_pauli(s, phase_m(rows[0][q]), rows[2][q], rows[1][q])
            pf *= res
            if res == 0:
                break
        if pf:
            thetas.append(s[0])
        if len(thetas) == count:
            break
    return np.array(thetas)


@pytest.mark.parametrize("t,k", [(1, 1), (2, 2), (3, 3), (6, 4), (12, 6), (24, 8), (31, 8), (33, 8), (40, 10),
                                 (57, 8), (63, 7), (64, 8)])
def test_pair_core_vs_oracle(tp, oracle, t, k):
    rs = np.random.RandomState(500 + t)
    L = np.array([rand_word(rs, t) for _ in range(k)], dtype=np.uint64)
    rows = random_projector_rows(rs, t, max(1, t // 3))
    r = oracle.rng(t)
    thetas = []
    for _ in range(40):
        s = oracle.random_state(t, r)
        pf = 1.0
        for q in range(len(rows[0])):
            res = oracle.measure_pauli(s, phase_m(rows[0][q]), rows[2][q], rows[1][q])
            pf *= res
            if res == 0:
                break
        if pf:
            thetas.append(s[0])
        if len(thetas) == 8:
            break
    thetas = np.array(thetas)
    js = np.unique(rs.randint(0, 2 ** k, size=48))
    xs = [oracle.codeword(int(j), L) for j in js]
    err, e, p, m = tp(thetas, xs)
    assert err == 0
    w = 0
    for a in range(len(thetas)):
        for jj, j in enumerate(js):
            want = oracle.inner_product(thetas[a:a + 1], oracle.prep_l(int(j), t, L))
            assert (e[w], p[w], m[w]) == want, (t, a, int(j))
            w += 1


def test_pair_core_golden(tp, golden_seeded):
    for ent in golden_seeded["term_pairs"]:
        t = ent["t"]
        L = [int(x, 16) for x in ent["L"]]
        thetas = states_from_json(ent["theta"])
        xs = []
        for j in ent["j"]:
            x = 0
            for rr in range(len(L)):
                if (j >> (len(L) - 1 - rr)) & 1:
                    x ^= L[rr]
            xs.append(x)
        err, e, p, m = tp(thetas, xs)
        assert err == 0
        got = np.stack([e, p, m], axis=1).reshape(len(thetas), len(xs), 3)
        assert got.tolist() == ent["prod_l"]


@pytest.mark.parametrize("t,k,d", [(3, 2, 1), (6, 3, 2), (12, 5, 4), (24, 6, 8), (33, 6, 10), (40, 8, 7),
                                   (40, 8, 16), (57, 6, 20), (64, 6, 24)])
def test_shared_prefix_vs_oracle(tp, oracle, t, k, d):
    """The kernels' block path (up to four codeword groups: halves split at the
    highest bit in which the codewords differ, each half at its own; each
    group's shared top-bit shrinks once per theta, then each pair from its
    group's state) against the oracle: codeword sets whose top d bits agree,
    split by the coefficient of the one row of L that has top bits (all-zero
    and mixed prefixes), the whole set (groups at the top bits), and a single
    codeword (every shrink shared)."""
    rs = np.random.RandomState(900 + t + d)
    low = (1 << (t - d)) - 1
    L = [rand_word(rs, t) & low for _ in range(k)]
    L[0] |= rand_word(rs, t) & ~low & ((1 << t) - 1)
    L = np.array(L, dtype=np.uint64)
    thetas = _projected_thetas(oracle, rs, t)
    js = np.unique(rs.randint(0, 2 ** k, size=40))
    top = 1 << (k - 1)  # j's bit of row 0 (codeword() takes row r at bit k-1-r)
    for subset in ([j for j in js if j & top], [j for j in js if not j & top], list(js), [js[0]]):
        if not subset:
            continue
        xs = [oracle.codeword(int(j), L) for j in subset]
        err, e, p, m = tp(thetas, xs, block=True)
        assert err == 0
        w = 0
        for a in range(len(thetas)):
            for j in subset:
                want = oracle.inner_product(thetas[a:a + 1], oracle.prep_l(int(j), t, L))
                assert (e[w], p[w], m[w]) == want, (t, d, a, int(j))
                w += 1


@pytest.mark.parametrize("t,k,run_len", [(3, 3, 4), (12, 6, 8), (24, 8, 32), (33, 9, 16), (40, 10, 32), (57, 8, 32),
                                         (64, 8, 16)])
def test_runs_vs_oracle(tp, oracle, t, k, run_len):
    """The run kernel's per-thread path: the 2^k codewords in numeric order,
    cut into runs of run_len; each run's common zeros in its agreed top bits
    shrunk once, then every pair from that state, against the oracle."""
    rs = np.random.RandomState(1300 + t)
    L = np.array([rand_word(rs, t) for _ in range(k)], dtype=np.uint64)
    thetas = _projected_thetas(oracle, rs, t, count=4)
    js = np.arange(2 ** k)
    xs = sorted((oracle.codeword(int(j), L), int(j)) for j in js)
    err, e, p, m = tp(thetas, [x for x, _ in xs], run_len=run_len)
    assert err == 0
    w = 0
    for a in range(len(thetas)):
        eo, po, mo = oracle.term_products(t, 0, L, k, thetas[a:a + 1], 0, 2 ** k, threads=os.cpu_count() or 1)
        for x, j in xs:
            assert (e[w], p[w], m[w]) == (eo[j], po[j], mo[j]), (t, a, j)
            w += 1


@pytest.mark.parametrize("t", [8, 24, 40, 64])
def test_j_diagonal_is_d1(oracle, t):
    """The direct kernel's exponential sum leaves out the J_aa, J_bb terms of its
    dimer steps and the bit-a mask of its dimer search (csim_pair_core.cuh,
    md_exp_step): it takes J's diagonal to be D1 (J_xx = D_x/2 mod 2), which is
    zero on the variables it eliminates.  That holds for every state the
    reference's own operations make: drawn (randomStabilizerState), projected
    (measurePauli) and shrunk."""
    rs = np.random.RandomState(4400 + t)
    thetas = list(_projected_thetas(oracle, rs, t, count=6))
    r = oracle.rng(t + 1)
    thetas += [oracle.random_state(t, r)[0] for _ in range(6)]
    checked = 0
    for th in thetas:
        one = np.array([th])
        for step in range(4):
            k = int(one["k"][0])
            d1 = int(one["D1"][0])
            for a in range(k):
                assert (int(one["J"][0][a]) >> a) & 1 == (d1 >> a) & 1, (t, step, a)
            checked += k
            oracle.shrink(one, rand_word(rs, t), int(rs.randint(2)), 0)
    assert checked > 0


@pytest.mark.parametrize("t,k,nshrink", [(1, 1, 0), (3, 3, 0), (8, 4, 0), (12, 6, 4), (24, 8, 0), (33, 8, 0),
                                         (40, 10, 0), (40, 10, 20), (44, 9, 0), (48, 9, 6), (57, 8, 0), (64, 9, 0),
                                         (64, 8, 40)])
def test_direct_vs_oracle(tp, oracle, t, k, nshrink):
    """The direct kernel's path: theta once in pivot coordinates
    (canon_theta), each pair by removing the variables at x's zero pivot
    coordinates, a constraint per zero at a non-pivot coordinate (md_shrink),
    then the exponential sum (md_exp_sum).  eps and p equal the oracle's and
    m equals it mod 8 (the reference's unreduced m depends on its basis; the
    inner product is the same complex number).  nshrink random shrinks first
    lower k, so many pairs carry several constraints."""
    rs = np.random.RandomState(1700 + t + nshrink)
    L = np.array([rand_word(rs, t) for _ in range(k)], dtype=np.uint64)
    thetas = _projected_thetas(oracle, rs, t, count=4)
    for i in range(len(thetas)):
        one = thetas[i:i + 1].copy()
        for _ in range(nshrink):
            oracle.shrink(one, rand_word(rs, t), int(rs.randint(2)), 0)
        thetas[i] = one[0]
    xs = [oracle.codeword(int(j), L) for j in range(2 ** k)]
    err, e, p, m = tp(thetas, xs, run_len=-1)
    assert err == 0
    eo, po, mo = oracle.term_products(t, 0, L, k, thetas, 0, 2 ** k, threads=os.cpu_count() or 1)
    ok = (e == eo) & ((e == 0) | ((p == po) & ((m % 8) == (mo % 8))))
    assert ok.all(), (t, k, nshrink, int((~ok).sum()))


def test_direct_odd_variable_above_32(tp, oracle):
    """Pairs whose exponential sum keeps its one odd-D variable (sidx) at a live
    index >= 32, with more than 32 live variables: in 64-bit mode the row of
    sidx stores column sidx of the rows below 32 and is updated apart from the
    row passes.  Every coordinate is a pivot (G = I), odd D only on coordinates
    56..63, J random symmetric with diagonal D1, codewords of about 45 ones."""
    rs = np.random.RandomState(77)
    t = 64
    thetas = []
    for _ in range(3):
        th = oracle.state(t, t)[0]
        hi = np.uint64(0xFF00000000000000)
        d1 = np.uint64(rand_word(rs, t)) & hi
        th["D1"] = d1
        th["D2"] = np.uint64(rand_word(rs, t))
        th["Q"] = int(rs.randint(8)) & 6
        J = np.zeros(t, dtype=np.uint64)
        for a in range(t):
            for b in range(a + 1, t):
                if rs.randint(2):
                    J[a] |= np.uint64(1 << b)
                    J[b] |= np.uint64(1 << a)
            if (int(d1) >> a) & 1:
                J[a] |= np.uint64(1 << a)
        th["J"] = J
        thetas.append(th)
    thetas = np.array(thetas)
    # codewords: random words of about 0.7 t ones, closed under XOR of a small code
    L = np.array([int("".join("1" if rs.rand() < 0.7 else "0" for _ in range(t)), 2) for _ in range(6)],
                 dtype=np.uint64)
    xs = [oracle.codeword(int(j), L) for j in range(2 ** len(L))]
    xs = [x for x in xs if bin(x).count("1") > 36]
    assert len(xs) >= 8
    err, e, p, m = tp(thetas, xs, run_len=-1)
    assert err == 0
    eo, po, mo = oracle.term_products(t, 0, L, len(L), thetas, 0, 2 ** len(L), threads=os.cpu_count() or 1)
    idx = [j for j in range(2 ** len(L)) if bin(oracle.codeword(j, L)).count("1") > 36]
    eo = eo.reshape(len(thetas), -1)[:, idx].reshape(-1)
    po = po.reshape(len(thetas), -1)[:, idx].reshape(-1)
    mo = mo.reshape(len(thetas), -1)[:, idx].reshape(-1)
    ok = (e == eo) & ((e == 0) | ((p == po) & ((m % 8) == (mo % 8))))
    assert ok.all(), int((~ok).sum())
    assert (e != 0).any()

"""Parity of the CUDA path (through the C ABI of libcsimgpu.so) with the
reference: its unit-test fixtures, vectors produced by the reference's own C
code, and the oracle restatement on seeded inputs up to the c2 workload's shape
(t = 40, chi = 2^16).  Integer results must be bit-exact, (eps, p, m) with m
unreduced; probabilities within 1e-12 relative (+1e-12 absolute floor, for
sums that cancel) of the reference's double accumulation on the same draws."""
import os

import numpy as np
import pytest

from circuitsimulator_gb300 import backend
from circuitsimulator_gb300.state import STATE_DTYPE
from golden.golden_io import state_from_json, states_from_json
from helpers import close, full_view, phase_m, rand_word, random_projector_rows

pytestmark = pytest.mark.gpu

REL = 1e-12
FLOOR = 1e-12


@pytest.fixture(scope="module")
def gpu():
    b = backend.Backend(0)
    yield b
    b.close()


def _words(xs):
    return np.array([int(x, 16) for x in xs], dtype=np.uint64)


# ---------------------------------------------------------------- reference unit-test fixtures
def test_fixture_exponential_sum(gpu, golden_fixtures):
    cases = golden_fixtures["exponential_sum"]
    s = states_from_json([c["in"] for c in cases])
    eps, p, m = gpu.exponentialSumExact(s)
    for i, c in enumerate(cases):
        assert [eps[i], p[i], m[i]] == list(c["ref"]), i
        f = c["fixture"]
        assert eps[i] == f[0] and p[i] == f[1] and m[i] % 8 == f[2] % 8
        assert full_view(s[i]) == full_view(state_from_json(c["ref_state"])), i


def test_fixture_shrink(gpu, golden_fixtures):
    cases = golden_fixtures["shrink"]
    s = states_from_json([c["in"] for c in cases])
    st = gpu.shrink(s, _words([c["xi"] for c in cases]), [c["alpha"] for c in cases], lazy=False)
    for i, c in enumerate(cases):
        assert st[i] == c["ref_status"] == c["fixture"]["status"]
        assert full_view(s[i]) == full_view(state_from_json(c["ref_state"])), i


def test_fixture_measure_pauli(gpu, golden_fixtures):
    cases = golden_fixtures["measure_pauli"]
    s = states_from_json([c["in"] for c in cases])
    res = gpu.measurePauli(s, [c["m"] for c in cases], _words([c["zeta"] for c in cases]),
                           _words([c["xi"] for c in cases]))
    for i, c in enumerate(cases):
        assert res[i] == c["ref_result"]
        assert full_view(s[i]) == full_view(state_from_json(c["ref_state"])), i


def test_fixture_extend(gpu, golden_fixtures):
    cases = golden_fixtures["extend"]
    s = states_from_json([c["in"] for c in cases])
    gpu.extend(s, _words([c["xi"] for c in cases]))
    for i, c in enumerate(cases):
        assert full_view(s[i]) == full_view(state_from_json(c["ref_state"])), i


def test_fixture_inner_product(gpu, golden_fixtures):
    cases = golden_fixtures["inner_product"]
    a = states_from_json([c["a"] for c in cases])
    b = states_from_json([c["b"] for c in cases])
    eps, p, m = gpu.innerProductExact(a, b)
    for i, c in enumerate(cases):
        assert [eps[i], p[i], m[i]] == list(c["ref"])


# ---------------------------------------------------------------- vectors from the reference's C code
def test_random_states_replay(gpu, golden_seeded):
    by_n = {}
    for rec in golden_seeded["random_states"]:
        by_n.setdefault(rec["n"], []).append(rec)
    for n, recs in by_n.items():
        words = np.concatenate([np.array(r["words"], dtype=np.uint32) for r in recs])
        offs = np.cumsum([0] + [len(r["words"]) for r in recs]).astype(np.int64)
        out = gpu.randomStabilizerStateReplay(n, words, offs)
        for i, r in enumerate(recs):
            assert full_view(out[i]) == full_view(state_from_json(r["state"])), (n, i)


def test_random_states_replay_short_segment_is_an_error(gpu, golden_seeded):
    rec = [r for r in golden_seeded["random_states"] if r["n"] == 12][0]
    words = np.array(rec["words"][:-3], dtype=np.uint32)
    with pytest.raises(backend.CsimError):
        gpu.randomStabilizerStateReplay(12, words, np.array([0, len(words)], dtype=np.int64))


def test_term_pairs(gpu, golden_seeded):
    for e in golden_seeded["term_pairs"]:
        t = e["t"]
        L = _words(e["L"])
        thetas = states_from_json(e["theta"])
        js = e["j"]
        j0, nj = min(js), max(js) - min(js) + 1
        eps, p, m = gpu.term_products(t, False, L, thetas, j0, nj)
        for a in range(len(thetas)):
            for jj, j in enumerate(js):
                assert [eps[a, j - j0], p[a, j - j0], m[a, j - j0]] == list(e["prod_l"][a][jj]), (t, a, j)
        if "jh" in e:
            jh = e["jh"]
            j0, nj = min(jh), max(jh) - min(jh) + 1
            eps, p, m = gpu.term_products(t, True, None, thetas, j0, nj)
            for a in range(len(thetas)):
                for jj, j in enumerate(jh):
                    assert [eps[a, j - j0], p[a, j - j0], m[a, j - j0]] == list(e["prod_h"][a][jj]), (t, a, j)
        phis = gpu.prepL(e["j"][: len(e["phi_l"])], t, L)
        for i, d in enumerate(e["phi_l"]):
            assert full_view(phis[i]) == full_view(state_from_json(d))
        if "phi_h" in e:
            phis = gpu.prepH(e["jh"][: len(e["phi_h"])], t)
            for i, d in enumerate(e["phi_h"]):
                assert full_view(phis[i]) == full_view(state_from_json(d))


def test_state_pairs(gpu, golden_seeded):
    cases = golden_seeded["state_pairs"]
    a = states_from_json([c["a"] for c in cases])
    b = states_from_json([c["b"] for c in cases])
    eps, p, m = gpu.innerProductExact(a, b)
    for i, c in enumerate(cases):
        assert [eps[i], p[i], m[i]] == list(c["ref"]), i


def test_estimators_same_draws(gpu, golden_seeded):
    for e in golden_seeded["estimators"]:
        t, exact = e["t"], e["exact"]
        pr = e["projector"]
        P = backend.projector(pr["phase"], _words(pr["xs"]), _words(pr["zs"]), t)
        L = None if exact else _words(e["L"])
        singles = gpu.singleProjectorSample(P, L, exact, len(e["singles"]), backend.RNG_LIBC, e["seed"])
        for a, b in zip(singles, e["singles"]):
            assert close(a, b, REL, FLOOR), (a, b)
        v = gpu.multiSampledProjector(P, L, exact, e["norm"], e["samples"], e["bins"], backend.RNG_LIBC, e["seed"])
        assert close(v, e["multi"], REL, FLOOR), (v, e["multi"])
        if e["exact_projector"] is not None:
            x = gpu.exactProjector(P, L, exact, e["norm"])
            assert close(x, e["exact_projector"], REL, FLOOR), (x, e["exact_projector"])


# ---------------------------------------------------------------- seeded inputs vs the oracle
def _project_all(gpu, states, rows):
    """measurePauli row by row on every state; drops annihilated ones (innerprod.c:104-116)."""
    ph, xs, zs = rows
    keep = np.ones(len(states), dtype=bool)
    pf = np.ones(len(states))
    for r in range(len(ph)):
        idx = np.nonzero(keep)[0]
        sub = states[idx].copy()
        res = gpu.measurePauli(sub, phase_m(ph[r]), zs[r], xs[r])
        states[idx] = sub
        pf[idx] *= res
        keep[idx[res == 0]] = False
    return states[keep], pf[keep]


@pytest.mark.parametrize("t,k,ntheta,nj", [(3, 3, 8, 8), (7, 5, 16, 32), (24, 10, 12, 96), (33, 9, 12, 64),
                                           (40, 16, 12, 96), (64, 14, 6, 48)])
def test_term_products_vs_oracle(gpu, oracle, t, k, ntheta, nj):
    rs = np.random.RandomState(1000 + t)
    L = np.array([rand_word(rs, t) for _ in range(k)], dtype=np.uint64)
    th = gpu.randomStabilizerState(t, 3 * ntheta, seed=77 + t)
    th, _ = _project_all(gpu, th, random_projector_rows(rs, t, max(1, t // 4)))
    th = th[:ntheta]
    assert len(th) > 0
    j0 = int(rs.randint(0, max(1, 2 ** k - nj)))
    nj = min(nj, 2 ** k - j0)
    eg, pg, mg = gpu.term_products(t, False, L, th, j0, nj)
    eo, po, mo = oracle.term_products(t, 0, L, k, th, j0, nj, threads=os.cpu_count() or 1)
    assert (eg.reshape(-1) == eo).all() and (pg.reshape(-1) == po).all() and (mg.reshape(-1) == mo).all()
    if t <= 24:
        nh = min(nj, 2 ** ((t + 1) // 2))
        eg, pg, mg = gpu.term_products(t, True, None, th, 0, nh)
        eo, po, mo = oracle.term_products(t, 1, None, 0, th, 0, nh, threads=os.cpu_count() or 1)
        assert (eg.reshape(-1) == eo).all() and (pg.reshape(-1) == po).all() and (mg.reshape(-1) == mo).all()


def test_random_states_philox_are_valid(gpu):
    """Counter-based draws keep the invariants of randomStabilizerState's output."""
    for n in (1, 5, 31, 32, 33, 40, 64):
        s = gpu.randomStabilizerState(n, 64, seed=9)
        for x in s:
            k = int(x["k"])
            G = [int(v) for v in x["G"][:n]]
            B = [int(v) for v in x["Gbar"][:n]]
            for a in range(n):
                for b in range(n):
                    assert bin(G[a] & B[b]).count("1") % 2 == (a == b)
            J = [int(v) for v in x["J"][:n]]
            for a in range(k):
                assert ((J[a] >> a) & 1) == ((int(x["D1"]) >> a) & 1)
                for b in range(k):
                    assert ((J[a] >> b) & 1) == ((J[b] >> a) & 1)
            assert int(x["Q"]) == 0


def test_philox_sampler_matches_its_own_states(gpu):
    """singleProjectorSample with the counter-based generator equals the
    explicit pipeline (same draws -> project -> all pairs -> exact sum)."""
    rs = np.random.RandomState(5)
    t, k, count = 12, 6, 24
    L = [rand_word(rs, t) for _ in range(k)]
    rows = random_projector_rows(rs, t, 3)
    P = backend.projector(rows[0], rows[1], rows[2], t)
    vals = gpu.singleProjectorSample(P, L, False, count, backend.RNG_PHILOX, 4242)
    th = gpu.randomStabilizerState(t, count, seed=4242, first=0)
    for i in range(count):
        s = th[i:i + 1].copy()
        pf = 1.0
        for r in range(len(rows[0])):
            res = gpu.measurePauli(s, phase_m(rows[0][r]), rows[2][r], rows[1][r])[0]
            pf *= res
            if res == 0:
                break
        if pf == 0:
            assert vals[i] == 0
            continue
        eps, p, m = gpu.term_products(t, False, L, s, 0, 2 ** k)
        tot = sum(complex((2.0 ** (pp / 2.0)) * np.exp(1j * np.pi * (mm % 8) / 4.0)) * e
                  for e, pp, mm in zip(eps[0], p[0], m[0]))
        want = 2.0 ** t * abs(tot * pf) ** 2
        assert close(vals[i], want, 1e-10, 1e-12), (i, vals[i], want)


@pytest.mark.slow
def test_c2_shape_subsample_bit_exact(gpu, oracle):
    """t = 40, chi = 2^16 (the c2 workload's code size): 10^5 (theta, term) pairs
    drawn at random from 8 projected thetas x all 2^16 terms, bit-exact against
    the oracle; plus a checksum of every pair's value against the fused
    per-theta accumulation of the sampler."""
    rs = np.random.RandomState(40)
    t, k = 40, 16
    L = np.array([rand_word(rs, t) for _ in range(k)], dtype=np.uint64)
    rows = random_projector_rows(rs, t, 10)
    th = gpu.randomStabilizerState(t, 32, seed=2024)
    th, pf = _project_all(gpu, th, rows)
    th, pf = th[:8], pf[:8]
    eps, p, m = gpu.term_products(t, False, L, th, 0, 2 ** k)
    # 10^5-pair subsample: 12 random blocks of 1024 consecutive terms per theta
    nthreads = os.cpu_count() or 1
    checked = 0
    for a in range(len(th)):
        for j0 in rs.choice(2 ** k // 1024, size=12, replace=False) * 1024:
            j0 = int(j0)
            eo, po, mo = oracle.term_products(t, 0, L, k, th[a:a + 1], j0, 1024, threads=nthreads)
            assert (eps[a, j0:j0 + 1024] == eo).all() and (p[a, j0:j0 + 1024] == po).all() \
                and (m[a, j0:j0 + 1024] == mo).all(), (a, j0)
            checked += 1024
    assert checked >= 98000
    # the reference's p lies in [-2t, t] (p_expsum - k1 - k2), m in [0, 14]
    assert (m >= 0).all() and (m <= 14).all() and (p <= t).all() and (p >= -2 * t).all()


def _exact_sum(eps, p, m, P):
    """sum of eps 2^{p/2} w^m as exact Z[w] coordinates scaled by 2^{P/2} (Python ints)."""
    z = [0, 0, 0, 0]
    for e, pp, mm in zip(eps.tolist(), p.tolist(), m.tolist()):
        if not e:
            continue
        q, mm = pp + P, mm % 8
        if q % 2 == 0:
            z[mm & 3] += -(1 << (q // 2)) if mm >= 4 else (1 << (q // 2))
        else:
            c = 1 << ((q - 1) // 2)
            a, b = (mm + 1) % 8, (mm + 3) % 8
            z[a & 3] += -c if a >= 4 else c
            z[b & 3] -= -c if b >= 4 else c
    return z


@pytest.mark.slow
def test_c2_shape_sampler_checksum(gpu):
    """t = 40, chi = 2^16: the fused sampler (draw -> project -> all 2^16 terms ->
    per-theta exact sum) equals the exact sum of the 2^16 per-pair results of
    the same draws, theta by theta (a checksum over 65536 pairs per theta)."""
    rs = np.random.RandomState(41)
    t, k, count, seed = 40, 16, 24, 99
    L = [rand_word(rs, t) for _ in range(k)]
    rows = random_projector_rows(rs, t, 6)
    P = backend.projector(rows[0], rows[1], rows[2], t)
    vals = gpu.singleProjectorSample(P, L, False, count, backend.RNG_PHILOX, seed)
    th = gpu.randomStabilizerState(t, count, seed=seed, first=0)
    s2 = 0.70710678118654752440
    checked = 0
    for i in range(count):
        s = th[i:i + 1].copy()
        pf = 1.0
        for r in range(len(rows[0])):
            res = gpu.measurePauli(s, phase_m(rows[0][r]), rows[2][r], rows[1][r])[0]
            pf *= res
            if res == 0:
                break
        if pf == 0:
            assert vals[i] == 0
            continue
        eps, p, m = gpu.term_products(t, False, L, s, 0, 2 ** k)
        z = _exact_sum(eps[0], p[0], m[0], 2 * t)
        re = (z[0] + (z[1] - z[3]) * s2) * 2.0 ** -t
        im = (z[2] + (z[1] + z[3]) * s2) * 2.0 ** -t
        want = 2.0 ** t * ((re * pf) ** 2 + (im * pf) ** 2)
        assert close(vals[i], want, 1e-13, 1e-300), (i, vals[i], want)
        checked += 1
        if checked == 4:
            break
    assert checked >= 2


@pytest.mark.parametrize("t,k,low", [(33, 8, 12), (40, 10, 20), (64, 12, 30)])
def test_shared_prefix_codes_vs_oracle(gpu, oracle, t, k, low):
    """Codes whose codewords share long top bits: two rows of L span all t bits,
    the rest only the low `low` bits, so each block's two codeword groups share
    t - low top bits and run their shrinks once (the block-prefix path of the
    pair kernels, through the C ABI).  Every pair bit-exact against the oracle,
    in term order; and the sampler (ordered table) equal to the exact sum of
    its own draws' pairs."""
    rs = np.random.RandomState(3000 + t)
    mask = (1 << low) - 1
    L = np.array([rand_word(rs, t) if r < 2 else rand_word(rs, t) & mask for r in range(k)], dtype=np.uint64)
    rows = random_projector_rows(rs, t, max(1, t // 5))
    th = gpu.randomStabilizerState(t, 24, seed=55 + t)
    th, _ = _project_all(gpu, th, rows)
    th = th[:6]
    assert len(th) > 0
    eg, pg, mg = gpu.term_products(t, False, L, th, 0, 2 ** k)
    eo, po, mo = oracle.term_products(t, 0, L, k, th, 0, 2 ** k, threads=os.cpu_count() or 1)
    assert (eg.reshape(-1) == eo).all() and (pg.reshape(-1) == po).all() and (mg.reshape(-1) == mo).all()
    P = backend.projector(rows[0], rows[1], rows[2], t)
    count, seed = 6, 17
    vals = gpu.singleProjectorSample(P, [int(v) for v in L], False, count, backend.RNG_PHILOX, seed)
    drawn = gpu.randomStabilizerState(t, count, seed=seed, first=0)
    s2 = 0.70710678118654752440
    for i in range(count):
        st = drawn[i:i + 1].copy()
        pf = 1.0
        for r in range(len(rows[0])):
            res = gpu.measurePauli(st, phase_m(rows[0][r]), rows[2][r], rows[1][r])[0]
            pf *= res
            if res == 0:
                break
        if pf == 0:
            assert vals[i] == 0
            continue
        eps, p, m = gpu.term_products(t, False, L, st, 0, 2 ** k)
        z = _exact_sum(eps[0], p[0], m[0], 2 * t)
        re = (z[0] + (z[1] - z[3]) * s2) * 2.0 ** -t
        im = (z[2] + (z[1] + z[3]) * s2) * 2.0 ** -t
        want = 2.0 ** t * ((re * pf) ** 2 + (im * pf) ** 2)
        assert close(vals[i], want, 1e-13, 1e-300), (i, vals[i], want)


@pytest.mark.parametrize("t,k", [(12, 6), (40, 16), (64, 12)])
def test_pair_kernels_agree(gpu, t, k):
    """Thread-per-pair and warp-per-pair kernels: identical per-pair results and
    identical sampler values (exact sums)."""
    rs = np.random.RandomState(7000 + t)
    L = [rand_word(rs, t) for _ in range(k)]
    rows = random_projector_rows(rs, t, max(1, t // 5))
    th = gpu.randomStabilizerState(t, 12, seed=31 + t)
    th, _ = _project_all(gpu, th, rows)
    nj = min(2 ** k, 8192)
    try:
        gpu.set_option(backend.OPT_PAIR_KERNEL, 0)
        a = gpu.term_products(t, False, L, th, 0, nj)
        P = backend.projector(rows[0], rows[1], rows[2], t)
        va = gpu.singleProjectorSample(P, L, False, 16, backend.RNG_PHILOX, 5)
        gpu.set_option(backend.OPT_PAIR_KERNEL, 1)
        b = gpu.term_products(t, False, L, th, 0, nj)
        vb = gpu.singleProjectorSample(P, L, False, 16, backend.RNG_PHILOX, 5)
    finally:
        gpu.set_option(backend.OPT_PAIR_KERNEL, 0)
    for x, y in zip(a, b):
        assert (x == y).all()
    assert (va == vb).all()


def test_philox_blocks_compose(gpu):
    """State i of a counter-based stream is the same whoever draws it: two
    blocks drawn separately (as two ranks would) equal one draw of both."""
    rs = np.random.RandomState(9)
    t, k = 24, 8
    L = [rand_word(rs, t) for _ in range(k)]
    rows = random_projector_rows(rs, t, 5)
    P = backend.projector(rows[0], rows[1], rows[2], t)
    whole = gpu.singleProjectorSample(P, L, False, 50, backend.RNG_PHILOX, 123)
    parts = []
    for lo, hi in ((0, 21), (21, 50)):
        gpu.rng_position(123, lo)
        parts.append(gpu.singleProjectorSample(P, L, False, hi - lo, backend.RNG_PHILOX, backend.SEED_CONTINUE))
    assert (np.concatenate(parts) == whole).all()


def _zl_reference_loop(t, L):
    """The reference's Z(L) loop (probability.c:391-398) in codeword order, in double."""
    k = len(L)
    j = np.arange(1 << k, dtype=np.uint64)
    x = np.zeros(1 << k, dtype=np.uint64)
    for r in range(k):
        x ^= np.where((j >> np.uint64(k - 1 - r)) & np.uint64(1), np.uint64(int(L[r])), np.uint64(0))
    w = np.array([bin(int(v)).count("1") // 2 for v in x], dtype=np.int64)
    return float(np.cumsum(2.0 ** (-w.astype(np.float64)))[-1])


@pytest.mark.gpu
def test_fidelity_sum_matches_reference_loop(gpu):
    rs = np.random.RandomState(41)
    for t, k in ((5, 3), (12, 6), (24, 11), (40, 16), (64, 12), (17, 17)):
        L = [rand_word(rs, t) for _ in range(k)]
        assert gpu.fidelity_sum(t, L) == _zl_reference_loop(t, L), (t, k)


@pytest.mark.gpu
def test_decompose_with_fidelity_on_gpu_equals_host(gpu):
    # k given (one draw of L) or small t with a loose bound: with the reference's
    # integer-division Z(L), an autopicked k at large t never reaches the bound
    for t, fb, kk, force_l in ((8, 0.3, 0, True), (9, 0.35, 0, True), (31, 0.02, 14, False), (40, 0.01, 16, False),
                               (48, 0.02, 12, False)):
        host = backend.decompose(t, fb, False, True, force_l, False, kk)
        dev = gpu.decompose(t, fb, False, True, force_l, False, kk)
        assert host[:3] == dev[:3], t
        assert (host[3] is None and dev[3] is None) or list(host[3]) == list(dev[3])


@pytest.mark.gpu
def test_decompose_fidelity_loop_is_bounded(gpu):
    """A fidelity bound out of reach fails after a bounded number of draws of L
    (the reference's loop, probability.c:355, never ends).  With delta = 1e-300
    the loop needs 2^k v^2t / Z(L) >= 1.0, and the integer-division Z(L) is at
    least the true one, whose fidelity is below 1; forceL keeps k = t = 12."""
    with pytest.raises(backend.CsimError):
        gpu.decompose(12, 1e-300, False, True, True, False, 0)

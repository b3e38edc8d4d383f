"""The drop-in sampler at the sample counts real queries use, and the committed
benchmark workloads, against the oracle and the reference backend.

* The reference-draw sampler (CSIM_RNG_LIBC) at counts that cross every
  hand-off of the host sampler: sub-batches of 64, 256, then 1024 states, and
  batches of 16384 states, with bins > 1.  Values within 1e-12
  relative of the oracle's multiSampledProjector on the same seed
  (libcirc/innerprod.c:23-84).
* workload_c1.txt (the c1 query: t = 12, exact decomposition chi = 2^6,
  2000 states per projector, forceSample) through the gpubackend executable,
  against the reference backend's own output on the same seeds
  (workload_c1_ref.json, recorded by make_workloads.py).
* workload_c2.txt (t = 40, the query's own k = 16 code and projectors):
  10^5 (theta, term) pairs bit-exact against the oracle, and the backend's
  numerator/denominator at 2 states per projector against the oracle.
"""
import json
import os

import numpy as np
import pytest

from circuitsimulator_gb300 import backend
from helpers import close, rand_word, random_projector_rows
from oracle_ffi import make_projector

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
REL = 1e-12
FLOOR = 1e-12


@pytest.fixture(scope="module")
def gpu():
    b = backend.Backend(0)
    yield b
    b.close()


@pytest.fixture(scope="module")
def exe():
    if not os.path.exists(backend.EXE_PATH):
        from circuitsimulator_gb300.build import build

        build()
    return backend.EXE_PATH


def _projectors(t, rows):
    return backend.projector(rows[0], rows[1], rows[2], t), make_projector(rows[0], rows[1], rows[2], t)


# ---------------------------------------------------------------- the libc-draw sampler at realistic L
@pytest.mark.parametrize("t,k,samples,bins", [(40, 3, 65, 1), (40, 3, 321, 1), (40, 3, 2000, 1), (40, 2, 5900, 3),
                                               (24, 6, 1500, 2)])
def test_libc_sampler_at_realistic_counts(gpu, oracle, t, k, samples, bins):
    """65 and 321 states: one past the first (64) and second (256) sub-batch;
    2000: the reference's default L, three sub-batch boundaries; 3 x 5900 =
    17700: past the 16384-state batch boundary, with a median over three bins."""
    rs = np.random.RandomState(500 + samples)
    L = [rand_word(rs, t) for _ in range(k)]
    rows = random_projector_rows(rs, t, max(2, t // 6))
    Pg, Po = _projectors(t, rows)
    seed = 1000 + samples
    Lo = np.array(L, dtype=np.uint64)
    want, want_vals = oracle.multi_sampled_projector_mt(Po, Lo, k, 0, 1.0, samples, bins, oracle.rng(seed))
    vals = gpu.singleProjectorSample(Pg, L, False, samples * bins, backend.RNG_LIBC, seed)
    bad = [i for i in range(len(vals)) if not close(vals[i], want_vals[i], REL, FLOOR)]
    assert not bad, (len(bad), bad[:5])
    assert (want_vals == 0).sum() < len(want_vals)  # not every state annihilated
    v = gpu.multiSampledProjector(Pg, L, False, 1.0, samples, bins, backend.RNG_LIBC, seed)
    assert close(v, want, REL, FLOOR), (v, want)


def test_libc_sampler_stream_continues_across_calls(gpu, oracle):
    """The numerator and the denominator draw from one stream (the second call
    passes SEED_CONTINUE), as probability.c:182-198 does."""
    rs = np.random.RandomState(77)
    t, k = 40, 3
    L = [rand_word(rs, t) for _ in range(k)]
    rg = random_projector_rows(rs, t, 7)
    rh = random_projector_rows(rs, t, 5)
    (Gg, Go), (Hg, Ho) = _projectors(t, rg), _projectors(t, rh)
    r = oracle.rng(31)
    Lo = np.array(L, dtype=np.uint64)
    num, _ = oracle.multi_sampled_projector_mt(Go, Lo, k, 0, 1.0, 300, 1, r)
    den, _ = oracle.multi_sampled_projector_mt(Ho, Lo, k, 0, 1.0, 300, 1, r)
    gnum = gpu.multiSampledProjector(Gg, L, False, 1.0, 300, 1, backend.RNG_LIBC, 31)
    gden = gpu.multiSampledProjector(Hg, L, False, 1.0, 300, 1, backend.RNG_LIBC, backend.SEED_CONTINUE)
    assert close(gnum, num, REL, FLOOR) and close(gden, den, REL, FLOOR), ((gnum, num), (gden, den))


# ---------------------------------------------------------------- workload c1 against the reference backend
def _c1_cases():
    with open(os.path.join(GOLDEN, "workload_c1_ref.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("case", _c1_cases(), ids=lambda c: "seed%d" % c["seed"])
def test_c1_workload_matches_reference_backend(exe, case):
    text = open(os.path.join(GOLDEN, "workload_c1.txt")).read()
    rc, lines = backend.run_backend(text, seed=case["seed"], timeout=600)
    assert rc == 0, lines[-5:]
    ref = case["ref"]
    for a, b in zip(lines[-2:], ref[-2:]):
        assert close(float(a), float(b), REL, FLOOR), (a, b)
    assert float(lines[-1]) > 0 and float(lines[-2]) > 0


# ---------------------------------------------------------------- workload c2: its own code and projectors
def _c2():
    text = open(os.path.join(GOLDEN, "workload_c2.txt")).read()
    cfg, projs = backend.parse_protocol(text)
    return text, cfg, projs


def _c2_code(oracle, cfg):
    e, k, norm, L = oracle.decompose(cfg["t"], cfg["fidbound"], cfg["rank"], cfg["fidelity"], cfg["forceL"],
                                     cfg["exact"], cfg["k"], oracle.rng(1))
    assert e == 0 and k == 16
    return L, norm


@pytest.mark.slow
def test_c2_workload_pairs_bit_exact(gpu, oracle):
    """The c2 query's k = 16 code (decompose on the unseeded rand() stream, as
    the backend runs it) and its G' projector: states drawn with the reference's
    rand() stream and projected by the oracle; all 2^16 terms of 8 surviving
    states on the GPU, and 98,304 of those pairs against the oracle."""
    _, cfg, projs = _c2()
    L, _ = _c2_code(oracle, cfg)
    t = cfg["t"]
    ph, xs, zs, nq = projs[0]
    Po = make_projector(ph, xs, zs, nq)
    r = oracle.rng(4096)
    th = []
    while len(th) < 8:
        s = oracle.random_state(t, r)
        if oracle.project(s, Po) != 0:
            th.append(s)
    th = np.concatenate([np.asarray(s).reshape(-1) for s in th])
    eps, p, m = gpu.term_products(t, False, L, th, 0, 1 << 16)
    rs = np.random.RandomState(16)
    nthreads = os.cpu_count() or 1
    checked = 0
    for a in range(len(th)):
        for j0 in rs.choice((1 << 16) // 1024, size=12, replace=False) * 1024:
            j0 = int(j0)
            eo, po, mo = oracle.term_products(t, 0, L, 16, th[a:a + 1], j0, 1024, threads=nthreads)
            assert (eps[a, j0:j0 + 1024] == eo).all() and (p[a, j0:j0 + 1024] == po).all() \
                and (m[a, j0:j0 + 1024] == mo).all(), (a, j0)
            checked += 1024
    assert checked >= 98000


@pytest.mark.slow
def test_c2_workload_backend_against_oracle(exe, oracle):
    """The c2 query through the gpubackend executable with 2 states per
    projector (the full query's 4096 would take the oracle hours): numerator
    and denominator within 1e-12 of the oracle's multiSampledProjector on the
    same rand() stream, 2 x 2 x 65,536 pairs."""
    text, cfg, projs = _c2()
    tok = text.split()
    tok[3] = "2"  # samples
    rc, lines = backend.run_backend("\n".join(tok) + "\n", seed=777, timeout=600)
    assert rc == 0, lines[-5:]
    L, norm = _c2_code(oracle, cfg)
    r = oracle.rng(777)
    want = []
    for (ph, xs, zs, nq) in projs:
        v, _ = oracle.multi_sampled_projector_mt(make_projector(ph, xs, zs, nq), L, 16, 0, norm, 2, 1, r)
        want.append(v)
    got = [float(x) for x in lines[-2:]]
    assert close(got[0], want[0], REL, FLOOR) and close(got[1], want[1], REL, FLOOR), (got, want)


# ---------------------------------------------------------------- exact projector by row ranges
@pytest.mark.parametrize("t,exact,k", [(9, True, 0), (14, False, 7), (33, False, 6)])
def test_exact_projector_rows_compose(gpu, t, exact, k):
    """Rows of exactProjector taken in ranges (as ranks of the sharded exact
    mode take them) and added in row order give csim_exact_projector's value
    bit for bit."""
    from circuitsimulator_gb300 import shard

    rs = np.random.RandomState(90 + t)
    L = None if exact else [rand_word(rs, t) for _ in range(k)]
    rows = random_projector_rows(rs, t, max(2, t // 4))
    P = backend.projector(rows[0], rows[1], rows[2], t)
    whole = gpu.exactProjector(P, L, exact, 1.0)
    chi = (1 << ((t + 1) // 2)) if exact else (1 << k)
    for world in (1, 2, 3):
        tr = ti = 0.0
        for r in range(world):
            lo, hi = shard.row_bounds(chi, r, world)
            re, im = gpu.exactProjectorRows(P, L, exact, lo, hi)
            for a in re:
                tr += float(a)
            for b in im:
                ti += float(b)
        assert float(np.sqrt(tr * tr + ti * ti)) == whole, world


# ---------------------------------------------------------------- autotuner
def test_autotuner_leaves_results_and_streams_unchanged():
    """A context that tunes on first use (the default) and one with the fixed
    rules give the same values, with the reference's rand() stream continued
    across a call that tunes a new t bucket in between; the tuned parameters
    are among the candidates."""
    rs = np.random.RandomState(12)
    a, b = backend.Backend(0), backend.Backend(0)
    try:
        b.set_option(backend.OPT_AUTOTUNE, 0)
        out = []
        for g in (a, b):
            vals = []
            for (t, k, seed) in ((22, 9, 5), (45, 10, backend.SEED_CONTINUE), (22, 9, backend.SEED_CONTINUE)):
                rr = np.random.RandomState(t)
                L = [rand_word(rr, t) for _ in range(k)]
                rows = random_projector_rows(rr, t, max(2, t // 3))
                P = backend.projector(rows[0], rows[1], rows[2], t)
                vals.append(g.singleProjectorSample(P, L, False, 40, backend.RNG_LIBC, seed))
            out.append(np.concatenate(vals))
        assert (out[0] == out[1]).all()
        for t in (22, 45):
            pt, lz, ms, kern = a.autotune(t)
            assert pt in (16, 32) and kern in (0, 1, 2, 3) and ms > 0, (t, pt, lz, kern)
            if kern == 3:  # the direct kernel's own bound: t - 33 above 32 qubits, else ceil(0.6 t)
                assert lz == (t - 33 if t > 32 else min(t, (3 * t + 4) // 5)), (t, lz)
            else:
                assert kern == 2 or lz in {min(t, (f * t + 99) // 100) for f in (50, 55, 60, 70)}, (t, lz)
        pt, lz, ms, kern = b.autotune(60)  # explicit tuning works with the automatic one off
        assert pt in (16, 32) and ms > 0
    finally:
        a.close()
        b.close()


# ---------------------------------------------------------------- the run kernel
@pytest.mark.parametrize("t,k,pt", [(24, 11, 16), (40, 16, 32), (40, 12, 16), (57, 12, 32), (64, 14, 16)])
def test_run_kernel_equals_block_kernel(gpu, t, k, pt):
    """The sampler through the run kernel (codewords in per-thread runs that
    share their top-bit shrinks), through the block-prefix kernel with heavy and
    light launches, with one launch per occupancy class, and through the
    direct kernel (alone, with its launch split by codeword weight above 32
    qubits, and split with the block-prefix kernel by each state's number of
    non-pivot coordinates): identical values for every state (the sums are
    exact), on the same counter-based draws."""
    rs = np.random.RandomState(4000 + t + k)
    L = [rand_word(rs, t) for _ in range(k)]
    rows = random_projector_rows(rs, t, int(0.7 * t))
    P = backend.projector(rows[0], rows[1], rows[2], t)
    out = []
    try:
        gpu.set_option(backend.OPT_PER_THREAD, pt)
        for kernel in (2, 3, 4, 5):
            gpu.set_option(backend.OPT_PAIR_KERNEL, kernel)
            out.append(gpu.singleProjectorSample(P, L, False, 96, backend.RNG_PHILOX, 606))
        # the direct kernel with one constraint slot: states with n - k > 1 go to the block-prefix kernel
        gpu.set_option(backend.OPT_DIRECT_SLOTS, 1)
        out.append(gpu.singleProjectorSample(P, L, False, 96, backend.RNG_PHILOX, 606))
    finally:
        gpu.set_option(backend.OPT_DIRECT_SLOTS, 0)
        gpu.set_option(backend.OPT_PAIR_KERNEL, 0)
        gpu.set_option(backend.OPT_PER_THREAD, 0)
    for o in out[1:]:
        assert (o == out[0]).all()
    assert (out[0] != 0).sum() > 48

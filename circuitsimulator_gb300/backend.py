"""Python view of libcsimgpu.so (include/csim.h) with the reference's names.

Each method calls one C-ABI entry point; all stabilizer work runs in the
sm_103a kernels.  There is no CPU fallback: if the library is missing or no
GB300 is visible, construction fails with an exception.

    innerProductExact      libcirc/stabilizer/stabilizer.c:589
    exponentialSumExact    libcirc/stabilizer/stabilizer.c:300
    shrink                 libcirc/stabilizer/stabilizer.c:500
    measurePauli / extend  libcirc/stabilizer/stabilizer.c:827 / :759
    randomStabilizerState  libcirc/stabilizer/stabilizer.c:689
    prepH / prepL          libcirc/stateprep.c:36 / :85
    singleProjectorSample  libcirc/innerprod.c:88
    multiSampledProjector  libcirc/innerprod.c:23
    exactProjector         libcirc/innerprod.c:148
    decompose              libcirc/probability.c:307
    run_queries            many backend runs (libcirc/probability.c:44-221) in shared launches
    Server                 the same as a long-lived server with continuous batching
"""
import ctypes as C
import os
import subprocess

import numpy as np

from .state import STATE_DTYPE

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcsimgpu.so")
EXE_PATH = os.path.join(PKG, "gpubackend")

OPT_PAIR_KERNEL = 1
OPT_PER_THREAD = 2
OPT_AUTOTUNE = 3
OPT_DIRECT_SLOTS = 4
RNG_PHILOX = 0
RNG_LIBC = 1
SEED_CONTINUE = (1 << 64) - 1

_ERRORS = {-1: "bad argument", -2: "CUDA error", -3: "device check failed", -4: "out of memory",
           -5: "no sm_103 device", -6: "protocol error"}


class CsimError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("csim error %d (%s): %s" % (code, _ERRORS.get(code, "?"), msg))
        self.code = code


class Stats(C.Structure):
    """csim_stats of include/csim.h."""
    _fields_ = [("device_ms", C.c_double), ("pair_kernel_ms", C.c_double), ("states", C.c_int64),
                ("states_live", C.c_int64), ("pairs", C.c_int64), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64), ("kernels", C.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class _Projector(C.Structure):
    _fields_ = [("nstabs", C.c_int32), ("nqubits", C.c_int32), ("phase", C.c_void_p), ("xs", C.c_void_p),
                ("zs", C.c_void_p)]


class _Query(C.Structure):
    """csim_query of include/csim.h."""
    _fields_ = ([(n, C.c_int32) for n in ("quiet", "verbose", "noapprox", "samples", "bins", "t", "k", "exact")]
                + [("fidbound", C.c_double)]
                + [(n, C.c_int32) for n in ("fidelity", "rank", "force_l", "force_sample")]
                + [("G", _Projector), ("H", _Projector), ("rng", C.c_int32), ("reserved", C.c_int32),
                   ("seed", C.c_uint64)])


class _QueryResult(C.Structure):
    """csim_query_result of include/csim.h."""
    _fields_ = [("numerator", C.c_double), ("denominator", C.c_double), ("norm", C.c_double),
                ("status", C.c_int32), ("exact", C.c_int32), ("k", C.c_int32), ("noapprox", C.c_int32),
                ("pairs", C.c_int64), ("latency_s", C.c_double)]


PROTOCOL_FIELDS = ["quiet", "verbose", "noapprox", "samples", "bins", "t", "k", "exact", "fidbound", "fidelity",
                   "rank", "forceL", "forceSample"]


def parse_protocol(text):
    """The backend's stdin input: 13 scalars, then the projectors G' and H'
    (libcirc/probability.py:249-272, libcirc/utils/comms.c:9-36).  Returns
    (cfg dict, [(phases, xs, zs, nqubits)] * 2) with x/z rows as bit masks."""
    tok = text.split()
    cfg = {}
    for i, name in enumerate(PROTOCOL_FIELDS):
        cfg[name] = float(tok[i]) if name == "fidbound" else int(tok[i])
    pos = len(PROTOCOL_FIELDS)
    projs = []
    for _ in range(2):
        ns, nq = int(tok[pos]), int(tok[pos + 1])
        pos += 2
        ph, xs, zs = [], [], []
        for _ in range(ns):
            ph.append(int(tok[pos]))
            pos += 1
            x = z = 0
            for j in range(nq):
                if int(tok[pos]) & 1:
                    x |= 1 << j
                if int(tok[pos + 1]) & 1:
                    z |= 1 << j
                pos += 2
            xs.append(x)
            zs.append(z)
        projs.append((ph, xs, zs, nq))
    return cfg, projs


_lib = None


def load_library(path=LIB_PATH):
    """Loads libcsimgpu.so once; raises if it is missing (run circuitsimulator_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError("%s not built: run python -m circuitsimulator_gb300.build" % path)
    lib = C.CDLL(path)
    vp, i32, i64, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64
    sig = {
        "csim_ctx_create": ([C.c_int, C.POINTER(C.c_void_p)], C.c_int),
        "csim_ctx_destroy": ([vp], None),
        "csim_last_error": ([vp], C.c_char_p),
        "csim_launch_count": ([vp], i64),
        "csim_last_stats": ([vp, vp], C.c_int),
        "csim_set_option": ([vp, i32, i64], C.c_int),
        "csim_rng_position": ([vp, u64, u64], C.c_int),
        "csim_inner_product_exact": ([vp, i64, vp, vp, vp, vp, vp], C.c_int),
        "csim_exponential_sum_exact": ([vp, i64, vp, vp, vp, vp], C.c_int),
        "csim_shrink": ([vp, i64, vp, vp, vp, i32, vp], C.c_int),
        "csim_measure_pauli": ([vp, i64, vp, vp, vp, vp, vp], C.c_int),
        "csim_extend": ([vp, i64, vp, vp], C.c_int),
        "csim_random_states": ([vp, i32, i64, u64, u64, vp], C.c_int),
        "csim_random_states_replay": ([vp, i32, i64, vp, vp, vp], C.c_int),
        "csim_prep_h": ([vp, i32, i64, vp, vp], C.c_int),
        "csim_prep_l": ([vp, i32, vp, i32, i64, vp, vp], C.c_int),
        "csim_term_products": ([vp, i32, i32, vp, i32, i64, vp, i64, i64, vp, vp, vp], C.c_int),
        "csim_single_projector_samples": ([vp, vp, vp, i32, i32, i64, i32, u64, vp], C.c_int),
        "csim_multi_sampled_projector": ([vp, vp, vp, i32, i32, C.c_double, i32, i32, i32, u64, vp], C.c_int),
        "csim_exact_projector": ([vp, vp, vp, i32, i32, C.c_double, vp], C.c_int),
        "csim_exact_projector_rows": ([vp, vp, vp, i32, i32, i64, i64, vp, vp], C.c_int),
        "csim_median_of_means": ([vp, i32, i32, vp], C.c_int),
        "csim_autotune": ([vp, i32, vp, vp, i32, vp, vp, vp, vp], C.c_int),
        "csim_decompose": ([i32, C.c_double, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp], C.c_int),
        "csim_decompose_on": ([vp, i32, C.c_double, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp], C.c_int),
        "csim_fidelity_sum": ([vp, i32, vp, i32, vp], C.c_int),
        "csim_run_queries": ([vp, i64, vp, vp, i32], C.c_int),
        "csim_server_create": ([vp, vp], C.c_int),
        "csim_submit": ([vp, vp, vp], C.c_int),
        "csim_poll": ([vp, i64, vp], C.c_int),
        "csim_wait": ([vp, i64, C.c_double, vp], C.c_int),
        "csim_release": ([vp, i64], C.c_int),
        "csim_server_get_stats": ([vp, vp], C.c_int),
        "csim_server_destroy": ([vp], None),
        "csim_libc_rand_size": ([], i64),
        "csim_libc_rand_seed": ([vp, C.c_uint32], None),
        "csim_libc_rand_next": ([vp], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _states(a):
    a = np.ascontiguousarray(a)
    if a.dtype != STATE_DTYPE:
        raise TypeError("expected csim_state records")
    return a.reshape(-1)


def projector(phases, xs, zs, nqubits):
    """Protocol-encoded projector -> ctypes struct (keeps its arrays alive)."""
    ph = np.ascontiguousarray(np.asarray(phases, dtype=np.int32).reshape(-1))
    xa = np.ascontiguousarray(np.asarray([int(x) for x in xs], dtype=np.uint64).reshape(-1))
    za = np.ascontiguousarray(np.asarray([int(z) for z in zs], dtype=np.uint64).reshape(-1))
    P = _Projector(len(ph), int(nqubits), _p(ph) if len(ph) else None, _p(xa) if len(ph) else None,
                   _p(za) if len(ph) else None)
    P._keep = (ph, xa, za)
    return P


def median_of_means(values, samples, bins):
    """multiSampledProjector's reduction of samples x bins values in draw order
    (libcirc/innerprod.c:17-41): bin means, then the median as the C library's
    qsort orders them with the truncating comparator.  The same native code
    reduces csim_multi_sampled_projector's values; needs no GPU."""
    v = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
    if len(v) != int(samples) * int(bins):
        raise ValueError("need samples * bins values")
    out = C.c_double(0)
    rc = load_library().csim_median_of_means(_p(v), int(samples), int(bins), C.byref(out))
    if rc:
        raise CsimError(rc, "median_of_means")
    return out.value


class LibcRand:
    """The C library's srand()/rand() sequence as a value (csim_libc_rand_*)."""

    def __init__(self, seed=1):
        lib = load_library()
        self._buf = C.create_string_buffer(int(lib.csim_libc_rand_size()))
        lib.csim_libc_rand_seed(self._buf, int(seed) & 0xFFFFFFFF)

    def rand(self):
        return load_library().csim_libc_rand_next(self._buf)


def decompose(t, fidbound=1e-5, rank=False, fidelity=False, forceL=False, exact=False, k=0, rng=None):
    """decompose() of libcirc/probability.c:307 -> (exact, k, norm, L or None)."""
    lib = load_library()
    rng = rng or LibcRand(1)
    e, kk, norm = C.c_int32(int(bool(exact))), C.c_int32(int(k or 0)), C.c_double(0)
    L = np.zeros(64, dtype=np.uint64)
    rc = lib.csim_decompose(int(t), float(fidbound), int(bool(rank)), int(bool(fidelity)), int(bool(forceL)), 0, 1,
                            C.byref(e), C.byref(kk), C.byref(norm), _p(L), rng._buf, None)
    if rc:
        raise CsimError(rc, "decompose")
    return bool(e.value), kk.value, norm.value, (None if e.value else L[: kk.value].copy())


class Backend:
    """One csim_ctx: a CUDA stream, device buffers and random streams on one GB300."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.csim_ctx_create(int(device), C.byref(h))
        if rc:
            raise CsimError(rc, "cannot open device %d" % device)
        self.ctx = h

    def close(self):
        if self.ctx:
            self.lib.csim_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise CsimError(rc, self.lib.csim_last_error(self.ctx).decode())

    @property
    def launches(self):
        return int(self.lib.csim_launch_count(self.ctx))

    def set_option(self, option, value):
        """CSIM_OPT_PAIR_KERNEL = 1 (0 thread-per-pair, 1 warp-per-pair), CSIM_OPT_PER_THREAD = 2,
        CSIM_OPT_AUTOTUNE = 3 (1 tune on first use, 0 fixed rules)."""
        self._check(self.lib.csim_set_option(self.ctx, int(option), int(value)))

    def autotune(self, t, P=None, L=None):
        """Tunes t's bucket if this process has not yet (csim_autotune), on
        projector P and code L when given; returns (terms per thread,
        light-launch zero bound, pair-kernel ms of the winning trial, kernel:
        0 block-prefix heavy/light, 1 per-thread runs, 2 per occupancy class)."""
        kern, pt, lz, ms = C.c_int32(0), C.c_int32(0), C.c_int32(0), C.c_double(0)
        Lp = np.ascontiguousarray(np.asarray([int(x) for x in (L if L is not None else [])] or [0], dtype=np.uint64))
        k = 0 if L is None else len(L)
        self._check(self.lib.csim_autotune(self.ctx, int(t), C.byref(P) if P is not None else None, _p(Lp), int(k),
                                           C.byref(kern), C.byref(pt), C.byref(lz), C.byref(ms)))
        return pt.value, lz.value, ms.value, kern.value

    def rng_position(self, seed, first):
        """Next CSIM_RNG_PHILOX draw (with SEED_CONTINUE) is state `first` of stream `seed`."""
        self._check(self.lib.csim_rng_position(self.ctx, int(seed), int(first)))

    def last_stats(self):
        st = Stats()
        self._check(self.lib.csim_last_stats(self.ctx, C.byref(st)))
        return st

    # ---------------------------------------------------------------- primitives
    def innerProductExact(self, a, b):
        a, b = _states(a), _states(b)
        n = len(a)
        eps, p, m = (np.zeros(n, dtype=np.int32) for _ in range(3))
        self._check(self.lib.csim_inner_product_exact(self.ctx, n, _p(a), _p(b), _p(eps), _p(p), _p(m)))
        return eps, p, m

    def exponentialSumExact(self, s):
        """Returns (eps, p, m) and updates the states in place."""
        s = _states(s)
        n = len(s)
        eps, p, m = (np.zeros(n, dtype=np.int32) for _ in range(3))
        self._check(self.lib.csim_exponential_sum_exact(self.ctx, n, _p(s), _p(eps), _p(p), _p(m)))
        return eps, p, m

    def shrink(self, s, xi, alpha, lazy=False):
        s = _states(s)
        n = len(s)
        xi = np.ascontiguousarray(np.broadcast_to(np.asarray(xi, dtype=np.uint64), (n,)))
        al = np.ascontiguousarray(np.broadcast_to(np.asarray(alpha, dtype=np.int32), (n,)))
        st = np.zeros(n, dtype=np.int32)
        self._check(self.lib.csim_shrink(self.ctx, n, _p(s), _p(xi), _p(al), int(bool(lazy)), _p(st)))
        return st

    def measurePauli(self, s, m, zeta, xi):
        s = _states(s)
        n = len(s)
        m = np.ascontiguousarray(np.broadcast_to(np.asarray(m, dtype=np.int32), (n,)))
        z = np.ascontiguousarray(np.broadcast_to(np.asarray(zeta, dtype=np.uint64), (n,)))
        x = np.ascontiguousarray(np.broadcast_to(np.asarray(xi, dtype=np.uint64), (n,)))
        norm = np.zeros(n, dtype=np.float64)
        self._check(self.lib.csim_measure_pauli(self.ctx, n, _p(s), _p(m), _p(z), _p(x), _p(norm)))
        return norm

    def extend(self, s, xi):
        s = _states(s)
        n = len(s)
        x = np.ascontiguousarray(np.broadcast_to(np.asarray(xi, dtype=np.uint64), (n,)))
        self._check(self.lib.csim_extend(self.ctx, n, _p(s), _p(x)))

    def randomStabilizerState(self, n, count=1, seed=0, first=0):
        out = np.zeros(int(count), dtype=STATE_DTYPE)
        self._check(self.lib.csim_random_states(self.ctx, int(n), int(count), int(seed), int(first), _p(out)))
        return out

    def randomStabilizerStateReplay(self, n, words, offsets):
        words = np.ascontiguousarray(words, dtype=np.uint32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        out = np.zeros(len(offsets) - 1, dtype=STATE_DTYPE)
        self._check(self.lib.csim_random_states_replay(self.ctx, int(n), len(out), _p(words), _p(offsets), _p(out)))
        return out

    def prepH(self, idx, t):
        idx = np.ascontiguousarray(np.atleast_1d(np.asarray(idx, dtype=np.int64)))
        out = np.zeros(len(idx), dtype=STATE_DTYPE)
        self._check(self.lib.csim_prep_h(self.ctx, int(t), len(idx), _p(idx), _p(out)))
        return out

    def prepL(self, idx, t, L):
        idx = np.ascontiguousarray(np.atleast_1d(np.asarray(idx, dtype=np.int64)))
        L = np.ascontiguousarray(np.asarray([int(x) for x in L], dtype=np.uint64))
        out = np.zeros(len(idx), dtype=STATE_DTYPE)
        self._check(self.lib.csim_prep_l(self.ctx, int(t), _p(L), len(L), len(idx), _p(idx), _p(out)))
        return out

    # ---------------------------------------------------------------- hot path
    def term_products(self, t, exact, L, theta, j0, nj):
        """(eps, p, m) of <theta_a|phi_j>, shape (len(theta), nj)."""
        theta = _states(theta)
        Lp = np.ascontiguousarray(np.asarray([int(x) for x in (L if L is not None else [])] or [0], dtype=np.uint64))
        k = 0 if L is None else len(L)
        na = len(theta)
        eps, p, m = (np.zeros(na * nj, dtype=np.int32) for _ in range(3))
        self._check(self.lib.csim_term_products(self.ctx, int(t), int(bool(exact)), _p(Lp), int(k), na, _p(theta),
                                                int(j0), int(nj), _p(eps), _p(p), _p(m)))
        return eps.reshape(na, nj), p.reshape(na, nj), m.reshape(na, nj)

    def singleProjectorSample(self, P, L, exact, count, rng=RNG_LIBC, seed=SEED_CONTINUE):
        Lp = np.ascontiguousarray(np.asarray([int(x) for x in (L if L is not None else [])] or [0], dtype=np.uint64))
        k = 0 if L is None else len(L)
        vals = np.zeros(int(count), dtype=np.float64)
        self._check(self.lib.csim_single_projector_samples(self.ctx, C.byref(P), _p(Lp), int(k), int(bool(exact)),
                                                           int(count), int(rng), int(seed), _p(vals)))
        return vals

    def multiSampledProjector(self, P, L, exact, norm, samples, bins=1, rng=RNG_LIBC, seed=SEED_CONTINUE):
        Lp = np.ascontiguousarray(np.asarray([int(x) for x in (L if L is not None else [])] or [0], dtype=np.uint64))
        k = 0 if L is None else len(L)
        out = C.c_double(0)
        self._check(self.lib.csim_multi_sampled_projector(self.ctx, C.byref(P), _p(Lp), int(k), int(bool(exact)),
                                                          float(norm), int(samples), int(bins), int(rng), int(seed),
                                                          C.byref(out)))
        return out.value

    def exactProjector(self, P, L, exact, norm):
        Lp = np.ascontiguousarray(np.asarray([int(x) for x in (L if L is not None else [])] or [0], dtype=np.uint64))
        k = 0 if L is None else len(L)
        out = C.c_double(0)
        self._check(self.lib.csim_exact_projector(self.ctx, C.byref(P), _p(Lp), int(k), int(bool(exact)),
                                                  float(norm), C.byref(out)))
        return out.value

    def exactProjectorRows(self, P, L, exact, i0, i1):
        """Rows [i0, i1) of exactProjector as (re, im) arrays (csim_exact_projector_rows)."""
        Lp = np.ascontiguousarray(np.asarray([int(x) for x in (L if L is not None else [])] or [0], dtype=np.uint64))
        k = 0 if L is None else len(L)
        n = max(0, int(i1) - int(i0))
        re, im = np.zeros(max(n, 1)), np.zeros(max(n, 1))
        self._check(self.lib.csim_exact_projector_rows(self.ctx, C.byref(P), _p(Lp), int(k), int(bool(exact)),
                                                       int(i0), int(i1), _p(re), _p(im)))
        return re[:n], im[:n]

    def decompose(self, t, fidbound=1e-5, rank=False, fidelity=False, forceL=False, exact=False, k=0, rng=None):
        """decompose() with the fidelity sum on this GPU (csim_decompose_on)."""
        rng = rng or LibcRand(1)
        e, kk, norm = C.c_int32(int(bool(exact))), C.c_int32(int(k or 0)), C.c_double(0)
        L = np.zeros(64, dtype=np.uint64)
        self._check(self.lib.csim_decompose_on(self.ctx, int(t), float(fidbound), int(bool(rank)),
                                               int(bool(fidelity)), int(bool(forceL)), 0, 1, C.byref(e),
                                               C.byref(kk), C.byref(norm), _p(L), rng._buf, None))
        return bool(e.value), kk.value, norm.value, (None if e.value else L[: kk.value].copy())

    def fidelity_sum(self, t, L):
        """Z(L) = sum over codewords x of 2^(-|x|/2) (probability.c:391-398) on the GPU."""
        Lp = np.ascontiguousarray(np.asarray([int(x) for x in L] or [0], dtype=np.uint64))
        out = C.c_double(0)
        self._check(self.lib.csim_fidelity_sum(self.ctx, int(t), _p(Lp), len(L), C.byref(out)))
        return out.value

    def run_queries(self, queries, batched=True, check=True):
        """Runs backend queries (libcirc/probability.c:44-221) through csim_run_queries.

        queries: list of dicts with the protocol text under "input" (or "cfg" and
        "projs" from parse_protocol), "seed", and optionally "rng" (RNG_LIBC by
        default, like the reference's rand()).  batched=False runs them one after
        another through the single-query entry points.  Returns one dict per
        query: numerator, denominator, norm, status, exact, k, noapprox, pairs."""
        n = len(queries)
        qs = (_Query * max(n, 1))()
        keep = []
        for i, q in enumerate(queries):
            _fill_query(qs[i], q, keep)
        rs = (_QueryResult * max(n, 1))()
        rc = self.lib.csim_run_queries(self.ctx, n, qs, rs, int(bool(batched)))
        if check:
            self._check(rc)
        return [_result_dict(rs[i]) for i in range(n)]


def _fill_query(qq, q, keep):
    cfg, projs = (q["cfg"], q["projs"]) if "cfg" in q else parse_protocol(q["input"])
    G = projector(*projs[0])
    H = projector(*projs[1])
    keep += [G, H]
    qq.quiet, qq.verbose, qq.noapprox = cfg["quiet"], cfg["verbose"], cfg["noapprox"]
    qq.samples, qq.bins, qq.t, qq.k, qq.exact = cfg["samples"], cfg["bins"], cfg["t"], cfg["k"], cfg["exact"]
    qq.fidbound = cfg["fidbound"]
    qq.fidelity, qq.rank, qq.force_l, qq.force_sample = cfg["fidelity"], cfg["rank"], cfg["forceL"], cfg["forceSample"]
    qq.G, qq.H = G, H
    qq.rng = int(q.get("rng", RNG_LIBC))
    qq.seed = int(q["seed"])


def _result_dict(r):
    return {f: getattr(r, f) for f, _ in r._fields_}


class _ServerConfig(C.Structure):
    """csim_server_config of include/csim.h."""
    _fields_ = [("device", C.c_int32), ("per_thread", C.c_int32), ("hbm_budget_bytes", C.c_int64),
                ("round_pairs", C.c_int64), ("round_states", C.c_int64)]


class _ServerStats(C.Structure):
    """csim_server_stats of include/csim.h."""
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "rounds", "pairs", "resident_bytes",
                                         "resident_decompositions", "queued")] + [("device_ms", C.c_double)]


PENDING = 1


class Server:
    """A query server on one GPU (csim_server_*): submit backend queries from
    any thread, poll or wait for their results.  Queries that arrive while
    others run join the next round of shared launches."""

    def __init__(self, device=0, hbm_budget_bytes=0, round_pairs=0, round_states=0, per_thread=0):
        self.lib = load_library()
        cfg = _ServerConfig(int(device), int(per_thread), int(hbm_budget_bytes), int(round_pairs),
                            int(round_states))
        h = C.c_void_p()
        rc = self.lib.csim_server_create(C.byref(cfg), C.byref(h))
        if rc:
            raise CsimError(rc, "csim_server_create on device %d" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.csim_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, query):
        qq = _Query()
        keep = []
        _fill_query(qq, query, keep)
        t = C.c_int64()
        rc = self.lib.csim_submit(self.h, C.byref(qq), C.byref(t))
        if rc:
            raise CsimError(rc, "csim_submit")
        return t.value

    def poll(self, ticket):
        r = _QueryResult()
        rc = self.lib.csim_poll(self.h, int(ticket), C.byref(r))
        if rc == PENDING:
            return None
        if rc:
            raise CsimError(rc, "csim_poll %d" % ticket)
        return _result_dict(r)

    def wait(self, ticket, timeout=None):
        r = _QueryResult()
        rc = self.lib.csim_wait(self.h, int(ticket), -1.0 if timeout is None else float(timeout), C.byref(r))
        if rc == PENDING:
            return None
        if rc:
            raise CsimError(rc, "csim_wait %d" % ticket)
        return _result_dict(r)

    def release(self, ticket):
        return self.lib.csim_release(self.h, int(ticket))

    def stats(self):
        st = _ServerStats()
        self.lib.csim_server_get_stats(self.h, C.byref(st))
        return _result_dict(st)


def serve_backend(protocol_texts, seed, rng=None, timeout=None, exe=EXE_PATH):
    """Runs `gpubackend serve` on back-to-back protocol inputs; returns one
    (status, numerator, denominator) per input, in input order.  Query i is
    seeded with seed + i."""
    env = dict(os.environ, CSIM_SEED=str(int(seed)))
    if rng is not None:
        env["CSIM_RNG"] = rng
    r = subprocess.run([exe, "serve"], input="".join(t if t.endswith("\n") else t + "\n" for t in protocol_texts)
                       .encode(), stdout=subprocess.PIPE, stderr=subprocess.PIPE, env=env, timeout=timeout)
    out = []
    for ln in r.stdout.decode().splitlines():
        f = ln.split()
        if len(f) == 4 and f[0].isdigit():
            out.append((int(f[1]), float(f[2]), float(f[3])))
    return r.returncode, out


def run_backend(protocol_text, seed=None, rng=None, timeout=None, exe=EXE_PATH):
    """Runs the gpubackend executable on one stdin-protocol input; returns its
    stdout lines (the last two are numerator and denominator)."""
    env = dict(os.environ)
    if seed is not None:
        env["CSIM_SEED"] = str(int(seed))
    if rng is not None:
        env["CSIM_RNG"] = rng
    r = subprocess.run([exe, "stdin"], input=protocol_text.encode(), stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       env=env, timeout=timeout)
    return r.returncode, r.stdout.decode().splitlines()

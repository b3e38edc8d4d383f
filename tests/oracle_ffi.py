"""ctypes bindings for the two CPU checkers used by the tests:

* ``Oracle``  — oracle/liboracle.so, the C restatement of the reference
  algorithm (oracle/csim_oracle.c).  Built by ``make -C oracle`` (and by
  ``__graft_entry__.build()``), available wherever the tests run.
* ``RefLib``  — oracle/_ref/libcsimref.so, the reference's own C sources
  compiled unchanged (``make -C oracle ref``).  Only exists where the reference
  checkout exists; tests that need it skip otherwise.

Both are test infrastructure; nothing in the product imports this module.
"""
import ctypes as C
import os

import numpy as np

from circuitsimulator_gb300.state import STATE_DTYPE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "liboracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libcsimref.so")

_st_p = C.c_void_p
_u64 = C.c_uint64
_i32p = C.POINTER(C.c_int32)
_ip = C.POINTER(C.c_int)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class RngState(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("idx", C.c_int32),
        ("ring", C.c_uint32 * 34),
        ("words", C.c_void_p),
        ("pos", C.c_int64),
        ("end", C.c_int64),
        ("overrun", C.c_int32),
    ]


class Projector(C.Structure):
    _fields_ = [
        ("nstabs", C.c_int32),
        ("nqubits", C.c_int32),
        ("phase", C.c_void_p),
        ("xs", C.c_void_p),
        ("zs", C.c_void_p),
    ]


def make_projector(phases, xs, zs, nqubits):
    ph = np.ascontiguousarray(np.asarray(phases, dtype=np.int32).reshape(-1))
    xa = np.ascontiguousarray(np.asarray(xs, dtype=np.uint64).reshape(-1))
    za = np.ascontiguousarray(np.asarray(zs, dtype=np.uint64).reshape(-1))
    P = Projector(len(ph), int(nqubits), _ptr(ph) if len(ph) else None, _ptr(xa) if len(ph) else None,
                  _ptr(za) if len(ph) else None)
    P._keep = (ph, xa, za)
    return P


class Oracle:
    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} missing: run make -C oracle")
        lib = C.CDLL(path)
        self.lib = lib
        lib.orc_rng_seed.argtypes = [C.POINTER(RngState), C.c_uint32]
        lib.orc_rng_replay.argtypes = [C.POINTER(RngState), C.c_void_p, C.c_int64, C.c_int64]
        lib.orc_rand.argtypes = [C.POINTER(RngState)]
        lib.orc_rand.restype = C.c_int32
        lib.orc_state_init.argtypes = [_st_p, C.c_int, C.c_int]
        lib.orc_exponential_sum_exact.argtypes = [_st_p, _ip, _ip, _ip]
        lib.orc_shrink.argtypes = [_st_p, _u64, C.c_int, C.c_int]
        lib.orc_shrink.restype = C.c_int
        lib.orc_inner_product_exact.argtypes = [_st_p, _st_p, _ip, _ip, _ip]
        lib.orc_random_state.argtypes = [C.c_int, C.POINTER(RngState), _st_p]
        lib.orc_measure_pauli.argtypes = [_st_p, C.c_int, _u64, _u64]
        lib.orc_measure_pauli.restype = C.c_double
        lib.orc_extend.argtypes = [_st_p, _u64]
        lib.orc_prep_h.argtypes = [C.c_int64, C.c_int, _st_p]
        lib.orc_prep_l.argtypes = [C.c_int64, C.c_int, C.c_void_p, C.c_int, _st_p]
        lib.orc_codeword.argtypes = [C.c_int64, C.c_void_p, C.c_int]
        lib.orc_codeword.restype = C.c_uint64
        lib.orc_project.argtypes = [_st_p, C.POINTER(Projector)]
        lib.orc_project.restype = C.c_double
        lib.orc_single_projector_sample.argtypes = [C.POINTER(Projector), C.c_void_p, C.c_int, C.c_int,
                                                    C.POINTER(RngState)]
        lib.orc_single_projector_sample.restype = C.c_double
        lib.orc_multi_sampled_projector.argtypes = [C.POINTER(Projector), C.c_void_p, C.c_int, C.c_int,
                                                    C.c_double, C.c_int, C.c_int, C.POINTER(RngState)]
        lib.orc_multi_sampled_projector.restype = C.c_double
        lib.orc_multi_sampled_projector_mt.argtypes = [C.POINTER(Projector), C.c_void_p, C.c_int, C.c_int,
                                                       C.c_double, C.c_int, C.c_int, C.POINTER(RngState), C.c_int,
                                                       C.c_void_p]
        lib.orc_multi_sampled_projector_mt.restype = C.c_double
        lib.orc_exact_projector.argtypes = [C.POINTER(Projector), C.c_void_p, C.c_int, C.c_int, C.c_double]
        lib.orc_exact_projector.restype = C.c_double
        lib.orc_decompose.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _ip, _ip,
                                      C.POINTER(C.c_double), C.c_void_p, C.POINTER(RngState)]
        lib.orc_term_products.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int64, _st_p, C.c_int64,
                                          C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.orc_pair_rowops.argtypes = [_st_p, C.c_uint64, _ip, _ip, _ip, C.POINTER(C.c_int64)]
        self.assert_failures = C.c_int.in_dll(lib, "orc_assert_failures")

    # -- rng
    def rng(self, seed):
        r = RngState()
        self.lib.orc_rng_seed(C.byref(r), int(seed) & 0xFFFFFFFF)
        return r

    def rng_replay(self, words, begin=0, end=None):
        words = np.ascontiguousarray(words, dtype=np.uint32)
        r = RngState()
        self.lib.orc_rng_replay(C.byref(r), _ptr(words), int(begin), int(len(words) if end is None else end))
        r._keep = words
        return r

    def rand(self, r):
        return self.lib.orc_rand(C.byref(r))

    # -- states
    def state(self, n, k=None):
        s = np.zeros(1, dtype=STATE_DTYPE)
        self.lib.orc_state_init(_ptr(s), n, n if k is None else k)
        return s

    def random_state(self, n, r):
        s = np.zeros(1, dtype=STATE_DTYPE)
        self.lib.orc_random_state(n, C.byref(r), _ptr(s))
        return s

    def inner_product(self, a, b):
        e, p, m = C.c_int(0), C.c_int(0), C.c_int(0)
        self.lib.orc_inner_product_exact(_ptr(a), _ptr(b), C.byref(e), C.byref(p), C.byref(m))
        return e.value, p.value, m.value

    def exponential_sum(self, s):
        e, p, m = C.c_int(0), C.c_int(0), C.c_int(0)
        self.lib.orc_exponential_sum_exact(_ptr(s), C.byref(e), C.byref(p), C.byref(m))
        return e.value, p.value, m.value

    def shrink(self, s, xi, alpha, lazy=0):
        return self.lib.orc_shrink(_ptr(s), int(xi), int(alpha), int(lazy))

    def measure_pauli(self, s, m, zeta, xi):
        return self.lib.orc_measure_pauli(_ptr(s), int(m), int(zeta), int(xi))

    def extend(self, s, xi):
        self.lib.orc_extend(_ptr(s), int(xi))

    def prep_h(self, i, t):
        s = np.zeros(1, dtype=STATE_DTYPE)
        self.lib.orc_prep_h(int(i), int(t), _ptr(s))
        return s

    def prep_l(self, i, t, L):
        L = np.ascontiguousarray(L, dtype=np.uint64)
        s = np.zeros(1, dtype=STATE_DTYPE)
        self.lib.orc_prep_l(int(i), int(t), _ptr(L), len(L), _ptr(s))
        return s

    def codeword(self, i, L):
        L = np.ascontiguousarray(L, dtype=np.uint64)
        return int(self.lib.orc_codeword(int(i), _ptr(L), len(L)))

    def pair_rowops(self, theta, x):
        e, p, m, ops = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int64(0)
        self.lib.orc_pair_rowops(_ptr(theta), int(x), C.byref(e), C.byref(p), C.byref(m), C.byref(ops))
        return (e.value, p.value, m.value), ops.value

    def project(self, s, P):
        return self.lib.orc_project(_ptr(s), C.byref(P))

    def single_projector_sample(self, P, L, k, exact, r):
        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        return self.lib.orc_single_projector_sample(C.byref(P), _ptr(L), int(k), int(exact), C.byref(r))

    def multi_sampled_projector(self, P, L, k, exact, norm, samples, bins, r):
        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        return self.lib.orc_multi_sampled_projector(C.byref(P), _ptr(L), int(k), int(exact), float(norm),
                                                    int(samples), int(bins), C.byref(r))

    def multi_sampled_projector_mt(self, P, L, k, exact, norm, samples, bins, r, threads=None):
        """orc_multi_sampled_projector on host threads: (value, per-state values)."""
        import os

        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        vals = np.zeros(max(1, int(samples) * int(bins)), dtype=np.float64)
        v = self.lib.orc_multi_sampled_projector_mt(C.byref(P), _ptr(L), int(k), int(exact), float(norm),
                                                    int(samples), int(bins), C.byref(r),
                                                    int(threads or os.cpu_count() or 1), _ptr(vals))
        return v, vals[: int(samples) * int(bins)]

    def exact_projector(self, P, L, k, exact, norm):
        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        return self.lib.orc_exact_projector(C.byref(P), _ptr(L), int(k), int(exact), float(norm))

    def decompose(self, t, fidbound, rank, fidelity, forceL, exact, k, r):
        e, kk, norm = C.c_int(int(exact)), C.c_int(int(k)), C.c_double(0)
        L = np.zeros(64, dtype=np.uint64)
        self.lib.orc_decompose(int(t), float(fidbound), int(rank), int(fidelity), int(forceL), C.byref(e),
                               C.byref(kk), C.byref(norm), _ptr(L), C.byref(r))
        return e.value, kk.value, norm.value, L[: kk.value].copy() if not e.value else None

    def term_products(self, t, exact, L, k, theta, j0, nj, threads=1):
        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        theta = np.ascontiguousarray(theta)
        na = len(theta)
        eps = np.zeros(na * nj, dtype=np.int32)
        p = np.zeros_like(eps)
        m = np.zeros_like(eps)
        self.lib.orc_term_products(int(t), int(exact), _ptr(L), int(k), na, _ptr(theta), int(j0), int(nj),
                                   _ptr(eps), _ptr(p), _ptr(m), int(threads))
        return eps, p, m


class RefLib:
    """The reference's own C code (compiled from its sources) behind flat entry points."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        self.lib = lib
        lib.csimref_srand.argtypes = [C.c_uint]
        lib.csimref_rand.restype = C.c_int
        lib.csimref_record_begin.argtypes = [C.c_void_p, C.c_int64]
        lib.csimref_record_end.restype = C.c_int64
        lib.csimref_inner_product_exact.argtypes = [_st_p, _st_p, _ip, _ip, _ip]
        lib.csimref_exponential_sum_exact.argtypes = [_st_p, _ip, _ip, _ip]
        lib.csimref_shrink.argtypes = [_st_p, _u64, C.c_int, C.c_int]
        lib.csimref_shrink.restype = C.c_int
        lib.csimref_measure_pauli.argtypes = [_st_p, C.c_int, _u64, _u64]
        lib.csimref_measure_pauli.restype = C.c_double
        lib.csimref_extend.argtypes = [_st_p, _u64]
        lib.csimref_random_state.argtypes = [C.c_int, _st_p]
        lib.csimref_prep_h.argtypes = [C.c_int, C.c_int, _st_p]
        lib.csimref_prep_l.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, _st_p]
        pa = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        lib.csimref_single_projector_sample.argtypes = pa
        lib.csimref_single_projector_sample.restype = C.c_double
        lib.csimref_multi_sampled_projector.argtypes = pa + [C.c_double, C.c_int, C.c_int]
        lib.csimref_multi_sampled_projector.restype = C.c_double
        lib.csimref_exact_projector.argtypes = pa + [C.c_double]
        lib.csimref_exact_projector.restype = C.c_double
        lib.csimref_decompose.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _ip, _ip,
                                          C.POINTER(C.c_double), C.c_void_p]

    def srand(self, seed):
        self.lib.csimref_srand(int(seed) & 0xFFFFFFFF)

    def rand(self):
        return self.lib.csimref_rand()

    def record(self, fn, cap=1 << 22):
        """Run fn() while recording every rand() value the reference draws."""
        buf = np.zeros(cap, dtype=np.uint32)
        self.lib.csimref_record_begin(_ptr(buf), cap)
        try:
            out = fn()
        finally:
            n = self.lib.csimref_record_end()
        if n > cap:
            raise RuntimeError("rand() record overflow")
        return out, buf[:n].copy()

    def random_state(self, n):
        s = np.zeros(1, dtype=STATE_DTYPE)
        self.lib.csimref_random_state(int(n), _ptr(s))
        return s

    def inner_product(self, a, b):
        e, p, m = C.c_int(0), C.c_int(0), C.c_int(0)
        self.lib.csimref_inner_product_exact(_ptr(a), _ptr(b), C.byref(e), C.byref(p), C.byref(m))
        return e.value, p.value, m.value

    def exponential_sum(self, s):
        e, p, m = C.c_int(0), C.c_int(0), C.c_int(0)
        self.lib.csimref_exponential_sum_exact(_ptr(s), C.byref(e), C.byref(p), C.byref(m))
        return e.value, p.value, m.value

    def shrink(self, s, xi, alpha, lazy=0):
        return self.lib.csimref_shrink(_ptr(s), int(xi), int(alpha), int(lazy))

    def measure_pauli(self, s, m, zeta, xi):
        return self.lib.csimref_measure_pauli(_ptr(s), int(m), int(zeta), int(xi))

    def extend(self, s, xi):
        self.lib.csimref_extend(_ptr(s), int(xi))

    def prep_h(self, i, t):
        s = np.zeros(1, dtype=STATE_DTYPE)
        self.lib.csimref_prep_h(int(i), int(t), _ptr(s))
        return s

    def prep_l(self, i, t, L):
        L = np.ascontiguousarray(L, dtype=np.uint64)
        s = np.zeros(1, dtype=STATE_DTYPE)
        self.lib.csimref_prep_l(int(i), int(t), _ptr(L), len(L), _ptr(s))
        return s

    def _proj(self, P):
        return [P.nstabs, P.nqubits, P.phase, P.xs, P.zs]

    def single_projector_sample(self, P, L, k, exact):
        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        return self.lib.csimref_single_projector_sample(*self._proj(P), _ptr(L), int(k), int(exact))

    def multi_sampled_projector(self, P, L, k, exact, norm, samples, bins):
        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        return self.lib.csimref_multi_sampled_projector(*self._proj(P), _ptr(L), int(k), int(exact), float(norm),
                                                        int(samples), int(bins))

    def exact_projector(self, P, L, k, exact, norm):
        L = np.ascontiguousarray(L if L is not None else np.zeros(1), dtype=np.uint64)
        return self.lib.csimref_exact_projector(*self._proj(P), _ptr(L), int(k), int(exact), float(norm))

    def decompose(self, t, fidbound, rank, fidelity, forceL, exact, k):
        e, kk, norm = C.c_int(int(exact)), C.c_int(int(k)), C.c_double(0)
        L = np.zeros(64, dtype=np.uint64)
        self.lib.csimref_decompose(int(t), float(fidbound), int(rank), int(fidelity), int(forceL), C.byref(e),
                                   C.byref(kk), C.byref(norm), _ptr(L))
        return e.value, kk.value, norm.value, L[: kk.value].copy() if not e.value else None

"""The codeword order of the sampled estimators (ordered_codewords and
light_split in csim_host_common.h, compiled for the host): a permutation of
all 2^k codewords; first the heavy part (more than light_zeros(t) zeros), then
the light part, light_split at the boundary; within each part by the top
ordered_prefix_bits(k, t) bits, then weight, then value.  The pair kernels'
results do not depend on the order; their speed does."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "order_check.cpp")
SO = os.path.join(HERE, "native", "_build", "liborder.so")
HDR = os.path.join(os.path.dirname(HERE), "circuitsimulator_gb300", "csrc", "csim_host_common.h")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


@pytest.fixture(scope="module")
def lib():
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    if not os.path.exists(SO) or os.path.getmtime(SO) < max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + CUDA_INC, SRC, "-o", SO])
    lb = C.CDLL(SO)
    lb.order_codewords.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lb.order_codewords.restype = C.c_int64
    lb.order_runs.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    lb.order_runs.restype = C.c_int64
    lb.order_classes.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    lb.order_classes.restype = None
    return lb


def _codewords(L, k):
    out = []
    for j in range(1 << k):
        x = 0
        for r in range(k):
            if (j >> r) & 1:
                x ^= int(L[r])
        out.append(x)
    return out


@pytest.mark.parametrize("t,k", [(4, 2), (12, 6), (24, 12), (40, 16), (57, 12), (64, 14)])
def test_ordered_codewords(lib, t, k):
    rs = np.random.RandomState(t * 100 + k)
    L = np.array([int(rs.randint(1, 1 << 62)) & ((1 << t) - 1) for _ in range(k)], dtype=np.uint64)
    out = np.zeros(1 << k, dtype=np.uint64)
    split = lib.order_codewords(L.ctypes.data, k, t, out.ctypes.data)
    got = [int(v) for v in out]
    assert sorted(got) == sorted(_codewords(L, k))
    wmin = t - lib.order_light_zeros(t)
    d = lib.order_prefix_bits(k, t)
    pc = [bin(v).count("1") for v in got]
    assert all(w < wmin for w in pc[:split]) and all(w >= wmin for w in pc[split:])

    def key(v):
        return ((v >> (t - d)) if d else 0, bin(v).count("1"), v)

    for part in (got[:split], got[split:]):
        assert [key(v) for v in part] == sorted(key(v) for v in part)


def test_items_per_thread_by_t(lib):
    """Terms per thread per work item: 32 up to t = 52, 16 above, unless fixed
    (CSIM_OPT_PER_THREAD).  Results never depend on it; the kernels' speed does."""
    assert [lib.order_per_thread(0, t) for t in (1, 24, 40, 52, 53, 64)] == [32, 32, 32, 32, 16, 16]
    assert lib.order_per_thread(8, 40) == 8 and lib.order_per_thread(16, 24) == 16


def _agree_top(dis, n):
    nm = (1 << n) - 1
    d = dis & nm
    return nm if d == 0 else nm & ~((1 << d.bit_length()) - 1)


@pytest.mark.parametrize("t,k,pt,gl", [(24, 11, 16, 12), (40, 16, 32, 22), (40, 13, 16, 20), (64, 14, 16, 35)])
def test_run_order(lib, t, k, pt, gl):
    """The run kernel's order: a permutation of all 2^k codewords; in each block
    of 64 runs, thread r's run sits at positions r + 64 i; a run is pt codewords
    consecutive in value, sorted by their zeros below the run's agreed top bits;
    runs with a codeword of more such zeros than gl come before the split, which
    is a whole number of blocks, and none after it."""
    rs = np.random.RandomState(t * 7 + k)
    L = np.array([int(rs.randint(1, 1 << 62)) & ((1 << t) - 1) for _ in range(k)], dtype=np.uint64)
    out = np.zeros(1 << k, dtype=np.uint64)
    split = lib.order_runs(L.ctypes.data, k, t, pt, gl, out.ctypes.data)
    got = [int(v) for v in out]
    allcw = sorted(_codewords(L, k))
    assert sorted(got) == allcw
    assert split % (64 * pt) == 0
    rank = {v: i for i, v in enumerate(allcw)}
    nm = (1 << t) - 1
    for b0 in range(0, len(got), 64 * pt):
        for r in range(64):
            run = [got[b0 + r + 64 * i] for i in range(pt)]
            idx = sorted(rank[v] for v in run)
            assert idx == list(range(idx[0], idx[0] + pt)) and idx[0] % pt == 0  # consecutive in value
            am, om = nm, 0
            for v in run:
                am &= v
                om |= v
            low = nm & ~_agree_top(am ^ om, t)
            rem = [bin(~v & low).count("1") for v in run]
            assert rem == sorted(rem)
            if b0 >= split:
                assert max(rem) <= gl


@pytest.mark.parametrize("t,k", [(24, 12), (57, 12), (64, 14)])
def test_zero_class_order(lib, t, k):
    """Launches per zero class: with bounds {t, light_zeros(t)} the order is the
    heavy/light order itself; with more bounds, class c (at most bounds[c]
    zeros, more than bounds[c + 1]) starts at starts[c], classes in order, each
    ordered by top bits, weight and value."""
    rs = np.random.RandomState(t * 11 + k)
    L = np.array([int(rs.randint(1, 1 << 62)) & ((1 << t) - 1) for _ in range(k)], dtype=np.uint64)
    ref = np.zeros(1 << k, dtype=np.uint64)
    split = lib.order_codewords(L.ctypes.data, k, t, ref.ctypes.data)
    for bounds in ([t, lib.order_light_zeros(t)], [t, (7 * t) // 10, (3 * t) // 5, t // 2]):
        b = np.array(bounds, dtype=np.int32)
        out = np.zeros(1 << k, dtype=np.uint64)
        starts = np.zeros(len(bounds) + 1, dtype=np.int64)
        lib.order_classes(L.ctypes.data, k, t, b.ctypes.data, len(bounds), out.ctypes.data, starts.ctypes.data)
        got = [int(v) for v in out]
        assert sorted(got) == sorted(_codewords(L, k))
        if len(bounds) == 2:
            assert got == [int(v) for v in ref] and starts[1] == split
        d = lib.order_prefix_bits(k, t)
        assert starts[0] == 0 and starts[-1] == 1 << k and list(starts) == sorted(starts)
        for c in range(len(bounds)):
            part = got[starts[c]:starts[c + 1]]
            lo = bounds[c + 1] if c + 1 < len(bounds) else -1
            assert all(lo < t - bin(v).count("1") <= bounds[c] for v in part)
            key = [((v >> (t - d)) if d else 0, bin(v).count("1"), v) for v in part]
            assert key == sorted(key)

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

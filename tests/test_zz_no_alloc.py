"""csim_single_projector_samples_static: the sampler for callers that cannot
allocate device memory (their GPU memory belongs to their own pool allocator,
or is planned to the byte).  Its scratch is one fixed array inside the
library, so the check here is that it gives the same values as the allocating
entry point, csim_single_projector_samples, on two calls in a row (the second
call must not see stale scratch), and refuses inputs beyond its stated size.

Collected last (file name) so that a stop-at-first-failure run has already
run every other test; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from circuitsimulator_gb300 import backend
from helpers import close, rand_word, random_projector_rows

pytestmark = pytest.mark.gpu


def _static_fn():
    lib = backend.load_library()
    f = lib.csim_single_projector_samples_static
    f.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p]
    f.restype = C.c_int
    return f


def _call(f, P, L, count, seed):
    Lw = np.ascontiguousarray(np.asarray([int(x) for x in L] or [0], dtype=np.uint64))
    out = np.full(count, np.nan)
    rc = f(0, C.addressof(P), Lw.ctypes.data, len(L), count, seed, out.ctypes.data)
    return rc, out


def _free_device_bytes():
    import torch

    return torch.cuda.mem_get_info(0)[0]


def test_static_scratch_matches_allocating_sampler():
    """t = 60 draws d from the upper end of the cumulative table, which this
    entry point shares with the allocating sampler; t = 40 and 12 are the
    workload sizes.  Free device memory is the same before and after the calls."""
    f = _static_fn()
    gpu = backend.Backend(0)
    rs = np.random.RandomState(2718)
    cases = []
    for (t, k, count, seed) in ((40, 16, 200, 77), (12, 6, 256, 5), (60, 8, 64, 31)):
        L = [rand_word(rs, t) for _ in range(k)]
        rows = random_projector_rows(rs, t, max(2, t // 5))
        P = backend.projector(rows[0], rows[1], rows[2], t)
        want = gpu.singleProjectorSample(P, L, False, count, backend.RNG_PHILOX, seed)
        cases.append((P, L, count, seed, want))
    for c in cases:  # warm-up: symbol lookup, and each kernel's lazy module load
        assert _call(f, *c[:4])[0] == 0
    free0 = _free_device_bytes()
    for (P, L, count, seed, want) in cases:
        for _ in range(2):  # two calls in a row share the scratch array
            rc, got = _call(f, P, L, count, seed)
            assert rc == 0
            for a, b in zip(got, want):
                assert close(a, b, 1e-12, 1e-12), (a, b)
    assert _free_device_bytes() == free0  # the calls allocated no device memory
    gpu.close()


def test_static_rejects_oversize_inputs():
    f = _static_fn()
    rs = np.random.RandomState(1)
    t = 20
    rows = random_projector_rows(rs, t, 3)
    P = backend.projector(rows[0], rows[1], rows[2], t)
    rc, _ = _call(f, P, [rand_word(rs, t) for _ in range(4)], 257, 1)
    assert rc == -1  # CSIM_ERR_ARG: more states than the scratch holds
    rc, _ = _call(f, P, [rand_word(rs, t) for _ in range(17)], 8, 1)
    assert rc == -1  # k beyond the codeword table

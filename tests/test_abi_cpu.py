"""C-ABI checks that need no GPU: libcsimgpu.so loads and exports every entry
point include/csim.h declares, and the host-only entry points (the libc rand()
sequence, decompose) reproduce the reference's values."""
import os
import re

import numpy as np
import pytest

from circuitsimulator_gb300 import backend

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "csim.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|int64_t|int32_t|const char \*)\s*\*?\s*(csim_\w+)\s*\(", text,
                                 re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(backend.LIB_PATH):
        from circuitsimulator_gb300.build import build

        build()
    return backend.load_library()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_backend_executable_links(lib):
    assert os.access(backend.EXE_PATH, os.X_OK)


def test_libc_rand_matches_reference_streams(lib, golden_seeded):
    for rec in golden_seeded["rand_streams"]:
        r = backend.LibcRand(rec["seed"])
        assert [r.rand() for _ in range(len(rec["values"]))] == rec["values"]


def test_decompose_matches_reference(lib, golden_seeded):
    for d in golden_seeded["decompose"]:
        e, k, norm, L = backend.decompose(d["t"], d["fidbound"], d["rank"], d["fidelity"], d["forceL"], False,
                                          d["k_in"])
        assert (int(e), k, norm) == (d["exact"], d["k"], d["norm"])
        if d["L"] is not None:
            assert ["%x" % int(x) for x in L] == d["L"]


def test_no_device_is_reported_not_faked(lib):
    """Without an sm_103 device the context refuses to open (no CPU fallback)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(backend.CsimError):
        backend.Backend(0)

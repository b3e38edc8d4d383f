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


def test_query_struct_layout_matches_header(tmp_path):
    """The query, result and server structs as gcc lays them out == the ctypes binding."""
    import ctypes
    import subprocess

    fields = [("csim_query", backend._Query, ["G", "H", "seed"]),
              ("csim_query_result", backend._QueryResult, ["pairs", "latency_s"]),
              ("csim_server_config", backend._ServerConfig, ["hbm_budget_bytes", "round_states"]),
              ("csim_server_stats", backend._ServerStats, ["queued", "device_ms"])]
    exprs = []
    want = []
    for cname, cls, names in fields:
        exprs.append("sizeof(%s)" % cname)
        want.append(ctypes.sizeof(cls))
        for nm in names:
            exprs.append("offsetof(%s, %s)" % (cname, nm))
            want.append(getattr(cls, nm).offset)
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "csim.h"\nint main(void) {\n' +
                   "".join('printf("%%zu\\n", (size_t)%s);\n' % e for e in exprs) + "return 0; }\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want


def test_parse_protocol_reads_the_e2e_inputs():
    import gzip
    import json

    with gzip.open(os.path.join(ROOT, "tests", "golden", "e2e_cases.json.gz"), "rt") as f:
        cases = json.load(f)
    for c in cases:
        cfg, projs = backend.parse_protocol(c["input"])
        assert set(cfg) == set(backend.PROTOCOL_FIELDS)
        assert len(projs) == 2
        for ph, xs, zs, nq in projs:
            assert len(ph) == len(xs) == len(zs)
            assert all(x < (1 << nq) and z < (1 << nq) for x, z in zip(xs, zs))

"""The gpubackend executable against the reference backend's own output
(tests/golden/e2e_cases.json.gz, produced by the reference C backend on the
same stdin input and seed).

CPU: everything the backend prints before it needs the GPU — the parameter
echo, decompose()'s messages and the L matrix — is line-for-line the
reference's.  GPU: the final numerator/denominator lines match the reference's
within 1e-12 relative on the same rand() draws."""
import gzip
import json
import os

import pytest

from circuitsimulator_gb300 import backend
from helpers import close

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    with gzip.open(os.path.join(HERE, "golden", "e2e_cases.json.gz"), "rt") as f:
        return json.load(f)


def _prefix(lines):
    """lines up to (not including) 'World Size', minus the matrix-backend banner."""
    out = []
    for ln in lines:
        if ln.startswith("World Size"):
            break
        if ln.startswith("Using ") and "matrix operations" in ln:
            continue
        out.append(ln)
    return out


def _l_block(lines):
    if "L:" not in lines:
        return None
    i = lines.index("L:")
    blk = []
    for ln in lines[i + 1:]:
        blk.append(ln)
        if ln.endswith("]]") or ln == "[]":
            break
    return blk


@pytest.fixture(scope="module")
def exe():
    if not os.path.exists(backend.EXE_PATH):
        from circuitsimulator_gb300.build import build

        build()
    return backend.EXE_PATH


@pytest.mark.parametrize("case", cases(), ids=lambda c: c["label"])
def test_echo_and_decompose_match_reference(exe, case):
    rc, lines = backend.run_backend(case["input"], seed=case["seed"], timeout=120)
    ref = case["ref"]
    # the reference's first two lines are the print-mode banners, which main() prints
    assert lines[:2] == ref[:2]
    assert _prefix(lines[2:]) == _prefix(ref[2:])
    assert _l_block(lines) == _l_block(ref)


def test_malformed_input_fails_loudly(exe):
    rc, lines = backend.run_backend("1 0 0 10\n", timeout=60)
    assert rc != 0
    assert any("malformed" in ln for ln in lines)


@pytest.mark.gpu
@pytest.mark.parametrize("case", cases(), ids=lambda c: c["label"])
def test_backend_output_matches_reference(exe, case):
    rc, lines = backend.run_backend(case["input"], seed=case["seed"], timeout=300)
    assert rc == 0, lines[-5:]
    ref = case["ref"]
    assert _l_block(lines) == _l_block(ref)
    for a, b in zip(lines[-2:], ref[-2:]):
        assert close(float(a), float(b), 1e-12, 1e-12), (a, b)


def test_serving_daemon_without_gpu_fails_loudly(exe):
    import subprocess

    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([exe, "serve"], input=cases()[0]["input"].encode(), stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, timeout=60)
    assert r.returncode != 0
    assert b"no usable GB300 device" in r.stdout

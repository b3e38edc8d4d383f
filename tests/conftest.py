import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (runs on the GPU box)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def oracle():
    from oracle_ffi import ORACLE_SO, Oracle

    if not os.path.exists(ORACLE_SO):
        import subprocess

        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    return Oracle()


@pytest.fixture(scope="session")
def golden_fixtures():
    from golden.golden_io import load

    return load("ref_fixtures.json.gz")


@pytest.fixture(scope="session")
def golden_seeded():
    from golden.golden_io import load

    return load("ref_seeded.json.gz")

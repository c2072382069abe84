"""Shared pytest configuration: the `gpu` marker and import paths."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "oracle", "dqmc-framework_gb300"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long CPU test (statistical pin)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def example_fixture():
    import json

    import numpy as np

    with open(os.path.join(ROOT, "tests", "golden", "example_8x8.json")) as f:
        d = json.load(f)
    bits = np.unpackbits(np.frombuffer(bytes.fromhex(d["fields_packed_hex"]), dtype=np.uint8))
    d["fields"] = np.where(bits[: d["Lt"] * d["N"]] > 0, 1, -1).astype(np.int8).reshape(d["Lt"], d["N"])
    return d

"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    from neuronephys_clean_gb300.build import build
    return build()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ctx(built_lib):
    import neuronephys_clean_gb300 as nn
    c = nn.Context(int(os.environ.get("NN_DEVICE", "0")))
    yield c
    c.close()


GOLDEN = ROOT / "tests" / "golden"

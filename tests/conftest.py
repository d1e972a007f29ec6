"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a CPU-only host."""

from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build the engine and the oracle once per session (fast no-op when up to date)."""
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def goldens():
    return json.loads((ROOT / "tests" / "golden" / "reference_goldens.json").read_text())


@pytest.fixture(scope="session")
def engine(built):
    import mcx_gb300

    return mcx_gb300


@pytest.fixture(scope="session")
def oracle(built):
    from oracle import oracle as o

    return o

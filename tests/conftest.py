"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def built_library():
    """Build libxenodon.so and the CLI in-tree (incremental)."""
    from xenodon_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx(built_library):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xenodon_gb300 as xg
    c = xg.Context(0)
    yield c
    c.close()

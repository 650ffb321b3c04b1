"""Shared pytest configuration: the `gpu` marker, import paths and session fixtures."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "procedural-fire_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA sm_103 device (GB300)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def firelib():
    """The CUDA library; GPU tests fail loudly when it is missing."""
    import fire_sim
    return fire_sim.load_library()


@pytest.fixture(scope="session")
def tables(oracle_mod):
    """Noise (seed 1) and curl tables computed by the oracle (half-rounded values)."""
    noise = oracle_mod.noise_table(128, 1)
    curl = oracle_mod.curl_table(noise)
    return noise, curl

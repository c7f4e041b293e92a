"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(GOLDEN))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import make_golden as G

    def load(name):
        return np.load(GOLDEN / f"{name}.npz")

    return G, load


def _build_native():
    import importlib.util

    spec = importlib.util.spec_from_file_location("lmc_native_build", ROOT / "latticemontecarlo_gb300" / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


_build_native()


@pytest.fixture(scope="session")
def native():
    from latticemontecarlo_gb300 import _native
    return _native


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle

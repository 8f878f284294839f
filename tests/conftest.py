"""Shared test fixtures.  GPU tests are marked ``gpu``; everything else runs
on a CPU-only host."""
from __future__ import annotations

import importlib
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

G = 1.48812e-34
THETA = 1.05
DT = 1.0 / 24.0


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbh_gpu.so")


@pytest.fixture(scope="session")
def bh():
    """The engine's Python bindings (package directory barnes-hut_gb300)."""
    return importlib.import_module("barnes-hut_gb300")


@pytest.fixture(scope="session")
def port():
    """The oracle: C restatement of the reference's path (test infrastructure)."""
    from oracle.oracle import Oracle
    return Oracle("port")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / name, allow_pickle=False)
    return load


def bits(a) -> np.ndarray:
    """Raw bytes of an array, for bit-exact comparisons."""
    return np.ascontiguousarray(a).view(np.uint8)


def assert_bits_equal(a, b, what=""):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} != {b.shape}"
    if not np.array_equal(bits(a), bits(b)):
        diff = np.flatnonzero(np.any(bits(a).reshape(len(a), -1) != bits(b).reshape(len(b), -1), axis=1)) \
            if a.ndim and len(a) else []
        raise AssertionError(f"{what}: {len(diff)} entries differ, first {list(diff[:5])}")

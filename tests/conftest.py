"""Shared fixtures. GPU tests carry @pytest.mark.gpu; the rest run on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def q():
    """The package (2022-qpesim_gb300 as `qpesim_gb300`)."""
    return graft.load_package()


@pytest.fixture(scope="session")
def oracle_mod():
    return graft.load_oracle()


@pytest.fixture(scope="session")
def orc(oracle_mod):
    return oracle_mod.Oracle()


@pytest.fixture(scope="session")
def gpu(q):
    """Skips unless a CUDA device is present; returns the package."""
    if q._native.device_count() < 1:
        pytest.skip("no CUDA device")
    return q


def reference_root():
    """The reference tree (its cpp/ directory's parent) where its sources are
    present, else None; located as the oracle's build recipe locates it."""
    src = graft.load_oracle().reference_cpp()
    return src.parent if src is not None else None


def load_golden(name):
    return np.load(GOLDEN / name)


def golden_segments(z, prefix=""):
    """kind -> TERM_DTYPE array stored by make_golden.py."""
    TERM_DTYPE = graft.load_package().TERM_DTYPE
    out = {}
    for k in ("pp", "pq", "pqqp", "pqqr", "pqrs"):
        raw = z[prefix + k]
        out[k] = np.frombuffer(raw.tobytes(), TERM_DTYPE).copy() if raw.size else np.zeros(0, TERM_DTYPE)
    return out


def evolve_cases():
    return sorted(p.name for p in GOLDEN.glob("evolve_*.npz"))

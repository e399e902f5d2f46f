"""Test configuration.

Markers: `gpu` tests need a CUDA device and call the CUDA path through the C
ABI; everything else runs on the CPU. The oracle (oracle/liboracle.so, test
infrastructure) is built on first use with make.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    from oracle.oracle import load_oracle
    return load_oracle()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(ROOT / "tests" / "golden" / "minidisk_golden.npz"))


@pytest.fixture(scope="session")
def srhd_golden():
    return dict(np.load(ROOT / "tests" / "golden" / "srhd_golden.npz"))


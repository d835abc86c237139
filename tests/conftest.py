"""Shared fixtures.  ``-m gpu`` tests need a CUDA device and call the library through its C ABI
(via the package's ctypes layer); everything else runs on the CPU."""

from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "hermite_golden.npz"
AUTOSHAPE_GOLDEN = ROOT / "tests" / "golden" / "autoshape_golden.npz"
BINOMIAL_GOLDEN = ROOT / "tests" / "golden" / "binomial_golden.npz"
DIAGONAL_GOLDEN = ROOT / "tests" / "golden" / "diagonal_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: larger parity cases")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def autoshape_golden():
    z = np.load(AUTOSHAPE_GOLDEN)
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def binomial_golden():
    z = np.load(BINOMIAL_GOLDEN)
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def diagonal_golden():
    z = np.load(DIAGONAL_GOLDEN)
    return {k: z[k] for k in z.files}


def diagonal_cases(z, kind):
    return [str(n) for n in z["names"] if str(z[f"{n}/kind"]) == kind]


def golden_cases(z, need=("G",)):
    names = sorted({k.split("/")[0] for k in z})
    return [n for n in names if all(f"{n}/{k}" in z for k in need) and f"{n}/A" in z and n != "batch"]


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build()
    oracle.set_numpy_division(False)
    return oracle

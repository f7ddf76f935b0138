import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product kernels")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.load()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "reference_kats.npz"))


@pytest.fixture(scope="session")
def ptlib():
    from pupiloptixlab_gb300 import abi, build
    if not build.LIB.exists():
        build.build_library()
    return abi.load()


@pytest.fixture(scope="session")
def cuda_ctx(ptlib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from pupiloptixlab_gb300.api import Context
    return Context(0)

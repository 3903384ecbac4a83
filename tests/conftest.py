"""Shared fixtures. `gpu`-marked tests need a CUDA device (run on a GB300);
everything else runs on the CPU. The product library and the C oracle are
built once per session (nvcc cross-compiles without a GPU)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from nsvf_gb300 import build
    build.build()
    from oracle import cpu
    cpu.build()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(GOLDEN, "golden_small.npz")))


@pytest.fixture(scope="session")
def golden_prune():
    return dict(np.load(os.path.join(GOLDEN, "golden_prune.npz")))


@pytest.fixture(scope="session")
def golden_next():
    return dict(np.load(os.path.join(GOLDEN, "golden_next.npz")))


@pytest.fixture(scope="session")
def golden_ops():
    return dict(np.load(os.path.join(GOLDEN, "golden_ops.npz")))


@pytest.fixture(scope="session")
def golden_train():
    return dict(np.load(os.path.join(GOLDEN, "golden_train.npz")))


@pytest.fixture(scope="session")
def golden_hier():
    return dict(np.load(os.path.join(GOLDEN, "golden_hier.npz")))


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test run without a CUDA device")
    return torch.device("cuda", 0)

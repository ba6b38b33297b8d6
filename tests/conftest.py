"""Shared fixtures.  GPU tests carry @pytest.mark.gpu and run only where a
CUDA device is present; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mlff-distiller_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running test")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden_cases():
    return np.load(os.path.join(GOLDEN, "golden_cases.npz"))


@pytest.fixture(scope="session")
def weights_seed0():
    return dict(np.load(os.path.join(GOLDEN, "weights_seed0.npz")))


@pytest.fixture(scope="session")
def weights_bias(weights_seed0):
    pert = dict(np.load(os.path.join(GOLDEN, "bias_perturbation.npz")))
    return {k: (v + pert[k] if k in pert else v) for k, v in weights_seed0.items()}


def case_names(golden):
    return sorted(set(k.split("/")[0] for k in golden.files))

"""Shared test setup: repository on sys.path, the `gpu` marker, oracle build, helpers."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libiane_gb300.so")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    from oracle import build as oracle_build

    oracle_build.build_oracle()
    yield


@pytest.fixture(scope="session")
def cuda():
    """The CUDA device for GPU tests. Fails (does not skip) when no GPU is visible, so that a
    GPU run can never pass without exercising the kernels."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import iane_gb300

    iane_gb300._lib.lib()  # load the extension now: a missing library fails loudly
    return torch.device("cuda:0")


def rel_err_bound(gpu: np.ndarray, ref: np.ndarray, magnitude: np.ndarray) -> float:
    """max |gpu - ref| / magnitude, the per-element error relative to conv(|src|, |k|)."""
    m = np.maximum(magnitude.astype(np.float64), np.finfo(np.float32).tiny)
    return float(np.max(np.abs(gpu.astype(np.float64) - ref.astype(np.float64)) / m)) if gpu.size else 0.0

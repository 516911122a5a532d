"""Failure detection without a GPU fault: a device-side wait that never completes gives up
after its bound, records IANE_GB_DEVICE_TIMEOUT in the status word, and leaves the context
usable (a convolution afterwards is correct)."""
from __future__ import annotations

import time

import numpy as np
import pytest

import iane_gb300
import oracle
from gpu_helpers import empty_like_np, to_gpu, to_host

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_stays_usable(cuda):
    iane_gb300.device_status()  # start clean
    t0 = time.perf_counter()
    iane_gb300.check(iane_gb300.lib().iane_gb_wait_probe(20000, None))  # a 20 ms bound
    with pytest.raises(iane_gb300.IaneError) as info:
        iane_gb300.device_status()
    assert info.value.status == iane_gb300.abi.DEVICE_TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    iane_gb300.device_status()  # reading cleared it
    rng = np.random.default_rng(1)
    src = rng.random((40, 50), dtype=np.float32)
    kernel = rng.random((5, 5), dtype=np.float32)
    out = empty_like_np(src.shape, np.float32)
    iane_gb300.convolve(to_gpu(src), to_gpu(kernel), out, "zero", exact=True)
    ref = np.zeros_like(src)
    oracle.convolve(src, kernel, ref, "zero")
    assert np.array_equal(to_host(out), ref)

"""Failure detection without a GPU fault: a device-side wait that never completes gives up
after its bound, records IANE_GB_DEVICE_TIMEOUT in the status word, and leaves the context
usable (a convolution afterwards is correct). Both kinds of wait are probed: the mbarrier
waits of the TMA pipelines and the completion-counter waits of the persistent queues, whose
abort flag must also end a wait at once."""
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
    iane_gb300.check(iane_gb300.lib().iane_gb_wait_probe(20000, iane_gb300.abi.PROBE_MBARRIER, None))  # 20 ms
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


def test_counter_wait_times_out_and_context_stays_usable(cuda):
    # the persistent queues' dependency wait on a counter that nothing raises
    iane_gb300.device_status()
    t0 = time.perf_counter()
    iane_gb300.check(iane_gb300.lib().iane_gb_wait_probe(20000, iane_gb300.abi.PROBE_COUNTER, None))
    with pytest.raises(iane_gb300.IaneError) as info:
        iane_gb300.device_status()
    assert info.value.status == iane_gb300.abi.DEVICE_TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    iane_gb300.device_status()
    rng = np.random.default_rng(2)
    src = rng.random((30, 60), dtype=np.float32)
    kernel = rng.random((3, 7), dtype=np.float32)
    out = empty_like_np(src.shape, np.float32)
    iane_gb300.convolve(to_gpu(src), to_gpu(kernel), out, "zero", exact=True)
    ref = np.zeros_like(src)
    oracle.convolve(src, kernel, ref, "zero")
    assert np.array_equal(to_host(out), ref)


def test_abort_flag_ends_a_counter_wait_at_once(cuda):
    # another warp raises the abort flag after 1 ms: the waiter (bounded to 5 s) returns then,
    # and nothing is recorded -- the way every other wait of a run ends after one times out
    iane_gb300.device_status()
    t0 = time.perf_counter()
    iane_gb300.check(iane_gb300.lib().iane_gb_wait_probe(5000000, iane_gb300.abi.PROBE_COUNTER_ABORT, None))
    iane_gb300.device_status()  # raises if the wait recorded a timeout
    assert time.perf_counter() - t0 < 2.0

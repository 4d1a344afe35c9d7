"""Failure detection on the GPU without a fault.  Each failure is made on the
host (a pool cap, a short host-side wait) or by a device wait that nothing
ends and that gives up on its own limit; each test checks that the error is
reported as the reference reports its failures (a typed exception, OpenCL.scala
:143-312) and that the context still computes bit-exact results afterwards."""

import time

import numpy as np
import pytest

from compute import _native
from oracle import rng

pytestmark = pytest.mark.gpu


def _still_computes(device):
    got = np.asarray(device.Tensor.random([4096], seed=7).flatArray(), np.float32)
    assert np.array_equal(got.view(np.int32), rng.random_uniform(4096, 7).view(np.int32))


def test_pool_limit_turns_allocations_into_errors(cuda_device):
    rt = cuda_device.runtime
    rt.synchronize()
    rt.pool_trim()  # a cached block of the size asked for would be reused within the cap
    in_use = rt.pool_stats()["in_use"]
    rt.pool_set_limit(in_use + (1 << 20))
    try:
        small = rt.alloc(1 << 16)
        with pytest.raises(_native.MemObjectAllocationFailure) as e:
            rt.alloc(64 << 20)
        assert "limit" in str(e.value)
        small.release()
    finally:
        rt.pool_set_limit(0)
    big = rt.alloc(64 << 20)
    big.release()
    _still_computes(cuda_device)


def test_device_wait_gives_up_and_the_context_stays_usable(cuda_device):
    rt = cuda_device.runtime
    assert rt.device_errors() == 0
    t0 = time.monotonic()
    rt.probe_bounded_wait(300_000_000, 0)  # 0.3 s; nothing sets the word
    ev = rt.event()
    try:
        with pytest.raises(_native.WaitTimeout):
            rt.event_wait(ev, 1_000_000)  # the host's own bounded wait: 1 ms
        rt.event_wait(ev, 10 ** 10)
    finally:
        rt.event_release(ev)
    assert time.monotonic() - t0 >= 0.25
    assert rt.device_errors() == rt.PROBE_TIMEOUT
    assert rt.device_errors() == 0  # read and cleared
    _still_computes(cuda_device)


def test_device_wait_on_a_set_word_ends_at_once(cuda_device):
    rt = cuda_device.runtime
    t0 = time.monotonic()
    rt.probe_bounded_wait(5_000_000_000, 1)
    ev = rt.event()
    try:
        rt.event_wait(ev, 10 ** 10)
    finally:
        rt.event_release(ev)
    assert time.monotonic() - t0 < 2.0
    assert rt.device_errors() == 0


def test_probe_limit_is_bounded(cuda_device):
    with pytest.raises(_native.InvalidValue):
        cuda_device.runtime.probe_bounded_wait(11_000_000_000, 0)

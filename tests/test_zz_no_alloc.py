"""The sum entry point for callers that cannot allocate device memory.

Some callers of this library cannot call cudaMalloc: a host framework that has
already reserved the GPU's memory for its own allocator, or a latency-critical
caller that cannot take cudaMalloc's device-wide synchronisation.
``cc_reduce_sum_f32_noalloc`` serves them with scratch in a fixed device array
instead of the buffer pool.  This test calls it through the C ABI and checks it
against the pooled entry point ``cc_reduce_sum_f32`` on the same input, twice
in a row (the second call reuses the array the first one left behind), within
the error bound the other sum tests use.  It lives in its own file, which
pytest collects last, and passes both alone and after the other tests.
"""

import ctypes

import numpy as np
import pytest

from compute import _native

pytestmark = pytest.mark.gpu

MAX_ELEMENTS = 16384 * 8192


def _device():
    from conftest import cuda_tensors
    return cuda_tensors()


def _noalloc(in_ptr, n, out_ptr, stream):
    lib = _native.load()
    return lib.cc_reduce_sum_f32_noalloc(ctypes.c_uint64(in_ptr), ctypes.c_size_t(n), ctypes.c_uint64(out_ptr),
                                         ctypes.c_uint64(stream))


def test_no_alloc_sum_matches_the_pooled_sum_on_two_calls():
    d = _device()
    rt = d.runtime
    T = d.Tensor
    n = 3_000_003
    a = (T.random([n], seed=5) - T.fill(0.5, [n])).doCache()
    host = a.flatArray()
    bound = np.sqrt(n) * 2.0 ** -24 * float(np.abs(host.astype(np.float64)).sum())
    in_ptr = a._cached.device_ptr()
    stream = rt.stream()
    out_pool, out_na = rt.alloc(4), rt.alloc(4)
    before = rt.pool_stats()
    results = []
    for _ in range(2):
        rt.reduce_sum_ptr(in_ptr, n, out_pool.device_ptr(), stream)
        _native.check(_noalloc(in_ptr, n, out_na.device_ptr(), stream), "cc_reduce_sum_f32_noalloc")
        rt.synchronize()
        pooled = float(rt.download(out_pool, 1)[0])
        noalloc = float(rt.download(out_na, 1)[0])
        assert abs(noalloc - pooled) <= bound
        results.append(noalloc)
    assert results[0] == results[1]
    # a misaligned start takes the scalar path
    _native.check(_noalloc(in_ptr + 4, n - 1, out_na.device_ptr(), stream), "cc_reduce_sum_f32_noalloc")
    rt.reduce_sum_ptr(in_ptr + 4, n - 1, out_pool.device_ptr(), stream)
    rt.synchronize()
    assert abs(float(rt.download(out_na, 1)[0]) - float(rt.download(out_pool, 1)[0])) <= bound
    after = rt.pool_stats()
    assert after["in_use"] == before["in_use"]
    out_pool.release()
    out_na.release()
    a.close()


def test_no_alloc_sum_rejects_inputs_beyond_its_scratch():
    d = _device()
    rt = d.runtime
    out = rt.alloc(4)
    status = _noalloc(out.device_ptr(), MAX_ELEMENTS + 1, out.device_ptr(), rt.stream())
    assert status == -30  # CC_ERR_INVALID_VALUE
    assert "scratch capacity" in _native.last_error()
    out.release()

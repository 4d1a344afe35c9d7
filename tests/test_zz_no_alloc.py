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
import os
import subprocess
import sys
import textwrap

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


@pytest.mark.parametrize("n", [0, 1, 8192, 8193, MAX_ELEMENTS])
def test_no_alloc_sum_at_the_edges_of_its_scratch(n):
    """n = 0 writes 0.0 from one block; 8192 is one full chunk; MAX_ELEMENTS
    (512 MB of floats) fills every partial of the array."""
    d = _device()
    rt = d.runtime
    buf = rt.alloc(max(4, 4 * n))
    if n:
        rt.random(buf, n, 11, False)
    out_pool, out_na = rt.alloc(4), rt.alloc(4)
    stream = rt.stream()
    rt.upload(out_na, np.array([123.0], np.float32))
    for _ in range(2):
        _native.check(_noalloc(buf.device_ptr(), n, out_na.device_ptr(), stream), "cc_reduce_sum_f32_noalloc")
        rt.reduce_sum_ptr(buf.device_ptr(), n, out_pool.device_ptr(), stream)
        rt.synchronize()
        got = float(rt.download(out_na, 1)[0])
        want = float(rt.download(out_pool, 1)[0])
        if n == 0:
            assert got == 0.0 and want == 0.0
        else:
            bound = np.sqrt(n) * 2.0 ** -24 * abs(want)
            assert abs(got - want) <= bound, (n, got, want)
    for b in (buf, out_pool, out_na):
        b.release()


_FRESH_PROCESS = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from compute import _native
    lib = _native.load()                         # the library only: cc_init is never called
    cu = ctypes.CDLL("libcuda.so.1")

    def ok(r, what):
        if r != 0:
            raise SystemExit("%s failed: %d" % (what, r))

    ok(cu.cuInit(0), "cuInit")
    dev = ctypes.c_int()
    ok(cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
    n = 1000003
    host = np.random.RandomState(3).uniform(-1, 1, n).astype(np.float32)
    exact = float(host.astype(np.float64).sum())
    bound = np.sqrt(n) * 2.0 ** -24 * float(np.abs(host.astype(np.float64)).sum())

    def sum_in_current_context():
        src, dst = ctypes.c_uint64(), ctypes.c_uint64()
        ok(cu.cuMemAlloc_v2(ctypes.byref(src), ctypes.c_size_t(4 * n)), "cuMemAlloc")
        ok(cu.cuMemAlloc_v2(ctypes.byref(dst), ctypes.c_size_t(4)), "cuMemAlloc")
        ok(cu.cuMemcpyHtoD_v2(src, host.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(4 * n)), "cuMemcpyHtoD")
        got = []
        for _ in range(2):
            r = lib.cc_reduce_sum_f32_noalloc(src, ctypes.c_size_t(n), dst, ctypes.c_uint64(0))
            if r != 0:
                raise SystemExit("cc_reduce_sum_f32_noalloc: %d %s" % (r, _native.last_error()))
            ok(cu.cuCtxSynchronize(), "cuCtxSynchronize")
            v = np.zeros(1, np.float32)
            ok(cu.cuMemcpyDtoH_v2(v.ctypes.data_as(ctypes.c_void_p), dst, ctypes.c_size_t(4)), "cuMemcpyDtoH")
            got.append(float(v[0]))
        ok(cu.cuMemFree_v2(src), "cuMemFree")
        ok(cu.cuMemFree_v2(dst), "cuMemFree")
        if got[0] != got[1] or abs(got[0] - exact) > bound:
            raise SystemExit("sum %r, exact %r" % (got, exact))

    # 1. the device's primary context, as a framework on the CUDA runtime has it
    primary = ctypes.c_void_p()
    ok(cu.cuDevicePrimaryCtxRetain(ctypes.byref(primary), dev), "cuDevicePrimaryCtxRetain")
    ok(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
    sum_in_current_context()
    # 2. a driver-API context of the caller's own on the same device
    own = ctypes.c_void_p()
    ok(cu.cuCtxCreate_v2(ctypes.byref(own), 0, dev), "cuCtxCreate")
    sum_in_current_context()
    ok(cu.cuCtxDestroy_v2(own), "cuCtxDestroy")
    # 3. back in the primary context
    ok(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
    sum_in_current_context()
    print("fresh-process no-alloc sums ok")
""")


def test_no_alloc_sum_needs_no_init_and_follows_the_current_context():
    """In a fresh process that never calls cc_init: sums in the device's
    primary context; then in a caller's own driver-API context on the same
    device, which gets its own scratch address (the array's address belongs
    to the context that loaded the module); then, after that context is
    destroyed, in the primary context again."""
    pkg = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "compute.scala_gb300")
    p = subprocess.run([sys.executable, "-c", _FRESH_PROCESS, pkg], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert p.returncode == 0, p.stdout
    assert "fresh-process no-alloc sums ok" in p.stdout

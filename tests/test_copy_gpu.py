"""Uploads and downloads through pinned host memory give the same bytes with
the DMA engines and with the SM copy kernel, for aligned and ragged sizes and
offsets (the kernel takes the 16-byte body, a DMA copy the remainder)."""

import ctypes

import numpy as np
import pytest

from compute._native import call

pytestmark = pytest.mark.gpu


def test_copy_kernel_round_trips(cuda_device):
    rt = cuda_device.runtime
    nbytes = (3 << 20) + 52
    host = ctypes.c_void_p()
    call("cc_host_alloc", ctypes.c_size_t(nbytes), ctypes.byref(host))
    back = ctypes.c_void_p()
    call("cc_host_alloc", ctypes.c_size_t(nbytes), ctypes.byref(back))
    try:
        src = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(host.value))
        dst = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(back.value))
        src[:] = np.random.RandomState(0).randint(0, 256, nbytes).astype(np.uint8)
        buf = rt.alloc(nbytes)
        for knob in (0, 1):
            rt.config_set("copy_kernel", knob)
            for off, size in ((0, nbytes), (16, nbytes - 16), (0, (1 << 20) + 7), (32, (2 << 20) + 3), (4, 1 << 21)):
                dst[:] = 0
                call("cc_buf_upload", ctypes.c_uint64(buf.handle), ctypes.c_size_t(off), ctypes.c_void_p(host.value + off),
                     ctypes.c_size_t(size))
                call("cc_buf_download", ctypes.c_uint64(buf.handle), ctypes.c_size_t(off),
                     ctypes.c_void_p(back.value + off), ctypes.c_size_t(size))
                assert np.array_equal(dst[off:off + size], src[off:off + size]), (knob, off, size)
        buf.release()
    finally:
        rt.config_set("copy_kernel", 0)
        call("cc_host_free", host)
        call("cc_host_free", back)


def test_async_uploads_are_ordered_before_launches(cuda_device):
    """cc_buf_upload_async copies many buffers without waiting; a launch and a
    download queued after them see the uploaded bytes; cc_buf_download_async
    reads them back without waiting, complete at the next synchronisation."""
    rt = cuda_device.runtime
    d = cuda_device
    from compute.tensors import NonInlineTensor
    n = (1 << 22) + 3
    p = NonInlineTensor(d, (n,), 0.0, None)
    prog = rt.program(d.serialize((p * d.Tensor.fill(2.0, [n])).closure, (n,)).text)
    hosts, bufs = [], []
    for k in range(6):
        h = ctypes.c_void_p()
        call("cc_host_alloc", ctypes.c_size_t(4 * n), ctypes.byref(h))
        arr = np.ctypeslib.as_array((ctypes.c_float * n).from_address(h.value))
        arr[:] = np.arange(n, dtype=np.float32) + k
        hosts.append((h, arr))
        bufs.append(rt.alloc(4 * n))
    outs = [rt.alloc(4 * n) for _ in bufs]
    try:
        for (h, _), b in zip(hosts, bufs):
            call("cc_buf_upload_async", ctypes.c_uint64(b.handle), ctypes.c_size_t(0), h, ctypes.c_size_t(4 * n))
        for b, o in zip(bufs, outs):
            rt.launch(prog, [b], o)
        for k, o in enumerate(outs):
            assert np.array_equal(rt.download(o, n), 2 * (np.arange(n, dtype=np.float32) + k))
        # non-blocking reads into the same pinned buffers, complete after one synchronisation
        for (h, arr), o in zip(hosts, outs):
            arr[:] = -1.0
            call("cc_buf_download_async", ctypes.c_uint64(o.handle), ctypes.c_size_t(0), h, ctypes.c_size_t(4 * n))
        rt.synchronize()
        for k, (_, arr) in enumerate(hosts):
            assert np.array_equal(arr, 2 * (np.arange(n, dtype=np.float32) + k))
    finally:
        for h, _ in hosts:
            call("cc_host_free", h)
        for b in bufs + outs:
            b.release()

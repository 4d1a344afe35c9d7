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

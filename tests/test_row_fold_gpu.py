"""The inner-axis fold `t.split(last).reduce(_ + _)` (Tensors.scala:1035-1074
with Scala's left-to-right reduce) on its TMA-staged skeleton.

Each output is the left fold ((t(g,0) + t(g,1)) + t(g,2)) + ... of its row, as
the reference's generated kernel computes it, so every result must be the
oracle's bits (the oracle taking exp/log/tanh values from the device, each
checked within 2 ulp): a plain tensor, a fused expression with a broadcast column
input, a rank-3 tensor, ragged row and column counts, a row input that is not
16-byte aligned (the direct-load kernel), and the generic fold (knob off) for
comparison.
"""

import ctypes

import numpy as np
import pytest

from compute import _native

pytestmark = pytest.mark.gpu


def _fold(t, axis):
    return t.split(axis).reduce(lambda a, b: a + b)


def _oracle_bits(d, expr):
    from device_functions import DeviceFunctions
    from oracle import interp
    ser = d.serialize(expr.closure, expr.shape)
    # exp/log/tanh from the device (each checked within 2 ulp), everything else the oracle's
    return interp.evaluate(ser.text, [p.flatArray() for p in ser.params], transcendental=DeviceFunctions(d)), ser


def _check(d, expr, expect_skeleton=True):
    rt = d.runtime
    want, ser = _oracle_bits(d, expr)
    src = rt.program(ser.text).source()
    assert ("cc_rowfold" in src) == expect_skeleton
    got = expr.flatArray()
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
    return got


@pytest.mark.parametrize("shape", [(16384, 4096), (1000, 4100), (64, 32), (3, 36), (130, 128)])
def test_plain_rows(cuda_device, shape):
    T = cuda_device.Tensor
    x = T.randomNormal(list(shape), seed=0x40000011).doCache()
    _check(cuda_device, _fold(x, 1))
    x.close()


def test_fused_rows_with_a_broadcast_column(cuda_device):
    T = cuda_device.Tensor
    R, J = 4096, 1024
    a, b, x = (T.randomNormal([R, J], seed=0x40000020 + s).doCache() for s in range(3))
    bias = T.randomNormal([1, J], seed=0x40000023).doCache()
    expr = _fold(T.tanh(a * b) + x * bias.broadcast([R, J]), 1)
    _check(cuda_device, expr)
    for t in (a, b, x, bias):
        t.close()


def test_rank_three(cuda_device):
    T = cuda_device.Tensor
    x = T.random([8, 300, 256], seed=0x40000031).doCache()
    _check(cuda_device, _fold(x * x, 2))
    x.close()


def test_short_or_unaligned_rows_stay_on_the_generic_fold(cuda_device):
    T = cuda_device.Tensor
    for shape in ([100, 30], [100, 102]):  # fewer than 32 terms; rows not a multiple of 16 bytes
        x = T.random(shape, seed=0x40000041).doCache()
        _check(cuda_device, _fold(x, 1), expect_skeleton=False)
        x.close()


def test_knob_off_gives_the_same_bits(cuda_device):
    rt = cuda_device.runtime
    T = cuda_device.Tensor
    x = T.randomNormal([512, 2048], seed=0x40000051).doCache()
    on = _fold(x, 1).flatArray()
    try:
        rt.config_set("row_fold", 0)
        off = _fold(x, 1).flatArray()
    finally:
        rt.config_set("row_fold", 1)
    assert np.array_equal(on.view(np.int32), off.view(np.int32))
    x.close()


def test_row_input_not_16_byte_aligned_takes_direct_loads(cuda_device):
    from compute.tensors import NonInlineTensor
    from oracle import interp
    d = cuda_device
    rt = d.runtime
    R, J = 300, 512
    p = NonInlineTensor(d, (R, J), 0.0, None)
    expr = _fold(p, 1)
    ser = d.serialize(expr.closure, expr.shape)
    prog = rt.program(ser.text)
    host = np.random.RandomState(2).standard_normal(R * J + 1).astype(np.float32)
    buf, out = rt.alloc(4 * (R * J + 1)), rt.alloc(4 * R)
    rt.upload(buf, host)
    for shift in (0, 1):  # 1: 4 bytes past the block's 256-byte alignment
        rt.launch_ptrs(prog, [buf.device_ptr() + 4 * shift], out.device_ptr())
        got = rt.download(out, R)
        want = interp.evaluate(ser.text, [host[shift:shift + R * J]])
        assert np.array_equal(got.view(np.int32), want.view(np.int32)), shift
    assert rt.device_errors() == 0
    buf.release()
    out.release()

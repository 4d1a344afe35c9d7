"""The reference's own Tensor tests, restated, against its own expected values.

Each test mirrors one block of Tensors/src/test/scala/com/thoughtworks/compute/
TensorsSpec.scala, cpu/src/test/scala/com/thoughtworks/compute/cpuSpec.scala or
an ``@example`` of cpu/src/main/scala/com/thoughtworks/compute/cpu.scala; the
expected values come from tests/golden/reference_goldens.json, which
tests/golden/make_golden.py extracted from those files.  The ``device`` fixture
runs every case twice: on the numpy oracle (CPU; this pins the oracle) and on
the CUDA runtime (GPU; this is parity of the sm_103a path).
"""

import functools
import json
import os

import numpy as np
import pytest

from compute import IllegalArgumentException

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def expected(spec, test, i=0):
    cases = [c for c in GOLDEN[spec] if c["test"] == test] or \
        [c for c in GOLDEN[spec] if c["test"].startswith(test)]
    if not cases:
        raise KeyError(test)
    e = cases[0]["expect"][i]
    return e.get("string", e.get("float", e.get("seq")))


def test_repeatedly_to_string(device):
    t = device.Tensor(42.0)
    for _ in range(20):
        assert t.toString() == expected("TensorsSpec", "repeatedly toString")


def test_create_a_tensor_of_a_constant(device):
    filled = device.Tensor.fill(42.0, [2, 3, 5])
    a = filled.flatArray()
    assert a.size == 30 and np.all(a == np.float32(42.0))


def test_tensor_literal(device):
    T = device.Tensor
    assert T(42.0).toString() == expected("TensorsSpec", "tensor literal", 0)
    assert T([1.0, 2.0]).toString() == expected("TensorsSpec", "tensor literal", 1)
    assert T([[1.0, 2.0], [3.0, 4.0]]).toString() == expected("TensorsSpec", "tensor literal", 2)


def test_wrong_tensor_shape(device):
    with pytest.raises(IllegalArgumentException):
        device.Tensor([[1.0], [3.0, 4.0]])


def test_translate(device):
    shape = (2, 3, 5)
    translated = device.Tensor.fill(42.0, shape, padding=99.0).translate([1, 2, -3])
    assert translated.toString() == expected("TensorsSpec", "translate")
    a = translated.flatArray().reshape(shape)
    for i in range(2):
        for j in range(3):
            for k in range(5):
                want = 42.0 if (i >= 1 and j >= 2 and 5 - k > 3) else 99.0
                assert a[i, j, k] == want


def test_unzip(device):
    t = device.Tensor([[[[1.0, 5.0]]]])
    assert [s.toString() for s in t.split(3)] == expected("TensorsSpec", "unzip")


def test_plus(device):
    t = device.Tensor([[[1.0, 5.0]]])
    assert (t + t).toString() == expected("TensorsSpec", "plus")


def test_plus_and_multiplication(device):
    t = device.Tensor([[[1.0, 5.0]]])
    t2 = t + t
    assert (t2 * t2).toString() == expected("TensorsSpec", "plus and multiplication")


def _convolute(T, inp, weight, bias):
    """TensorsSpec.scala:140-219: a 3x3 convolution out of translate, split and join."""
    batch, height, width, depth = inp.shape
    kh, kw, d2, filters = weight.shape
    assert d2 == depth and bias.shape == (filters,)
    input_seq = list(inp.split(3))
    weight_seq = [[[list(d.split(0)) for d in kwd.split(0)] for kwd in khkwd.split(0)]
                  for khkwd in weight.split(3)]
    bias_seq = list(bias.split(0))
    outputs = []
    for weight_per_filter, bias_per_filter in zip(weight_seq, bias_seq):
        summands = []
        for offset_y, weight_per_row in zip(range(-1, 2), weight_per_filter):
            for offset_x, weight_per_pixel in zip(range(-1, 2), weight_per_row):
                for input_per_channel, weight_per_channel in zip(input_seq, weight_per_pixel):
                    assert weight_per_channel.shape == ()
                    summands.append(input_per_channel.translate([0, offset_y, offset_x]) *
                                    weight_per_channel.broadcast([batch, height, width]))
        outputs.append(bias_per_filter.broadcast([batch, height, width]) +
                       functools.reduce(lambda a, b: a + b, summands))
    return T.join(outputs)


def test_convolution(device):
    T = device.Tensor
    inp = np.zeros((2, 4, 5, 3), np.float32)
    inp[0, 0, 0, 0] = 1.0
    inp[0, 1, 0, 0] = 10.0
    inp[1, 0, 0, 0] = 100.0
    w = np.zeros((3, 3, 3, 2), np.float32)
    w[1, 1, 0, 0] = 3.0
    w[1, 1, 0, 1] = 4.0
    w[0, 1, 0, 0] = 5.0
    w[2, 2, 0, 1] = 6.0
    b = np.array([100000.0, 200000.0], np.float32)
    out = _convolute(T, T(inp), T(w), T(b))
    assert out.shape == (2, 4, 5, 2)
    o = out.flatArray().reshape(2, 4, 5, 2)
    spec = [c for c in GOLDEN["TensorsSpec"] if c["test"] == "convolution"][0]["expect"]
    floats = [e["float"] for e in spec if "float" in e][1:]  # the first is the group length check
    idx = [(0, 0, 0, 0), (0, 1, 1, 1), (1, 1, 1, 1), (0, 2, 1, 1), (0, 0, 0, 1), (0, 1, 0, 0), (1, 0, 0, 0)]
    assert len(floats) == len(idx)
    for (i, j, k, l), want in zip(idx, floats):
        assert o[i, j, k, l] == np.float32(want)


def test_sum(device):
    assert device.Tensor.fill(15625.0, [8, 8]).sum().toString() == expected("TensorsSpec", "sum")


def test_random_normal_scalar(device):
    got = device.Tensor.randomNormal([], seed=54321).flatArray()
    assert got.tolist() == [np.float32(v) for v in expected("TensorsSpec", "randomNormal scalar")]


def test_read_scalar(device):
    assert device.Tensor(42.0).readScalar() == expected("TensorsSpec", "readScalar")


def test_read_nd(device):
    T = device.Tensor
    assert T([1.0, 2.0]).read1DArray().tolist() == [1.0, 2.0]
    a2 = [[1, 2], [3, 4], [5, 6]]
    assert T(a2).read2DArray().tolist() == a2
    a3 = [[[1, 2], [3, 4], [5, 6]], [[7, 8], [9, 10], [11, 12]]]
    assert T(a3).read3DArray().tolist() == a3
    a4 = [a3, [[[13, 14], [15, 16], [17, 18]], [[19, 20], [21, 22], [23, 24]]]]
    assert T(a4).read4DArray().tolist() == a4
    assert T(a4).read4DSeq() == a4
    assert T([1.0, 2.0]).read1DSeq() == [1.0, 2.0]
    assert T(a2).read2DSeq() == a2


def test_random(device):
    assert device.Tensor.random([3, 3], seed=12345).toString() == expected("TensorsSpec", "random")


def test_random_normal(device):
    assert device.Tensor.randomNormal([3, 3, 3], seed=54321).toString() == expected("TensorsSpec", "randomNormal")


def test_transposes(device):
    T = device.Tensor
    assert T(42.0).transpose().toString() == expected("TensorsSpec", "scalar transpose")
    assert T([1.0, 2.0, 3.0]).transpose().toString() == expected("TensorsSpec", "1d transpose")
    assert T([[1.0, 2.0], [3.0, 4.0]]).transpose().toString() == expected("TensorsSpec", "2d transpose")
    t = T([[[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]], [[7.0, 8.0, 9.0], [10.0, 11.0, 12.0]]])
    assert t.transpose().toString() == expected("TensorsSpec", "3d transpose")


def _matrix_multiply(m1, m2):
    """TensorsSpec.scala:472-478."""
    i, j = m1.shape
    j2, k = m2.shape
    assert j == j2
    product = m1.broadcast([i, j, k]) * m2.reshape([1, j, k]).broadcast([i, j, k])
    return product.split(1).reduce(lambda a, b: a + b)


M1 = [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]
M2 = [[7.0, 8.0, 9.0, 10.0], [11.0, 12.0, 13.0, 14.0], [15.0, 16.0, 17.0, 18.0]]


def test_matrix_multiplication(device):
    T = device.Tensor
    assert _matrix_multiply(T(M1), T(M2)).toString() == expected("TensorsSpec", "matrix multiplication")


def test_broadcast(device):
    assert device.Tensor(M1).broadcast([2, 3, 4]).toString() == expected("TensorsSpec", "broadcast")


def test_unrolled_matrix_multiplication(device):
    """TensorsSpec.scala:502-528."""
    T = device.Tensor

    def mm(a, b):
        cols1 = list(a.split(1))
        cols2 = list(b.split(1))
        result_columns = []
        for col2 in cols2:
            terms = [l * r.broadcast(l.shape) for l, r in zip(cols1, col2.split(0))]
            result_columns.append(functools.reduce(lambda x, y: x + y, terms))
        return T.join(result_columns)

    assert mm(T(M1), T(M2)).toString() == expected("TensorsSpec", "unrolled matrix multiplication")


def test_cpu_examples(device):
    """cpu.scala:15-101."""
    T = device.Tensor
    assert T([[1.0, 2.0], [3.0, 4.0]]).toString() == expected("cpu", "example: In Compute.scala")
    my3d = T([[[float(a * 12 + b * 4 + c) for c in range(4)] for b in range(3)] for a in range(2)])
    assert my3d.shape == (2, 3, 4)
    s0 = my3d.split(0)
    assert s0.toString() == expected("cpu", "example: A `Tensor` can be `split`", 1)
    assert [t.shape for t in s0] == [(3, 4), (3, 4)]
    s1 = my3d.split(1)
    spec = [c for c in GOLDEN["cpu"] if c["test"].startswith("example: A `Tensor` can be `split`")][0]["expect"]
    strings = [e["string"] for e in spec if "string" in e]
    assert s1.toString() == strings[-1]
    assert [t.shape for t in s1] == [(2, 4)] * 3
    subs = [T([[1.0, 2.0], [3.0, 4.0]]), T([[5.0, 6.0], [7.0, 8.0]]), T([[9.0, 10.0], [11.0, 12.0]])]
    merged = T.join(subs)
    assert merged.toString() == expected("cpu", "example: Multiple `Tensor`s", 0)
    assert merged.shape == (2, 2, 3)
    s = T.scalar(42.0)
    assert s.broadcast([2, 3]).toString() == expected("cpu", "example: A [[Tensor]] of scalar")


def test_computational_graph(device):
    """cpuSpec.scala:9-16."""
    T = device.Tensor
    a = T.fill(2.0, [2, 3]).nonInline()
    b = T.fill(2.0, [2, 3]).nonInline()
    c = (a + b).nonInline()
    d = (c + b).nonInline()
    assert d.toString() == expected("cpuSpec", "computational graph")


def test_join(device):
    """cpuSpec.scala:18-38."""
    T = device.Tensor
    a = T.fill(42.0, [3, 4])
    b = T.fill(43.0, [3, 4])
    t0 = T.join([a, b], 0)
    assert t0.shape == (2, 3, 4)
    assert t0.toString() == expected("cpuSpec", "join", 1)
    t1 = T.join([a, b], 1)
    assert t1.shape == (3, 2, 4)
    assert t1.toString() == expected("cpuSpec", "join", 3)
    t2 = T.join([a, b], 2)
    assert t2.shape == (3, 4, 2)
    assert t2.toString() == expected("cpuSpec", "join", 5)

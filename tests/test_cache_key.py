"""The kernel-cache key: structural equality modulo parameter names.

The reference caches compiled kernels by the alpha-converted tree
(Trees.scala:266-298, :807-822; Tensors.scala:1267-1293) and pins that
equality in Trees/src/test/scala/com/thoughtworks/compute/TreesSpec.scala:13-93:
a term equals itself and its alpha-conversion (`reflexive`), terms that differ
only in parameter names are equal (`sameStructuralDifferentParameterName`), and
terms of different structure, padding or shape differ (`differentStructural`).
Here the alpha-converted form is the IR text that ``trees.serialize`` writes
and the runtime's program cache keys on, so these cases are restated over it.
"""

import pytest

from compute import trees


class _Id:
    """A parameter identity (the reference's parameter id string)."""

    def __init__(self, name):
        self.name = name


def _param(name, padding=0.0, shape=(12, 34)):
    return trees.ArrayParameter(_Id(name), padding, shape)


def _read(param, frame=None):
    """The parameter read at the frame's coordinates (ArrayParameter.extract)."""
    return trees.Extract(param)


def _key(root, shape=(12, 34), kind="ew"):
    return trees.serialize(root, shape, kind).text


def _same(t0, t1, shape=(12, 34)):
    assert _key(t0, shape) == _key(t1, shape)


def _different(t0, t1, shape0=(12, 34), shape1=None):
    assert _key(t0, shape0) != _key(t1, shape1 or shape0)


def _reflexive(make, shape=(12, 34)):
    t0, t1 = make(), make()
    assert _key(t0, shape) == _key(t0, shape)
    assert _key(t1, shape) == _key(t1, shape)
    assert _key(t0, shape) == _key(t1, shape)


def test_float():
    # TreesSpec "float": a parameter and a literal are reflexive; two names are one structure
    _reflexive(lambda: _read(_param("my_id")))
    _reflexive(lambda: trees.Literal(42.0))
    _same(_read(_param("my_id_1")), _read(_param("my_id_2")))


def test_array():
    # TreesSpec "array": padding 42 over [12, 34]; other names, same structure;
    # other padding and shape, different structure
    _reflexive(lambda: _read(_param("my_id", 42.0, (12, 34))))
    _same(_read(_param("my_id_3", 42.0, (12, 34))), _read(_param("my_id_4", 42.0, (12, 34))))
    _different(_read(_param("my_id", 0.1, (12, 34))), _read(_param("my_id2", 99.9, (56, 78)), (56, 78)),
               (12, 34), (56, 78))


def test_padding_and_shape_each_change_the_key():
    # the reference's key includes the parameter's padding and shape (Trees.scala:779-798)
    _different(_read(_param("a", 0.1)), _read(_param("a", 99.9)))
    _different(_read(_param("a", 0.0, (12, 34))), _read(_param("a", 0.0, (34, 12))), (12, 34), (34, 12))
    # and here the output shape too (the reference reuses the first shape's ND-range)
    _different(trees.Literal(1.0), trees.Literal(1.0), (12, 34), (12, 35))


def test_tuple_join():
    # TreesSpec "tuple.zip"
    _reflexive(lambda: trees.Concatenate([_read(_param("my_id")), trees.Literal(2.0), trees.Literal(3.0)]))
    _same(trees.Concatenate([_read(_param("my_id1")), _read(_param("my_id2")), trees.Literal(0.0)]),
          trees.Concatenate([_read(_param("my_id2")), _read(_param("my_id3")), trees.Literal(0.0)]))
    _different(trees.Concatenate([trees.Literal(1.0), trees.Literal(0.0)]),
               trees.Concatenate([trees.Literal(0.0), trees.Literal(1.0)]))


def test_parameter_sharing_is_structure():
    # one parameter read twice is not two parameters read once each (alphaConversion
    # keeps the identity pattern, Trees.scala:807-822)
    a, b = _param("a"), _param("b")
    twice = trees.Binary("add", _read(a), _read(a))
    two = trees.Binary("add", _read(a), _read(b))
    _different(twice, two)
    c, d = _param("c"), _param("d")
    _same(two, trees.Binary("add", _read(c), _read(d)))
    _same(twice, trees.Binary("add", _read(c), _read(c)))
    # parameters are numbered by first appearance: (a + b) - a is (c + d) - c, not (c + d) - d
    _same(trees.Binary("sub", two, _read(a)), trees.Binary("sub", trees.Binary("add", _read(c), _read(d)), _read(c)))
    _different(trees.Binary("sub", two, _read(a)),
               trees.Binary("sub", trees.Binary("add", _read(c), _read(d)), _read(d)))


def test_operators_literals_and_views_are_structure():
    a = _param("a")
    _different(trees.Unary("exp", _read(a)), trees.Unary("log", _read(a)))
    _different(trees.Binary("sub", _read(a), trees.Literal(1.0)), trees.Binary("sub", trees.Literal(1.0), _read(a)))
    _different(trees.Binary("add", _read(a), trees.Literal(1.0)), trees.Binary("add", _read(a), trees.Literal(2.0)))
    # a translated view of the same parameter is another kernel
    moved = trees.Extract(trees.Transform(a, [1, 0, 0, 0, 1, -1]))
    _different(_read(a), moved)
    _same(trees.Extract(trees.Transform(_param("b"), [1, 0, 0, 0, 1, -1])), moved)
    # an elementwise store and a sum of the same tree are different programs
    assert _key(_read(a), kind="ew") != _key(_read(a), kind="sum")


def test_tensor_api_trees_share_a_key():
    """Through the Tensor API: the same expression over other tensors of the same
    shape is one cache entry; another shape or padding is another."""
    from compute import Tensors
    from oracle_runtime import OracleRuntime
    d = Tensors(runtime=OracleRuntime())
    T = d.Tensor
    x, y, z = (T.random([8, 16], seed=s).doCache() for s in (1, 2, 3))
    e1 = T.tanh(x * y + x)
    e2 = T.tanh(z * x + z)
    e3 = T.tanh(x * y + z)
    k1, k2, k3 = (d.serialize(e.closure, e.shape).text for e in (e1, e2, e3))
    assert k1 == k2
    assert k1 != k3
    w = T.random([16, 8], seed=4).doCache()
    assert d.serialize(T.tanh(w * w + w).closure, w.shape).text != k1


@pytest.mark.gpu
def test_alpha_equivalent_programs_hit_the_runtime_cache(cuda_device):
    d = cuda_device
    rt = d.runtime
    T = d.Tensor
    x, y, z = (T.random([64, 48], seed=s).doCache() for s in (21, 22, 23))
    import ctypes
    from compute import _native
    first = T.exp(x - y * T.fill(0.5, [64, 48]))
    first.flatArray()
    before = rt.cache_stats()
    again = T.exp(z - x * T.fill(0.5, [64, 48]))
    got = again.flatArray()
    after = rt.cache_stats()
    assert after["entries"] == before["entries"]
    # the C ABI's program lookup of the alpha-equivalent text is a cache hit on the same handle
    raw = [d.serialize(t.closure, t.shape).text.encode() for t in (first, again)]
    handles = []
    for r in raw:
        h = ctypes.c_uint64()
        _native.call("cc_program_get", r, ctypes.c_size_t(len(r)), ctypes.byref(h))
        handles.append(h.value)
    assert handles[0] == handles[1]
    assert rt.cache_stats()["hits"] >= after["hits"] + 2
    import numpy as np
    want = np.exp(z.flatArray().astype(np.float64) - np.float32(x.flatArray() * np.float32(0.5)))
    assert np.allclose(got, want, rtol=1e-6)
    other = T.exp(z - x * T.fill(0.25, [64, 48]))  # another literal: another program
    other.flatArray()
    assert rt.cache_stats()["entries"] == after["entries"] + 1
    for t in (x, y, z):
        t.close()

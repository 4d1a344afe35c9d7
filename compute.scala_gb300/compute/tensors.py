"""The Tensor API of Compute.scala over the GB300 runtime.

This mirrors ``trait Tensors`` (Tensors/src/main/scala/com/thoughtworks/compute/
Tensors.scala:199-1442) name for name, so code written against the reference's
``cpu``/``gpu`` objects reads the same against the ``cuda`` object here:

* the companion ``Tensor``: ``apply`` (call it), ``scalar``, ``fill``,
  ``random``, ``randomNormal``, ``abs``, ``sqrt``, ``tanh``, ``exp``, ``log``,
  ``min``, ``max``, ``join`` (:395-600);
* tensor methods: ``nonInline``, ``doCache``, ``sum``, ``toString``,
  ``broadcast``, ``reshape``, unary ``-``/``+``, ``* + - / %``, ``scale``,
  ``translate``, ``permute``, ``transpose``, ``split``, ``shape``, ``padding``,
  ``flatArray``, ``flatBuffer``, ``readScalar``, ``read1DArray`` ..
  ``read5DArray``, ``read1DSeq`` .. ``read5DSeq`` (:636-1261).

The three kinds of tensor keep the reference's meaning (:614-634):
``InlineTensor``/``TransformedTensor`` are expressions merged into the kernel
that consumes them, ``NonInlineTensor`` owns a buffer computed by its own
kernel, and ``CachedTensor`` holds a buffer until it is closed.  Where the
reference always materialises an inline tensor that is viewed
(``TransformedTensor.closure``, :1423-1426), the planner in ``trees.py`` may
instead evaluate the expression at the view's coordinates inside the consuming
kernel; the values are identical, only the memory traffic differs.

Slow actions (``toString``, ``flatArray``, ``read*``, ``doCache``) evaluate the
lazy graph: each distinct tensor is computed once per action, in dependency
order, and intermediate buffers go back to the pool when the action ends.
"""

from __future__ import annotations

import functools
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import affine
from . import trees
from .javafmt import tensor_to_string
from ._native import IllegalArgumentException

__all__ = ["Tensors", "Tensor", "InlineTensor", "TransformedTensor", "NonInlineTensor", "CachedTensor",
           "FillTensor", "TensorSeq", "IllegalArgumentException"]


def _shape_tuple(shape) -> tuple:
    return tuple(int(s) for s in shape)


def _product(shape) -> int:
    p = 1
    for s in shape:
        p *= int(s)
    return p


class _Evaluation:
    """One slow action: memoises each tensor's buffer and releases the
    intermediates at the end (the reference's ``Do`` resource scope).

    With the device's queue pool on, a buffer may still be pending: ``events``
    maps its handle to the event after which it holds its values (the
    reference's ``PendingBuffer.eventOption``, Tensors.scala:253-299)."""

    def __init__(self, device: "Tensors"):
        self.device = device
        self.memo: Dict[int, object] = {}
        self.owned: List[object] = []
        self.keep: List[object] = []
        self.events: Dict[int, int] = {}

    def event_of(self, buf) -> Optional[int]:
        return self.events.get(buf.handle) if self.events else None

    def wait(self, buf) -> None:
        """Blocks until ``buf`` holds its values (Event.waitFor)."""
        e = self.event_of(buf)
        if e is not None:
            self.device.runtime.event_wait(e, 600 * 10 ** 9)

    def close(self, keep=None):
        for e in self.events.values():
            self.device.runtime.event_release(e)
        self.events.clear()
        for b in self.owned:
            if b is not keep:
                b.release()
        self.owned.clear()
        self.memo.clear()


# ----------------------------------------------------------------- tensors

class Tensor:
    """Tensors.scala:636-1261."""

    __slots__ = ("device", "shape", "padding", "_array_term", "__weakref__")

    def __init__(self, device: "Tensors", shape, padding=0.0):
        self.device = device
        self.shape = _shape_tuple(shape)
        self.padding = np.float32(padding)
        self._array_term = None

    # -- the expression of this tensor
    @property
    def closure(self) -> trees.Node:
        raise NotImplementedError

    def arrayTerm(self) -> trees.ArrayParameter:
        """Tensors.scala:1253-1260: this tensor as a kernel input."""
        if self._array_term is None:
            self._array_term = trees.ArrayParameter(self, self.padding, self.shape)
        return self._array_term

    def _compute(self, ev: _Evaluation):
        raise NotImplementedError

    def _buffer(self, ev: _Evaluation):
        key = id(self)
        b = ev.memo.get(key)
        if b is None:
            ev.keep.append(self)
            b = self._compute(ev)
            ev.memo[key] = b
        return b

    # -- delayed operators
    def nonInline(self) -> "NonInlineTensor":
        raise NotImplementedError

    def broadcast(self, newShape) -> "Tensor":
        """Tensors.scala:816-855 (left-aligned: missing trailing dimensions are added)."""
        newShape = _shape_tuple(newShape)
        if newShape == self.shape:
            return self
        if isinstance(self, FillTensor):
            return FillTensor(self.device, self.value, newShape, self.padding)
        n_new, n = len(newShape), len(self.shape)
        if n_new < n:
            raise IllegalArgumentException("Cannot broadcast %s to %s" % (list(self.shape), list(newShape)))
        m = [0.0] * ((n_new + 1) * n)
        for i in range(n):
            if self.shape[i] == newShape[i]:
                m[i * (n_new + 1) + i] = 1.0
            elif self.shape[i] == 1:
                pass
            else:
                raise IllegalArgumentException("Cannot broadcast %s to %s" % (list(self.shape), list(newShape)))
        return self._transform(newShape, m)

    def reshape(self, newShape) -> "NonInlineTensor":
        """Tensors.scala:879-888: same buffer, new shape (row-major)."""
        newShape = _shape_tuple(newShape)
        if _product(newShape) != _product(self.shape):
            raise IllegalArgumentException("reshape from %s to %s" % (list(self.shape), list(newShape)))
        src = self
        return NonInlineTensor(self.device, newShape, self.padding, lambda ev: src._buffer(ev), kind="reshape")

    def _derived(self, closure: trees.Node) -> "InlineTensor":
        return InlineTensor(self.device, closure, self.shape, self.padding)

    def __neg__(self):
        return self._derived(trees.Unary("neg", self.closure))

    def __pos__(self):
        return self

    def _binary(self, op: str, other: "Tensor") -> "InlineTensor":
        left, right = self.device._auto_broadcast(self, other)
        return left._derived(trees.Binary(op, left.closure, right.closure))

    def __mul__(self, other):
        return self._binary("mul", other)

    def __add__(self, other):
        return self._binary("add", other)

    def __sub__(self, other):
        return self._binary("sub", other)

    def __truediv__(self, other):
        return self._binary("div", other)

    def __mod__(self, other):
        return self._binary("mod", other)

    def scale(self, newShape) -> "TransformedTensor":
        """Tensors.scala:950-965."""
        newShape = _shape_tuple(newShape)
        n = len(newShape)
        if n != len(self.shape):
            raise IllegalArgumentException("scale must keep the rank")
        m = [0.0] * (n * (n + 1))
        for i in range(n):
            m[i * (n + 1) + i] = float(self.shape[i]) / newShape[i]
        return self._transform(newShape, m)

    def translate(self, offset: Sequence[float], newShape=None) -> "TransformedTensor":
        """Tensors.scala:970-976: element i of the result is element i - offset of this tensor."""
        if len(offset) != len(self.shape):
            raise IllegalArgumentException("translate offset rank %d != tensor rank %d" % (len(offset), len(self.shape)))
        newShape = self.shape if newShape is None else _shape_tuple(newShape)
        m = affine.translate([-float(o) for o in offset])
        return self._transform(newShape, m)

    def _transform(self, newShape, matrix) -> "TransformedTensor":
        """Tensors.scala:978-1003: views of a view compose into one matrix."""
        if isinstance(self, TransformedTensor):
            m = affine.pre_concatenate(matrix, self.matrix, len(newShape))
            return TransformedTensor(self.device, self.checkpoint, m, newShape, self.padding)
        return TransformedTensor(self.device, self, list(matrix), newShape, self.padding)

    def permute(self, dimensions: Sequence[int]) -> "TransformedTensor":
        """Tensors.scala:1008-1025: result dimension i is this tensor's dimension dimensions[i]."""
        n = len(self.shape)
        if len(dimensions) != n:
            raise IllegalArgumentException("permute needs %d dimensions" % n)
        new_shape = [0] * n
        m = [0.0] * (n * (n + 1))
        for new_i in range(n):
            old_i = int(dimensions[new_i])
            new_shape[new_i] = self.shape[old_i]
            m[old_i * (n + 1) + new_i] = 1.0
        return self._transform(tuple(new_shape), m)

    def transpose(self) -> "TransformedTensor":
        """Tensors.scala:1030."""
        return self.permute(list(reversed(range(len(self.shape)))))

    def split(self, dimension: int) -> "TensorSeq":
        """Tensors.scala:1035-1074."""
        return TensorSeq(self, int(dimension))

    def sum(self) -> "NonInlineTensor":
        """Tensors.scala:673-771: the sum of all elements, as a scalar tensor.

        The reference materialises this tensor, then reduces the buffer.  Here the
        tensor's expression is evaluated inside the reduction kernel (one pass over
        its inputs); the sum is compensated, so it is at least as close to the
        exact sum as the reference's plain float accumulation.
        """
        src = self

        def compute(ev: _Evaluation):
            return ev.device._enqueue(src.closure, src.shape, ev, kind="sum")

        return NonInlineTensor(self.device, (), self.padding, compute, kind="sum")

    # -- slow actions
    def doCache(self) -> "CachedTensor":
        """Tensors.scala:642-666: a tensor whose buffer stays on the device until closed."""
        ev = _Evaluation(self.device)
        try:
            buf = self._buffer(ev)
            ev.wait(buf)
            buf.retain()
        finally:
            ev.close()
        return CachedTensor(self.device, self.shape, self.padding, buf)

    def flatArray(self) -> np.ndarray:
        """Tensors.scala:1099-1118: the elements in row-major order, as float32."""
        ev = _Evaluation(self.device)
        try:
            buf = self._buffer(ev)
            rt = self.device.runtime
            if ev.event_of(buf) is None:
                return rt.download(buf, _product(self.shape))
            # toHostBuffer: a read that waits for the buffer's event (OpenCL.scala:698-715)
            out = np.empty(_product(self.shape), dtype=np.float32)
            done = rt.download_ev(buf, out.ctypes.data, out.nbytes, wait=[ev.event_of(buf)])
            try:
                rt.event_wait(done, 600 * 10 ** 9)
            finally:
                rt.event_release(done)
            return out
        finally:
            ev.close()

    flatBuffer = flatArray

    def toString(self) -> str:
        """Tensors.scala:776-811."""
        return tensor_to_string(self.shape, self.flatArray())

    def __str__(self):
        return self.toString()

    def __repr__(self):
        return "%s(shape=%s)" % (type(self).__name__, list(self.shape))

    def readScalar(self) -> float:
        return float(self.flatArray()[0])

    def read1DArray(self) -> np.ndarray:
        return self.flatArray()

    def _read_nd(self, nd: int) -> np.ndarray:
        if len(self.shape) < nd:
            raise IllegalArgumentException("tensor of rank %d read as %dD" % (len(self.shape), nd))
        return self.flatArray().reshape(self.shape[:nd] + (-1,) if len(self.shape) > nd else self.shape)

    def read2DArray(self):
        return self._read_nd(2)

    def read3DArray(self):
        return self._read_nd(3)

    def read4DArray(self):
        return self._read_nd(4)

    def read5DArray(self):
        return self._read_nd(5)

    def read1DSeq(self):
        return [float(v) for v in self.flatArray()]

    def read2DSeq(self):
        return self._read_nd(2).tolist()

    def read3DSeq(self):
        return self._read_nd(3).tolist()

    def read4DSeq(self):
        return self._read_nd(4).tolist()

    def read5DSeq(self):
        return self._read_nd(5).tolist()


class InlineTensor(Tensor):
    """Tensors.scala:1400-1411: an expression merged into the kernel that uses it."""

    __slots__ = ("_closure",)

    def __init__(self, device, closure, shape, padding=0.0):
        super().__init__(device, shape, padding)
        self._closure = closure

    @property
    def closure(self):
        return self._closure

    def _compute(self, ev):
        return ev.device._enqueue(self.closure, self.shape, ev, kind="ew")

    def nonInline(self) -> "NonInlineTensor":
        src = self
        return NonInlineTensor(self.device, self.shape, self.padding, lambda ev: src._buffer(ev), kind="nonInline")


class FillTensor(InlineTensor):
    """Tensors.scala:1393-1396: a constant."""

    __slots__ = ("value",)

    def __init__(self, device, value, shape, padding=0.0):
        self.value = np.float32(value)
        super().__init__(device, trees.Literal(self.value), shape, padding)


class TransformedTensor(InlineTensor):
    """Tensors.scala:1413-1428: a view (``matrix``) of ``checkpoint``."""

    __slots__ = ("checkpoint", "matrix")

    def __init__(self, device, checkpoint, matrix, shape, padding):
        self.checkpoint = checkpoint
        self.matrix = list(matrix)
        super().__init__(device, None, shape, padding)

    @property
    def closure(self):
        if self._closure is None:
            self._closure = trees.Extract(trees.Transform(self.checkpoint.arrayTerm(), self.matrix))
        return self._closure


class NonInlineTensor(Tensor):
    """Tensors.scala:1431-1440: a tensor backed by its own buffer."""

    __slots__ = ("_make", "kind", "_closure")

    def __init__(self, device, shape, padding, make, kind="buffer"):
        super().__init__(device, shape, padding)
        self._make = make
        self.kind = kind
        self._closure = None

    @property
    def closure(self):
        if self._closure is None:
            self._closure = trees.Extract(self.arrayTerm())
        return self._closure

    def _compute(self, ev):
        return self._make(ev)

    def nonInline(self):
        return self


class CachedTensor(NonInlineTensor):
    """Tensors.scala:602, :642-666: keeps its buffer until ``close``."""

    __slots__ = ("_cached",)

    def __init__(self, device, shape, padding, buf):
        self._cached = buf
        super().__init__(device, shape, padding, lambda ev: buf, kind="cached")

    def close(self):
        if self._cached is not None:
            self._cached.release()
            self._cached = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _compute(self, ev):
        if self._cached is None:
            raise IllegalArgumentException("the cached tensor has been closed")
        return self._cached


class TensorSeq:
    """The IndexedSeq ``split`` returns (Tensors.scala:1035-1074)."""

    __slots__ = ("tensor", "dimension", "newShape")

    def __init__(self, tensor: Tensor, dimension: int):
        n = len(tensor.shape)
        if not 0 <= dimension < n:
            raise IllegalArgumentException("split dimension %d of a rank-%d tensor" % (dimension, n))
        self.tensor = tensor
        self.dimension = dimension
        self.newShape = tensor.shape[:dimension] + tensor.shape[dimension + 1:]

    def __len__(self):
        return self.tensor.shape[self.dimension]

    def __getitem__(self, index):
        if isinstance(index, slice):
            return [self[i] for i in range(*index.indices(len(self)))]
        if index < 0:
            index += len(self)
        if not 0 <= index < len(self):
            raise IndexError(index)
        n = len(self.tensor.shape)
        d = self.dimension
        m = [0.0] * (n * n)
        for i in range(d):
            m[i * n + i] = 1.0
        m[d * n + n - 1] = float(index)
        for i in range(d + 1, n):
            m[i * n + i - 1] = 1.0
        return self.tensor._transform(self.newShape, m)

    def __iter__(self):
        for i in range(len(self)):
            yield self[i]

    def reduce(self, f):
        """Scala's ``Seq.reduce``: a left fold."""
        return functools.reduce(f, iter(self))

    def map(self, f):
        return [f(t) for t in self]

    def toString(self):
        return "TensorSeq(" + ", ".join(t.toString() for t in self) + ")"

    def __str__(self):
        return self.toString()


# ----------------------------------------------------------------- the device object

class _TensorCompanion:
    """``object Tensor`` (Tensors.scala:395-600)."""

    def __init__(self, device: "Tensors"):
        self._d = device

    def __call__(self, elements, padding=0.0) -> NonInlineTensor:
        """Tensor.apply (:445-463): a tensor from nested sequences of floats."""
        shape, flat = _flatten(elements)
        data = np.asarray(flat, dtype=np.float32)
        device = self._d

        def compute(ev):
            buf = device.runtime.alloc(max(1, data.size) * 4)
            ev.owned.append(buf)
            device.runtime.upload(buf, data)
            return buf

        return NonInlineTensor(device, shape, padding, compute, kind="literal")

    def scalar(self, value, padding=0.0) -> FillTensor:
        return self.fill(value, (), padding)

    def fill(self, value, shape, padding=0.0) -> FillTensor:
        return FillTensor(self._d, value, shape, padding)

    def random(self, shape, seed: Optional[int] = None, padding=0.0) -> NonInlineTensor:
        """Tensors.scala:479-497: uniform floats hash(i ^ seed) / 2^32."""
        return self._random(shape, seed, padding, normal=False)

    def randomNormal(self, shape, seed: Optional[int] = None, padding=0.0) -> NonInlineTensor:
        """Tensors.scala:500-524: Box-Muller normal floats."""
        return self._random(shape, seed, padding, normal=True)

    def _random(self, shape, seed, padding, normal):
        shape = _shape_tuple(shape)
        if seed is None:
            seed = int(np.random.randint(-2 ** 31, 2 ** 31))
        seed32 = int(seed) & 0xFFFFFFFF
        size = _product(shape)
        alloc = size + (size & 1) if normal else size
        device = self._d

        def compute(ev):
            buf = device.runtime.alloc(max(1, alloc) * 4)
            ev.owned.append(buf)
            device.runtime.random(buf, size, seed32, normal)
            if device.queues:
                ev.events[buf.handle] = device.runtime.event()  # on the context stream
            return buf

        return NonInlineTensor(device, shape, padding, compute, kind="randomNormal" if normal else "random")

    def abs(self, t: Tensor):
        return t._derived(trees.Unary("abs", t.closure))

    def sqrt(self, t: Tensor):
        return t._derived(trees.Unary("sqrt", t.closure))

    def tanh(self, t: Tensor):
        return t._derived(trees.Unary("tanh", t.closure))

    def exp(self, t: Tensor):
        return t._derived(trees.Unary("exp", t.closure))

    def log(self, t: Tensor):
        return t._derived(trees.Unary("log", t.closure))

    def min(self, a: Tensor, b: Tensor):
        left, right = self._d._auto_broadcast(a, b)
        return left._derived(trees.Binary("min", left.closure, right.closure))

    def max(self, a: Tensor, b: Tensor):
        left, right = self._d._auto_broadcast(a, b)
        return left._derived(trees.Binary("max", left.closure, right.closure))

    def join(self, tensors: Sequence[Tensor], dimension: Optional[int] = None) -> Tensor:
        """Tensors.scala:560-598: stack along a new last dimension (then permute to ``dimension``)."""
        tensors = list(tensors)
        if not tensors:
            raise IllegalArgumentException("join of no tensors")
        head = tensors[0]
        device = self._d
        out_shape = head.shape + (len(tensors),)

        def compute(ev):
            return device._enqueue(trees.Concatenate([t.closure for t in tensors]), head.shape, ev, kind="ew",
                                   tuple_len=len(tensors))

        joined = NonInlineTensor(device, out_shape, head.padding, compute, kind="join")
        if dimension is None or dimension == len(out_shape) - 1:
            return joined
        n = len(out_shape)
        perm = [i if i < dimension else (n - 1 if i == dimension else i - 1) for i in range(n)]
        return joined.permute(perm)


def _flatten(elements):
    """Shape and row-major elements of nested sequences (the reference's TensorBuilder, Tensors.scala:43-94)."""
    if isinstance(elements, np.ndarray):
        return tuple(elements.shape), elements.astype(np.float32).ravel().tolist()
    if isinstance(elements, (list, tuple, range)):
        if len(elements) == 0:
            return (0,), []
        parts = [_flatten(e) for e in elements]
        s0 = parts[0][0]
        for s, _ in parts[1:]:
            if s != s0:
                raise IllegalArgumentException("ragged nested sequence: %s vs %s" % (list(s0), list(s)))
        flat = []
        for _, f in parts:
            flat.extend(f)
        return (len(elements),) + s0, flat
    return (), [float(elements)]


class Tensors:
    """A device object: the tensors of one GPU.

    ``cuda = Tensors(device=0)`` is the counterpart of the reference's ``gpu``
    object (gpu/src/main/scala/com/thoughtworks/compute/gpu.scala:15-27).  The
    runtime (``_native``/``runtime.NativeRuntime``) is created on first use.
    """

    def __init__(self, device: int = 0, flags: int = 0, planner: Optional[trees.Planner] = None, runtime=None,
                 queues: bool = False, tuner: str = "learned"):
        self.device_ordinal = device
        self.flags = flags
        # launch configurations of the native runtime's programs: "learned" (the shipped
        # cost model's choice, timed against the standard kernel at a program's first
        # launch; the faster is kept), "exhaustive" (every configuration timed) or "off"
        # (the standard kernels); programs of more than 64 nodes are never tuned
        if tuner not in ("learned", "exhaustive", "off"):
            raise IllegalArgumentException("tuner must be 'learned', 'exhaustive' or 'off'")
        self.tuner = tuner
        self._cost_model = None
        # queues=True: every kernel of an action goes to the runtime's queue pool and
        # waits only for the events of the buffers it reads, as the reference's
        # CompiledKernel.run enqueues with its inputs' events (Tensors.scala:1331-1381);
        # independent subgraphs then run concurrently.  False: one ordered stream.
        self.queues = queues
        self.planner = planner if planner is not None else trees.Planner()
        self._runtime = runtime
        self.Tensor = _TensorCompanion(self)

    @property
    def runtime(self):
        if self._runtime is None:
            from .runtime import NativeRuntime
            rt = NativeRuntime(self.device_ordinal, self.flags)
            if self.tuner == "learned":
                from . import tuner as tuner_mod
                if os.path.exists(tuner_mod.DEFAULT_MODEL):
                    self._cost_model = tuner_mod.use_learned_tuner(rt)
                else:
                    rt.config_set("tuner", 0)
            else:
                rt.config_set("tuner", 1 if self.tuner == "exhaustive" else 0)
            self._runtime = rt
        return self._runtime

    @staticmethod
    def _auto_broadcast_shape(s1, s2):
        """Tensors.scala:208-222."""
        out = []
        for i in range(max(len(s1), len(s2))):
            if i >= len(s1) or s1[i] == 1:
                out.append(s2[i])
            elif i >= len(s2) or s2[i] == 1:
                out.append(s1[i])
            elif s1[i] == s2[i]:
                out.append(s1[i])
            else:
                raise IllegalArgumentException(
                    "Failed to automatically broadcast between shape [%s] and [%s]}"
                    % (",".join(map(str, s1)), ",".join(map(str, s2))))
        return tuple(out)

    def _auto_broadcast(self, a: Tensor, b: Tensor):
        shape = self._auto_broadcast_shape(a.shape, b.shape)
        return a.broadcast(shape), b.broadcast(shape)

    def _is_inline(self, t) -> bool:
        return isinstance(t, InlineTensor) and not isinstance(t, TransformedTensor)

    def serialize(self, closure, shape, kind="ew") -> trees.Serialized:
        return trees.serialize(closure, shape, kind, self.planner, self._is_inline)

    def _enqueue(self, closure, shape, ev: _Evaluation, kind="ew", tuple_len=1):
        """Tensors.scala:1291-1392: compile (or find) the kernel, evaluate its inputs, launch."""
        ser = self.serialize(closure, shape, kind)
        prog = self.runtime.program(ser.text)
        inputs = [t._buffer(ev) for t in ser.params]
        n_out = 1 if kind == "sum" else _product(shape) * tuple_len
        out = self.runtime.alloc(max(1, n_out) * 4)
        ev.owned.append(out)
        if self.queues:
            wait = [e for e in (ev.event_of(b) for b in inputs) if e is not None]
            ev.events[out.handle] = self.runtime.launch_ev(prog, inputs, out, wait)
        else:
            self.runtime.launch(prog, inputs, out)
        return out

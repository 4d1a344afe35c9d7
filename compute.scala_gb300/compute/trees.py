"""Expression trees of lazily evaluated tensors, and their wire format.

The node set is the reference's term algebra for the fused-tensor path
(Trees/src/main/scala/com/thoughtworks/compute/Trees.scala): float literals
(:368-377), the unary operators ``Exp/Log/Abs/Tanh/Sqrt/UnaryMinus`` (:380-447,
:604-615), the binary operators ``Plus/Minus/Times/Div/Percent/Min/Max``
(:450-602), ``ArrayParameter`` (:755-823), ``Transform`` (:676-690), ``Extract``
(:660-672) and the tuple ``Concatenate`` used by ``join`` (:956-973).

Two trees are the same kernel when their *alpha-converted* forms are equal
(Trees.scala:266-298, :807-822): parameter identities are replaced by their
order of first appearance.  Here the alpha-converted form is the IR text that
crosses the C ABI (``serialize``), so the runtime's program cache keys on
exactly the structure the reference's Guava kernel cache keys on
(Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala:1267-1293),
plus the output shape (the reference forgets it, see ``serialize``).

IR text (one item per line, nodes numbered from 0 in line order)::

    ccir 1 <kind>                  kind: ew (elementwise store) | sum (full sum)
    o <rank> <dims...>             the output frame's shape
    p <rank> <dims...> <pad>       array parameter; kernel input #k is the k-th p line
    l <bits>                       float literal (IEEE-754 binary32 bits, 8 hex digits)
    x <param> <cols> <m...>        Extract of a parameter through a view matrix
                                   (rows = parameter rank, cols = frame rank + 1)
    v <node> <rank> <dims...> <pad> <cols> <m...>
                                   evaluate <node> at view coordinates of a tensor
                                   of shape <dims>; outside it the value is <pad>
    u <op> <a>                     neg exp log tanh abs sqrt
    b <op> <a> <b>                 add sub mul div mod min max
    t <n> <a1> ... <an>            tuple of n values (root only; ``join``)
    r <node>                       the root

Matrix coefficients are written as shortest round-trip decimal doubles, so the
runtime recovers the exact doubles the view composition produced.
"""

from __future__ import annotations

import struct
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


def f32_bits(value: float) -> str:
    return "%08x" % struct.unpack("<I", struct.pack("<f", np.float32(value)))[0]


def _double_text(v: float) -> str:
    if v == 0.0:
        return "0"
    if float(v).is_integer() and abs(v) < 2 ** 53:
        return str(int(v))
    return repr(float(v))


class Node:
    __slots__ = ()


class Literal(Node):
    __slots__ = ("value",)

    def __init__(self, value):
        self.value = np.float32(value)


class Unary(Node):
    __slots__ = ("op", "a")
    OPS = ("neg", "exp", "log", "tanh", "abs", "sqrt")

    def __init__(self, op: str, a: Node):
        assert op in self.OPS
        self.op = op
        self.a = a


class Binary(Node):
    __slots__ = ("op", "a", "b")
    OPS = ("add", "sub", "mul", "div", "mod", "min", "max")

    def __init__(self, op: str, a: Node, b: Node):
        assert op in self.OPS
        self.op = op
        self.a = a
        self.b = b


class ArrayParameter(Node):
    """A tensor used as a kernel input (Trees.scala:755-823).  ``id`` is the tensor."""

    __slots__ = ("id", "padding", "shape")

    def __init__(self, id, padding, shape: Sequence[int]):
        self.id = id
        self.padding = np.float32(padding)
        self.shape = tuple(int(s) for s in shape)


class Transform(Node):
    __slots__ = ("array", "matrix")

    def __init__(self, array: ArrayParameter, matrix: Sequence[float]):
        self.array = array
        self.matrix = [float(m) for m in matrix]


class Extract(Node):
    __slots__ = ("array",)

    def __init__(self, array: Node):
        self.array = array


class Concatenate(Node):
    __slots__ = ("elements",)

    def __init__(self, elements: Sequence[Node]):
        self.elements = list(elements)


def identity_matrix(source_rank: int, target_rank: int) -> List[float]:
    """The matrix of ``ArrayParameter.extract`` (OpenCLKernelBuilder.scala:435-455):
    source dimension i reads the i-th global id."""
    cols = target_rank + 1
    m = [0.0] * (source_rank * cols)
    for i in range(source_rank):
        m[i * cols + i] = 1.0
    return m


class Planner:
    """Decides, per view of an inline (not yet materialised) tensor, whether the
    view reads a materialised buffer (what the reference always does,
    Tensors.scala:1413-1428 with :1253-1260) or evaluates the tensor's expression
    at the view's coordinates inside the consuming kernel.

    Both give identical bits: a materialised element is the same float the
    inlined expression computes, and out-of-range view coordinates yield the
    tensor's padding either way.  Inlining is chosen when the view does not
    make the kernel recompute elements: the expression is a bare literal, or
    the number of element evaluations it causes is at most ``max_recompute``
    times the tensor's own size.
    """

    def __init__(self, max_recompute: float = 1.5, enabled: bool = True, merge_common: bool = None):
        self.max_recompute = max_recompute
        self.enabled = enabled
        # write structurally identical subexpressions once (see serialize); off with
        # fusion off, which keeps the reference's kernel structure
        self.merge_common = enabled if merge_common is None else merge_common

    def inline(self, tensor, uses: int, frame_elements: int) -> bool:
        if not self.enabled:
            return False
        closure = tensor.closure
        if isinstance(closure, Literal):
            return True
        size = max(1, int(np.prod(tensor.shape, dtype=np.int64)))
        return uses * frame_elements <= self.max_recompute * size


class Serialized:
    __slots__ = ("text", "params", "n_nodes")

    def __init__(self, text: str, params: List, n_nodes: int):
        self.text = text
        self.params = params  # tensors, in kernel-argument order
        self.n_nodes = n_nodes


def _count_views(root: Node) -> Dict[int, int]:
    """Number of Extract sites per parameter tensor (keyed by ``id(tensor)``) in one tree."""
    counts: Dict[int, int] = {}
    seen = set()
    stack = [root]
    while stack:
        n = stack.pop()
        if id(n) in seen:
            continue
        seen.add(id(n))
        if isinstance(n, Extract):
            arr = n.array
            p = arr.array if isinstance(arr, Transform) else arr
            if isinstance(p, ArrayParameter):
                counts[id(p.id)] = counts.get(id(p.id), 0) + 1
        elif isinstance(n, Unary):
            stack.append(n.a)
        elif isinstance(n, Binary):
            stack.append(n.a)
            stack.append(n.b)
        elif isinstance(n, Concatenate):
            stack.extend(n.elements)
    return counts


def serialize(root: Node, out_shape: Sequence[int], kind: str = "ew",
              planner: Optional[Planner] = None, is_inline=None) -> Serialized:
    """Alpha-convert ``root`` into IR text.

    ``is_inline(tensor)`` tells whether a parameter's tensor is an inline
    (unmaterialised) expression that the planner may fuse.  Parameters are
    numbered in order of first appearance in a left-to-right walk, which is the
    reference's ``parameterDescendants`` order (Tensors.scala:230-251).

    The output shape is part of the text.  The reference keys its kernel cache
    on the closure alone (Tensors.scala:1293) and reuses the first shape's
    ND-range for a structurally equal closure of another shape; keying on the
    shape too avoids that.
    """
    import sys
    if sys.getrecursionlimit() < 200000:
        sys.setrecursionlimit(200000)  # a J-term fold (split(d).reduce) nests J deep
    out_shape = tuple(int(s) for s in out_shape)
    lines: List[str] = ["ccir 1 %s" % kind, "o %d%s" % (len(out_shape), "".join(" %d" % d for d in out_shape))]
    params: List = []
    # id(node) -> node number.  A node's line does not depend on the frame it is
    # evaluated in (its matrices are sized by its own tensor's shape), so a
    # subtree reached through several views is written once and shared.
    node_ids: Dict[int, int] = {}
    param_ids: Dict[int, int] = {}  # id(ArrayParameter) -> node number
    inline_memo: Dict[int, bool] = {}
    counts_memo: Dict[int, Dict[int, int]] = {}

    # Identical lines (children already numbered canonically) denote the same
    # function of the frame coordinates, so each is written once: common
    # subexpressions -- the same translated input channel used by every filter
    # of a convolution -- become one node, which the code generator evaluates
    # (and loads) once per point.  Parameter lines are never merged.
    line_ids: Dict[str, int] = {}
    merge = planner is None or planner.merge_common

    def emit(line: str) -> int:
        if merge and not line.startswith("p "):
            got = line_ids.get(line)
            if got is not None:
                return got
        lines.append(line)
        nid = len(lines) - 3  # node numbers start after the two header lines
        if merge and not line.startswith("p "):
            line_ids[line] = nid
        return nid

    def elements(shape) -> int:
        return int(np.prod(shape, dtype=np.int64)) if shape else 1

    def counts_of(tree: Node) -> Dict[int, int]:
        c = counts_memo.get(id(tree))
        if c is None:
            c = _count_views(tree)
            counts_memo[id(tree)] = c
        return c

    def gen(node: Node, frame_shape: Tuple[int, ...], evals: float, counts: Dict[int, int]) -> int:
        # ``evals``: how many times each element of this frame is evaluated per output element
        key = id(node)
        got = node_ids.get(key)
        if got is not None:
            return got
        if isinstance(node, Literal):
            nid = emit("l " + f32_bits(node.value))
        elif isinstance(node, Unary):
            a = gen(node.a, frame_shape, evals, counts)
            nid = emit("u %s %d" % (node.op, a))
        elif isinstance(node, Binary):
            a = gen(node.a, frame_shape, evals, counts)
            b = gen(node.b, frame_shape, evals, counts)
            nid = emit("b %s %d %d" % (node.op, a, b))
        elif isinstance(node, Extract):
            arr = node.array
            if isinstance(arr, Transform):
                param, matrix = arr.array, arr.matrix
            else:
                param, matrix = arr, None
            if not isinstance(param, ArrayParameter):
                raise TypeError("Extract of a non-parameter array")
            rank = len(param.shape)
            if matrix is None:
                if rank > len(frame_shape):
                    raise ValueError("parameter rank %d exceeds the kernel rank %d" % (rank, len(frame_shape)))
                matrix = identity_matrix(rank, len(frame_shape))
            cols = len(frame_shape) + 1
            if len(matrix) != rank * cols:
                raise ValueError("view matrix has %d entries, expected %d x %d" % (len(matrix), rank, cols))
            tensor = param.id
            fuse = False
            if is_inline is not None and planner is not None and is_inline(tensor):
                k = id(tensor)
                if k not in inline_memo:
                    uses = counts.get(k, 1)
                    inline_memo[k] = planner.inline(tensor, uses, int(elements(frame_shape) * evals))
                fuse = inline_memo[k]
            mtext = " ".join(_double_text(m) for m in matrix)
            if fuse:
                inner_shape = tuple(param.shape)
                closure = tensor.closure
                sub = gen(closure, inner_shape,
                          evals * elements(frame_shape) / max(1, elements(inner_shape)), counts_of(closure))
                nid = emit("v %d %d%s %s %d%s" % (sub, rank, "".join(" %d" % d for d in inner_shape),
                                                  f32_bits(param.padding), cols, (" " + mtext) if mtext else ""))
            else:
                pid = param_ids.get(id(param))
                if pid is None:
                    pid = emit("p %d%s %s" % (rank, "".join(" %d" % d for d in param.shape), f32_bits(param.padding)))
                    param_ids[id(param)] = pid
                    params.append(tensor)
                nid = emit("x %d %d%s" % (pid, cols, (" " + mtext) if mtext else ""))
        elif isinstance(node, Concatenate):
            raise ValueError("a tuple may only be the root of a kernel")
        else:
            raise TypeError("unknown node %r" % (node,))
        node_ids[key] = nid
        return nid

    counts = counts_of(root)
    if isinstance(root, Concatenate):
        ids = [gen(e, out_shape, 1.0, counts) for e in root.elements]
        t = emit("t %d%s" % (len(ids), "".join(" %d" % i for i in ids)))
        lines.append("r %d" % t)
    else:
        r = gen(root, out_shape, 1.0, counts)
        lines.append("r %d" % r)
    n_nodes = len(lines) - 3
    return Serialized("\n".join(lines) + "\n", params, n_nodes)

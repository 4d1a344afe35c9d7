"""ORACLE (test infrastructure only): a CPU restatement of the reference kernels' semantics.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may use
this module, and only as the checker.  The product path never calls it.

``evaluate(ir_text, inputs)`` computes what the reference's generated OpenCL
kernel computes for the same expression tree, point by point, in numpy:

* every operator node is one binary32 operation, rounded once, like one
  ``const float _N = ...;`` statement of OpenCLKernelBuilder.scala:245-326 and
  :516-571 (``+ - * /`` and ``sqrt`` are correctly rounded in IEEE binary32;
  ``fmin``/``fmax`` return the non-NaN operand; ``exp``/``log``/``tanh`` are
  evaluated in binary64 and rounded, i.e. correctly rounded in practice, which
  is the yardstick the device's <= 2 ulp functions are measured against; ``%``
  is ``fmod``, which OpenCL C does not accept on floats, see below);
* a view index is ``(int)(sum of gid * coefficient + constant)`` where each
  coefficient is the text java.text.DecimalFormat prints for it (at most three
  fraction digits, HALF_EVEN): integer texts are C ``int`` literals, others
  ``double`` literals, and the sum is typed and evaluated left to right like
  the C expression (OpenCLKernelBuilder.scala:14-32, :348-386);
* a row with no non-zero coefficient reads index 0 without a bounds check, any
  other index outside ``[0, dim)`` yields the padding (:383-411);
* ``v`` nodes (an inline tensor evaluated at view coordinates) are the same
  thing as the reference's materialise-then-view: the padding outside, the
  tensor's own expression inside.

Divergences from the reference that are deliberate and documented:
``%`` on floats fails to compile in the reference's OpenCL C; here it is
C's ``fmodf`` (the meaning of Scala's ``Float.%``).  Infinite literals print
as the invalid identifier ``INFINITE`` there (:252-262); here they are
infinities.
"""

from __future__ import annotations

import decimal
import struct
from typing import Dict, List, Sequence, Tuple

import numpy as np


def bits_to_f32(bits: str) -> np.float32:
    return np.frombuffer(struct.pack("<I", int(bits, 16)), dtype=np.float32)[0]


_CTX = decimal.Context(prec=2000, rounding=decimal.ROUND_HALF_EVEN)


def decimal_format3(v: float) -> str:
    """java.text.DecimalFormat("#,##0.###") without grouping, HALF_EVEN (OpenCLKernelBuilder.scala:14-32)."""
    q = decimal.Decimal(float(v)).quantize(decimal.Decimal("0.001"), context=_CTX)
    s = format(q, "f")  # the sign survives rounding to zero: -0.0001 -> "-0.000"
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


class _Frame:
    __slots__ = ("gid", "n")

    def __init__(self, gid: List[np.ndarray], n: int):
        self.gid = gid
        self.n = n


def _index_rows(m: Sequence[float], cols: int, dims: Sequence[int], frame: _Frame):
    """Returns (indices per row, in-bounds mask) for one view, as the C expression computes them."""
    idx = []
    ok = np.ones(frame.n, dtype=bool)
    for y, dim in enumerate(dims):
        acc = None  # (value array, is_double)
        for x in range(cols):
            s = float(m[y * cols + x])
            if s == 0.0:
                continue
            text = decimal_format3(s)
            is_double = "." in text
            lit = float(text) if is_double else int(text)
            if x < cols - 1:
                g = frame.gid[x]
                if s == 1.0:
                    term, tdouble = g.astype(np.int64), False
                elif is_double:
                    term, tdouble = g.astype(np.float64) * lit, True
                else:
                    term, tdouble = (g.astype(np.int64) * lit).astype(np.int64), False
            else:
                if is_double:
                    term, tdouble = np.full(frame.n, lit, dtype=np.float64), True
                else:
                    term, tdouble = np.full(frame.n, lit, dtype=np.int64), False
            if acc is None:
                acc = (term, tdouble)
            else:
                a, ad = acc
                if ad or tdouble:
                    acc = (a.astype(np.float64) + term.astype(np.float64), True)
                else:
                    acc = (a + term, False)
        if acc is None:
            idx.append(np.zeros(frame.n, dtype=np.int64))
            if dim == 0:
                ok &= False
            continue
        a, ad = acc
        if ad:
            a = np.trunc(a)
            a = np.clip(a, -2 ** 31, 2 ** 31 - 1).astype(np.int64)
        i = a.astype(np.int64)
        idx.append(i)
        ok &= (i >= 0) & (i < dim)
    return idx, ok


def _flat_offset(idx: List[np.ndarray], dims: Sequence[int]) -> np.ndarray:
    off = np.zeros_like(idx[0]) if idx else np.zeros(1, dtype=np.int64)
    for i, d in zip(idx, dims):
        off = off * int(d) + i
    return off


def _f64(fn, a):
    with np.errstate(all="ignore"):
        return fn(a.astype(np.float64)).astype(np.float32)


def parse(ir_text: str):
    lines = [ln.split() for ln in ir_text.strip().split("\n")]
    assert lines[0][0] == "ccir" and lines[0][1] == "1"
    kind = lines[0][2]
    out_rank = int(lines[1][1])
    out_shape = tuple(int(v) for v in lines[1][2:2 + out_rank])
    nodes = []
    root = None
    for ln in lines[2:]:
        if ln[0] == "r":
            root = int(ln[1])
            break
        nodes.append(ln)
    return kind, out_shape, nodes, root


def evaluate(ir_text: str, inputs: Sequence[np.ndarray]):
    """Evaluates an IR text on float32 inputs (flat arrays, in parameter order).

    Returns the flat float32 output (tuple roots interleaved as the kernel
    stores them) for an ``ew`` program, or the float32 element values that a
    ``sum`` program adds up.
    """
    kind, out_shape, nodes, root = parse(ir_text)
    params: Dict[int, Tuple[int, Tuple[int, ...], np.float32]] = {}
    k = 0
    for i, ln in enumerate(nodes):
        if ln[0] == "p":
            r = int(ln[1])
            params[i] = (k, tuple(int(v) for v in ln[2:2 + r]), bits_to_f32(ln[2 + r]))
            k += 1
    if len(inputs) != k:
        raise ValueError("program takes %d inputs, got %d" % (k, len(inputs)))
    flat_inputs = [np.ascontiguousarray(a, dtype=np.float32).ravel() for a in inputs]

    n = int(np.prod(out_shape, dtype=np.int64)) if out_shape else 1
    lin = np.arange(n, dtype=np.int64)
    gid = list(np.unravel_index(lin, out_shape)) if out_shape else []
    frame0 = _Frame([g.astype(np.int64) for g in gid], n)
    memo: Dict[Tuple[int, int], np.ndarray] = {}
    counter = [0]

    def ev(i: int, fr: _Frame, fid: int) -> np.ndarray:
        key = (i, fid)
        if key in memo:
            return memo[key]
        ln = nodes[i]
        tag = ln[0]
        if tag == "l":
            out = np.full(fr.n, bits_to_f32(ln[1]), dtype=np.float32)
        elif tag == "u":
            a = ev(int(ln[2]), fr, fid)
            op = ln[1]
            with np.errstate(all="ignore"):
                if op == "neg":
                    out = -a
                elif op == "abs":
                    out = np.abs(a)
                elif op == "sqrt":
                    out = np.sqrt(a)
                elif op == "exp":
                    out = _f64(np.exp, a)
                elif op == "log":
                    out = _f64(np.log, a)
                elif op == "tanh":
                    out = _f64(np.tanh, a)
                else:
                    raise ValueError(op)
        elif tag == "b":
            a = ev(int(ln[2]), fr, fid)
            b = ev(int(ln[3]), fr, fid)
            op = ln[1]
            with np.errstate(all="ignore"):
                if op == "add":
                    out = a + b
                elif op == "sub":
                    out = a - b
                elif op == "mul":
                    out = a * b
                elif op == "div":
                    out = a / b
                elif op == "mod":
                    out = np.fmod(a, b)
                elif op == "min":
                    out = np.fmin(a, b)
                elif op == "max":
                    out = np.fmax(a, b)
                else:
                    raise ValueError(op)
        elif tag == "x":
            pk, pdims, pad = params[int(ln[1])]
            cols = int(ln[2])
            m = [float(v) for v in ln[3:]]
            data = flat_inputs[pk]
            if not pdims:
                out = np.full(fr.n, data[0], dtype=np.float32)
            else:
                idx, ok = _index_rows(m, cols, pdims, fr)
                out = np.full(fr.n, pad, dtype=np.float32)
                if ok.any():
                    off = _flat_offset([ix[ok] for ix in idx], pdims)
                    out[ok] = data[off]
        elif tag == "v":
            sub = int(ln[1])
            r = int(ln[2])
            vdims = tuple(int(v) for v in ln[3:3 + r])
            pad = bits_to_f32(ln[3 + r])
            cols = int(ln[4 + r])
            m = [float(v) for v in ln[5 + r:]]
            idx, ok = _index_rows(m, cols, vdims, fr)
            out = np.full(fr.n, pad, dtype=np.float32)
            if ok.any():
                counter[0] += 1
                inner = _Frame([ix[ok] for ix in idx], int(ok.sum()))
                out[ok] = ev(sub, inner, counter[0])
        elif tag == "t":
            raise ValueError("tuple below the root")
        else:
            raise ValueError("unknown node " + tag)
        memo[key] = out
        return out

    rl = nodes[root]
    if rl[0] == "t":
        cnt = int(rl[1])
        parts = [ev(int(v), frame0, 0) for v in rl[2:2 + cnt]]
        out = np.stack(parts, axis=-1).ravel() if parts else np.zeros(0, np.float32)
    else:
        out = ev(root, frame0, 0)
    if kind == "sum":
        return out.astype(np.float32)
    return out.astype(np.float32)


def exact_sum(values: np.ndarray) -> float:
    """The sum of float32 values, exact up to one final rounding to binary64."""
    import math
    return math.fsum(np.asarray(values, dtype=np.float64).tolist())


def window_text(ir_text: str, length: int) -> str:
    """The IR text of a contiguous elementwise program (every input read at the
    output's own index, no views) over ``length`` points instead of its own
    length: its value at a point depends only on the inputs at that point, so
    any window of its inputs evaluates the matching window of its output."""
    kind, out_shape, nodes, root = parse(ir_text)
    if kind != "ew" or len(out_shape) != 1:
        raise ValueError("not a one-dimensional elementwise program")
    lines = ["ccir 1 ew", "o 1 %d" % length]
    for ln in nodes:
        if ln[0] == "p":
            if ln[1] != "1" or int(ln[2]) != out_shape[0]:
                raise ValueError("parameter is not read contiguously")
            lines.append("p 1 %d %s" % (length, ln[3]))
        elif ln[0] == "x":
            if ln[2:] != ["2", "1", "0"]:
                raise ValueError("parameter read through a view")
            lines.append(" ".join(ln))
        elif ln[0] in ("l", "u", "b"):
            lines.append(" ".join(ln))
        else:
            raise ValueError("node %s in a contiguous program" % ln[0])
    lines.append("r %d" % root)
    return "\n".join(lines) + "\n"


_TRANSCENDENTAL = ("exp", "log", "tanh")


def evaluate_with_bound(ir_text: str, inputs: Sequence[np.ndarray], ulps: float = 2.0, safety: float = 4.0,
                        perturb=None):
    """The oracle's values of a contiguous elementwise program (no views), and
    per point a bound on how far a device whose exp/log/tanh are within
    ``ulps`` ulp of the correctly rounded value (and whose other operations
    round exactly like the oracle's) can be from them.

    The bound is first-order error propagation: at each transcendental node the
    device may differ by ``ulps`` ulp of the node's value; every node above one
    may then round to a neighbouring float, one more ulp of its value; each
    such difference reaches the output scaled by the output's partial
    derivative with respect to that node (reverse-mode adjoints on the oracle's
    values, in binary64, with max/min counted as 1-Lipschitz in both operands).
    ``safety`` covers second-order terms.  Points where the bound is not finite
    (a derivative overflows) come back with an infinite bound; the caller
    decides how to treat them.  Without transcendentals the bound is 0: the
    device must give the oracle's bits.

    ``perturb`` (a numpy RandomState) turns the evaluation into a model of such
    a device, for testing the bound itself: every exp/log/tanh result moves by
    a random whole number of ulps in [-ulps, ulps].
    """
    kind, out_shape, nodes, root = parse(ir_text)
    if kind != "ew":
        raise ValueError("elementwise programs only")
    values = []  # per node: float32 values
    k = 0
    param_input = {}
    for i, ln in enumerate(nodes):
        if ln[0] == "p":
            param_input[i] = k
            k += 1
    if len(inputs) != k:
        raise ValueError("program takes %d inputs, got %d" % (k, len(inputs)))
    n = int(np.prod(out_shape, dtype=np.int64)) if out_shape else 1
    flat = [np.ascontiguousarray(a, dtype=np.float32).ravel()[:n] for a in inputs]
    affected = [False] * len(nodes)  # has a transcendental at or below it
    for i, ln in enumerate(nodes):
        tag = ln[0]
        with np.errstate(all="ignore"):
            if tag == "p":
                v = None
            elif tag == "x":
                if ln[2:] != ["2", "1", "0"]:
                    raise ValueError("views are not supported here")
                v = flat[param_input[int(ln[1])]]
            elif tag == "l":
                v = np.full(n, bits_to_f32(ln[1]), dtype=np.float32)
            elif tag == "u":
                a = values[int(ln[2])]
                op = ln[1]
                affected[i] = affected[int(ln[2])] or op in _TRANSCENDENTAL
                if op == "neg":
                    v = -a
                elif op == "abs":
                    v = np.abs(a)
                elif op == "sqrt":
                    v = np.sqrt(a)
                elif op in _TRANSCENDENTAL:
                    v = _f64(getattr(np, op), a)
                    if perturb is not None:
                        for _ in range(int(ulps)):
                            step = perturb.randint(-1, 2, size=v.shape)
                            v = np.where(step > 0, np.nextafter(v, np.float32(np.inf)),
                                         np.where(step < 0, np.nextafter(v, np.float32(-np.inf)), v))
                        v = v.astype(np.float32)
                else:
                    raise ValueError(op)
            elif tag == "b":
                a, b = values[int(ln[2])], values[int(ln[3])]
                affected[i] = affected[int(ln[2])] or affected[int(ln[3])]
                op = ln[1]
                v = {"add": np.add, "sub": np.subtract, "mul": np.multiply, "div": np.divide,
                     "mod": np.fmod, "min": np.fmin, "max": np.fmax}[op](a, b)
            else:
                raise ValueError("node %s is not supported here" % tag)
        values.append(v)
    out = values[root].astype(np.float32)
    if not affected[root]:
        return out, np.zeros(n, dtype=np.float64)
    # reverse-mode adjoints d out / d node, in binary64
    adj = [None] * len(nodes)
    adj[root] = np.ones(n, dtype=np.float64)
    with np.errstate(all="ignore"):
        for i in range(root, -1, -1):
            a_i = adj[i]
            ln = nodes[i]
            if a_i is None or ln[0] in ("p", "x", "l"):
                continue

            def add(j, g):
                g = np.where(a_i == 0.0, 0.0, g)  # no sensitivity stays none (0 * inf is not NaN here)
                adj[j] = g if adj[j] is None else adj[j] + g

            if ln[0] == "u":
                j = int(ln[2])
                x = values[j].astype(np.float64)
                op = ln[1]
                if op == "neg":
                    add(j, -a_i)
                elif op == "abs":
                    add(j, a_i * np.sign(x))
                elif op == "sqrt":
                    add(j, a_i / (2.0 * np.sqrt(x)))
                elif op == "exp":
                    add(j, a_i * np.exp(x))
                elif op == "log":
                    add(j, a_i / x)
                elif op == "tanh":
                    add(j, a_i * (1.0 - np.tanh(x) ** 2))
            else:
                ja, jb = int(ln[2]), int(ln[3])
                x = values[ja].astype(np.float64)
                y = values[jb].astype(np.float64)
                op = ln[1]
                if op == "add":
                    add(ja, a_i)
                    add(jb, a_i)
                elif op == "sub":
                    add(ja, a_i)
                    add(jb, -a_i)
                elif op == "mul":
                    add(ja, a_i * y)
                    add(jb, a_i * x)
                elif op == "div":
                    add(ja, a_i / y)
                    add(jb, -a_i * x / (y * y))
                elif op in ("max", "min", "mod"):
                    add(ja, np.abs(a_i))
                    add(jb, np.abs(a_i) * (np.abs(x / y) + 1.0 if op == "mod" else 1.0))
        bound = np.zeros(n, dtype=np.float64)
        for i, ln in enumerate(nodes):
            if not affected[i] or adj[i] is None:
                continue
            ulp = np.spacing(np.abs(values[i])).astype(np.float64)
            own = ulps if (ln[0] == "u" and ln[1] in _TRANSCENDENTAL) else 0.0
            bound += np.where(adj[i] == 0.0, 0.0, np.abs(adj[i]) * ulp * (own + 1.0))
        bound *= safety
        bound[~np.isfinite(bound)] = np.inf
    return out, bound

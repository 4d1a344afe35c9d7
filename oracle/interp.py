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


def fma32(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    """fmaf(a, b, c) on float32 arrays: a*b + c rounded once to binary32.

    The product of two binary32 values is exact in binary64 (48 significant
    bits); the sum s = p + c is rounded to binary64 and TwoSum gives its exact
    error e.  Rounding s to binary32 is then the correct rounding of p + c,
    except when s lies exactly halfway between two binary32 values and e is
    not zero: the true sum lies on e's side of that midpoint."""
    with np.errstate(all="ignore"):
        p = a.astype(np.float64) * b.astype(np.float64)
        c64 = c.astype(np.float64)
        s = p + c64
        bb = s - p
        e = (p - (s - bb)) + (c64 - bb)
        r = s.astype(np.float32)
        r64 = r.astype(np.float64)
        other = np.where(s > r64, np.nextafter(r, np.float32(np.inf)), np.nextafter(r, np.float32(-np.inf)))
        tie = np.isfinite(s) & (s != r64) & ((s - r64) == (other.astype(np.float64) - s))
        up = tie & (e > 0)
        down = tie & (e < 0)
        out = np.where(up, np.maximum(r, other), np.where(down, np.minimum(r, other), r))
    return out.astype(np.float32)


def evaluate(ir_text: str, inputs: Sequence[np.ndarray], transcendental=None, fma: bool = False):
    """Evaluates an IR text on float32 inputs (flat arrays, in parameter order).

    Returns the flat float32 output (tuple roots interleaved as the kernel
    stores them) for an ``ew`` program, or the float32 element values that a
    ``sum`` program adds up.

    ``transcendental(op, args)``, when given, supplies the float32 values of
    exp/log/tanh ("exp", "log" or "tanh" of a float32 array) instead of the
    correctly rounded ones.  The reference takes these three functions from the
    vendor's math library, outside its own semantics; a caller that supplies a
    device's values (checked against their error bound separately) gets that
    device's bits for everything else the reference specifies: operation order,
    rounding of every statement, views, padding.

    ``fma``: the FMA-contraction mode (the runtime's CC_FLAG_FMA_CONTRACT):
    every add or sub whose operand is a mul node computes that product and the
    sum with one rounding (the left operand when both are products):
    p*q + c and c + p*q -> fma(p, q, c), p*q - c -> fma(p, q, -c),
    c - p*q -> fma(-p, q, c).
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
                elif op in ("exp", "log", "tanh"):
                    if transcendental is not None:
                        out = np.asarray(transcendental(op, a.astype(np.float32)), dtype=np.float32)
                    else:
                        out = _f64(getattr(np, op), a)
                else:
                    raise ValueError(op)
        elif tag == "b" and fma and ln[1] in ("add", "sub") and (
                nodes[int(ln[2])][:2] == ["b", "mul"] or nodes[int(ln[3])][:2] == ["b", "mul"]):
            left = nodes[int(ln[2])][:2] == ["b", "mul"]
            m = nodes[int(ln[2]) if left else int(ln[3])]
            p = ev(int(m[2]), fr, fid)
            q = ev(int(m[3]), fr, fid)
            c = ev(int(ln[3]) if left else int(ln[2]), fr, fid)
            if ln[1] == "add":
                out = fma32(p, q, c)
            elif left:
                out = fma32(p, q, -c)
            else:
                out = fma32(-p, q, c)
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

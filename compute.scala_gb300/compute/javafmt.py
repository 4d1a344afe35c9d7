"""``Tensor.toString`` formatting: the JVM's ``Float.toString`` and the nested-bracket layout.

``Tensors.scala:776-811`` renders a tensor as nested ``[a,b,...]`` groups of
``Float.toString`` values (a scalar prints bare).  ``Float.toString`` prints the
shortest decimal that round-trips the float, in plain notation when
``1e-3 <= |x| < 1e7`` (always with a fractional digit, ``42.0``) and in
``d.dddE<n>`` notation otherwise.
"""

from __future__ import annotations

import numpy as np


def float_to_string(value) -> str:
    f = np.float32(value)
    if np.isnan(f):
        return "NaN"
    if np.isinf(f):
        return "Infinity" if f > 0 else "-Infinity"
    if f == 0:
        return "-0.0" if np.signbit(f) else "0.0"
    sign = "-" if f < 0 else ""
    a = abs(f)
    sci = np.format_float_scientific(a, unique=True, trim="k")  # e.g. '4.8931676e-01'
    mant, exp = sci.split("e")
    exp = int(exp)
    digits = mant.replace(".", "").rstrip("0") or "0"
    if np.float32(1e-3) <= a < np.float32(1e7):
        point = exp + 1  # digits before the decimal point
        if point <= 0:
            s = "0." + "0" * (-point) + digits
        elif point >= len(digits):
            s = digits + "0" * (point - len(digits)) + ".0"
        else:
            s = digits[:point] + "." + digits[point:]
        return sign + s
    frac = digits[1:] or "0"
    return "%s%s.%sE%d" % (sign, digits[0], frac, exp)


def tensor_to_string(shape, flat) -> str:
    """Tensors.scala:776-811."""
    flat = list(flat)

    def rec(shape, values):
        if len(shape) == 0:
            if len(values) == 1:
                return float_to_string(values[0])
            raise ValueError("shape() does not match the data size (%d)" % len(values))
        head = shape[0]
        tail = shape[1:]
        if not tail:
            if head != len(values):
                raise ValueError("shape does not match the data size")
            return "[" + ",".join(float_to_string(v) for v in values) + "]"
        group = len(values) // head if head else 0
        return "[" + ",".join(rec(tail, values[i * group:(i + 1) * group]) for i in range(head)) + "]"

    return rec(tuple(shape), flat)

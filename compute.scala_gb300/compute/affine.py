"""View matrices: the N-dimensional affine transforms behind every tensor view.

A view matrix maps coordinates of a *target* tensor (the view) to coordinates of
its *source* tensor.  It is stored row-major as a flat list of doubles with
``rows = source rank`` and ``cols = target rank + 1``; the last column holds the
constant offset, so ``source[y] = sum_x M[y][x] * target[x] + M[y][cols-1]``.

Follows NDimensionalAffineTransform/src/main/scala/com/thoughtworks/compute/
NDimensionalAffineTransform.scala: ``translate`` (:13-26), ``preConcatenate``
(:28-35), ``concatenate`` (:37-95) and ``transform`` (:97-127).  The
accumulation order of every dot product is the same as there (partial sums in
index order, the constant column seeded with the outer matrix's offset), so the
doubles that reach the kernel builder are bit-identical to the reference's.
"""

from __future__ import annotations

from typing import List, Sequence

MatrixData = List[float]


def translate(offset: Sequence[float]) -> MatrixData:
    """Identity plus a constant offset column (NDimensionalAffineTransform.scala:13-26)."""
    n = len(offset)
    m = [0.0] * (n * (n + 1))
    for i in range(n):
        m[i * (n + 1) + i] = 1.0
        m[i * (n + 1) + n] = float(offset[i])
    return m


def _concatenate(m01: Sequence[float], m12: Sequence[float], len0: int, len1: int, len2: int) -> MatrixData:
    """m02 = m12 . m01 with the reference's summation order (NDimensionalAffineTransform.scala:48-95)."""
    m02 = [0.0] * ((len0 + 1) * len2)
    for i2 in range(len2):
        for i0 in range(len0):
            acc = 0.0
            for i1 in range(len1):
                acc = acc + m12[i2 * (len1 + 1) + i1] * m01[i1 * (len0 + 1) + i0]
            m02[i2 * (len0 + 1) + i0] = acc
        acc = m12[i2 * (len1 + 1) + len1]
        for i1 in range(len1):
            acc = acc + m12[i2 * (len1 + 1) + i1] * m01[i1 * (len0 + 1) + len0]
        m02[i2 * (len0 + 1) + len0] = acc
    return m02


def pre_concatenate(m01: Sequence[float], m12: Sequence[float], len0: int) -> MatrixData:
    """Compose a new view ``m01`` (target rank ``len0``) in front of an existing view ``m12``.

    NDimensionalAffineTransform.scala:28-35.
    """
    len1 = len(m01) // (len0 + 1)
    len2 = len(m12) // (len1 + 1)
    return _concatenate(m01, m12, len0, len1, len2)


def concatenate(m12: Sequence[float], m01: Sequence[float], len2: int) -> MatrixData:
    """NDimensionalAffineTransform.scala:37-46 (argument order as there)."""
    len1 = len(m12) // len2 - 1
    len0 = len(m01) // len1 - 1
    return _concatenate(m01, m12, len0, len1, len2)


def transform(matrix: Sequence[float], source: Sequence[float]) -> List[float]:
    """Apply a matrix to one coordinate vector (NDimensionalAffineTransform.scala:97-127)."""
    n = len(source)
    rows = len(matrix) // (n + 1)
    if len(matrix) != (n + 1) * rows:
        raise ValueError("matrix does not match the coordinate vector")
    out = []
    for y in range(rows):
        acc = matrix[y * (n + 1) + n]
        for x in range(n):
            acc = acc + matrix[y * (n + 1) + x] * source[x]
        out.append(acc)
    return out

"""ORACLE (test infrastructure only): the reference's random-number kernels in numpy.

Follows Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala:
Wang hash (:106-117), xorshift (:402-406), ``random`` (:431-443) and
``random_normal`` (:397-429).  Integer steps are exact uint32 arithmetic; the
float steps round to binary32 after every operation, with log/sqrt/cos/sin
taken in binary64 and rounded once (correctly rounded in practice).
"""

from __future__ import annotations

import numpy as np


def wang_hash(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint32)
    with np.errstate(over="ignore"):
        v = (v ^ np.uint32(61)) ^ (v >> np.uint32(16))
        v = v * np.uint32(9)
        v = v ^ (v << np.uint32(4))
        v = v * np.uint32(0x27D4EB2D)
        v = v ^ (v >> np.uint32(15))
    return v.astype(np.uint32)


def xorshift(s: np.ndarray) -> np.ndarray:
    s = s.astype(np.uint32)
    t1 = s ^ (s << np.uint32(13))
    t2 = t1 ^ (t1 >> np.uint32(17))
    return (t2 ^ (t2 << np.uint32(5))).astype(np.uint32)


def _unit(h: np.ndarray) -> np.ndarray:
    # (float)uint with round-to-nearest-even, then an exact division by 2^32
    return (h.astype(np.float32) * np.float32(2.0 ** -32)).astype(np.float32)


def random_uniform(n: int, seed: int) -> np.ndarray:
    i = np.arange(n, dtype=np.uint64).astype(np.uint32)
    return _unit(wang_hash(i ^ np.uint32(seed & 0xFFFFFFFF)))


def random_normal(n: int, seed: int) -> np.ndarray:
    pairs = (n + 1) // 2
    i = np.arange(pairs, dtype=np.uint64).astype(np.uint32)
    r1 = wang_hash(i ^ np.uint32(seed & 0xFFFFFFFF))
    r2 = xorshift(r1)
    u1 = _unit(r1)
    u2 = _unit(r2)
    with np.errstate(all="ignore"):
        lg = np.log(u1.astype(np.float64)).astype(np.float32)
        r = np.sqrt((np.float32(-2.0) * lg).astype(np.float32).astype(np.float64)).astype(np.float32)
        theta = ((np.float32(2.0) * np.float32(np.pi)) * u2).astype(np.float32)  # 2 * M_PI_F
        z0 = (r * np.cos(theta.astype(np.float64)).astype(np.float32)).astype(np.float32)
        z1 = (r * np.sin(theta.astype(np.float64)).astype(np.float32)).astype(np.float32)
    out = np.empty(pairs * 2, dtype=np.float32)
    out[0::2] = z0
    out[1::2] = z1
    return out[:n]

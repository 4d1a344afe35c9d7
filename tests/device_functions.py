"""Test helper: exp/log/tanh values from the device, for the oracle.

The reference takes exp, log and tanh from the vendor's math library, outside
its own semantics, so parity for them is a bound (2 ulp of the correctly
rounded value), not bits.  A parity test that wants the bits of everything the
reference does specify -- the order of the statements, the rounding of each,
views and padding -- passes ``DeviceFunctions`` to ``oracle.interp.evaluate``:
the oracle then takes each transcendental value from the device's own
single-operation kernel, after checking it against that bound.
"""

import numpy as np


def _ulp_distance(a, b):
    """Distance in units in the last place between float32 arrays (finite values)."""
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


class DeviceFunctions:
    """exp/log/tanh of float32 arrays from the device's single-operation
    generated kernels, each value checked within 2 ulp of the correctly
    rounded one (an infinity where the correctly rounded value is the largest
    finite float, or the reverse, counts as one ulp)."""

    def __init__(self, device):
        self.rt = device.runtime
        self.values = 0
        self.worst = 0

    def __call__(self, op, a):
        rt = self.rt
        n = int(a.size)
        prog = rt.program("ccir 1 ew\no 1 %d\np 1 %d 00000000\nx 0 2 1 0\nu %s 1\nr 2\n" % (n, n, op))
        src, dst = rt.alloc(4 * n), rt.alloc(4 * n)
        try:
            rt.upload(src, a)
            rt.launch(prog, [src], dst)
            got = rt.download(dst, n)
        finally:
            src.release()
            dst.release()
        with np.errstate(all="ignore"):
            want = getattr(np, op)(a.astype(np.float64)).astype(np.float32)
        nan = np.isnan(want)
        assert np.array_equal(nan, np.isnan(got)), op
        fin = ~nan & np.isfinite(want) & np.isfinite(got)
        dist = _ulp_distance(got[fin], want[fin])
        assert dist.size == 0 or dist.max() <= 2, (op, int(dist.max()))
        edge = ~nan & ~fin
        big = np.float32(np.finfo(np.float32).max)
        ok_edge = (got[edge] == want[edge]) | ((np.abs(got[edge]) >= big) & (np.abs(want[edge]) >= big) &
                                               (np.sign(got[edge]) == np.sign(want[edge])))
        assert ok_edge.all(), op
        self.values += n
        self.worst = max(self.worst, int(dist.max()) if dist.size else 0)
        return got

"""Programmatic dependent launch keeps stream order: a chain of kernels, each
reading the buffer the previous one wrote (elementwise, view and sum programs),
gives the bits of the same chain launched without it."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _chain(d, n):
    T = d.Tensor
    x = T.random([n, 64], seed=7).doCache()
    t = x
    for k in range(12):
        t = (t * T.fill(1.0001, [n, 64]) + T.fill(0.5, [n, 64])).doCache()  # one kernel per step, reading the last
        if k % 4 == 3:
            t = t.transpose().transpose().translate([1, 0]).doCache()  # a view program in the chain
    s = t.sum().readScalar()
    return t.flatArray(), s


def test_pdl_chain_matches_plain_launches(cuda_device):
    rt = cuda_device.runtime
    for n in (1000, 300000):
        rt.config_set("pdl", 0)
        want, want_s = _chain(cuda_device, n)
        rt.config_set("pdl", 1)
        try:
            got, got_s = _chain(cuda_device, n)
        finally:
            rt.config_set("pdl", 0)
        assert np.array_equal(got.view(np.int32), want.view(np.int32))
        assert got_s == want_s

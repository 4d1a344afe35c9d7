"""doCache / CachedTensor lifetime over the buffer pool.

The reference keeps a cached tensor's buffer until its resource is released
(Tensors.scala:602, :642-666) and shows the mutable-variable idiom over it
(README.md:212-229): a weight cached, replaced each step by a new cached
tensor computed from it, and the old one released.  Over the pool, such a loop
must reuse the released blocks (reuses grow, no new allocations) and keep the
bytes in use flat, while every step's weight holds the bits the oracle
computes from the previous one.
"""

import numpy as np
import pytest

from compute.tensors import IllegalArgumentException

pytestmark = pytest.mark.gpu


def test_mutable_weight_loop_reuses_pool_blocks(cuda_device):
    from oracle import rng
    d = cuda_device
    rt = d.runtime
    T = d.Tensor
    shape = [32, 32]
    weight = T.random(shape, seed=100).doCache()
    host = weight.flatArray().copy()
    rt.synchronize()
    steady = None
    for step in range(40):
        new = (weight * T.random(shape, seed=200 + step)).doCache()
        got = new.flatArray()
        want = (host * rng.random_uniform(1024, 200 + step)).astype(np.float32)
        assert np.array_equal(got.view(np.int32), want.view(np.int32))
        weight.close()  # releaseWeight
        weight, host = new, got
        stats = rt.pool_stats()
        if step == 4:
            steady = stats
        elif step > 4:
            assert stats["in_use"] == steady["in_use"], (step, stats, steady)
            assert stats["allocs"] == steady["allocs"], (step, stats, steady)
    assert rt.pool_stats()["reuses"] >= steady["reuses"] + 35
    weight.close()


def test_closed_cache_returns_its_block_and_refuses_use(cuda_device):
    d = cuda_device
    rt = d.runtime
    T = d.Tensor
    rt.synchronize()
    before = rt.pool_stats()
    w = T.randomNormal([1000, 1000], seed=0x40000005).doCache()  # bit 30: no zero hash (log 0) below 2^30
    mid = rt.pool_stats()
    assert mid["in_use"] >= before["in_use"] + 4 * 10 ** 6
    total = (w * w).sum().readScalar()
    assert total > 0
    w.close()
    after = rt.pool_stats()
    assert after["in_use"] == before["in_use"]
    assert after["cached"] > mid["cached"]  # the block went back to the pool's free list
    with pytest.raises(IllegalArgumentException):
        (w + w).flatArray()
    again = T.randomNormal([1000, 1000], seed=0x40000006).doCache()
    assert rt.pool_stats()["reuses"] > after["reuses"]  # the released block serves the next cache
    again.close()

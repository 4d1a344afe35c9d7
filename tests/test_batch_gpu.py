"""Batched evaluation: one persistent launch, per-program launches and a CUDA
graph of them all give the bits a single evaluation through the API gives."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_modes_agree_with_single_launches(cuda_device):
    import bench
    from compute.batch import Batch
    T = cuda_device.Tensor
    progs = bench.c4_programs(T, seed=3, count=40, lo=1, hi=70000)
    tensors = [t for t, _ in progs]
    single = [t.flatArray() for t in tensors]
    b = Batch(cuda_device, tensors).bind()
    for mode in (Batch.PERSISTENT, Batch.PER_PROGRAM, Batch.GRAPH, Batch.GRAPH, Batch.PERSISTENT):
        for out in b.outputs:
            cuda_device.runtime.upload(out, np.full(out.nbytes // 4, np.nan, np.float32))
        b.run(mode)
        for k, (t, want) in enumerate(zip(tensors, single)):
            got = cuda_device.runtime.download(b.outputs[k], want.size)
            assert np.array_equal(got.view(np.int32), want.view(np.int32)), (mode, k)
    n, structures, regs, resident = cuda_device.runtime.batch_info(b.handle)
    assert n == 40 and 1 <= structures <= 40
    b.close()
    for _, inputs in progs:
        for i in inputs:
            i.close()


@pytest.mark.parametrize("lanes,inline,rolled", [(0, 1, 0), (4, 1, 0), (8, 1, 0), (4, 0, 0), (8, 2, 0), (4, 1, 1),
                                                  (8, 1, 1)])
def test_batch_lane_widths_give_the_single_launch_bits(cuda_device, lanes, inline, rolled):
    """Tile functions evaluating 1, 4 or 8 points per call (and each inlining
    level) run the same per-point arithmetic: every program's output is the
    single launch's, bit for bit, ragged ends included."""
    import bench
    from compute.batch import Batch
    rt = cuda_device.runtime
    T = cuda_device.Tensor
    saved = {k: rt.config_get(k) for k in ("batch_lanes", "batch_inline", "batch_rolled", "batch_max_loads")}
    progs = bench.c4_programs(T, seed=11, count=24, lo=1, hi=40000)
    # and every other operator, through the lane helpers
    for k, n in enumerate((4099, 8192, 33)):
        a, b = (T.random([n], seed=900 + 2 * k + j) * T.fill(4.0, [n]) - T.fill(2.0, [n]) for j in (0, 1))
        a, b = a.doCache(), b.doCache()
        e = [T.abs(a - b) % (b + T.fill(3.0, [n])), -T.sqrt(T.abs(a)) * T.min(a, b),
             T.min(T.max(a, b), T.fill(0.5, [n])) / (T.abs(b) + T.fill(0.25, [n]))][k]
        progs.append((e, [a, b]))
    tensors = [t for t, _ in progs]
    single = [t.flatArray() for t in tensors]
    try:
        rt.config_set("batch_lanes", lanes)
        rt.config_set("batch_inline", inline)
        rt.config_set("batch_rolled", rolled)
        rt.config_set("batch_max_loads", 2 if rolled else 4)  # rolled: loops of one or two positions
        b = Batch(cuda_device, tensors).bind()
        b.run(Batch.PERSISTENT)
        for k, want in enumerate(single):
            got = rt.download(b.outputs[k], want.size)
            assert np.array_equal(got.view(np.int32), want.view(np.int32)), k
        b.close()
    finally:
        for k, v in saved.items():
            rt.config_set(k, v)
        for _, inputs in progs:
            for i in inputs:
                i.close()


def test_batch_rejects_programs_with_views(cuda_device):
    from compute._native import InvalidProgram
    from compute.batch import Batch
    T = cuda_device.Tensor
    a = T.random([64, 8], seed=1).doCache()
    with pytest.raises(InvalidProgram):
        Batch(cuda_device, [a.transpose() * T.fill(2.0, [8, 64])])
    a.close()

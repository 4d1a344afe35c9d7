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


def test_batch_rejects_programs_with_views(cuda_device):
    from compute._native import InvalidProgram
    from compute.batch import Batch
    T = cuda_device.Tensor
    a = T.random([64, 8], seed=1).doCache()
    with pytest.raises(InvalidProgram):
        Batch(cuda_device, [a.transpose() * T.fill(2.0, [8, 64])])
    a.close()

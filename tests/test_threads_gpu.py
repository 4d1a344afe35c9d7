"""The C ABI is called from several threads at once (the reference's tensors
are evaluated from any thread of its execution context, OpenCL.scala:414-416):
program compiles, cache hits, allocations, launches, sums and downloads
interleave, and every thread gets the bits a single thread gets."""

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _work(T, k):
    shape = [37, 29, 5]
    a = T.random(shape, seed=100 + k)
    b = T.random(shape, seed=200 + k)
    e = (a * b + T.fill(0.25 * (k + 1), shape)).permute([2, 0, 1]).translate([0, k % 3, -1])
    e = T.max(e, -e * T.fill(0.5, e.shape))
    return np.asarray(e.flatArray(), np.float32), np.float32((a - b).sum().flatArray()[0])


def test_threads_get_single_thread_bits(cuda_device):
    T = cuda_device.Tensor
    want = [_work(T, k) for k in range(8)]
    got = {}
    errors = []

    def run(t):
        try:
            for rep in range(3):
                for k in range(t, 8, 4):
                    got[(t, rep, k)] = _work(T, k)
        except Exception as exc:  # reported below, with the thread's index
            errors.append((t, repr(exc)))

    threads = [threading.Thread(target=run, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=300)
    assert not any(th.is_alive() for th in threads)
    assert not errors, errors
    assert len(got) == 4 * 3 * 2
    for (t, rep, k), (e, s) in got.items():
        assert np.array_equal(e.view(np.int32), want[k][0].view(np.int32)), (t, rep, k)
        assert s.view(np.int32) == want[k][1].view(np.int32), (t, rep, k)

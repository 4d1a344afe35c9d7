"""Loads staged through the shared-memory ring (cp.async into per-thread
slots) give the bits of loads into registers: the view-heavy channel sum and
random view programs with zero padding, in elementwise and sum kernels."""

import numpy as np
import pytest

from compute import tuner

pytestmark = pytest.mark.gpu


def _run(rt, text, arrays, n_out):
    bufs = []
    for a in arrays:
        b = rt.alloc(max(1, a.size) * 4)
        rt.upload(b, a)
        bufs.append(b)
    out = rt.alloc(max(1, n_out) * 4)
    rt.launch(rt.program(text), bufs, out)
    got = rt.download(out, n_out)
    for b in bufs + [out]:
        b.release()
    return got


@pytest.mark.parametrize("slots", [8, 32])
def test_ring_matches_register_loads(cuda_device, slots):
    import bench
    from compute.tensors import NonInlineTensor
    rt = cuda_device.runtime
    d = cuda_device
    cases = []
    n, c, h, w = 2, 128, 9, 11
    x = NonInlineTensor(d, (n, c, h, w), 0.0, None)
    bias = NonInlineTensor(d, (1, 1, 1, c), 0.0, None)
    s = bench.build_c2(d.Tensor, x, bias, n, c, h, w)
    r = np.random.RandomState(0)
    cases.append((d.serialize(s.closure, s.shape).text,
                  [r.normal(size=n * c * h * w).astype(np.float32), r.normal(size=c).astype(np.float32)],
                  n * h * w))
    for p in tuner.random_programs(12, seed=31, max_points=1 << 16, max_dim=300):
        arrays = [r.uniform(0.1, 2.0, size=int(np.prod(sh))).astype(np.float32) for sh in p["params"]]
        cases.append((p["ir"], arrays, 1 if p["kind"] == "sum" else p["points"]))
    try:
        for text, arrays, n_out in cases:
            rt.config_set("ew_smem_ring", 0)
            want = _run(rt, text, arrays, n_out)
            rt.config_set("ew_smem_ring", slots)
            got = _run(rt, text, arrays, n_out)
            nan = np.isnan(want)
            assert np.array_equal(nan, np.isnan(got))
            assert np.array_equal(want[~nan].view(np.int32), got[~nan].view(np.int32))
    finally:
        rt.config_set("ew_smem_ring", 0)

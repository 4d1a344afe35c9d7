"""Batched programs against the oracle at the benchmark's configuration.

2048 independent fused programs (seed 0), lengths log-uniform on [1K, 4M]
(about 1.0e9 points), each a random 3-12-node tree over
{+,-,*,/,exp,log,tanh,max} on 1-4 inputs uniform in [0.1, 2], evaluated by one
persistent launch, by one launch per program and by a replayed CUDA graph.  The
reference evaluates each tensor with its own kernel (Tensors.scala:1331-1381),
so every program's output must be what its own kernel computes:

* programs without exp/log/tanh: the oracle's bits (every operation is one
  correctly rounded binary32 statement on both sides);
* programs with them: within a per-point bound from first-order error
  propagation (``oracle.interp.evaluate_with_bound``: the device's exp/log/tanh
  within 2 ulp of the correctly rounded value, one more ulp of rounding at
  every node above one, each scaled by the output's derivative with respect to
  that node, times 4); a NaN must be a NaN, an infinity the same infinity.

Each program is checked on up to three 4096-point windows: its first, its last
and one at a seeded random place (the whole program when it is shorter).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WINDOW = 4096


def _windows(n, rs):
    if n <= 3 * WINDOW:
        return [(0, n)]
    mid = int(rs.randint(WINDOW, n - 2 * WINDOW))
    return [(0, WINDOW), (mid, WINDOW), (n - WINDOW, WINDOW)]


def _check(got, want, bound, where):
    nan = np.isnan(want)
    assert np.array_equal(nan, np.isnan(got)), where
    exact = (bound == 0) & ~nan
    assert np.array_equal(got[exact].view(np.int32), want[exact].view(np.int32)), where
    inf = np.isinf(want) & ~exact
    assert np.array_equal(got[inf], want[inf]), where
    rest = ~nan & ~exact & ~inf & np.isfinite(bound)
    g = got[rest].astype(np.float64)
    w = want[rest].astype(np.float64)
    # a finite oracle value next to the overflow threshold may round to infinity on the device
    near_overflow = np.isinf(g) & (np.abs(w) > 1e38) & (np.sign(g) == np.sign(w))
    ok = (np.abs(g - w) <= bound[rest]) | near_overflow
    assert ok.all(), (where, g[~ok][:4], w[~ok][:4], bound[rest][~ok][:4])
    return int(rest.sum()), int((~nan & ~np.isfinite(bound) & ~inf).sum())


def test_every_batched_program_matches_the_oracle_at_the_benchmark_config(cuda_device):
    import bench
    from compute.batch import Batch
    from oracle import interp
    d = cuda_device
    rt = d.runtime
    progs = bench.c4_programs(d.Tensor, seed=0, count=2048)
    tensors = [t for t, _ in progs]
    b = Batch(d, tensors).bind()
    try:
        rs = np.random.RandomState(0)
        plan = []  # per program: windows, oracle values and bounds
        n_transcendental = 0
        total_points = 0
        for k, (t, ser) in enumerate(zip(tensors, b.serialized)):
            n = int(t.shape[0])
            total_points += n
            entries = []
            for start, length in _windows(n, rs):
                ins = [rt.download(p._cached, length, offset=4 * start) for p in ser.params]
                want, bound = interp.evaluate_with_bound(interp.window_text(ser.text, length), ins)
                entries.append((start, length, want, bound))
            if any(("u %s " % op) in ser.text for op in ("exp", "log", "tanh")):
                n_transcendental += 1
            plan.append(entries)
        assert len(plan) == 2048 and total_points > 9e8
        assert 0 < n_transcendental < 2048
        checked = unbounded = 0
        for mode in (Batch.PERSISTENT, Batch.GRAPH, Batch.PER_PROGRAM):
            for k, entries in enumerate(plan):
                for start, length, _, _ in entries:
                    rt.upload(b.outputs[k], np.full(length, np.nan, np.float32), offset=4 * start)
            b.run(mode)
            for k, entries in enumerate(plan):
                for start, length, want, bound in entries:
                    got = rt.download(b.outputs[k], length, offset=4 * start)
                    c, u = _check(got, want, bound, (mode, k, start))
                    checked += c
                    unbounded += u
        # points whose bound overflows (an infinity that reaches the output) are checked for NaN-ness only
        assert checked > 0 and unbounded < checked
        print("checked %d points within the bound, %d without a finite bound" % (checked, unbounded))
    finally:
        b.close()
        for _, inputs in progs:
            for i in inputs:
                i.close()

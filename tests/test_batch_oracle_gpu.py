"""Batched programs against the oracle at the benchmark's configuration.

2048 independent fused programs (seed 0), lengths log-uniform on [1K, 4M]
(about 1.0e9 points), each a random 3-12-node tree over
{+,-,*,/,exp,log,tanh,max} on 1-4 inputs uniform in [0.1, 2], evaluated by one
persistent launch, by a replayed CUDA graph and by one launch per program.  The
reference evaluates each tensor with its own kernel (Tensors.scala:1331-1381),
so every program's output must be what the oracle computes for its tree:

* the oracle takes exp/log/tanh of each transcendental node from the device's
  own single-operation kernel (the reference takes them from the vendor's math
  library, outside its own semantics), and every such value is checked within
  2 ulp of the correctly rounded one; everything else -- the order of the
  statements, the rounding of each, the operands -- is the oracle's, so every
  program, with or without transcendentals, must give the oracle's bits.
  (A derivative bound cannot serve here: one ulp of a logarithm near 1 turns
  log(log(e)) from -6e-8 into 0 and a following 0/0 into NaN.)

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


from device_functions import DeviceFunctions  # noqa: E402


def _same_bits(got, want):
    nan = np.isnan(want)
    return np.array_equal(nan, np.isnan(got)) and np.array_equal(got[~nan].view(np.int32), want[~nan].view(np.int32))


def test_every_batched_program_matches_the_oracle_at_the_benchmark_config(cuda_device):
    import bench
    from compute.batch import Batch
    from oracle import interp
    d = cuda_device
    rt = d.runtime
    progs = bench.c4_programs(d.Tensor, seed=0, count=2048)
    tensors = [t for t, _ in progs]
    b = Batch(d, tensors).bind()
    fns = DeviceFunctions(d)
    try:
        rs = np.random.RandomState(0)
        plan = []  # per program: windows, and the oracle's values on them
        n_transcendental = 0
        total_points = 0
        for k, (t, ser) in enumerate(zip(tensors, b.serialized)):
            n = int(t.shape[0])
            total_points += n
            wins = _windows(n, rs)
            length = sum(w for _, w in wins)
            # the program is pointwise: its windows, side by side, are one program of their total length
            ins = [np.concatenate([rt.download(p._cached, w, offset=4 * s) for s, w in wins]) for p in ser.params]
            want = interp.evaluate(interp.window_text(ser.text, length), ins, transcendental=fns)
            if any(("u %s " % op) in ser.text for op in ("exp", "log", "tanh")):
                n_transcendental += 1
            plan.append((wins, want))
        assert len(plan) == 2048 and total_points > 9e8
        assert 0 < n_transcendental < 2048
        for mode in (Batch.PERSISTENT, Batch.GRAPH, Batch.PER_PROGRAM):
            for k, (wins, _) in enumerate(plan):
                for s, w in wins:
                    rt.upload(b.outputs[k], np.full(w, np.nan, np.float32), offset=4 * s)
            b.run(mode)
            for k, (wins, want) in enumerate(plan):
                got = np.concatenate([rt.download(b.outputs[k], w, offset=4 * s) for s, w in wins])
                assert _same_bits(got, want), (mode, k)
        print("device exp/log/tanh: %d values, worst %d ulp" % (fns.values, fns.worst))
    finally:
        b.close()
        for _, inputs in progs:
            for i in inputs:
                i.close()

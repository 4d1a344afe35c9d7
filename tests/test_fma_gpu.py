"""FMA contraction mode (CC_FLAG_FMA_CONTRACT) against the oracle's FMA mode.

The reference builds its kernels with -cl-unsafe-math-optimizations
(OpenCL.scala:1131-1135), which lets a vendor compiler fuse a*b+c into one
rounding.  With the flag, the runtime's code generator applies one stated rule
(every + or - with a product operand becomes one fmaf of that product, the left
one when both are products) and the oracle evaluates the same rule with an
exact fused multiply-add, so results are again bit-exact: random trees over
views, the fused elementwise+sum and view-heavy shapes, the inner-axis fold and
a batch.  The context's flags are fixed at cc_init, so this runs in a child
process of its own.
"""

import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

_CHILD = textwrap.dedent("""
    import sys
    import numpy as np
    root = sys.argv[1]
    sys.path[:0] = [root, root + "/compute.scala_gb300"]
    from compute import Tensors
    from compute.batch import Batch
    from oracle import interp

    d = Tensors(device=0, flags=1, tuner="off")  # CC_FLAG_FMA_CONTRACT; the standard kernels
    T = d.Tensor

    def check(expr, kind="ew"):
        ser = d.serialize(expr.closure, expr.shape, kind)
        ins = [p.flatArray() for p in ser.params]
        want = interp.evaluate(ser.text, ins, fma=True)
        plain = interp.evaluate(ser.text, ins)
        got = expr.flatArray()
        nan = np.isnan(want)
        assert np.array_equal(nan, np.isnan(got))
        assert np.array_equal(got[~nan].view(np.int32), want[~nan].view(np.int32)), ser.text[:200]
        return int((plain[~nan].view(np.int32) != want[~nan].view(np.int32)).sum())

    contracted = 0
    r = np.random.RandomState(11)
    shape = [33, 17, 5]
    leaves = [T.randomNormal(shape, seed=0x40000100 + s) for s in range(4)]
    for trial in range(24):
        pool = list(leaves)
        for _ in range(r.randint(4, 12)):
            op = r.choice(["+", "-", "*", "*", "max", "tr", "perm"])
            a = pool[r.randint(len(pool))]
            b = pool[r.randint(len(pool))]
            if op in "+-*":
                t = {"+": a + b, "-": a - b, "*": a * b}[op]
            elif op == "max":
                t = T.max(a, b)
            elif op == "perm":
                t = a.permute([0, 1, 2]).translate([1, 0, -1])
            else:
                t = a.translate([-2, 3, 0])
            pool.append(t)
        contracted += check(pool[-1])
    # the fused elementwise + sum's producer and the view-heavy op
    a, b, c = (T.random([256, 256], seed=s) * T.fill(2.0, [256, 256]) - T.fill(1.0, [256, 256]) for s in (0, 1, 2))
    contracted += check(a * b + c)
    x = T.randomNormal([4, 16, 12, 12], seed=0x40000000)
    bias = (T.randomNormal([16], seed=0x40000001) * T.fill(0.1, [16])).reshape([1, 1, 1, 16])
    y = T.max(x.permute([0, 2, 3, 1]) * T.fill(1.5, [4, 12, 12, 16]) + bias.broadcast([4, 12, 12, 16]),
              T.fill(0.0, [4, 12, 12, 16]))
    contracted += check(y.translate([0, 0, 1, 0]).split(3).reduce(lambda u, v: u + v))
    # the inner-axis fold: acc + a*b terms
    m = T.randomNormal([200, 256], seed=0x40000005)
    n = T.randomNormal([200, 256], seed=0x40000006)
    contracted += check((m * n - m).split(1).reduce(lambda u, v: u + v))
    # a batch: every program's bits are its single launch's
    def contractible(k):
        n = 5000 + 7 * k
        u, w = T.random([n], seed=k), T.random([n], seed=100 + k)
        return [u * T.fill(1.25, [n]) + T.fill(0.5, [n]), T.fill(0.5, [n]) - u * w, u * w - T.exp(u),
                T.tanh(u * w + u * u)][k % 4]
    progs = [contractible(k) for k in range(8)]
    single = [p.flatArray() for p in progs]
    for lanes in (0, 4, 8):  # one, four and eight points per tile-function call
        d.runtime.config_set("batch_lanes", lanes)
        bt = Batch(d, progs).bind()
        bt.run(Batch.PERSISTENT)
        for k, want in enumerate(single):
            got = d.runtime.download(bt.outputs[k], want.size)
            assert np.array_equal(got.view(np.int32), want.view(np.int32)), (lanes, k)
        bt.close()
    assert contracted > 0
    print("fma mode bit-exact; %d points differ from the uncontracted oracle" % contracted)
""")


def test_fma_contraction_mode_matches_the_oracle():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.run([sys.executable, "-c", _CHILD, root], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stdout[-4000:]
    assert "fma mode bit-exact" in p.stdout

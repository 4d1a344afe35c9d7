"""The two CPU restatements pin each other beyond the reference's goldens: the
numpy IR interpreter (fused programs) and the reference's generated OpenCL C
compiled for the host (the reference's unfused kernel structure) give the same
bits on seeded random expression trees over views, and agree on the
convolution idiom."""

import numpy as np
import pytest


def _devices():
    from compute import Tensors, trees
    from oracle.cref import CRuntime
    from oracle_runtime import OracleRuntime
    return (Tensors(runtime=OracleRuntime()),
            Tensors(runtime=CRuntime(), planner=trees.Planner(enabled=False)))


def _tree(T, r, shape):
    leaves = [T.random(shape, seed=s) for s in range(3)] + [T.fill(0.75, shape)]
    pool = list(leaves)
    for _ in range(r.randint(3, 9)):
        op = r.choice(["+", "-", "*", "/", "max", "min", "neg", "abs", "perm", "tr"])
        a = pool[r.randint(len(pool))]
        b = pool[r.randint(len(pool))]
        if op in "+-*/":
            t = {"+": a + b, "-": a - b, "*": a * b, "/": a / b}[op]
        elif op == "max":
            t = T.max(a, b)
        elif op == "min":
            t = T.min(a, b)
        elif op == "neg":
            t = -a
        elif op == "abs":
            t = T.abs(a)
        elif op == "perm":
            t = a.permute([0, 2, 1]).permute([0, 2, 1]).translate([0, 1, -1])
        else:
            t = a.translate([-1, 2, 0])
        pool.append(t)
    return pool[-1]


@pytest.mark.parametrize("seed", range(6))
def test_interpreter_and_generated_c_agree(seed):
    shape = [5, 7, 3]
    results = []
    for d in _devices():
        r = np.random.RandomState(seed)
        results.append(np.asarray(_tree(d.Tensor, r, shape).flatArray(), np.float32))
    a, b = results
    nan = np.isnan(a)
    assert np.array_equal(nan, np.isnan(b))
    assert np.array_equal(a[~nan].view(np.int32), b[~nan].view(np.int32))


def test_convolution_agrees():
    import bench
    outs = []
    for d in _devices():
        T = d.Tensor
        x = T.randomNormal([2, 5, 6, 3], seed=0x40000003)
        w = T.randomNormal([3, 3, 3, 2], seed=0x40000004)
        b = T.randomNormal([2], seed=0x40000005)
        outs.append(np.asarray(bench.conv_expr(T, x, w, b).flatArray(), np.float32))
    assert np.array_equal(outs[0].view(np.int32), outs[1].view(np.int32))


def test_scaled_joined_and_reshaped_views_agree():
    """Non-integer `scale` coefficients (DecimalFormat text, truncation of a
    double index), `join` along the last and a middle dimension, `transpose`,
    `reshape` and `broadcast`: the same bits from both restatements."""
    outs = []
    for d in _devices():
        T = d.Tensor
        a = T.random([7, 9], seed=4)
        b = T.random([7, 9], seed=5)
        s = a.scale([12, 5]).translate([0.5, -1.25])
        j = T.join([a, b * T.fill(2.0, [7, 9]), T.abs(a - b)])
        j1 = T.join([a, b], 1)
        t = (a.transpose() + b.transpose()).reshape([3, 21])
        c = T.random([1, 9], seed=6).broadcast([7, 9]) * a
        outs.append([np.asarray(v.flatArray(), np.float32) for v in (s, j, j1, t, c)])
    for x, y in zip(*outs):
        assert x.shape == y.shape
        assert np.array_equal(x.view(np.int32), y.view(np.int32))

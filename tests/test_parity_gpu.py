"""Parity of the sm_103a path with the oracle, through the C ABI.

Every GPU result is compared with ``oracle.interp`` evaluating the same IR text
on the same input values (read back from the device).  The bars:

* views, permutes, copies and plain arithmetic: bit-exact (FMA contraction off,
  so every statement rounds once, as the reference's SSA code is written);
* one transcendental at the root: within 2 ulp of the correctly rounded value;
* sums: within sqrt(n) * 2^-24 relative to the exact sum of the element values.
"""

import functools

import numpy as np
import pytest

from oracle import interp, rng

pytestmark = pytest.mark.gpu


def oracle_of(device, tensor, kind="ew"):
    ser = device.serialize(tensor.closure, tensor.shape, kind)
    return interp.evaluate(ser.text, [p.flatArray() for p in ser.params])


def bits(a):
    return np.asarray(a, dtype=np.float32).view(np.int32)


def ulp_diff(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


@pytest.mark.parametrize("n", [0, 1, 7, 1000, 4096 + 3, 1 << 20])
def test_random_uniform_bit_exact(cuda_device, n):
    got = cuda_device.Tensor.random([n], seed=12345).flatArray()
    assert np.array_equal(bits(got), bits(rng.random_uniform(n, 12345)))


def test_random_normal_infinities_follow_the_reference():
    """hash == 0 gives log(0) = -inf, hence infinite normals, in the reference too (Tensors.scala:419-426)."""
    n = 3 << 20
    want = rng.random_normal(n, 9)
    assert not np.isfinite(want).all()


@pytest.mark.parametrize("n", [1, 2, 27, 1001, 1 << 20, 3 << 20])
def test_random_normal_matches_the_oracle(cuda_device, n):
    seed = 54321 if n < (3 << 20) else 9
    got = cuda_device.Tensor.randomNormal([n], seed=seed).flatArray()
    want = rng.random_normal(n, seed)
    fin = np.isfinite(want)
    assert np.array_equal(np.isinf(got), np.isinf(want))
    # log/sin/cos are taken in double and rounded once on both sides: bit-exact except, in
    # vanishingly rare cases, a double-rounding difference of one ulp
    d = ulp_diff(got[fin], want[fin])
    assert d.max() <= 1 and (d > 0).sum() <= max(1, n // 10 ** 6)


def _c2(T, n, c, h, w):
    x = T.randomNormal([n, c, h, w], seed=0).doCache()
    bias = (T.randomNormal([c], seed=1) * T.fill(0.1, [c])).reshape([1, 1, 1, c]).doCache()
    y = T.max(x.permute([0, 2, 3, 1]) + bias.broadcast([n, h, w, c]), T.fill(0.0, [n, h, w, c]))
    t = y.translate([0, 0, 1, 0])
    s = t.split(3).reduce(lambda a, b: a + b)
    return x, bias, y, t, s


@pytest.mark.parametrize("shape", [(1, 1, 1, 1), (2, 3, 4, 5), (2, 16, 7, 9), (4, 128, 56, 56), (64, 128, 56, 56)])
def test_view_heavy_fused_op_bit_exact(cuda_device, shape):
    T = cuda_device.Tensor
    x, bias, y, t, s = _c2(T, *shape)
    got = s.flatArray()
    want = oracle_of(cuda_device, s)
    assert np.array_equal(bits(got), bits(want))
    # the permuted and translated views themselves, materialised, are bit-exact too
    for view in (x.permute([0, 2, 3, 1]), t):
        assert np.array_equal(bits(view.flatArray()), bits(oracle_of(cuda_device, view)))
    x.close()
    bias.close()


def test_fusion_does_not_change_bits(cuda_device):
    """The planner's inlined form and the reference's materialise-then-view form agree bit for bit."""
    from compute import trees
    T = cuda_device.Tensor
    x, bias, y, t, s = _c2(T, 2, 32, 9, 11)
    assert "\nv " in cuda_device.serialize(s.closure, s.shape).text
    fused = s.flatArray()
    saved = cuda_device.planner
    cuda_device.planner = trees.Planner(enabled=False)
    try:
        assert "\nv " not in cuda_device.serialize(s.closure, s.shape).text
        unfused = s.flatArray()
    finally:
        cuda_device.planner = saved
    assert np.array_equal(bits(fused), bits(unfused))
    x.close()
    bias.close()


def test_elementwise_arithmetic_bit_exact(cuda_device):
    T = cuda_device.Tensor
    a = T.random([333, 77], seed=1).doCache()
    b = T.random([333, 77], seed=2).doCache()
    c = T.randomNormal([333, 77], seed=3).doCache()
    e = ((a * b + c) / (a + T.fill(0.5, [333, 77])) - b) % T.fill(0.3, [333, 77])
    e = T.min(T.abs(-e), T.sqrt(T.abs(c)))
    assert np.array_equal(bits(e.flatArray()), bits(oracle_of(cuda_device, e)))
    for t in (a, b, c):
        t.close()


@pytest.mark.parametrize("fn", ["exp", "log", "tanh"])
def test_transcendentals_within_2ulp(cuda_device, fn):
    T = cuda_device.Tensor
    a = (T.randomNormal([1 << 16], seed=7) * T.fill(3.0, [1 << 16])).doCache()
    arg = T.abs(a) if fn == "log" else a
    e = getattr(T, fn)(arg)
    got, want = e.flatArray(), oracle_of(cuda_device, e)
    fin = np.isfinite(want)
    assert np.array_equal(np.isfinite(got), fin)
    assert ulp_diff(got[fin], want[fin]).max() <= 2
    a.close()


@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 1000, 1 << 20, (1 << 22) + 5])
def test_fused_sum_within_bound(cuda_device, n):
    T = cuda_device.Tensor
    a = T.random([n], seed=0).doCache()
    b = T.random([n], seed=1).doCache()
    expr = T.tanh(a * b + a)
    got = expr.sum().readScalar()
    vals = oracle_of(cuda_device, expr, "sum")
    exact = interp.exact_sum(vals)
    bound = max(np.sqrt(max(n, 1)) * 2.0 ** -24 * abs(exact), 1e-30)
    assert abs(got - exact) <= bound
    a.close()
    b.close()


def test_c1_fused_elementwise_sum(cuda_device):
    """((a*b+c).tanh).sum over three [1024,1024] tensors uniform in [-1,1] (seeds 0,1,2)."""
    T = cuda_device.Tensor
    shape = [1024, 1024]
    two, one = T.fill(2.0, shape), T.fill(1.0, shape)
    a, b, c = [(T.random(shape, seed=s) * two - one).doCache() for s in (0, 1, 2)]
    expr = T.tanh(a * b + c)
    got = expr.sum().readScalar()
    exact = interp.exact_sum(oracle_of(cuda_device, expr, "sum"))
    assert abs(got - exact) <= np.sqrt(1 << 20) * 2.0 ** -24 * abs(exact)
    # the elementwise part alone: within 2 ulp per element
    ew = expr.flatArray()
    assert ulp_diff(ew, oracle_of(cuda_device, expr)).max() <= 2
    for t in (a, b, c):
        t.close()


def test_sum_is_deterministic(cuda_device):
    T = cuda_device.Tensor
    n = 3 << 20
    a = (T.random([n], seed=9) - T.fill(0.5, [n])).doCache()
    r = {a.sum().readScalar() for _ in range(5)}
    assert len(r) == 1
    a.close()


def test_plain_sum_entry_point(cuda_device):
    T = cuda_device.Tensor
    rt = cuda_device.runtime
    n = (1 << 20) + 3
    a = (T.random([n], seed=11) - T.fill(0.5, [n])).doCache()
    ev = a._cached
    out = rt.alloc(4)
    for off in (0, 1):  # aligned (float4 loads) and misaligned (scalar loads)
        rt.reduce_sum_ptr(ev.device_ptr() + 4 * off, (1 << 20) + 3 - off, out.device_ptr())
        got = rt.download(out, 1)[0]
        exact = interp.exact_sum(a.flatArray()[off:])
        assert abs(got - exact) <= np.sqrt(1 << 20) * 2.0 ** -24 * np.abs(a.flatArray()).sum()
    out.release()
    a.close()


def test_tuple_join_and_padding(cuda_device):
    T = cuda_device.Tensor
    a = T.random([5, 6], seed=1, padding=7.0)
    b = T.random([5, 6], seed=2, padding=-3.0)
    j = T.join([a.translate([1, -2]), b.translate([-1, 3]), a * b], 1)
    assert j.shape == (5, 3, 6)
    assert np.array_equal(bits(j.flatArray()), bits(oracle_of(cuda_device, j)))


def test_scale_non_integer_view(cuda_device):
    """scale() gives non-integer coefficients: the index is computed in double and truncated, as the reference does."""
    T = cuda_device.Tensor
    a = T.random([7, 9], seed=4)
    v = a.scale([12, 5]).translate([0.5, -1.25])
    assert np.array_equal(bits(v.flatArray()), bits(oracle_of(cuda_device, v)))


def test_matmul_via_broadcast_and_split(cuda_device):
    T = cuda_device.Tensor
    m1 = T.randomNormal([19, 23], seed=1)
    m2 = T.randomNormal([23, 17], seed=2)
    prod = m1.broadcast([19, 23, 17]) * m2.reshape([1, 23, 17]).broadcast([19, 23, 17])
    c = prod.split(1).reduce(lambda x, y: x + y)
    assert np.array_equal(bits(c.flatArray()), bits(oracle_of(cuda_device, c)))


def test_kernel_cache_hit(cuda_device):
    """TensorsSpec.scala:50-52: structurally equal trees reuse one compiled program."""
    T = cuda_device.Tensor
    before = cuda_device.runtime.cache_stats()
    f1 = T.fill(42.0, [2, 3, 5]).translate([0, 1, 0])
    f1.flatArray()
    mid = cuda_device.runtime.cache_stats()
    f2 = T.fill(42.0, [2, 3, 5]).translate([0, 1, 0])
    f2.flatArray()
    after = cuda_device.runtime.cache_stats()
    assert after["entries"] == mid["entries"] >= before["entries"]


def test_random_expression_trees(cuda_device):
    """Seeded random trees over + - * / max min neg abs on views: bit-exact."""
    T = cuda_device.Tensor
    r = np.random.RandomState(5)
    shape = [31, 17, 3]
    leaves = [T.random(shape, seed=s) for s in range(4)] + [T.fill(0.25, shape)]
    for trial in range(12):
        pool = list(leaves)
        for _ in range(r.randint(3, 12)):
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
                t = a.permute([0, 1, 2]).translate([1, 0, -1])
            else:
                t = a.translate([-2, 3, 0])
            pool.append(t)
        e = pool[-1]
        assert np.array_equal(bits(e.flatArray()), bits(oracle_of(cuda_device, e))), trial


@pytest.mark.parametrize("shape", [(2, 6, 5, 3, 4), (3, 32, 32, 8, 8)])
def test_convolution_idiom_bit_exact(cuda_device, shape):
    """The library's 3x3 convolution (translate + split + join), with its shared
    translated channels written once, against the oracle and against the same
    expression without merged subexpressions."""
    import bench
    from compute import Tensors, trees
    n, h, w, c, f = shape
    T = cuda_device.Tensor
    # seeds with bit 30 set: the reference's randomNormal of small seeds meets a zero
    # hash (log 0) at some index, and NaN payloads are not comparable bit for bit
    x = T.randomNormal([n, h, w, c], seed=0x40000003).doCache()
    wt = T.randomNormal([3, 3, c, f], seed=0x40000004).doCache()
    b = T.randomNormal([f], seed=0x40000005).doCache()
    parts = bench.conv_expr(T, x, wt, b, parts=True)
    ser = cuda_device.serialize(trees.Concatenate([t.closure for t in parts]), parts[0].shape)
    got = bench.conv_expr(T, x, wt, b).flatArray()
    want = interp.evaluate(ser.text, [p.flatArray() for p in ser.params])
    assert np.array_equal(bits(got), bits(want))
    plain = Tensors(device=0, runtime=cuda_device.runtime, planner=trees.Planner(merge_common=False))
    unmerged = plain.serialize(trees.Concatenate([t.closure for t in parts]), parts[0].shape)
    assert unmerged.text.count("\nx ") > ser.text.count("\nx ")
    assert np.array_equal(bits(bench.conv_expr(plain.Tensor, x, wt, b).flatArray()), bits(got))


def test_wide_indices_past_2_31(cuda_device):
    """A view program over 5 x 2^29 = 2.7e9 points (10.7 GB per tensor): the
    coordinate decode and the view offsets run in 64-bit arithmetic past 2^31.
    Checked bit-exactly at chunks around the 2^31 and 2^32-byte boundaries and
    at the end, from the reference RNG's values at the mapped indices."""
    rt = cuda_device.runtime
    T = cuda_device.Tensor
    rows, cols = 5, 1 << 29
    seed = 0x40000007
    x = T.random([rows, cols], seed=seed).doCache()
    e = x.translate([1, -3]) + x
    ser = cuda_device.serialize(e.closure, e.shape)
    assert [id(p) for p in ser.params] == [id(x)]
    out = rt.alloc(rows * cols * 4)
    try:
        rt.launch(rt.program(ser.text), [x._cached], out)
        starts = [0, (1 << 29) - 8, (1 << 31) - 8, (1 << 31) + 1000, 3 * (1 << 29) + 7, rows * cols - 4096]
        for s0 in starts:
            got = rt.download(out, 4096, offset=4 * s0)
            lin = np.arange(s0, s0 + 4096, dtype=np.int64)
            i0, i1 = lin // cols, lin % cols
            src0, src1 = i0 - 1, i1 + 3  # translate negates its offsets: source = target - offset
            inside = (src0 >= 0) & (src1 < cols)
            xv = lambda j: rng._unit(rng.wang_hash(j.astype(np.uint32) ^ np.uint32(seed)))
            shifted = np.where(inside, xv(np.where(inside, src0 * cols + src1, 0)), np.float32(0.0))
            want = (shifted + xv(lin)).astype(np.float32)
            assert np.array_equal(got.view(np.int32), want.view(np.int32)), s0
    finally:
        out.release()
        x.close()

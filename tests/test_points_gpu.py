"""Several output points per thread in the generic elementwise kernel (the
`ew_points` knob) and float4 grouped reads (cc_ew_vl, the `ew_vector_loads`
knob): the 3x3 convolution idiom and random view programs give the bits of the
one-point scalar kernel, and the oracle's; misaligned inputs fall back to the
scalar kernel."""

import numpy as np
import pytest

from compute import tuner
from oracle import interp

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


def _same_bits(want, got):
    nan = np.isnan(want)
    assert np.array_equal(nan, np.isnan(got))
    assert np.array_equal(want[~nan].view(np.int32), got[~nan].view(np.int32))


@pytest.mark.parametrize("vl", [0, 1])
@pytest.mark.parametrize("points", [1, 2, 4, 8])
@pytest.mark.parametrize("shape", [(2, 6, 8, 3, 4), (3, 32, 32, 8, 8), (2, 5, 4, 12, 3)])
def test_convolution_points_bit_exact(cuda_device, shape, points, vl):
    import bench
    from compute import trees
    n, h, w, c, f = shape
    T = cuda_device.Tensor
    rt = cuda_device.runtime
    x = T.randomNormal([n, h, w, c], seed=0x40000003).doCache()
    wt = T.randomNormal([3, 3, c, f], seed=0x40000004).doCache()
    b = T.randomNormal([f], seed=0x40000005).doCache()
    parts = bench.conv_expr(T, x, wt, b, parts=True)
    ser = cuda_device.serialize(trees.Concatenate([t.closure for t in parts]), parts[0].shape)
    arrays = [np.asarray(p.flatArray(), np.float32) for p in ser.params]
    want = interp.evaluate(ser.text, arrays)
    before = rt.config_get("ew_vector_loads")
    try:
        rt.config_set("ew_points", points)
        rt.config_set("ew_vector_loads", vl)
        got = _run(rt, ser.text, arrays, n * h * w * f)
    finally:
        rt.config_set("ew_points", 1)
        rt.config_set("ew_vector_loads", before)
    _same_bits(np.asarray(want, np.float32), got)


def test_vector_loads_need_aligned_inputs(cuda_device):
    """The same program through pointers 4 bytes past a 16-byte boundary runs the
    scalar kernel and gives the same bits as the aligned (float4) launch."""
    import bench
    from compute import trees
    from compute.tensors import NonInlineTensor
    rt = cuda_device.runtime
    d = cuda_device
    x, w, b = (NonInlineTensor(d, s, 0.0, None) for s in [(2, 9, 7, 8), (3, 3, 8, 5), (5,)])
    parts = bench.conv_expr(d.Tensor, x, w, b, parts=True)
    ser = d.serialize(trees.Concatenate([t.closure for t in parts]), parts[0].shape)
    r = np.random.RandomState(2)
    by_id = {id(x): r.normal(size=2 * 9 * 7 * 8), id(w): r.normal(size=3 * 3 * 8 * 5), id(b): r.normal(size=5)}
    arrays = [by_id[id(p)].astype(np.float32) for p in ser.params]
    n_out = 2 * 9 * 7 * 5
    prog = rt.program(ser.text)
    assert "cc_ew_vl" in prog.source()
    aligned = _run(rt, ser.text, arrays, n_out)
    bufs = []
    for a in arrays:
        buf = rt.alloc(a.size * 4 + 16)
        rt.upload(buf, a, offset=4)
        bufs.append(buf)
    out = rt.alloc(n_out * 4 + 16)
    rt.launch_ptrs(prog, [buf.device_ptr() + 4 for buf in bufs], out.device_ptr() + 4)
    rt.synchronize()
    shifted = rt.download(out, n_out, offset=4)
    for buf in bufs + [out]:
        buf.release()
    _same_bits(aligned, shifted)
    want = interp.evaluate(ser.text, arrays)
    _same_bits(np.asarray(want, np.float32), aligned)


@pytest.mark.parametrize("points", [2, 4])
def test_random_programs_points_match_one_point(cuda_device, points):
    rt = cuda_device.runtime
    r = np.random.RandomState(3)
    cases = []
    for p in tuner.random_programs(24, seed=41, max_points=1 << 16, max_dim=64):
        if p["kind"] != "ew":
            continue
        arrays = [r.uniform(0.1, 2.0, size=int(np.prod(sh))).astype(np.float32) for sh in p["params"]]
        cases.append((p["ir"], arrays, p["points"]))
    assert len(cases) >= 6
    divisible = 0
    try:
        for text, arrays, n_out in cases:
            rt.config_set("ew_points", 1)
            want = _run(rt, text, arrays, n_out)
            rt.config_set("ew_points", points)
            got = _run(rt, text, arrays, n_out)
            _same_bits(want, got)
            last = int(text.split("\n")[1].split()[-1])
            divisible += last % points == 0
    finally:
        rt.config_set("ew_points", 1)
    assert divisible >= 2


@pytest.mark.parametrize("c", [4, 8, 16])
def test_channel_split_programs(cuda_device, c):
    """Channel reads of a translated NHWC tensor (float4 groups at the edges
    too, where the translate pads) against the oracle, for 1 and 3 points."""
    from compute.tensors import NonInlineTensor
    rt = cuda_device.runtime
    d = cuda_device
    x = NonInlineTensor(d, (3, 7, 9, c), 0.0, None)
    chans = x.split(3)
    acc = chans[0].translate([0, 1, -1])
    for ch in chans[1:]:
        acc = acc * ch + ch.translate([1, 0, 0])
    ser = d.serialize(acc.closure, acc.shape)
    arrays = [np.random.RandomState(c).uniform(-1, 1, size=3 * 7 * 9 * c).astype(np.float32)]
    want = np.asarray(interp.evaluate(ser.text, arrays), np.float32)
    before = rt.config_get("ew_vector_loads")
    try:
        for vl in (0, 1):
            for points in (1, 3):
                rt.config_set("ew_vector_loads", vl)
                rt.config_set("ew_points", points)
                _same_bits(want, _run(rt, ser.text, arrays, 3 * 7 * 9))
    finally:
        rt.config_set("ew_points", 1)
        rt.config_set("ew_vector_loads", before)


def test_vector_load_sum_keeps_the_bits(cuda_device):
    """cc_sum_vl folds the same point values in the same order as cc_sum: the
    sum of the view-heavy op has the same bits with and without float4 reads,
    and is within the sum bound of the exact sum of the oracle's values."""
    import bench
    from compute.tensors import NonInlineTensor
    rt = cuda_device.runtime
    d = cuda_device
    n, c, h, w = 4, 128, 28, 28
    x = NonInlineTensor(d, (n, c, h, w), 0.0, None)
    bias = NonInlineTensor(d, (1, 1, 1, c), 0.0, None)
    s = bench.build_c2(d.Tensor, x, bias, n, c, h, w)
    text = d.serialize(s.closure, s.shape, "sum").text
    r = np.random.RandomState(9)
    arrays = [r.normal(size=n * c * h * w).astype(np.float32), r.normal(size=c).astype(np.float32)]
    before = rt.config_get("ew_vector_loads")
    try:
        rt.config_set("ew_vector_loads", 1)
        assert "cc_sum_vl" in rt.program(text).source()
        got = _run(rt, text, arrays, 1)
        rt.config_set("ew_vector_loads", 0)
        want = _run(rt, text, arrays, 1)
    finally:
        rt.config_set("ew_vector_loads", before)
    assert got.view(np.int32)[0] == want.view(np.int32)[0]
    ew = text.replace("ccir 1 sum", "ccir 1 ew", 1)
    vals = np.asarray(interp.evaluate(ew, arrays), np.float64)
    exact = float(np.sum(vals))
    assert abs(float(got[0]) - exact) <= np.sqrt(vals.size) * 2.0 ** -24 * float(np.sum(np.abs(vals))) + 1e-30


def test_batched_loads_keep_the_bits(cuda_device):
    """`ew_batch_loads`: scalar loads of one condition share a predicate in
    blocks of 8 (the view-heavy op's 128 channel reads); same bits."""
    import bench
    from compute.tensors import NonInlineTensor
    rt = cuda_device.runtime
    d = cuda_device
    r = np.random.RandomState(6)
    n, c, h, w = 4, 128, 28, 28
    x = NonInlineTensor(d, (n, c, h, w), 0.0, None)
    bias = NonInlineTensor(d, (1, 1, 1, c), 0.0, None)
    s = bench.build_c2(d.Tensor, x, bias, n, c, h, w)
    arrays = [r.normal(size=n * c * h * w).astype(np.float32), r.normal(size=c).astype(np.float32)]
    try:
        for kind in ("ew", "sum"):
            text = d.serialize(s.closure, s.shape, kind).text
            n_out = n * h * w if kind == "ew" else 1
            rt.config_set("ew_batch_loads", 0)
            want = _run(rt, text, arrays, n_out)
            rt.config_set("ew_batch_loads", 1)
            assert "@q ld.global.nc.f32 %7" in rt.program(text).source()
            _same_bits(want, _run(rt, text, arrays, n_out))
        ref = interp.evaluate(d.serialize(s.closure, s.shape).text, arrays)
        _same_bits(np.asarray(ref, np.float32), _run(rt, d.serialize(s.closure, s.shape).text, arrays, n * h * w))
    finally:
        rt.config_set("ew_batch_loads", 0)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_channel_view_programs_in_every_form(cuda_device, seed):
    """Random channel splits of translated NHWC tensors weighted by a staged
    vector: the oracle's bits with scalar reads, float4 groups, batched
    predicates and two points per thread; sums bit-identical across forms."""
    from compute.tensors import NonInlineTensor
    rt = cuda_device.runtime
    d = cuda_device
    r = np.random.RandomState(seed)
    n, h, w = 2, int(r.randint(3, 9)), 2 * int(r.randint(2, 6))
    c = int(r.choice([4, 8, 12]))
    x = NonInlineTensor(d, (n, h, w, c), 0.0, None)
    wt = NonInlineTensor(d, (c,), 0.0, None)
    chans, ws = x.split(3), wt.split(0)
    acc = None
    for k in range(c):
        t = chans[k].translate([0, int(r.randint(-1, 2)), int(r.randint(-1, 2))]) * ws[k].broadcast([n, h, w])
        acc = t if acc is None else acc + t
    ser = d.serialize(acc.closure, acc.shape)
    by_id = {id(x): r.normal(size=n * h * w * c).astype(np.float32), id(wt): r.normal(size=c).astype(np.float32)}
    arrays = [by_id[id(p)] for p in ser.params]
    want = np.asarray(interp.evaluate(ser.text, arrays), np.float32)
    sum_text = d.serialize(acc.closure, acc.shape, "sum").text
    knobs = ("ew_vector_loads", "ew_batch_loads", "ew_points")
    saved = [rt.config_get(k) for k in knobs]
    sums = []
    try:
        for vl, bl, pts in ((0, 0, 1), (1, 0, 1), (1, 1, 1), (1, 0, 2)):
            for k, v in zip(knobs, (vl, bl, pts)):
                rt.config_set(k, v)
            _same_bits(want, _run(rt, ser.text, arrays, n * h * w))
            sums.append(_run(rt, sum_text, arrays, 1))
    finally:
        for k, v in zip(knobs, saved):
            rt.config_set(k, v)
    for s in sums[1:]:
        _same_bits(sums[0], s)

"""The C ABI library: loads without a GPU, exports every declared entry point,
and its GPU-free entry points generate and compile the fused kernels."""

import ctypes
import os
import re

import pytest

from compute import _native
from compute.runtime import codegen, compile_check

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^int\s+(cc_\w+)\s*\(", text, flags=re.M)
    return names


def test_library_loads_and_exports_every_declared_symbol():
    lib = _native.load()
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
        assert n in _native._SIGNATURES, "no ctypes signature for " + n


def test_init_without_gpu_fails_cleanly():
    lib = _native.load()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    st = lib.cc_init(0, 0)
    assert st == -1  # CC_ERR_DEVICE_NOT_FOUND
    assert "CUDA" in _native.last_error() or "device" in _native.last_error()


C2_SMALL = None


def c2_ir():
    from compute import Tensors
    d = Tensors(runtime=object())
    T = d.Tensor
    x = T.randomNormal([2, 8, 5, 5], seed=0)
    bias = (T.randomNormal([8], seed=1) * T.fill(0.1, [8])).reshape([1, 1, 1, 8])
    y = T.max(x.permute([0, 2, 3, 1]) + bias.broadcast([2, 5, 5, 8]), T.fill(0.0, [2, 5, 5, 8]))
    s = y.translate([0, 0, 1, 0]).split(3).reduce(lambda a, b: a + b)
    return d.serialize(s.closure, s.shape).text


def test_codegen_and_nvrtc_compile_for_sm103a():
    ir = c2_ir()
    src = codegen(ir)
    assert "cc_ew" in src and "__launch_bounds__" in src
    compile_check(ir, (10, 3))
    compile_check(ir.replace("ccir 1 ew", "ccir 1 sum"), (10, 3))


def test_contiguous_programs_get_a_float4_variant():
    ir = "ccir 1 sum\no 1 100\np 1 100 00000000\nx 0 2 1 0\np 1 100 00000000\nx 2 2 1 0\nb mul 1 3\nu tanh 4\nr 5\n"
    src = codegen(ir)
    assert "cc_sum_v4" in src and "float4" in src
    compile_check(ir)


def test_invalid_ir_is_rejected():
    with pytest.raises(_native.InvalidProgram):
        codegen("ccir 1 ew\no 1 4\nb add 0 1\nr 0\n")
    with pytest.raises(_native.InvalidProgram):
        codegen("not an ir")
    with pytest.raises(_native.InvalidProgram):
        codegen("ccir 1 ew\no 1 4\np 1 4 00000000\nx 0 3 1 0 0\nr 1\n")  # matrix/frame mismatch


def test_compile_failure_carries_the_nvrtc_log():
    ir = "ccir 1 ew\no 1 4\nl 3f800000\nr 0\n"
    with pytest.raises(_native.BuildProgramFailure) as e:
        compile_check(ir, (1, 0))
    assert "NVRTC" in str(e.value)


def _matmul_ir(i, j, k, swap=False):
    from compute import Tensors
    d = Tensors(runtime=object())
    T = d.Tensor
    m1 = T.randomNormal([i, j], seed=1)
    m2 = T.randomNormal([j, k], seed=2)
    a = m1.broadcast([i, j, k])
    b = m2.reshape([1, j, k]).broadcast([i, j, k])
    prod = b * a if swap else a * b
    c = prod.split(1).reduce(lambda x, y: x + y)
    return d.serialize(c.closure, c.shape).text


def test_the_matmul_idiom_is_recognised_as_a_contraction():
    """TensorsSpec.scala:472-478's matmul reaches the runtime as one fused fold, recognised as C = A * B."""
    src = codegen(_matmul_ir(5, 7, 3))
    assert src.startswith("// contraction m=5 n=3 k=7 a=0 b=1")
    src = codegen(_matmul_ir(5, 7, 3, swap=True))
    assert src.startswith("// contraction m=5 n=3 k=7 a=1 b=0")
    # a fold whose terms are not the split views of one product is not a contraction
    from compute import Tensors
    d = Tensors(runtime=object())
    T = d.Tensor
    t = T.randomNormal([4, 6, 3], seed=1)
    s = t.split(1).reduce(lambda x, y: x + y)
    assert not codegen(d.serialize(s.closure, s.shape).text).startswith("// contraction")


def test_a_long_fold_serialises():
    text = _matmul_ir(8, 2048, 8)
    assert text.count("\nv ") == 2048


def test_batch_module_compiles_for_sm103a():
    """A batch of contiguous programs of several structures and lengths builds (parts compile; no GPU to link)."""
    from compute import Tensors
    from compute.runtime import batch_compile_check
    from compute.tensors import NonInlineTensor
    d = Tensors(runtime=object())
    T = d.Tensor
    texts = []
    for k, n in enumerate([5, 4096, 70001, 3, 4096]):
        a = NonInlineTensor(d, (n,), 0.0, None)
        b = NonInlineTensor(d, (n,), 0.0, None)
        e = [T.tanh(a * b + a), T.exp(a) / b, T.max(a, b) - T.log(b), T.tanh(a * b + a), a * b][k]
        texts.append(d.serialize(e.closure, e.shape).text)
    structures, seconds = batch_compile_check(texts)
    assert structures == 4  # programs 0 and 3 share code although their lengths differ


def test_shared_memory_ring_codegen_compiles():
    import bench
    from compute import Tensors, runtime
    from compute.tensors import NonInlineTensor
    d = Tensors(device=0)
    n, c, h, w = 64, 128, 56, 56
    x = NonInlineTensor(d, (n, c, h, w), 0.0, None)
    bias = NonInlineTensor(d, (1, 1, 1, c), 0.0, None)
    s = bench.build_c2(d.Tensor, x, bias, n, c, h, w)
    text = d.serialize(s.closure, s.shape).text
    src = runtime.codegen(text, "block=128 ring=32 lookahead=32 min_blocks=11")
    assert "extern __shared__ float cc_ring[];" in src
    assert src.count("cc_cp4(&cc_ring") == 128  # every x load staged; the bias loads (uniform) are not
    assert "cc_cp4(&cc_ring" not in runtime.codegen(text)
    runtime.compile_check(text, options="block=128 ring=32 lookahead=32 min_blocks=11")


def test_merged_subexpressions_keep_the_oracle_bits():
    """Structurally identical subexpressions are written once in the IR; the
    oracle gives the same bits for the merged and the unmerged text."""
    import bench
    import numpy as np
    from compute import Tensors, trees
    from compute.tensors import NonInlineTensor
    from oracle import interp
    d = Tensors(device=0)
    plain = Tensors(device=0, planner=trees.Planner(merge_common=False))
    shapes = [(2, 5, 4, 3), (3, 3, 3, 2), (2,)]
    r = np.random.RandomState(0)
    arrays = [r.normal(size=int(np.prod(s))).astype(np.float32) for s in shapes]
    texts = []
    for dev in (d, plain):
        x, w, b = (NonInlineTensor(dev, s, 0.0, None) for s in shapes)
        parts = bench.conv_expr(dev.Tensor, x, w, b, parts=True)
        ser = dev.serialize(trees.Concatenate([t.closure for t in parts]), parts[0].shape)
        order = {id(x): 0, id(w): 1, id(b): 2}
        texts.append((ser.text, [arrays[order[id(p)]] for p in ser.params]))
    (merged, m_in), (unmerged, u_in) = texts
    assert merged.count("\nx ") < unmerged.count("\nx ")
    a = interp.evaluate(merged, m_in)
    b_ = interp.evaluate(unmerged, u_in)
    assert np.array_equal(a.view(np.int32), b_.view(np.int32))


def test_points_per_thread_codegen():
    """Two points per thread of the 3x3 convolution: the x reads the two points
    share and the weight reads are emitted once; a last extent the point count
    does not divide keeps the one-point kernel."""
    import bench
    from compute import Tensors, runtime, trees
    from compute.tensors import NonInlineTensor
    d = Tensors(device=0)
    x, w, b = (NonInlineTensor(d, s, 0.0, None) for s in [(4, 16, 16, 8), (3, 3, 8, 8), (8,)])
    parts = bench.conv_expr(d.Tensor, x, w, b, parts=True)
    text = d.serialize(trees.Concatenate([t.closure for t in parts]), parts[0].shape).text
    one = runtime.codegen(text, "vl=0")
    two = runtime.codegen(text, "points=2 vl=0")
    assert runtime.codegen(text, "points=1 vl=0") == one
    assert runtime.codegen(text, "points=3 vl=0") == one  # 16 % 3 != 0
    # 9 offsets x 8 channels of x per point; two points along w share 2 of 3 columns
    assert one.count("cc_ld(_") == 72 and two.count("cc_ld(_") == 96
    assert one.count("cc_sp2[") == two.count("cc_sp2[") == 2 + 576  # declaration, copy, reads
    assert "* 2; lin < n; lin += stride * 2)" in two
    runtime.compile_check(text, options="points=2 vl=0")


def test_vector_load_codegen():
    """Reads of the 8 channels of a pixel (NHWC, constant innermost index)
    become two float4 loads per pixel in cc_ew_vl; cc_ew keeps scalar reads."""
    import bench
    from compute import Tensors, runtime, trees
    from compute.tensors import NonInlineTensor
    d = Tensors(device=0)
    x, w, b = (NonInlineTensor(d, s, 0.0, None) for s in [(4, 16, 16, 8), (3, 3, 8, 8), (8,)])
    parts = bench.conv_expr(d.Tensor, x, w, b, parts=True)
    text = d.serialize(trees.Concatenate([t.closure for t in parts]), parts[0].shape).text
    assert "cc_ew_vl" not in runtime.codegen(text, "vl=0")
    src = runtime.codegen(text)  # vl=1 by default
    scalar, vl = src.split("cc_ew_vl(")
    assert scalar.count("cc_ld(_") == 72 and "cc_ld4(_" not in scalar
    assert vl.count("cc_ld4(_") == 18 and "cc_ld(_" not in vl  # 9 offsets x 2 groups of 4 channels
    # the staged weights (filters innermost) and bias as float4 shared reads: 9 x 8 x 2 + 2
    assert vl.count("reinterpret_cast<const float4 *>(cc_sp") == 146
    assert "__align__(16) float cc_sp2[576]" in vl and "__align__(16) float cc_sp" not in scalar
    assert runtime.codegen(text, "vl=1 points=2").split("cc_ew_vl(")[1].count("cc_ld4(_") == 24
    runtime.compile_check(text, options="vl=1 points=2")
    # a view whose innermost index varies with the output has nothing to group
    y = NonInlineTensor(d, (6, 8), 0.0, None)
    t = y.translate([0, 1]) + y
    assert "cc_ew_vl" not in runtime.codegen(d.serialize(t.closure, t.shape).text, "vl=1")


def test_vector_load_sum_codegen():
    """A sum over the view-heavy op gets cc_sum_vl (the bias read as float4
    groups), compiled for sm_103a."""
    import bench
    from compute import Tensors, runtime
    from compute.tensors import NonInlineTensor
    d = Tensors(device=0)
    n, c, h, w = 2, 16, 5, 7
    x = NonInlineTensor(d, (n, c, h, w), 0.0, None)
    bias = NonInlineTensor(d, (1, 1, 1, c), 0.0, None)
    s = bench.build_c2(d.Tensor, x, bias, n, c, h, w)
    text = d.serialize(s.closure, s.shape, "sum").text
    src = runtime.codegen(text)
    assert "cc_sum_vl(" in src and src.split("cc_sum_vl(")[1].count("cc_ld4(_") == 4
    assert "cc_sum_vl(" not in runtime.codegen(text, "vl=0")
    runtime.compile_check(text)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_channel_view_programs_compile_in_every_form(seed):
    """Random channel splits of translated/permuted NHWC tensors (reads at known
    view indices, float4 groups, staged weights), as elementwise programs and
    sums, compile for sm_103a with every read form: scalar, float4 groups,
    batched predicates, two points per thread."""
    import numpy as np
    from compute import Tensors, runtime
    from compute.tensors import NonInlineTensor
    r = np.random.RandomState(seed)
    d = Tensors(device=0)
    n, h, w = 2, int(r.randint(3, 9)), 2 * int(r.randint(2, 6))
    c = int(r.choice([4, 8, 12]))
    x = NonInlineTensor(d, (n, h, w, c), 0.0, None)
    wt = NonInlineTensor(d, (c,), 0.0, None)
    chans = x.split(3)
    ws = wt.split(0)
    acc = None
    for k in range(c):
        t = chans[k].translate([0, int(r.randint(-1, 2)), int(r.randint(-1, 2))]) * ws[k].broadcast([n, h, w])
        acc = t if acc is None else acc + t
    for kind in ("ew", "sum"):
        text = d.serialize(acc.closure, acc.shape, kind).text
        for opts in ("vl=0", "vl=1", "vl=1 batch=1", "vl=1 points=2"):
            runtime.compile_check(text, options=opts)
        assert ("cc_ew_vl(" if kind == "ew" else "cc_sum_vl(") in runtime.codegen(text)

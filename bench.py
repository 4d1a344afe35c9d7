"""Benchmark of the fused-tensor hot path on GB300.

Default workload (``--workload c2``): the view-heavy fused op on
x[64,128,56,56] ~ N(0,1) and bias[128] ~ N(0,0.1): permute NCHW->NHWC,
broadcast-add the bias, max(.,0), translate by 1 along W, then sum over the
channel axis to [64,56,56].  ``--workload c1``: ((a*b+c).tanh).sum over three
[1024,1024] tensors uniform in [-1,1].

A step is one evaluation of the op with its inputs resident in HBM.  The value
is algorithmic bytes / time (the bytes a single fused pass must move: every
input read once, the output written once).  Inputs rotate over enough copies
that the working set exceeds the 129 MB L2 between uses of one copy.

``--impl reference`` times the reference's CPU implementation of the same op
(the oracle's restatement of the generated OpenCL C, compiled with OpenMP, on
all host cores) on a bounded sample of the workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "compute.scala_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

L2_BYTES = 129 * 1024 * 1024


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic(workload):
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(workload)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock/throttle samples while the GPU is busy."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        busy = [v for v in sm if mx and v > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ------------------------------------------------------------------ workloads

C2 = dict(n=64, c=128, h=56, w=56)
C1 = dict(n=1024, m=1024)


def c2_bytes(n, c, h, w):
    return 4 * (n * c * h * w + c + n * h * w)


def c1_bytes(n, m):
    return 4 * (3 * n * m) + 4


def build_c2(T, x, bias, n, c, h, w):
    y = T.max(x.permute([0, 2, 3, 1]) + bias.broadcast([n, h, w, c]), T.fill(0.0, [n, h, w, c]))
    return y.translate([0, 0, 1, 0]).split(3).reduce(lambda a, b: a + b)


C6 = {"n": 128, "h": 32, "w": 32, "c": 8, "k": 3}


def conv_expr(T, x, weight, bias, parts=False):
    """The library's 3x3 convolution idiom (benchmarks.scala:463-556): per filter,
    the sum over kernel offsets and input channels of translated channel views
    times broadcast weight scalars, plus the bias, joined along a new last axis
    (``parts``: the per-filter tensors instead of their join)."""
    n, h, w, depth = x.shape
    kh, kw, _, filters = weight.shape
    channels = x.split(3)
    out = []
    for f_weights, f_bias in zip(weight.split(3), bias.split(0)):
        terms = []
        for oy, row in zip(range(-(kh // 2), kh // 2 + 1), f_weights.split(0)):
            for ox, pixel in zip(range(-(kw // 2), kw // 2 + 1), row.split(0)):
                for ch, wch in zip(channels, pixel.split(0)):
                    terms.append(ch.translate([0, oy, ox]) * wch.broadcast([n, h, w]))
        acc = terms[0]
        for t in terms[1:]:
            acc = acc + t
        out.append(f_bias.broadcast([n, h, w]) + acc)
    return out if parts else T.join(out)


C3 = {"c3": (4096, 4096, 4096), "c3s": (16384, 256, 16384)}
# The inner-axis fold t.split(1).reduce(_ + _) over x[16384, 4096] ~ N(0,1).
C7 = {"rows": 16384, "cols": 4096}
# Exactly one index per seed makes the Wang hash 0 (log(0) = -inf in Box-Muller);
# seeds with bit 30 set move it past 2^30, beyond these tensors.
C3_SEED = 0x40000000


def matmul_expr(T, a, b):
    """The library's matmul (TensorsSpec.scala:472-478): broadcast product, then a left fold of split(1)."""
    i, j = a.shape
    _, k = b.shape
    prod = a.broadcast([i, j, k]) * b.reshape([1, j, k]).broadcast([i, j, k])
    return prod.split(1).reduce(lambda x, y: x + y)


def c4_programs(T, seed=0, count=2048, lo=1024, hi=4194304, shapes_only=False):
    """The batched-programs workload: `count` independent fused programs, lengths
    log-uniform on [lo, hi], each a random expression tree of 3-12 operator
    nodes over {+,-,*,/,exp,log,tanh,max} on 1-4 inputs uniform in [0.1, 2]."""
    import numpy as np
    r = np.random.RandomState(seed)
    progs = []
    for p in range(count):
        n = int(round(float(np.exp(r.uniform(np.log(lo), np.log(hi))))))
        n_in = int(r.randint(1, 5))
        n_nodes = int(r.randint(3, 13))
        ops = [r.choice(["+", "-", "*", "/", "exp", "log", "tanh", "max"]) for _ in range(n_nodes)]
        picks = [(int(r.randint(0, 1 << 30)), int(r.randint(0, 1 << 30))) for _ in range(n_nodes)]
        progs.append((n, n_in, ops, picks, int(r.randint(0, 1 << 30))))
    if shapes_only:
        return progs
    out = []
    for n, n_in, ops, picks, in_seed in progs:
        inputs = [(T.random([n], seed=in_seed + i) * T.fill(1.9, [n]) + T.fill(0.1, [n])).doCache() for i in range(n_in)]
        pool = list(inputs)
        for op, (pa, pb) in zip(ops, picks):
            a = pool[-1]  # keep the tree connected: every node uses the previous one
            b = pool[pb % len(pool)]
            if op == "+":
                t = a + b
            elif op == "-":
                t = a - b
            elif op == "*":
                t = a * b
            elif op == "/":
                t = a / b
            elif op == "max":
                t = T.max(a, b)
            else:
                t = getattr(T, op)(a)
            pool.append(t)
        out.append((pool[-1], inputs))
    return out


def setup(workload, d):
    """Returns (program, list of input-buffer lists to rotate over, output buffer, bytes, description)."""
    T = d.Tensor
    rt = d.runtime
    if workload == "c2":
        n, c, h, w = C2["n"], C2["c"], C2["h"], C2["w"]
        x = T.randomNormal([n, c, h, w], seed=0).doCache()
        bias = (T.randomNormal([c], seed=1) * T.fill(0.1, [c])).reshape([1, 1, 1, c]).doCache()
        s = build_c2(T, x, bias, n, c, h, w)
        ser = d.serialize(s.closure, s.shape)
        assert [id(p) for p in ser.params] == [id(x), id(bias)]
        prog = rt.program(ser.text)
        xbytes = n * c * h * w * 4
        copies = max(2, -(-4 * L2_BYTES // xbytes))
        sets = []
        for _ in range(copies):
            buf = rt.alloc(xbytes)
            rt.random(buf, n * c * h * w, 0, True)
            sets.append([buf, bias._cached])
        out = rt.alloc(n * h * w * 4)
        return dict(prog=prog, sets=sets, out=out, bytes=c2_bytes(n, c, h, w), copies=copies,
                    owned=[s_[0] for s_ in sets],
                    keep=[x, bias], ser=ser, shape=(n, c, h, w),
                    config={"workload": arm_workload("c2"),
                            "x": [n, c, h, w], "bias": [c], "out": [n, h, w],
                            "l2": "inputs rotate over %d copies of x (%.0f MB > 4x L2)" % (copies, copies * xbytes / 1e6)})
    if workload == "c1":
        n, m = C1["n"], C1["m"]
        two, one = T.fill(2.0, [n, m]), T.fill(1.0, [n, m])
        abc = [(T.random([n, m], seed=s) * two - one).doCache() for s in (0, 1, 2)]
        expr = T.tanh(abc[0] * abc[1] + abc[2])
        ser = d.serialize(expr.closure, expr.shape, "sum")
        prog = rt.program(ser.text)
        copies = max(2, -(-4 * L2_BYTES // (3 * n * m * 4)))
        sets = []
        for k in range(copies):
            trip = []
            for t in abc:
                buf = rt.alloc(n * m * 4)
                d.runtime.launch(rt.program(d.serialize(t.closure, t.shape).text), [t._cached], buf)
                trip.append(buf)
            sets.append(trip)
        out = rt.alloc(4)
        return dict(prog=prog, sets=sets, out=out, bytes=c1_bytes(n, m), copies=copies, keep=abc, ser=ser,
                    owned=[b_ for trip in sets for b_ in trip],
                    shape=(n, m),
                    config={"workload": arm_workload("c1"),
                            "l2": "inputs rotate over %d copies of (a,b,c) (%.0f MB > 4x L2)"
                                  % (copies, copies * 3 * n * m * 4 / 1e6)})
    if workload == "c6":
        from compute import trees
        n, h, w, c, k = C6["n"], C6["h"], C6["w"], C6["c"], C6["k"]
        x = T.randomNormal([n, h, w, c], seed=C3_SEED).doCache()
        weight = T.randomNormal([k, k, c, c], seed=C3_SEED + 1).doCache()
        bias = T.randomNormal([c], seed=C3_SEED + 2).doCache()
        chans = conv_expr(T, x, weight, bias, parts=True)
        ser = d.serialize(trees.Concatenate([t.closure for t in chans]), chans[0].shape)
        assert sorted(id(p) for p in ser.params) == sorted((id(x), id(weight), id(bias)))
        prog = rt.program(ser.text)
        xbytes = n * h * w * c * 4
        copies = max(2, -(-4 * L2_BYTES // xbytes))
        sets = []
        owned = []
        for i in range(copies):
            buf = rt.alloc(xbytes)
            owned.append(buf)
            rt.random(buf, n * h * w * c, C3_SEED, True)
            by_param = {id(x): buf, id(weight): weight._cached, id(bias): bias._cached}
            sets.append([by_param[id(p)] for p in ser.params])  # parameters in first-use order
        out = rt.alloc(n * h * w * c * 4)
        nbytes = 2 * xbytes + k * k * c * c * 4 + c * 4
        return dict(prog=prog, sets=sets, out=out, bytes=nbytes, copies=copies, keep=(x, weight, bias), ser=ser,
                    owned=owned,
                    shape=(n, h, w, c),
                    config={"workload": arm_workload("c6"),
                            "flops_per_step": 2 * n * h * w * c * k * k * c,
                            "l2": "inputs rotate over %d copies of x (%.0f MB > 4x L2)"
                                  % (copies, copies * xbytes / 1e6)})
    if workload == "c7":
        R, J = C7["rows"], C7["cols"]
        x = T.randomNormal([R, J], seed=C3_SEED).doCache()
        s = x.split(1).reduce(lambda a, b: a + b)
        ser = d.serialize(s.closure, s.shape)
        prog = rt.program(ser.text)
        xbytes = R * J * 4
        copies = max(2, -(-4 * L2_BYTES // xbytes))
        sets, owned = [], []
        for _ in range(copies):
            buf = rt.alloc(xbytes)
            rt.random(buf, R * J, C3_SEED, True)
            sets.append([buf])
            owned.append(buf)
        out = rt.alloc(R * 4)
        return dict(prog=prog, sets=sets, out=out, bytes=xbytes + R * 4, copies=copies, keep=[x], ser=ser,
                    owned=owned, shape=(R, J),
                    config={"workload": arm_workload("c7"),
                            "kernel": "TMA-staged row tiles (64 rows x 32 floats, 128-byte swizzle), one output "
                                      "per thread folded left to right",
                            "l2": "inputs rotate over %d copies of x (%.0f MB > 4x L2)" % (copies, copies * xbytes / 1e6)})
    if workload in C3:
        m, k, n = C3[workload]
        rt.config_set("contraction", 3)  # split-BF16 on the tensor cores
        a = T.randomNormal([m, k], seed=C3_SEED).doCache()
        b = T.randomNormal([k, n], seed=C3_SEED + 1).doCache()
        c = matmul_expr(T, a, b)
        ser = d.serialize(c.closure, c.shape)
        # inputs: A, and B's [1,J,K] reshape (which shares B's buffer)
        assert len(ser.params) == 2 and ser.params[0] is a
        prog = rt.program(ser.text)
        out = rt.alloc(m * n * 4)
        return dict(prog=prog, sets=[[a._cached, b._cached]], out=out, flops=2.0 * m * n * k, bytes=4 * (m * k + k * n + m * n),
                    owned=[],
                    keep=[a, b], ser=ser, shape=(m, k, n), copies=1,
                    config={"workload": arm_workload(workload),
                            "method": "split-BF16 (3 planes, 6 products) on tcgen05 tensor cores, FP32 accumulate",
                            "seeds": [C3_SEED, C3_SEED + 1],
                            "l2": "operands %.0f MB; no rotation (compute-bound)" % (4 * (m * k + k * n) / 1e6)})
    raise SystemExit("unknown workload " + workload)


def release(st):
    """Returns a workload's buffers to the pool."""
    for b in st["owned"]:
        b.release()
    for t in st["keep"]:
        t.close()
    st["out"].release()


def contraction_extras(d, st):
    """Error of the split-BF16 result against float64 (512 sampled rows), and the
    FP32 CUDA-core GEMM's speed, fraction of the FP32 CUDA-core peak and error."""
    import numpy as np
    rt = d.runtime
    m, k, n = st["shape"]
    a, b = st["keep"]
    rt.launch(st["prog"], st["sets"][0], st["out"])
    rows = np.sort(np.random.RandomState(0).choice(m, size=min(m, 512), replace=False))
    c = np.stack([rt.download(st["out"], n, offset=int(r) * n * 4) for r in rows]).astype(np.float64)
    A = a.flatArray().reshape(m, k)[rows].astype(np.float64)
    B = b.flatArray().reshape(k, n).astype(np.float64)
    ref = A @ B
    err = float(np.linalg.norm(c - ref) / np.linalg.norm(ref))
    out = rt.alloc(m * n * 4)
    args = (a._cached.device_ptr(), b._cached.device_ptr(), out.device_ptr(), m, n, k, rt.GEMM_FP32)
    rt.gemm_ptr(*args)
    e0 = rt.event()
    for _ in range(3):
        rt.gemm_ptr(*args)
    e1 = rt.event()
    rt.event_wait(e1)
    ms = rt.event_elapsed_ms(e0, e1) / 3
    c32 = np.stack([rt.download(out, n, offset=int(r) * n * 4) for r in rows]).astype(np.float64)
    err32 = float(np.linalg.norm(c32 - ref) / np.linalg.norm(ref))
    # the exact fold (the default contraction mode: the reference's rounding order), timed once
    exact_args = args[:-1] + (rt.GEMM_EXACT,)
    rt.gemm_ptr(*exact_args)
    e0 = rt.event()
    rt.gemm_ptr(*exact_args)
    e1 = rt.event()
    rt.event_wait(e1)
    ms_exact = rt.event_elapsed_ms(e0, e1)
    out.release()
    info = rt.device_info()
    # FP32 CUDA-core peak: 128 FP32 lanes per SM, one FMA (2 flops) each per clock, at the maximum SM clock
    fp32_peak = info["sm_count"] * 128 * 2 * 2070e6 / 1e12
    fp32 = 2.0 * m * n * k / (ms * 1e-3) / 1e12
    return {"rel_fro_err_vs_fp64": err, "rows_checked": int(len(rows)),
            "fp32_cuda_core_tflops": fp32, "fp32_cuda_core_rel_fro_err": err32,
            "fp32_cuda_core_peak_tflops": fp32_peak, "fp32_cuda_core_frac_of_peak": fp32 / fp32_peak,
            "fp32_cuda_core_peak_note": "SMs x 128 FP32 lanes x 2 flops x 2070 MHz (nominal)",
            "exact_fold_tflops": 2.0 * m * n * k / (ms_exact * 1e-3) / 1e12,
            "exact_fold_note": "the default contraction mode: per output, products and sums rounded separately "
                               "in the reference's order (one mul and one add per term)"}


def time_device(rt, st, steps, warmup):
    prog, sets, out = st["prog"], st["sets"], st["out"]
    ptr_sets = [[b.device_ptr() for b in s] for s in sets]
    out_ptr = out.device_ptr()
    for i in range(warmup):
        rt.launch_ptrs(prog, ptr_sets[i % len(sets)], out_ptr)
    rt.synchronize()
    e0 = rt.event()
    for i in range(steps):
        rt.launch_ptrs(prog, ptr_sets[i % len(sets)], out_ptr)
    e1 = rt.event()
    rt.event_wait(e1, 120 * 10 ** 9)
    ms = rt.event_elapsed_ms(e0, e1)
    rt.event_release(e0)
    rt.event_release(e1)
    return ms


def launch_floor(d, steps=200, warmup=10):
    """Per-launch time of the fused elementwise+sum program on 4 points (one
    block, one partial), launched back to back like the benchmark: the fixed
    cost a launch of this kernel pays whatever its size."""
    T = d.Tensor
    rt = d.runtime
    tiny = [(T.random([1, 4], seed=s) * T.fill(2.0, [1, 4]) - T.fill(1.0, [1, 4])).doCache() for s in (0, 1, 2)]
    expr = T.tanh(tiny[0] * tiny[1] + tiny[2])
    prog = rt.program(d.serialize(expr.closure, expr.shape, "sum").text)
    out = rt.alloc(4)
    st = {"prog": prog, "sets": [[t._cached for t in tiny]], "out": out}
    for i in range(warmup):
        rt.launch_ptrs(prog, [t._cached.device_ptr() for t in tiny], out.device_ptr())
    ms = time_device(rt, st, steps, warmup) / steps
    out.release()
    for t in tiny:
        t.close()
    return ms


def time_isolated(rt, st, reps):
    """Median device time of single launches, each alone between two synchronisations."""
    prog, sets, out = st["prog"], st["sets"], st["out"]
    ptr_sets = [[b.device_ptr() for b in s] for s in sets]
    out_ptr = out.device_ptr()
    times = []
    for i in range(reps):
        rt.synchronize()
        e0 = rt.event()
        rt.launch_ptrs(prog, ptr_sets[i % len(sets)], out_ptr)
        e1 = rt.event()
        rt.event_wait(e1, 60 * 10 ** 9)
        times.append(rt.event_elapsed_ms(e0, e1))
        rt.event_release(e0)
        rt.event_release(e1)
    return statistics.median(times)


def keep_busy(rt, st, seconds):
    """Untimed launches of the same kernel so the clock sampler sees the GPU under this load."""
    prog, sets, out = st["prog"], st["sets"], st["out"]
    ptr_sets = [[b.device_ptr() for b in s] for s in sets]
    t_end = time.time() + seconds
    i = 0
    while time.time() < t_end:
        for _ in range(200):
            rt.launch_ptrs(prog, ptr_sets[i % len(sets)], out.device_ptr())
            i += 1
        rt.synchronize()


def time_e2e(d, st, steps, pipelined=True, depth=2):
    """Host buffers in, result out, through the C ABI, every step: upload the
    inputs from pinned host memory, launch, read the result back.

    pipelined: `depth` steps in flight through the event API (cc_buf_upload_ev,
    cc_launch_ev, cc_buf_download_ev: the reference's enqueue with wait lists),
    each on its own device buffers, the host waiting for a step's result before
    issuing the step `depth` later; else one step at a time (non-blocking
    uploads, launch, blocking read).  Returns (seconds per step, H2D bytes, D2H
    bytes, whether every result read back has the bits of a launch on the inputs)."""
    import ctypes
    import numpy as np
    from compute._native import call
    rt = d.runtime
    inputs = st["sets"][0]
    hosts = []
    h2d = 0
    for b in inputs:
        ptr = ctypes.c_void_p()
        call("cc_host_alloc", ctypes.c_size_t(b.nbytes), ctypes.byref(ptr))
        arr = np.ctypeslib.as_array((ctypes.c_float * (b.nbytes // 4)).from_address(ptr.value))
        arr[:] = rt.download(b, b.nbytes // 4)
        hosts.append((ptr, arr))
        h2d += b.nbytes
    out = st["out"]
    out_elems = st["prog"].out_elems
    d2h = 4 * max(1, out_elems)
    depth = depth if pipelined else 1
    results = []  # the results land in pinned host memory too
    for _ in range(depth):
        res = ctypes.c_void_p()
        call("cc_host_alloc", ctypes.c_size_t(d2h), ctypes.byref(res))
        results.append(res)
    owned = []

    def blocking_step():
        for (ptr, arr), b in zip(hosts, inputs):
            call("cc_buf_upload_async", ctypes.c_uint64(b.handle), ctypes.c_size_t(0), ptr, ctypes.c_size_t(b.nbytes))
        rt.launch(st["prog"], inputs, out)
        call("cc_buf_download", ctypes.c_uint64(out.handle), ctypes.c_size_t(0), results[0], ctypes.c_size_t(d2h))

    if pipelined:
        slots = []
        for _ in range(depth):
            ins = [rt.alloc(b.nbytes) for b in inputs]
            o = rt.alloc(max(d2h, out.nbytes))
            owned.extend(ins + [o])
            slots.append((ins, o))
        launched = [None] * depth
        pending = []

        def run(n_steps):
            for k in range(n_steps):
                s = k % depth
                ins, o = slots[s]
                # the slot's buffers are free once its previous launch has read them
                wait = [launched[s]] if launched[s] else []
                ups = [rt.upload_ev(b, ptr.value, b.nbytes, wait=wait) for (ptr, _), b in zip(hosts, ins)]
                if launched[s]:
                    rt.event_release(launched[s])
                launched[s] = rt.launch_ev(st["prog"], ins, o, wait=ups)
                for e in ups:
                    rt.event_release(e)
                pending.append(rt.download_ev(o, results[s].value, d2h, wait=[launched[s]]))
                if len(pending) >= depth:  # this step's slot comes round again next: its result must be read
                    e = pending.pop(0)
                    rt.event_wait(e, 60 * 10 ** 9)
                    rt.event_release(e)
            while pending:
                e = pending.pop(0)
                rt.event_wait(e, 60 * 10 ** 9)
                rt.event_release(e)
    else:
        def run(n_steps):
            for _ in range(n_steps):
                blocking_step()

    try:
        run(2)
        t0 = time.perf_counter()
        run(steps)
        dt = (time.perf_counter() - t0) / steps
        # every slot's last result against one launch on the original inputs
        rt.launch(st["prog"], inputs, out)
        want = rt.download(out, d2h // 4)
        match = all(np.array_equal(np.ctypeslib.as_array((ctypes.c_float * (d2h // 4)).from_address(r.value)).view(
            np.int32), want.view(np.int32)) for r in results)
    finally:
        if pipelined:
            for e in launched:
                if e:
                    rt.event_release(e)
            rt.synchronize()
        for b in owned:
            b.release()
        for ptr, _ in hosts:
            call("cc_host_free", ptr)
        for r in results:
            call("cc_host_free", r)
    return dt, h2d, d2h, match


_LINK = {}


def link_rates(d, nbytes=64 << 20, reps=8):
    """The host link's copy rates through the C ABI (pinned host memory of
    cc_host_alloc, cc_buf_upload_async / cc_buf_download_async of nbytes, reps
    back to back, one cc_synchronize), in GB/s; measured once per process."""
    if _LINK:
        return _LINK
    import ctypes
    from compute._native import call
    rt = d.runtime
    buf = rt.alloc(nbytes)
    ptr = ctypes.c_void_p()
    call("cc_host_alloc", ctypes.c_size_t(nbytes), ctypes.byref(ptr))
    try:
        ctypes.memset(ptr, 0, nbytes)
        for name, fn in (("h2d_gbs", "cc_buf_upload_async"), ("d2h_gbs", "cc_buf_download_async")):
            best = None
            for _ in range(3):
                call(fn, ctypes.c_uint64(buf.handle), ctypes.c_size_t(0), ptr, ctypes.c_size_t(nbytes))
                call("cc_synchronize")
                t0 = time.perf_counter()
                for _ in range(reps):
                    call(fn, ctypes.c_uint64(buf.handle), ctypes.c_size_t(0), ptr, ctypes.c_size_t(nbytes))
                call("cc_synchronize")
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            _LINK[name] = nbytes * reps / best / 1e9
    finally:
        call("cc_host_free", ptr)
        buf.release()
    _LINK["how"] = "%d MB copies from/to pinned host memory, %d back to back, best of 3" % (nbytes >> 20, reps)
    return _LINK


def with_link_bound(d, e2e):
    """Adds the host link's bound to an e2e record: the time the step's copies
    take at the link's measured rates (each direction alone, the two overlapping),
    and the step's fraction of it."""
    if not e2e or not e2e.get("ms_per_step"):
        return e2e
    rates = link_rates(d)
    t_h2d = e2e["h2d_bytes_per_step"] / (rates["h2d_gbs"] * 1e9)
    t_d2h = e2e["d2h_bytes_per_step"] / (rates["d2h_gbs"] * 1e9)
    bound_ms = max(t_h2d, t_d2h) * 1e3
    e2e["link"] = {"h2d_gbs": rates["h2d_gbs"], "d2h_gbs": rates["d2h_gbs"], "how": rates["how"],
                   "bound_ms_per_step": bound_ms, "frac": bound_ms / e2e["ms_per_step"],
                   "note": "bound = the step's host->device bytes at the measured H2D rate, or its device->host "
                           "bytes at the D2H rate, whichever is longer (the two directions overlapping)"}
    return e2e


def e2e_record(d, st, steps, work, unit):
    """The e2e record: the step timed both ways (three steps in flight through
    the event API, and one step at a time), `work` units per step; the value is
    the faster way's, and the record names it and carries both."""
    dt_p, h2d, d2h, match_p = time_e2e(d, st, steps=steps, depth=3)
    dt_b, _, _, match_b = time_e2e(d, st, steps=steps, pipelined=False)
    modes = {"three_in_flight": {"value": work / dt_p, "unit": unit, "ms_per_step": dt_p * 1e3,
                                 "how": "cc_buf_upload_ev, cc_launch_ev, cc_buf_download_ev with wait lists, three "
                                        "steps in flight on their own device buffers"},
             "one_at_a_time": {"value": work / dt_b, "unit": unit, "ms_per_step": dt_b * 1e3,
                               "how": "cc_buf_upload_async, cc_launch, blocking cc_buf_download"}}
    best = min(modes, key=lambda k: modes[k]["ms_per_step"])
    return with_link_bound(d, {
        "value": modes[best]["value"], "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
        "ms_per_step": modes[best]["ms_per_step"], "mode": best, "modes": modes,
        "note": "every step uploads its inputs from pinned host memory and reads its result back inside the "
                "timed region",
        "results_match": bool(match_p and match_b)})


def time_e2e_batch(d, b, progs, nbytes, steps):
    """The batch through the C ABI with host buffers, every step: every input
    uploaded from pinned memory, one persistent launch, every output read back.
    Timed both ways, the value being the faster's:
      two_in_flight: cc_batch_upload_ev / cc_batch_run_ev / cc_batch_download_ev
        with wait lists (uploads after the previous run, the run after them and
        the previous step's reads), a step's reads overlapping the next step's
        uploads, each step reading into its own host buffers;
      one_at_a_time: a non-blocking upload per input, the run, a non-blocking
        read per output, one synchronisation."""
    import ctypes
    import numpy as np
    from compute._native import call
    rt = d.runtime
    # bound inputs: per program its parameters in the program's order
    bufs = [prm._cached for ser in b.serialized for prm in ser.params]
    pinned = []

    def host(nb):
        ptr = ctypes.c_void_p()
        call("cc_host_alloc", ctypes.c_size_t(max(16, nb)), ctypes.byref(ptr))
        pinned.append(ptr)
        return ptr

    hosts = []
    h2d = 0
    for buf in bufs:
        ptr = host(buf.nbytes)
        ctypes.memmove(ptr, rt.download(buf, buf.nbytes // 4).ctypes.data, buf.nbytes)
        hosts.append(ptr)
        h2d += buf.nbytes
    outs = [[host(out.nbytes) for out in b.outputs] for _ in range(2)]
    d2h = sum(out.nbytes for out in b.outputs)

    def one_at_a_time():
        for ptr, buf in zip(hosts, bufs):
            call("cc_buf_upload_async", ctypes.c_uint64(buf.handle), ctypes.c_size_t(0), ptr,
                 ctypes.c_size_t(buf.nbytes))
        b.run(0)
        for ptr, out in zip(outs[0], b.outputs):
            call("cc_buf_download_async", ctypes.c_uint64(out.handle), ctypes.c_size_t(0), ptr,
                 ctypes.c_size_t(out.nbytes))
        call("cc_synchronize")

    host_in = [p.value for p in hosts]
    host_out = [[p.value for p in o] for o in outs]

    def two_in_flight(n_steps):
        prev_run = prev_read = None
        pending = []
        for k in range(n_steps):
            up = b.upload_ev(host_in, wait=[prev_run] if prev_run else [])
            run = b.run_ev(0, wait=[up] + ([prev_read] if prev_read else []))
            read = b.download_ev(host_out[k % 2], wait=[run])
            rt.event_release(up)
            if prev_run:
                rt.event_release(prev_run)
            prev_run, prev_read = run, read
            pending.append(read)
            if len(pending) >= 2:  # the step whose host buffers come round next: its results are read
                e = pending.pop(0)
                rt.event_wait(e, 600 * 10 ** 9)
                rt.event_release(e)
        for e in pending:
            rt.event_wait(e, 600 * 10 ** 9)
            rt.event_release(e)
        if prev_run:
            rt.event_release(prev_run)

    def timed(fn):
        fn(2)  # both host output sets seen once (the copy tables are built on first use)
        t0 = time.perf_counter()
        fn(steps)
        return (time.perf_counter() - t0) / steps

    try:
        dt_b = timed(lambda n: [one_at_a_time() for _ in range(n)])
        want = [np.ctypeslib.as_array((ctypes.c_float * (o.nbytes // 4)).from_address(p.value)).copy()
                for p, o in zip(outs[0], b.outputs)]
        dt_p = timed(two_in_flight)
        match = all(np.array_equal(np.ctypeslib.as_array((ctypes.c_float * (o.nbytes // 4)).from_address(p.value))
                                   .view(np.int32), w.view(np.int32))
                    for slot in outs for p, o, w in zip(slot, b.outputs, want))
    finally:
        rt.synchronize()
        for ptr in pinned:
            call("cc_host_free", ptr)
    copier = "one SM copy kernel over a table of the copies" if rt.config_get("batch_copy_kernel") else \
        "the DMA engines, one copy per buffer over four streams"
    modes = {"two_in_flight": {"value": nbytes / dt_p / 1e9, "unit": "GB/s", "ms_per_step": dt_p * 1e3,
                               "how": "cc_batch_upload_ev, cc_batch_run_ev, cc_batch_download_ev with wait lists; "
                                      "copies by " + copier},
             "one_at_a_time": {"value": nbytes / dt_b / 1e9, "unit": "GB/s", "ms_per_step": dt_b * 1e3,
                               "how": "cc_buf_upload_async per input, cc_batch_run, cc_buf_download_async per "
                                      "output, cc_synchronize"}}
    best = min(modes, key=lambda k: modes[k]["ms_per_step"])
    return with_link_bound(d, {
        "value": modes[best]["value"], "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
        "ms_per_step": modes[best]["ms_per_step"], "mode": best, "modes": modes,
        "note": "every step uploads its inputs from pinned host memory and reads every output back inside "
                "the timed region",
        "results_match": bool(match)})


_KNOBS = []


def emit(line):
    """Prints the result line; runtime settings changed by --knob are recorded in its config."""
    if _KNOBS and isinstance(line.get("config"), dict):
        line["config"]["knobs"] = list(_KNOBS)
    print(json.dumps(line), flush=True)


def arm_workload(workload):
    """The `config.workload` string of a workload, shared by both arms."""
    if workload == "c2":
        n = C2["n"]
        return ("view-heavy fused op: x[%d,128,56,56] permute->+bias[128]->max0"
                "->translate W+1->channel sum [%d,56,56]") % (n, n)
    if workload == "c1":
        return "fused elementwise+sum: ((a*b+c).tanh).sum, a,b,c [%d,%d] U[-1,1]" % (C1["n"], C1["m"])
    if workload == "c6":
        return ("3x3 convolution via translate/split/join: x[128,32,32,8] NHWC ~N(0,1), "
                "weight[3,3,8,8], bias[8] -> [128,32,32,8]")
    if workload in C3:
        m, k, n = C3[workload]
        return "contraction via broadcast+split(1).reduce: A[%d,%d] x B[%d,%d] ~ N(0,1)" % (m, k, k, n)
    if workload == "c7":
        return "inner-axis sum: x[%d,%d] ~ N(0,1) .split(1).reduce(_+_) -> [%d]" % (C7["rows"], C7["cols"], C7["rows"])
    raise SystemExit("unknown workload " + workload)


def apply_knobs(rt, knobs):
    _KNOBS[:] = list(knobs)
    for kv in knobs:
        k, v = kv.split("=", 1)
        rt.config_set(k, int(v))


def max_over_ranks(dist, value: float) -> float:
    """The largest of every rank's value (the replicas' slowest timing)."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_reference(workload, budget_s=15.0, threads=None, contract="off"):
    """Times the reference's CPU implementation (the oracle's C restatement of the
    generated OpenCL C, OpenMP over all host threads) on a bounded sample;
    ``contract`` is gcc's -ffp-contract mode for the generated C."""
    from oracle import cref
    if contract != "off":
        return cref.time_workload(workload, budget_s=budget_s, threads=threads, contract=contract)
    if workload == "c7":
        R, J = 1024, C7["cols"]

        def make_fold(T):
            x = T.randomNormal([R, J], seed=C3_SEED).doCache()
            return x.split(1).reduce(lambda a, b: a + b)

        r = cref.time_expression(make_fold, 4 * (R * J + R), budget_s=budget_s, threads=threads)
        r["config"] = {"workload": "inner-axis sum (reference CPU path, OpenCL C on host cores)"}
        r["sample"] = ("x[%d,%d] (%d of %d rows), %d reps; one work item per output, its %d-term fold of "
                       "split views" % (R, J, R, C7["rows"], r["reps"], J))
        return r
    if workload == "c6":
        n, h, w, c, k = C6["n"], C6["h"], C6["w"], C6["c"], C6["k"]

        def make(T):
            x = T.randomNormal([n, h, w, c], seed=C3_SEED).doCache()
            weight = T.randomNormal([k, k, c, c], seed=C3_SEED + 1).doCache()
            bias = T.randomNormal([c], seed=C3_SEED + 2).doCache()
            return conv_expr(T, x, weight, bias)

        r = cref.time_expression(make, 2 * n * h * w * c * 4 + k * k * c * c * 4 + c * 4, budget_s=budget_s,
                                 threads=threads)
        r["config"] = {"workload": "3x3 convolution (reference CPU path, OpenCL C on host cores)"}
        r["sample"] = "full workload, %d reps; one kernel joins the 8 filters, 576 loads per point" % r["reps"]
        return r
    return cref.time_workload(workload, budget_s=budget_s, threads=threads)


# ------------------------------------------------------------------ main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c3s", "c4", "c5", "c6", "c7"])
    ap.add_argument("--programs", type=int, default=2048,
                    help="c4: programs in the batch; c5: tuning workloads to time (the last 10%% held out)")
    ap.add_argument("--max-len", type=int, default=4194304, help="c4: longest program (lengths log-uniform from 1024)")
    ap.add_argument("--c1-side", type=int, default=1024, help="c1: side of the square inputs (1024 = the benchmark)")
    ap.add_argument("--c2-batch", type=int, default=64, help="c2: images in x (64 = the benchmark)")
    ap.add_argument("--db", default=None, help="c5: append the timing records (JSON lines) to this file")
    ap.add_argument("--collect-budget-s", type=float, default=None, help="c5: stop collecting after this long")
    ap.add_argument("--db-in", default=None, help="c5: train and evaluate on these timing records instead of timing")
    ap.add_argument("--save-model", default=None, help="c5: write the trained cost model (.npz) here")
    ap.add_argument("--epochs", type=int, default=40, help="c5: training epochs")
    ap.add_argument("--seed", type=int, default=0, help="c5: seed of the generated tuning workloads")
    ap.add_argument("--eval-model", default=None,
                    help="c5: evaluate this trained model (.npz) on all timed programs instead of training one")
    ap.add_argument("--knob", action="append", default=[], metavar="KEY=VALUE",
                    help="runtime setting (cc_config_set) applied before the run; repeatable")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-clocks", action="store_true", help="skip the clock sampling (and its untimed busy loop)")
    ap.add_argument("--tuner", default="learned", choices=["off", "exhaustive", "learned"],
                    help="launch configurations (the device object's setting): the shipped cost model's choice "
                         "timed against the standard kernel at a program's first launch (learned, the default), "
                         "every configuration timed (exhaustive), or the standard kernels (off)")
    ap.add_argument("--no-workloads", action="store_true",
                    help="default workload only: skip the records of the other configurations")
    ap.add_argument("--c5-eval-programs", type=int, default=400,
                    help="tuning workloads the shipped cost model is evaluated on in the default run")
    args = ap.parse_args()
    warmup = max(3, args.warmup)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    metric = "fused-op GB/s"
    if args.workload in C3:
        return main_contraction(args, warmup, rank, world, local_rank)
    if args.workload == "c4":
        return main_batch(args, warmup, rank, world, local_rank)
    if args.workload == "c5":
        return main_tuner(args, warmup, rank, world, local_rank)

    if args.impl == "reference":
        if rank != 0:
            return
        r = cpu_reference(args.workload)
        config = dict(r["config"], workload=arm_workload(args.workload), path=r["config"]["workload"])
        line = {"impl": "reference", "metric": metric, "value": r["gbs"], "unit": "GB/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded reference RNG)",
                "config": config,
                "cpu_baseline": {"value": r["gbs"], "unit": "GB/s", "cores": r["threads"], "kind": "port",
                                 "sample": r["sample"]},
                "e2e": {"value": r["gbs"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        emit(line)
        return

    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo", init_method="env://")
        dist = dist_mod

    from compute import Tensors
    d = Tensors(device=local_rank, tuner=args.tuner)
    rt = d.runtime
    apply_knobs(rt, args.knob)
    if args.workload == "c1":
        C1["n"] = C1["m"] = args.c1_side
    if args.workload == "c2":
        C2["n"] = args.c2_batch
    line = measure_fused(d, args.workload, args.steps, warmup, rank=rank, world=world, local_rank=local_rank,
                         dist=dist, e2e_on=not args.no_e2e, cpu_on=rank == 0 and not args.no_cpu_baseline,
                         clocks_on=not args.no_clocks)
    if rank == 0 and world == 1 and args.workload == "c2" and not args.no_workloads:
        line["workloads"] = measure_all_configs(d, args, warmup, local_rank)
    line["config"]["tuner"] = args.tuner
    if rank == 0:
        emit(line)
    if dist:
        dist.destroy_process_group()


def measure_fused(d, workload, steps, warmup, rank=0, world=1, local_rank=0, dist=None, e2e_on=True, cpu_on=True,
                  clocks_on=True, cpu_budget_s=12.0):
    """One fused-op workload (c1, c2, c6): the result line, without printing it."""
    rt = d.runtime
    st = setup(workload, d)
    sampler = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    rt.synchronize()
    if clocks_on:
        sampler.start()
    ms_total = time_device(rt, st, steps, warmup)
    clocks = None
    if clocks_on:
        keep_busy(rt, st, 1.5)
        clocks = sampler.stop()
    if dist:
        ms_total = max_over_ranks(dist, ms_total)
        dist.barrier()
    ms_step = ms_total / steps
    gbs_step = st["bytes"] / (ms_step * 1e-3) / 1e9
    value = gbs_step * world
    # the same launches on one input set, which then stays in L2 (reported beside, never as the value)
    hot_ms = time_device(rt, dict(st, sets=st["sets"][:1]), steps, warmup) / steps
    hot = {"value": st["bytes"] / (hot_ms * 1e-3) / 1e9, "unit": "GB/s", "ms_per_step": hot_ms}
    iso_ms = time_isolated(rt, st, 50)
    overlap = {"pdl": rt.config_get("pdl") == 1,
               "rule": "programmatic dependent launch: a launch whose inputs do not overlap the previous "
                       "kernel's output issues its loads while that kernel drains; its stores wait for it",
               "isolated_launch": {"value": st["bytes"] / (iso_ms * 1e-3) / 1e9, "unit": "GB/s",
                                   "ms": iso_ms, "note": "one launch between two synchronisations, median of 50"}}
    e2e = None
    if e2e_on:
        n_e2e = max(3, min(steps, 20))
        e2e = e2e_record(d, st, n_e2e, st["bytes"] / 1e9 * world, "GB/s")
    peak, peak_kind = _peaks()
    roofline = {"bound": "hbm", "achieved": gbs_step, "peak": peak, "unit": "GB/s", "frac": gbs_step / peak,
                "traffic": _traffic(workload), "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": st["bytes"]}
    cpu = cpu_fast = None
    if cpu_on:
        try:
            r = cpu_reference(workload, budget_s=cpu_budget_s)
            cpu = {"value": r["gbs"], "unit": "GB/s", "cores": r["threads"], "kind": "port", "sample": r["sample"],
                   "fp_contract": "off"}
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": "GB/s", "cores": None, "kind": "port", "sample": "failed: %s" % e}
        if workload in ("c1", "c2"):
            try:
                r = cpu_reference(workload, budget_s=cpu_budget_s / 2, contract="fast")
                cpu_fast = {"value": r["gbs"], "unit": "GB/s", "cores": r["threads"], "kind": "port",
                            "sample": r["sample"], "fp_contract": "fast"}
            except Exception as e:
                cpu_fast = {"value": None, "unit": "GB/s", "sample": "failed: %s" % e, "fp_contract": "fast"}
    line = {"metric": "fused-op GB/s", "value": value, "unit": "GB/s", "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded reference RNG)",
            "config": dict(st["config"], parallelism="replicas" if world > 1 else "single GPU"),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": steps,
            "clocks": clocks, "hot_l2": hot, "launch_overlap": overlap}
    if cpu_fast is not None:
        line["cpu_baseline_fp_contract_fast"] = cpu_fast
    if workload == "c1":
        floor_ms = launch_floor(d, steps, warmup)
        bytes_ms = st["bytes"] / (peak * 1e9) * 1e3
        line["launch_floor"] = {
            "ms": floor_ms, "note": "the same kernel on 4 points (one block), back to back",
            "bound_ms": bytes_ms + floor_ms, "frac_of_bound": (bytes_ms + floor_ms) / ms_step,
            "bound_note": "algorithmic bytes at the measured HBM peak plus the per-launch floor"}
    release(st)
    return line


def measure_all_configs(d, args, warmup, local_rank):
    """Every other configuration of the benchmark, each as its own record (value,
    roofline, cpu_baseline, e2e and clocks): the fused elementwise+sum, both
    contractions, the batched programs and the shipped cost model on programs it
    has not seen.  A configuration that fails records its error instead."""
    out = {}
    rt = d.runtime

    def attempt(name, fn):
        t0 = time.time()
        try:
            rec = fn()
        except Exception as e:  # one configuration's failure does not hide the others
            rec = {"error": "%s: %s" % (type(e).__name__, e)}
        rec["wall_s"] = round(time.time() - t0, 1)
        out[name] = rec
        rt.synchronize()

    attempt("c1", lambda: measure_fused(d, "c1", args.steps, warmup, local_rank=local_rank, cpu_budget_s=6.0,
                                        clocks_on=not args.no_clocks))
    attempt("c7", lambda: measure_fused(d, "c7", min(args.steps, 50), warmup, local_rank=local_rank,
                                        cpu_budget_s=6.0, clocks_on=not args.no_clocks))
    for w in ("c3", "c3s"):
        attempt(w, lambda w=w: measure_contraction(d, w, 20, warmup, local_rank=local_rank, cpu_budget_s=6.0,
                                                   clocks_on=not args.no_clocks))
    attempt("c4", lambda: measure_batch(d, 2048, 4194304, 20, warmup, local_rank=local_rank, cpu_budget_s=6.0,
                                        clocks_on=not args.no_clocks))
    attempt("c5_eval", lambda: measure_tuner_eval(rt, args.c5_eval_programs, 1, SHIPPED_MODEL))
    return out


SHIPPED_MODEL = os.path.join(ROOT, "compute.scala_gb300", "compute", "costmodel_gb300.npz")


def measure_tuner_eval(rt, programs, seed, model_path):
    """The shipped cost model on tuning workloads it was not trained on: every
    program timed in all 48 configurations (exhaustive), the model's pick, the
    fixed default and the best fixed configuration compared with the best."""
    from compute import tuner
    sm = rt.device_info()["sm_count"]
    t0 = time.time()
    progs = tuner.random_programs(programs, seed=seed)
    recs = tuner.collect(rt, progs, reps=5, flush_l2=True, standard=True)
    collect_s = time.time() - t0
    model = tuner.CostModel(rt, seed=0)
    try:
        model.load(model_path)
        res = tuner.evaluate(model, recs, sm, fixed=30)
    finally:
        model.close()
    return {"metric": "learned-tuner regret (geometric-mean slowdown vs exhaustive best), shipped model on "
                      "unseen programs",
            "value": res["learned"]["geomean_slowdown"], "unit": "fraction", "n_gpus": 1, "steps": 0,
            "warmup": 0, "ms_per_step": None, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded tuning workloads, seed %d)" % seed,
            "config": {"workload": "tuning workloads as c5, %d programs, all evaluated" % len(recs),
                       "model": os.path.relpath(model_path, ROOT),
                       "timing": "median of 5 launches per config, L2 flushed"},
            "tuner": res, "seconds": {"compile_and_time": round(collect_s, 1)},
            "roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": None}


def main_tuner(args, warmup, rank, world, local_rank):
    """C5: the exhaustive tuner times every configuration of seeded tuning
    workloads; the cost model trains on the first 90% of programs (its own CUDA
    kernels) and picks configurations for the held-out 10%.  The value is the
    held-out geometric-mean slowdown of the learned pick against the exhaustive
    best (0 = always the best); the default configuration's and the best single
    fixed configuration's figures are reported beside it."""
    if rank != 0:
        return
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no tuner (the OpenCL runtime picks "
                          "its local size)"}), flush=True)
        return
    from compute.runtime import NativeRuntime
    from compute import tuner
    rt = NativeRuntime(local_rank)
    apply_knobs(rt, args.knob)
    sm = rt.device_info()["sm_count"]
    if args.eval_model and not args.db_in:
        line = measure_tuner_eval(rt, args.programs, args.seed, args.eval_model)
        emit(line)
        return
    t0 = time.time()
    if args.db_in:
        recs = [json.loads(line) for line in open(args.db_in)][:args.programs]
        gen_s = 0.0
        collect_s = 0.0
    else:
        progs = tuner.random_programs(args.programs, seed=args.seed)
        gen_s = time.time() - t0
        log = open(args.db, "a") if args.db else None
        t0 = time.time()
        try:
            recs = tuner.collect(rt, progs, reps=5, flush_l2=True, log=log, time_budget_s=args.collect_budget_s)
        finally:
            if log:
                log.close()
        collect_s = time.time() - t0
    if args.eval_model:
        model = tuner.CostModel(rt, seed=0)
        model.load(args.eval_model)
        res = tuner.evaluate(model, recs, sm, fixed=30)
        model.close()
        line = {"metric": "learned-tuner regret (geometric-mean slowdown vs exhaustive best), trained model on "
                          "recorded programs",
                "value": res["learned"]["geomean_slowdown"], "unit": "fraction", "n_gpus": 1, "steps": 0,
                "warmup": 0, "ms_per_step": None, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "recorded timings (%s)" % args.db_in,
                "config": {"workload": "tuning workloads as c5, %d programs evaluated" % len(recs),
                           "model": args.eval_model},
                "tuner": res, "roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": None,
                "clocks": None}
        emit(line)
        return
    split = int(len(recs) * 0.9)
    train, test = recs[:split], recs[split:]
    x, y = tuner.training_arrays(train, sm)
    model = tuner.CostModel(rt, seed=0)
    t0 = time.time()
    losses = model.fit(x, y, epochs=args.epochs, batch=4096, lr=2e-3, lr_final=1e-4)
    rt.synchronize()
    train_s = time.time() - t0
    steps = args.epochs * max(1, x.shape[0] // 4096)
    if args.save_model:
        model.save(args.save_model)
    fixed = tuner.best_fixed_config(train)
    res = tuner.evaluate(model, test, sm, fixed=fixed)
    xt = tuner.feature_matrix([r["ir"] for r in test], sm)
    t0 = time.time()
    model.predict(xt)
    predict_s = time.time() - t0
    kinds = {}
    for r in recs:
        kinds[r["kind"]] = kinds.get(r["kind"], 0) + 1
    line = {"metric": "learned-tuner regret (held-out geometric-mean slowdown vs exhaustive best)",
            "value": res["learned"]["geomean_slowdown"], "unit": "fraction", "n_gpus": 1, "steps": steps,
            "warmup": 0, "ms_per_step": train_s * 1e3 / steps, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tuning workloads)",
            "config": {"workload": "tuning workloads: rank 1-4, dims 1-4096, <= 64M points, inputs through "
                                   "random permute/broadcast/translate views, 3-12-node trees over "
                                   "+,-,*,/,exp,log,tanh,max, optional full or inner-axis sum; 48 configs each",
                       "programs_timed": len(recs), "train": len(train), "held_out": len(test), "kinds": kinds,
                       "timing": "median of 5 launches per config, L2 flushed (256 MiB write) before each",
                       "model": "MLP 64-256-256-256-1 ReLU, Adam, %d epochs, batch 4096, own CUDA kernels" % args.epochs,
                       "timings_from": args.db_in or "collected in this run"},
            "tuner": res, "train_loss_first_last": [losses[0], losses[-1]],
            "seconds": {"generate": round(gen_s, 1), "compile_and_time": round(collect_s, 1),
                        "train": round(train_s, 2), "predict_held_out": round(predict_s, 3)},
            "roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": None}
    emit(line)
    model.close()


def measure_batch(d, programs, max_len, steps, warmup, local_rank=0, e2e_on=True, cpu_on=True, clocks_on=True,
                  cpu_budget_s=12.0, world=1):
    """The batched-programs workload: `programs` independent fused programs
    evaluated by one persistent launch; the same programs launched one by one,
    and replayed from a CUDA graph, are the comparison."""
    from compute.batch import Batch
    rt = d.runtime
    T = d.Tensor
    t0 = time.time()
    progs = c4_programs(T, seed=0, count=programs, hi=max_len)
    tensors = [t for t, _ in progs]
    b = Batch(d, tensors).bind()
    setup_s = time.time() - t0
    nbytes = 0
    for t, ser in zip(tensors, b.serialized):
        n = 1
        for s_ in t.shape:
            n *= s_
        nbytes += 4 * n * (len(ser.params) + 1)
    n_progs, n_structs, regs, resident = rt.batch_info(b.handle)

    def timed(mode, k):
        for _ in range(max(3, warmup)):
            b.run(mode)
        rt.synchronize()
        e0 = rt.event()
        for _ in range(k):
            b.run(mode)
        e1 = rt.event()
        rt.event_wait(e1, 600 * 10 ** 9)
        ms = rt.event_elapsed_ms(e0, e1) / k
        rt.event_release(e0)
        rt.event_release(e1)
        return ms

    sampler = ClockSampler(local_rank)
    if clocks_on:
        sampler.start()
    ms_persistent = timed(Batch.PERSISTENT, steps)
    clocks = None
    if clocks_on:
        t_end = time.time() + 1.5
        while time.time() < t_end:
            b.run(Batch.PERSISTENT)
            rt.synchronize()
        clocks = sampler.stop()
    k2 = max(3, min(steps, 20))
    ms_each = timed(Batch.PER_PROGRAM, k2)
    ms_graph = timed(Batch.GRAPH, k2)
    gbs = nbytes / (ms_persistent * 1e-3) / 1e9
    e2e = None
    if e2e_on:
        e2e = time_e2e_batch(d, b, progs, nbytes, steps=3)
    cpu = None
    if cpu_on:
        try:
            from oracle import cref
            r = cref.time_programs(lambda T_: c4_programs(T_, seed=0, count=48, hi=max_len), budget_s=cpu_budget_s)
            cpu = {"value": r["gbs"], "unit": "GB/s", "cores": r["threads"], "kind": "port", "sample": r["sample"]}
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": "GB/s", "cores": None, "kind": "port", "sample": "failed: %s" % e}
    peak, peak_kind = _peaks()
    line = {"metric": "fused-op GB/s", "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": ms_persistent, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded reference RNG)",
            "config": {"workload": "batched uneven programs: %d random fused programs (3-12 nodes over "
                                   "+,-,*,/,exp,log,tanh,max; 1-4 inputs U[0.1,2]), lengths log-uniform [1K,%d]"
                                   % (programs, max_len),
                       "programs": n_progs, "distinct_structures": n_structs, "bytes_per_step": nbytes,
                       "persistent_registers": regs, "persistent_blocks_per_sm": resident,
                       "l2": "inputs %.1f GB > L2" % (nbytes / 1e9), "setup_s": round(setup_s, 1),
                       "parallelism": "single GPU"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "traffic": _traffic("c4"), "peak_source": peak_kind, "algorithmic_bytes_per_launch": nbytes},
            "batch": {"persistent_ms": ms_persistent, "per_program_ms": ms_each, "graph_ms": ms_graph,
                      "speedup_vs_per_program": ms_each / ms_persistent, "speedup_vs_graph": ms_graph / ms_persistent},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": steps, "clocks": clocks}
    b.close()
    for _, inputs in progs:
        for i in inputs:
            i.close()
    return line


def main_batch(args, warmup, rank, world, local_rank):
    from compute import Tensors
    d = Tensors(device=local_rank, tuner=args.tuner)
    apply_knobs(d.runtime, args.knob)
    line = measure_batch(d, args.programs, args.max_len, args.steps, warmup, local_rank=local_rank,
                         e2e_on=not args.no_e2e, cpu_on=not args.no_cpu_baseline, clocks_on=not args.no_clocks,
                         world=world)
    emit(line)


def measure_contraction(d, workload, steps, warmup, local_rank=0, e2e_on=True, cpu_on=True, clocks_on=True,
                        cpu_budget_s=10.0, world=1):
    """A contraction workload: TFLOP/s (2*M*N*K per step, counted once) of the
    split-BF16 tensor-core path, reached through the Tensor API's matmul idiom."""
    rt = d.runtime
    saved = rt.config_get("contraction")
    st = setup(workload, d)
    try:
        sampler = ClockSampler(local_rank)
        rt.synchronize()
        if clocks_on:
            sampler.start()
        ms_total = time_device(rt, st, steps, warmup)
        clocks = None
        if clocks_on:
            keep_busy(rt, st, 1.5)
            clocks = sampler.stop()
        ms_step = ms_total / steps
        tflops = st["flops"] / (ms_step * 1e-3) / 1e12
        extras = contraction_extras(d, st)
        e2e = None
        if e2e_on:
            e2e = e2e_record(d, st, max(3, min(steps, 12)), st["flops"] / 1e12, "TFLOP/s")
    finally:
        release(st)
        rt.config_set("contraction", saved)
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        peak, peak_kind = float(peaks["bf16_tflops"]), "measured"
        sustained = float(peaks.get("bf16_tflops_sustained", peak))
    except Exception:
        peak, peak_kind, sustained = 1900.0, "fallback", 1700.0
    roofline = {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                "traffic": _traffic(workload), "peak_source": peak_kind,
                "tensor_work_frac": 6 * tflops / peak,
                "tensor_work_frac_of_sustained": 6 * tflops / sustained,
                "note": "achieved counts 2*M*N*K once; the tensor cores execute 6 bf16 products per output term; "
                        "peak is the burst BF16 rate, the loop runs under the power cap (sustained rate %.1f)"
                        % sustained}
    cpu = None
    if cpu_on:
        try:
            from oracle import cref
            r = cref.time_contraction(C3[workload], budget_s=cpu_budget_s)
            cpu = {"value": r["tflops"], "unit": "TFLOP/s", "cores": r["threads"], "kind": "port", "sample": r["sample"]}
        except Exception as e:
            cpu = {"value": None, "unit": "TFLOP/s", "cores": None, "kind": "port", "sample": "failed: %s" % e}
    return {"metric": "matmul TFLOP/s", "value": tflops, "unit": "TFLOP/s", "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3 split of f32 (fp32 accumulate)",
            "data": "synthetic (seeded reference RNG)",
            "config": dict(st["config"], parallelism="single GPU"), "roofline": roofline, "accuracy": extras,
            "speedup_vs_fp32_cuda_core": tflops / extras["fp32_cuda_core_tflops"],
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": steps * 3, "clocks": clocks}


def main_contraction(args, warmup, rank, world, local_rank):
    metric = "matmul TFLOP/s"
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import cref
        r = cref.time_contraction(C3[args.workload])
        config = dict(r["config"], workload=arm_workload(args.workload), path=r["config"]["workload"])
        line = {"impl": "reference", "metric": metric, "value": r["tflops"], "unit": "TFLOP/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded reference RNG)",
                "config": config,
                "cpu_baseline": {"value": r["tflops"], "unit": "TFLOP/s", "cores": r["threads"], "kind": "port",
                                 "sample": r["sample"]},
                "e2e": {"value": r["tflops"], "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        emit(line)
        return
    from compute import Tensors
    d = Tensors(device=local_rank, tuner=args.tuner)
    apply_knobs(d.runtime, args.knob)
    line = measure_contraction(d, args.workload, args.steps, warmup, local_rank=local_rank, e2e_on=not args.no_e2e,
                               cpu_on=not args.no_cpu_baseline, clocks_on=not args.no_clocks, world=world)
    emit(line)


if __name__ == "__main__":
    main()

"""The asynchronous DAG: launches and copies on a pool of streams, ordered only
by event wait lists.

The reference enqueues every kernel on a queue of its CommandQueuePool with the
events of the buffers it reads as its wait list (Kernel.enqueue, OpenCL.scala:
787-844, dispatch :1298-1329; CompiledKernel.run, Tensors.scala:1331-1381), so
independent subgraphs run concurrently and a kernel starts once its inputs
exist.  Here the *_ev entry points do the same over eight CUDA streams; these
tests check that such graphs compute the oracle's bits, that the chains of a
graph really overlap, and that buffers released while other streams may still
use them are not reused too early.
"""

import ctypes
import time

import numpy as np
import pytest

from compute import _native

pytestmark = pytest.mark.gpu


def _queued():
    from conftest import cuda_tensors
    return cuda_tensors(queues=True)


def _oracle():
    from compute import Tensors
    from oracle_runtime import OracleRuntime
    return Tensors(runtime=OracleRuntime())


def test_computational_graph_of_cpu_spec():
    """cpuSpec.scala:9-16: a and b are independent kernels, c waits for both, d for c and b."""
    d = _queued()
    T = d.Tensor
    a = T.fill(2.0, [2, 3]).nonInline()
    b = T.fill(2.0, [2, 3]).nonInline()
    c = (a + b).nonInline()
    e = (c + b).nonInline()
    assert e.toString() == "[[6.0,6.0,6.0],[6.0,6.0,6.0]]"


def _two_chains(dev, n, depth):
    T = dev.Tensor
    x = T.random([n, 64], seed=31)  # uniform: the oracle's random numbers are the device's bits
    y = T.random([n, 64], seed=32) - T.fill(0.5, [n, 64])
    cx, cy = x, y
    for k in range(depth):
        cx = (T.abs(cx) * T.fill(-1.5, [n, 64]) + T.fill(0.25, [n, 64])).nonInline()
        cy = (cy * T.fill(0.5, [n, 64]) - T.fill(1.0, [n, 64])).nonInline()
        if k % 3 == 2:
            cx = cx.transpose().transpose().translate([1, 0]).nonInline()  # a view kernel in the chain
    joined = (cx * cy + cx).nonInline()
    return joined, (cx - cy).sum()


def test_independent_chains_joined_by_wait_lists_match_the_oracle():
    """Two chains of nonInline kernels (no transcendentals: every statement is
    correctly rounded on both sides) that share nothing until the end run on
    different queues; the kernel that joins them waits for both.  Elementwise
    results are the oracle's bits; the final sum (on a queue, with that queue's
    own partials) is within sqrt(n) * 2^-24 of the oracle's."""
    from conftest import cuda_tensors
    got_t, got_s = _two_chains(_queued(), 4096, 9)
    want_t, want_s = _two_chains(_oracle(), 4096, 9)
    g, w = got_t.flatArray(), want_t.flatArray()
    assert np.array_equal(g.view(np.int32), w.view(np.int32))
    one_stream = _two_chains(cuda_tensors(), 4096, 9)[0].flatArray()
    assert np.array_equal(g.view(np.int32), one_stream.view(np.int32))
    s_dev, s_ref = got_s.readScalar(), want_s.readScalar()
    n = 4096 * 64
    assert abs(s_dev - s_ref) <= np.sqrt(n) * 2.0 ** -24 * max(1.0, abs(s_ref)) * 4


def test_events_and_wait_lists_through_the_c_abi():
    """Two chains of uploads and launches on the queue pool, joined by one
    launch that waits for both, read back by a download that waits for it."""
    from compute.tensors import NonInlineTensor
    d = _queued()
    rt = d.runtime
    T = d.Tensor
    n = 1 << 20
    p = NonInlineTensor(d, (n,), 0.0, None)
    q = NonInlineTensor(d, (n,), 0.0, None)
    step = rt.program(d.serialize((p * T.fill(3.0, [n]) + T.fill(1.0, [n])).closure, (n,)).text)
    join = rt.program(d.serialize((p - q).closure, (n,)).text)
    r = np.random.RandomState(5)
    ha = r.uniform(-1, 1, n).astype(np.float32)
    hb = r.uniform(-1, 1, n).astype(np.float32)
    A, B, A2, B2, C = (rt.alloc(4 * n) for _ in range(5))
    evs = []
    ea = rt.upload_ev(A, ha.ctypes.data, 4 * n)
    eb = rt.upload_ev(B, hb.ctypes.data, 4 * n)
    evs += [ea, eb]
    cur_a, cur_b, nxt_a, nxt_b = A, B, A2, B2
    for _ in range(6):
        ea = rt.launch_ev(step, [cur_a], nxt_a, [ea])
        eb = rt.launch_ev(step, [cur_b], nxt_b, [eb])
        evs += [ea, eb]
        cur_a, nxt_a = nxt_a, cur_a
        cur_b, nxt_b = nxt_b, cur_b
    ej = rt.launch_ev(join, [cur_a, cur_b], C, [ea, eb])
    out = np.empty(n, np.float32)
    ed = rt.download_ev(C, out.ctypes.data, 4 * n, wait=[ej])
    rt.event_wait(ed, 60 * 10 ** 9)
    assert rt.event_query(ed) and rt.event_query(ej)
    wa, wb = ha.copy(), hb.copy()
    for _ in range(6):
        wa = (wa * np.float32(3.0)).astype(np.float32) + np.float32(1.0)
        wb = (wb * np.float32(3.0)).astype(np.float32) + np.float32(1.0)
    want = (wa - wb).astype(np.float32)
    assert np.array_equal(out.view(np.int32), want.view(np.int32))
    for e in evs + [ej, ed]:
        rt.event_release(e)
    for b in (A, B, A2, B2, C):
        b.release()
    rt.synchronize()


def test_invalid_wait_handle_is_rejected_before_anything_is_enqueued():
    from compute.tensors import NonInlineTensor
    d = _queued()
    rt = d.runtime
    T = d.Tensor
    p = NonInlineTensor(d, (16,), 0.0, None)
    prog = rt.program(d.serialize((p + T.fill(1.0, [16])).closure, (16,)).text)
    a, o = rt.alloc(64), rt.alloc(64)
    with pytest.raises(_native.InvalidEvent):
        rt.launch_ev(prog, [a], o, [12345])
    a.release()
    o.release()


def test_chains_on_different_queues_overlap():
    """Two chains of launches ordered by their events, each launch a kernel of
    one block that runs long (an inner-axis fold of 4096 terms of tanh(x) per
    output, 64 outputs): independent, the chains take about as long as one;
    forced into one order by their wait lists, about twice as long."""
    from compute.tensors import NonInlineTensor
    d = _queued()
    rt = d.runtime
    T = d.Tensor
    rows, cols = 64, 4096
    p = NonInlineTensor(d, (rows, cols), 0.0, None)
    fold = T.tanh(p).split(1).reduce(lambda u, v: u + v)
    prog = rt.program(d.serialize(fold.closure, fold.shape).text)
    assert "cc_rowfold" in prog.source()
    x = rt.alloc(4 * rows * cols)
    rt.upload(x, np.random.RandomState(4).uniform(-1, 1, rows * cols).astype(np.float32))
    outs = [rt.alloc(4 * rows) for _ in range(2)]

    def run(independent, launches=6):
        rt.synchronize()
        t0 = time.perf_counter()
        ea = eb = None
        evs = []
        for k in range(launches):
            wait_a = [ea] if ea else []
            if not independent and eb:
                wait_a.append(eb)  # one order: a0, b0, a1, b1, ...
            ea = rt.launch_ev(prog, [x], outs[0], wait_a)
            wait_b = [eb] if eb else []
            if not independent:
                wait_b.append(ea)
            eb = rt.launch_ev(prog, [x], outs[1], wait_b)
            evs += [ea, eb]
        rt.event_wait(ea, 60 * 10 ** 9)
        rt.event_wait(eb, 60 * 10 ** 9)
        dt = time.perf_counter() - t0
        for ev in evs:
            rt.event_release(ev)
        return dt

    run(True)
    together = min(run(True) for _ in range(3))
    ordered = min(run(False) for _ in range(3))
    print("two independent chains %.3f ms, forced into one order %.3f ms" % (together * 1e3, ordered * 1e3))
    assert together < 0.8 * ordered
    a, b = rt.download(outs[0], rows), rt.download(outs[1], rows)
    assert np.array_equal(a.view(np.int32), b.view(np.int32))
    for buf in outs + [x]:
        buf.release()


def test_released_buffers_wait_for_every_stream_that_used_them():
    """A buffer read by a slow launch on one queue and released at once must not
    be handed out and overwritten before that launch has read it."""
    from compute.tensors import NonInlineTensor
    d = _queued()
    rt = d.runtime
    T = d.Tensor
    n = 1 << 24
    p = NonInlineTensor(d, (n,), 0.0, None)
    slow = rt.program(d.serialize(T.tanh(T.exp(T.tanh(p) * T.fill(0.5, [n]))).closure, (n,)).text)
    fill = rt.program(d.serialize((p * T.fill(0.0, [n]) + T.fill(7.0, [n])).closure, (n,)).text)
    src = np.random.RandomState(9).uniform(-1, 1, n).astype(np.float32)
    want = None
    for it in range(4):
        a, out = rt.alloc(4 * n), rt.alloc(4 * n)
        e0 = rt.upload_ev(a, src.ctypes.data, 4 * n)
        e1 = rt.launch_ev(slow, [a], out, [e0])
        a.release()  # still read by the launch behind e1
        b = rt.alloc(4 * n)  # must not be a's block while that launch may run
        e2 = rt.launch_ev(fill, [b], b, [])  # overwrites b on another queue at once
        res = np.empty(n, np.float32)
        e3 = rt.download_ev(out, res.ctypes.data, 4 * n, wait=[e1])
        rt.event_wait(e3, 60 * 10 ** 9)
        rt.event_wait(e2, 60 * 10 ** 9)
        if want is None:
            want = res.copy()
        assert np.array_equal(res.view(np.int32), want.view(np.int32)), it
        for e in (e0, e1, e2, e3):
            rt.event_release(e)
        b.release()
        out.release()
    rt.synchronize()
    stats = rt.pool_stats()
    assert stats["reuses"] > 0

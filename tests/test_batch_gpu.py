"""Batched evaluation: one persistent launch, per-program launches and a CUDA
graph of them all give the bits a single evaluation through the API gives."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_modes_agree_with_single_launches(cuda_device):
    import bench
    from compute.batch import Batch
    T = cuda_device.Tensor
    progs = bench.c4_programs(T, seed=3, count=40, lo=1, hi=70000)
    tensors = [t for t, _ in progs]
    single = [t.flatArray() for t in tensors]
    b = Batch(cuda_device, tensors).bind()
    for mode in (Batch.PERSISTENT, Batch.PER_PROGRAM, Batch.GRAPH, Batch.GRAPH, Batch.PERSISTENT):
        for out in b.outputs:
            cuda_device.runtime.upload(out, np.full(out.nbytes // 4, np.nan, np.float32))
        b.run(mode)
        for k, (t, want) in enumerate(zip(tensors, single)):
            got = cuda_device.runtime.download(b.outputs[k], want.size)
            assert np.array_equal(got.view(np.int32), want.view(np.int32)), (mode, k)
    n, structures, regs, resident = cuda_device.runtime.batch_info(b.handle)
    assert n == 40 and 1 <= structures <= 40
    b.close()
    for _, inputs in progs:
        for i in inputs:
            i.close()


@pytest.mark.parametrize("lanes,inline,rolled", [(0, 1, 0), (4, 1, 0), (8, 1, 0), (4, 0, 0), (8, 2, 0), (4, 1, 1),
                                                  (8, 1, 1)])
def test_batch_lane_widths_give_the_single_launch_bits(cuda_device, lanes, inline, rolled):
    """Tile functions evaluating 1, 4 or 8 points per call (and each inlining
    level) run the same per-point arithmetic: every program's output is the
    single launch's, bit for bit, ragged ends included."""
    import bench
    from compute.batch import Batch
    rt = cuda_device.runtime
    T = cuda_device.Tensor
    saved = {k: rt.config_get(k) for k in ("batch_lanes", "batch_inline", "batch_rolled", "batch_max_loads")}
    progs = bench.c4_programs(T, seed=11, count=24, lo=1, hi=40000)
    # and every other operator, through the lane helpers
    for k, n in enumerate((4099, 8192, 33)):
        a, b = (T.random([n], seed=900 + 2 * k + j) * T.fill(4.0, [n]) - T.fill(2.0, [n]) for j in (0, 1))
        a, b = a.doCache(), b.doCache()
        e = [T.abs(a - b) % (b + T.fill(3.0, [n])), -T.sqrt(T.abs(a)) * T.min(a, b),
             T.min(T.max(a, b), T.fill(0.5, [n])) / (T.abs(b) + T.fill(0.25, [n]))][k]
        progs.append((e, [a, b]))
    tensors = [t for t, _ in progs]
    single = [t.flatArray() for t in tensors]
    try:
        rt.config_set("batch_lanes", lanes)
        rt.config_set("batch_inline", inline)
        rt.config_set("batch_rolled", rolled)
        rt.config_set("batch_max_loads", 2 if rolled else 4)  # rolled: loops of one or two positions
        b = Batch(cuda_device, tensors).bind()
        b.run(Batch.PERSISTENT)
        for k, want in enumerate(single):
            got = rt.download(b.outputs[k], want.size)
            assert np.array_equal(got.view(np.int32), want.view(np.int32)), k
        b.close()
    finally:
        for k, v in saved.items():
            rt.config_set(k, v)
        for _, inputs in progs:
            for i in inputs:
                i.close()


@pytest.mark.parametrize("prefetch,run", [(1, 4), (2, 4), (2, 3), (1, 16)])
def test_batch_l2_prefetch_keeps_the_bits(cuda_device, prefetch, run):
    """The L2 bulk prefetches of a run's later tiles and of a block's next run
    (whose tiles may start in another program, or past the last one) change no
    result: every program's output is the single launch's, bit for bit."""
    import bench
    from compute.batch import Batch
    rt = cuda_device.runtime
    T = cuda_device.Tensor
    saved = {k: rt.config_get(k) for k in ("batch_prefetch", "batch_run_tiles")}
    progs = bench.c4_programs(T, seed=17, count=32, lo=1, hi=60000)
    tensors = [t for t, _ in progs]
    single = [t.flatArray() for t in tensors]
    try:
        rt.config_set("batch_prefetch", prefetch)
        rt.config_set("batch_run_tiles", run)
        b = Batch(cuda_device, tensors).bind()
        for _ in range(2):
            for out in b.outputs:
                rt.upload(out, np.full(out.nbytes // 4, np.nan, np.float32))
            b.run(Batch.PERSISTENT)
            for k, want in enumerate(single):
                got = rt.download(b.outputs[k], want.size)
                assert np.array_equal(got.view(np.int32), want.view(np.int32)), k
        b.close()
    finally:
        for k, v in saved.items():
            rt.config_set(k, v)
        for _, inputs in progs:
            for i in inputs:
                i.close()


def test_batch_rejects_programs_with_views(cuda_device):
    from compute._native import InvalidProgram
    from compute.batch import Batch
    T = cuda_device.Tensor
    a = T.random([64, 8], seed=1).doCache()
    with pytest.raises(InvalidProgram):
        Batch(cuda_device, [a.transpose() * T.fill(2.0, [8, 64])])
    a.close()


@pytest.mark.parametrize("copy_kernel", [1, 0])
def test_batch_transfers_in_the_event_model(cuda_device, copy_kernel):
    """Three steps in flight: each uploads its own inputs, runs after them and
    the previous step's reads, and reads into its own host buffers; every step's
    outputs are the bits of the same step run one call at a time.  The copies
    go through one SM kernel over a copy table (copy_kernel 1) or the DMA engines."""
    import ctypes
    import bench
    from compute._native import call
    from compute.batch import Batch
    rt = cuda_device.runtime
    T = cuda_device.Tensor
    saved = rt.config_get("batch_copy_kernel")
    rt.config_set("batch_copy_kernel", copy_kernel)
    progs = bench.c4_programs(T, seed=21, count=20, lo=1, hi=60000)
    b = Batch(cuda_device, [t for t, _ in progs]).bind()
    lengths = [int(np.prod(t.shape)) for t, _ in progs]
    # the bound inputs: per program, its parameters in the order the program numbers them
    in_lengths = [n for ser, n in zip(b.serialized, lengths) for _ in ser.params]
    in_bufs = [prm._cached for ser in b.serialized for prm in ser.params]
    pinned = []

    def host(n):
        p = ctypes.c_void_p()
        call("cc_host_alloc", ctypes.c_size_t(max(1, 4 * n)), ctypes.byref(p))
        pinned.append(p)
        return p.value, np.ctypeslib.as_array((ctypes.c_float * max(1, n)).from_address(p.value))[:n]

    r = np.random.RandomState(5)
    steps = 3
    hin = [[host(n) for n in in_lengths] for _ in range(steps)]
    hout = [[host(n) for n in lengths] for _ in range(steps)]
    for k in range(steps):
        for _, arr in hin[k]:
            arr[:] = r.uniform(0.1, 2.0, arr.size).astype(np.float32)
    try:
        # one call at a time: blocking uploads, a run, blocking reads
        want = []
        for k in range(steps):
            for (_, arr), buf in zip(hin[k], in_bufs):
                rt.upload(buf, arr)
            b.run()
            want.append([rt.download(o, n) for o, n in zip(b.outputs, lengths)])
        for k in range(steps):  # the outputs are overwritten before the pipelined run reads them
            for _, arr in hout[k]:
                arr[:] = np.nan
        events, prev_run, prev_read = [], None, None
        for k in range(steps):
            up = b.upload_ev([p for p, _ in hin[k]], wait=[prev_run] if prev_run else [])
            run = b.run_ev(0, wait=[up] + ([prev_read] if prev_read else []))
            read = b.download_ev([p for p, _ in hout[k]], wait=[run])
            events += [up, run, read]
            prev_run, prev_read = run, read
        rt.event_wait(prev_read, 60 * 10 ** 9)
        rt.synchronize()
        for e in events:
            rt.event_release(e)
        for k in range(steps):
            for p, ((_, got), exp) in enumerate(zip(hout[k], want[k])):
                assert np.array_equal(got.view(np.int32), exp.view(np.int32)), (k, p)
    finally:
        rt.synchronize()
        rt.config_set("batch_copy_kernel", saved)
        for p in pinned:
            call("cc_host_free", p)
        b.close()
        for _, inputs in progs:
            for i in inputs:
                i.close()


def test_batch_event_calls_check_their_arguments(cuda_device):
    from compute._native import InvalidValue
    from compute.batch import Batch
    T = cuda_device.Tensor
    a = T.random([64], seed=1).doCache()
    b = Batch(cuda_device, [a * a, a + a]).bind()
    with pytest.raises(InvalidValue):
        b.upload_ev([0])  # two inputs (one per program), one pointer
    with pytest.raises(InvalidValue):
        b.download_ev([0, 0, 0])
    b.close()
    a.close()

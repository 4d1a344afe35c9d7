"""Programmatic dependent launch keeps stream order: a chain of kernels, each
reading the buffer the previous one wrote (elementwise, view and sum programs),
gives the bits of the same chain launched without it."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _chain(d, n):
    T = d.Tensor
    x = T.random([n, 64], seed=7).doCache()
    t = x
    for k in range(12):
        t = (t * T.fill(1.0001, [n, 64]) + T.fill(0.5, [n, 64])).doCache()  # one kernel per step, reading the last
        if k % 4 == 3:
            t = t.transpose().transpose().translate([1, 0]).doCache()  # a view program in the chain
    s = t.sum().readScalar()
    return t.flatArray(), s


def test_pdl_chain_matches_plain_launches(cuda_device):
    rt = cuda_device.runtime
    for n in (1000, 300000):
        rt.config_set("pdl", 0)
        want, want_s = _chain(cuda_device, n)
        rt.config_set("pdl", 1)
        try:
            got, got_s = _chain(cuda_device, n)
        finally:
            rt.config_set("pdl", 1)
        assert np.array_equal(got.view(np.int32), want.view(np.int32))
        assert got_s == want_s


def test_early_start_keeps_write_after_read_and_write_after_write(cuda_device):
    """Kernels whose inputs do not overlap the previous kernel's output start
    early; their stores still wait, so a kernel that overwrites what the
    previous one reads (or writes) leaves the same bits as plain launches."""
    from compute.tensors import NonInlineTensor
    d = cuda_device
    rt = d.runtime
    T = d.Tensor
    n = 1 << 24
    p = NonInlineTensor(d, (n,), 0.0, None)
    f = rt.program(d.serialize((T.exp(p) * T.fill(0.5, [n])).closure, (n,)).text)     # C = exp(A) / 2
    g = rt.program(d.serialize((p * T.fill(3.0, [n]) + T.fill(1.0, [n])).closure, (n,)).text)  # A = 3B + 1
    h = rt.program(d.serialize(T.tanh(p).closure, (n,)).text)                          # C = tanh(B)
    r = np.random.RandomState(0)
    a0 = r.uniform(-1, 1, n).astype(np.float32)
    b0 = r.uniform(-1, 1, n).astype(np.float32)

    def run(pdl):
        rt.config_set("pdl", pdl)
        A, B, C = rt.alloc(4 * n), rt.alloc(4 * n), rt.alloc(4 * n)
        rt.upload(A, a0)
        rt.upload(B, b0)
        pa, pb, pc = A.device_ptr(), B.device_ptr(), C.device_ptr()
        outs = []
        for _ in range(20):
            rt.launch_ptrs(f, [pa], pc)   # reads A, writes C
            rt.launch_ptrs(g, [pb], pa)   # early (B not written by f); overwrites A, which f reads
            rt.launch_ptrs(f, [pa], pc)   # reads g's output: waits at entry
            rt.launch_ptrs(h, [pb], pc)   # early; writes C, which the previous kernel writes
            rt.launch_ptrs(g, [pc], pb)   # reads h's output: waits at entry; overwrites B, which h reads
        outs = [rt.download(buf, n) for buf in (A, B, C)]
        for buf in (A, B, C):
            buf.release()
        return outs

    try:
        want = run(0)
        got = run(1)
    finally:
        rt.config_set("pdl", 1)
    for w, g_ in zip(want, got):
        nan = np.isnan(w)
        assert np.array_equal(nan, np.isnan(g_))
        assert np.array_equal(w[~nan].view(np.int32), g_[~nan].view(np.int32))


def test_precompiled_kernels_between_generated_ones_keep_their_writes_visible(cuda_device):
    """A generated kernel G1 writes Z; a precompiled kernel (random numbers, the
    pooled sum, the sum without a context, the FP32 GEMM) writes X; a generated
    kernel G2 reads X.  The precompiled kernels never release their dependents
    early, so G2 must not load X before they end: the results are the bits of
    the same sequence launched without programmatic dependent launch."""
    import ctypes
    from compute import _native
    from compute.tensors import NonInlineTensor
    d = cuda_device
    rt = d.runtime
    T = d.Tensor
    n = 1 << 22
    p = NonInlineTensor(d, (n,), 0.0, None)
    g1 = rt.program(d.serialize((p * T.fill(2.0, [n])).closure, (n,)).text)            # Z = 2A
    g2 = rt.program(d.serialize((p + T.fill(1.0, [n])).closure, (n,)).text)            # Y = X + 1
    lib = _native.load()
    a0 = np.random.RandomState(1).uniform(-1, 1, n).astype(np.float32)

    def run(pdl):
        rt.config_set("pdl", pdl)
        A, Z, X, Y = (rt.alloc(4 * n) for _ in range(4))
        rt.upload(A, a0)
        pa, pz, px, py = A.device_ptr(), Z.device_ptr(), X.device_ptr(), Y.device_ptr()
        outs = []
        for seed in range(6):
            rt.launch_ptrs(g1, [pa], pz)
            rt.random(X, n, seed, seed % 2 == 1)           # X = random numbers
            rt.launch_ptrs(g2, [px], py)                    # reads X
            outs.append(rt.download(Y, n))
            rt.launch_ptrs(g1, [pa], pz)
            rt.reduce_sum_ptr(pz, n, px)                     # X[0] = sum(Z)
            rt.launch_ptrs(g2, [px], py)
            outs.append(rt.download(Y, 1))
            rt.launch_ptrs(g1, [pa], pz)
            _native.check(lib.cc_reduce_sum_f32_noalloc(ctypes.c_uint64(pa), ctypes.c_size_t(n), ctypes.c_uint64(px + 4),
                                                        ctypes.c_uint64(rt.stream())),
                          "cc_reduce_sum_f32_noalloc")     # X[1] = sum(A), without the context
            rt.launch_ptrs(g2, [px], py)
            outs.append(rt.download(Y, 2))
            rt.launch_ptrs(g1, [pa], pz)
            rt.gemm_ptr(pa, pa, px, 64, 64, 64, rt.GEMM_FP32)  # X[:4096] = A[:64,:64] @ A[:64,:64]
            rt.launch_ptrs(g2, [px], py)
            outs.append(rt.download(Y, 4096))
        rt.synchronize()
        for buf in (A, Z, X, Y):
            buf.release()
        return outs

    try:
        want = run(0)
        got = run(1)
    finally:
        rt.config_set("pdl", 1)
    for w, g_ in zip(want, got):
        assert np.array_equal(w.view(np.int32), g_.view(np.int32))

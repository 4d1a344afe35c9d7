"""The contraction kernels (cc_gemm_f32) against the reference's fold and FP64.

* CC_GEMM_EXACT must equal, bit for bit, the reference's matmul: the left fold
  over k of float products (TensorsSpec.scala:468-485), computed here in numpy
  float32 one k at a time.
* CC_GEMM_FP32 (fused multiply-adds) and CC_GEMM_BF16X6 (three bfloat16 planes,
  six products, FP32 accumulation on the tensor cores) are measured by their
  relative Frobenius error against float64: at most 1e-6 for the split-BF16
  path (the bar: <= 1e-6 relative error).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_fold(a, b):
    """C[i][j] = ((a[i,0]*b[0,j] + a[i,1]*b[1,j]) + ...) in float32, the reference's order."""
    acc = (a[:, 0:1] * b[0:1, :]).astype(np.float32)
    for k in range(1, a.shape[1]):
        acc = (acc + (a[:, k:k + 1] * b[k:k + 1, :])).astype(np.float32)
    return acc


def rel_fro(c, ref):
    return float(np.linalg.norm(c.astype(np.float64) - ref) / np.linalg.norm(ref))


# Exactly one index per seed makes the Wang hash 0 and log(0) = -inf, so a
# normal tensor of that seed holds an infinity there (also in the reference).
# Seeds with bit 30 set move that index past 2^30, beyond these tensors.
SEED = 0x40000000


def _operands(device, m, k, n, seed=SEED):
    T = device.Tensor
    a = T.randomNormal([m, k], seed=seed).doCache()
    b = T.randomNormal([k, n], seed=seed + 1).doCache()
    return a, b


def _run(device, a, b, m, k, n, mode):
    rt = device.runtime
    out = rt.alloc(m * n * 4)
    rt.gemm_ptr(a._cached.device_ptr(), b._cached.device_ptr(), out.device_ptr(), m, n, k, mode)
    c = rt.download(out, m * n).reshape(m, n)
    out.release()
    assert rt.device_errors() == 0
    return c


@pytest.mark.parametrize("shape", [(19, 23, 17), (128, 32, 256), (200, 50, 300), (256, 129, 512)])
def test_exact_mode_is_the_reference_fold(cuda_device, shape):
    m, k, n = shape
    a, b = _operands(cuda_device, m, k, n)
    c = _run(cuda_device, a, b, m, k, n, 0)
    want = reference_fold(a.flatArray().reshape(m, k), b.flatArray().reshape(k, n))
    assert np.array_equal(c.view(np.int32), want.view(np.int32))
    a.close()
    b.close()


@pytest.mark.parametrize("shape", [(128, 32, 256), (300, 100, 700), (1024, 1024, 1024)])
def test_fp32_mode(cuda_device, shape):
    m, k, n = shape
    a, b = _operands(cuda_device, m, k, n)
    c = _run(cuda_device, a, b, m, k, n, 1)
    ref = a.flatArray().reshape(m, k).astype(np.float64) @ b.flatArray().reshape(k, n).astype(np.float64)
    assert rel_fro(c, ref) <= 1e-6
    a.close()
    b.close()


@pytest.mark.parametrize("shape", [(128, 32, 256), (256, 64, 512), (300, 100, 700), (1024, 1024, 1024),
                                   (2048, 256, 2048)])
def test_split_bf16_tensor_core_mode(cuda_device, shape):
    m, k, n = shape
    a, b = _operands(cuda_device, m, k, n)
    c = _run(cuda_device, a, b, m, k, n, 2)
    ref = a.flatArray().reshape(m, k).astype(np.float64) @ b.flatArray().reshape(k, n).astype(np.float64)
    err = rel_fro(c, ref)
    assert err <= 1e-6, err
    a.close()
    b.close()


@pytest.mark.parametrize("variant", [3, 4, 5])
@pytest.mark.parametrize("shape", [(300, 100, 700), (1024, 1024, 1024), (512, 4096, 768), (200, 1000, 520),
                                   (256, 300, 512), (2560, 512, 2048), (2500, 600, 2000)])
def test_tensor_core_kernel_variants(cuda_device, variant, shape):
    """Every K-chunked kernel (128-column tiles restarting every 256 / 512 of K;
    256-column tiles restarting hi*hi every 256 of K) within the error bar, on
    ragged shapes, on K long enough for many chunks and on a last partial chunk
    (K = 300: ten k-blocks of 32, chunks of 8 then 2).  The last two shapes
    have 160 256-column tiles, more than one round of 152 SMs, so variant 5
    runs its last 8 tiles as column halves (ragged ones in the second)."""
    rt = cuda_device.runtime
    m, k, n = shape
    a, b = _operands(cuda_device, m, k, n)
    saved = rt.config_get("tc_variant")
    try:
        rt.config_set("tc_variant", variant)
        c = _run(cuda_device, a, b, m, k, n, 2)
    finally:
        rt.config_set("tc_variant", saved)
    ref = a.flatArray().reshape(m, k).astype(np.float64) @ b.flatArray().reshape(k, n).astype(np.float64)
    err = rel_fro(c, ref)
    assert err <= 1e-6, err
    a.close()
    b.close()


def _api_matmul(device, m1, m2):
    """TensorsSpec.scala:472-478, through the Tensor API."""
    i, j = m1.shape
    _, k = m2.shape
    prod = m1.broadcast([i, j, k]) * m2.reshape([1, j, k]).broadcast([i, j, k])
    return prod.split(1).reduce(lambda x, y: x + y)


def test_matmul_idiom_through_the_api_in_every_contraction_mode(cuda_device):
    rt = cuda_device.runtime
    T = cuda_device.Tensor
    m, k, n = 64, 300, 96
    a = T.randomNormal([m, k], seed=SEED).doCache()
    b = T.randomNormal([k, n], seed=SEED + 1).doCache()
    want = reference_fold(a.flatArray().reshape(m, k), b.flatArray().reshape(k, n))
    ref64 = a.flatArray().reshape(m, k).astype(np.float64) @ b.flatArray().reshape(k, n).astype(np.float64)
    saved = rt.config_get("contraction")
    got = {}
    try:
        for mode in (0, 1, 2, 3):
            rt.config_set("contraction", mode)
            c = _api_matmul(cuda_device, a, b)
            got[mode] = c.flatArray().reshape(m, n)
            assert rt.device_errors() == 0
    finally:
        rt.config_set("contraction", saved)
    assert np.array_equal(got[0].view(np.int32), want.view(np.int32))  # the generated fold
    assert np.array_equal(got[1].view(np.int32), want.view(np.int32))  # the exact GEMM
    assert rel_fro(got[2], ref64) <= 1e-6
    assert rel_fro(got[3], ref64) <= 1e-6
    a.close()
    b.close()


@pytest.mark.parametrize("shape", [(4096, 4096, 4096), (16384, 256, 16384)])
def test_benchmark_shapes_through_the_api(cuda_device, shape):
    """The two contraction configurations at full size (A[4096,4096] x B[4096,4096];
    A[16384,256] x B[256,16384], both ~ N(0,1)), through the Tensor API's matmul
    idiom on the split-BF16 tensor cores, and the FP32 CUDA-core GEMM on the same
    operands: relative Frobenius error of 512 sampled rows against float64 at
    most 1e-6 for both, and no device error."""
    rt = cuda_device.runtime
    m, k, n = shape
    a, b = _operands(cuda_device, m, k, n)
    saved = rt.config_get("contraction")
    try:
        rt.config_set("contraction", 3)
        c = _api_matmul(cuda_device, a, b)
        ser = cuda_device.serialize(c.closure, c.shape)
        prog = rt.program(ser.text)
        out = rt.alloc(m * n * 4)
        rt.launch(prog, [a._cached, b._cached], out)
        assert rt.device_errors() == 0
        rows = np.sort(np.random.RandomState(1).choice(m, size=512, replace=False))
        got = np.stack([rt.download(out, n, offset=int(r) * n * 4) for r in rows])
        fp32 = rt.alloc(m * n * 4)
        rt.gemm_ptr(a._cached.device_ptr(), b._cached.device_ptr(), fp32.device_ptr(), m, n, k, rt.GEMM_FP32)
        got32 = np.stack([rt.download(fp32, n, offset=int(r) * n * 4) for r in rows])
        out.release()
        fp32.release()
    finally:
        rt.config_set("contraction", saved)
    A = a.flatArray().reshape(m, k)[rows].astype(np.float64)
    B = b.flatArray().reshape(k, n).astype(np.float64)
    ref = A @ B
    err, err32 = rel_fro(got, ref), rel_fro(got32, ref)
    assert err <= 1e-6, err
    assert err32 <= 1e-5, err32  # the plain FP32 GEMM, for comparison (about 1e-6 at K = 4096)
    a.close()
    b.close()

"""ORACLE (test infrastructure only): the reference's CPU path, as a timed baseline and a checker.

``CRuntime`` is a runtime for the Tensor API that runs every program as the
reference's own generated OpenCL C (``clgen``), compiled as C through
``cl_shim.h`` with gcc and OpenMP over all host threads, with the fusion
planner off so the kernels have the reference's structure (an inline tensor
that is viewed is materialised first, Tensors.scala:1413-1428).  Full sums use
the reference's CPU reduction: one work item, sixteen lanes, then the tail
(Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala:313-351).
Random numbers come from ``oracle.rng``.

``time_workload`` times the benchmark's workloads with it on a bounded sample.
"""

from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import sys
import time

import numpy as np

from . import clgen, rng

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "_ref")

REDUCE_C = r"""
/* Tensors.scala:313-351 (sequentialReductionProgram), one work item. */
float cc_reduce_sequential(const float *restrict buffer, unsigned int length) {
  const unsigned int vector_length = length / 16;
  if (vector_length >= 1) {
    const int stage1_length = 16 * vector_length;
    const int stage2_length = length - stage1_length;
    float acc[16];
    for (int j = 0; j < 16; ++j) acc[j] = buffer[j];
    for (unsigned int gi = 1; gi < vector_length; ++gi)
      for (int j = 0; j < 16; ++j) acc[j] = ((acc[j]) + (buffer[16 * gi + j]));
    float f8[8], f4[4], f2[2];
    for (int j = 0; j < 8; ++j) f8[j] = ((acc[8 + j]) + (acc[j]));
    for (int j = 0; j < 4; ++j) f4[j] = ((f8[4 + j]) + (f8[j]));
    for (int j = 0; j < 2; ++j) f2[j] = ((f4[2 + j]) + (f4[j]));
    float a = ((f2[0]) + (f2[1]));
    const float *rest = buffer + stage1_length;
    for (int gi = 0; gi < stage2_length; ++gi) a = ((a) + (rest[gi]));
    return a;
  }
  float a = 0.0f;
  for (unsigned int gi = 0; gi < length; ++gi) a = ((a) + (buffer[gi]));
  return a;
}
"""


def _compile(source: str, tag: str, contract: str = "off") -> ctypes.CDLL:
    """Builds the generated C.  ``contract``: gcc's -ffp-contract mode, "off"
    (every statement rounds as written) or "fast" (gcc fuses a*b+c where the
    target has FMA, as a vendor OpenCL compiler may under the reference's
    -cl-unsafe-math-optimizations)."""
    if contract not in ("off", "fast"):
        raise ValueError(contract)
    os.makedirs(CACHE, exist_ok=True)
    h = hashlib.sha1((contract + source).encode()).hexdigest()[:16]
    so = os.path.join(CACHE, "%s_%s.so" % (tag, h))
    if not os.path.exists(so):
        c = so[:-3] + ".c"
        with open(c, "w") as f:
            f.write(source)
        cmd = ["gcc", "-O3", "-std=gnu11", "-fopenmp", "-ffp-contract=" + contract, "-fPIC", "-shared",
               "-I", HERE, c, "-o", so + ".tmp", "-lm"]
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError("gcc failed:\n" + p.stdout[-4000:])
        os.replace(so + ".tmp", so)
    return ctypes.CDLL(so)


def _driver(src: str, info) -> str:
    gws = info["global_work_size"]
    nd = len(gws)
    lines = ['#include "cl_shim.h"', src,
             "void cc_run(void **ins, void *out, const int *size_args) {"]
    for d in range(3):
        lines.append("  cl_gsz_[%d] = %d;" % (d, gws[d] if d < nd else 1))
    if nd == 0:
        call_args = ["size_args[%d]" % k for k in range(len(info["size_args"]))]
        call_args += ["(%s)ins[%d]" % (t, k) for k, (t, _) in enumerate(info["param_types"])]
        call_args.append("(%s *)out" % info["out_type"])
        lines.append("  jit_kernel(%s);" % ", ".join(call_args))
        lines.append("}")
        return "\n".join(lines)
    lines.append("  #pragma omp parallel for collapse(%d) schedule(static)" % nd)
    for d in range(nd):
        lines.append("  for (long i%d = 0; i%d < %d; ++i%d)" % (d, d, gws[d], d))
    lines.append("  {")
    for d in range(nd):
        lines.append("    cl_gid_[%d] = i%d;" % (d, d))
    call_args = ["size_args[%d]" % k for k in range(len(info["size_args"]))]
    call_args += ["(%s)ins[%d]" % (t, k) for k, (t, _) in enumerate(info["param_types"])]
    call_args.append("(%s *)out" % info["out_type"])
    lines.append("    jit_kernel(%s);" % ", ".join(call_args))
    lines.append("  }")
    lines.append("}")
    return "\n".join(lines)


class CBuffer:
    def __init__(self, nbytes):
        self.data = np.zeros(max(1, (nbytes + 3) // 4), dtype=np.float32)
        self.nbytes = nbytes

    def retain(self):
        pass

    def release(self):
        pass


class CProgram:
    def __init__(self, text, contract="off"):
        self.text = text
        self.kind = text.split("\n", 1)[0].split()[2]
        ew_text = text.replace("ccir 1 sum", "ccir 1 ew", 1)
        src, info = clgen.kernel_source(ew_text)
        info["param_types"], info["out_type"] = _param_types(src, info)
        self.info = info
        self.lib = _compile(_driver(src, info), "k", contract)
        self.lib.cc_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        self.lib.cc_run.restype = None


def _param_types(src, info):
    import re
    types = re.findall(r"typedef global const float \(\* (float_array_\d+)\)", src)
    out_type = "float"
    m = re.search(r"typedef struct (float_tuple_\d+)", src)
    if info["tuple_len"] > 1 and m:
        out_type = m.group(1)
    return [(t, None) for t in types], out_type


_reduce_lib = None


def _reducer():
    global _reduce_lib
    if _reduce_lib is None:
        _reduce_lib = _compile(REDUCE_C, "reduce")
        _reduce_lib.cc_reduce_sequential.argtypes = [ctypes.c_void_p, ctypes.c_uint]
        _reduce_lib.cc_reduce_sequential.restype = ctypes.c_float
    return _reduce_lib


class CRuntime:
    """Runs Tensor programs as the reference's OpenCL C compiled for the host."""

    def __init__(self, threads=None, contract="off"):
        if threads:
            os.environ["OMP_NUM_THREADS"] = str(threads)
        self.contract = contract
        self._programs = {}

    def alloc(self, nbytes):
        return CBuffer(nbytes)

    def upload(self, buf, array, offset=0):
        a = np.ascontiguousarray(array, dtype=np.float32).ravel()
        buf.data[offset // 4: offset // 4 + a.size] = a

    def download(self, buf, count, dtype=np.float32, offset=0):
        return buf.data[offset // 4: offset // 4 + count].copy()

    def program(self, text):
        p = self._programs.get(text)
        if p is None:
            p = CProgram(text, self.contract)
            self._programs[text] = p
        return p

    def launch(self, prog, inputs, out):
        info = prog.info
        n = len(inputs)
        ins = (ctypes.c_void_p * max(1, n))(*[b.data.ctypes.data for b in inputs])
        sa = (ctypes.c_int * max(1, len(info["size_args"])))(*info["size_args"])
        if prog.kind == "sum":
            count = int(np.prod(info["out_shape"])) if info["out_shape"] else 1
            tmp = np.zeros(max(1, count), dtype=np.float32)
            prog.lib.cc_run(ins, tmp.ctypes.data, sa)
            out.data[0] = _reducer().cc_reduce_sequential(tmp.ctypes.data, count)
        else:
            prog.lib.cc_run(ins, out.data.ctypes.data, sa)

    def random(self, buf, n, seed, normal):
        buf.data[:n] = rng.random_normal(n, seed) if normal else rng.random_uniform(n, seed)


def _threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def time_workload(workload: str, budget_s: float = 15.0, threads=None, contract="off"):
    """GB/s of the reference's CPU path on a bounded sample of a benchmark workload."""
    root = os.path.dirname(HERE)
    sys.path.insert(0, os.path.join(root, "compute.scala_gb300"))
    from compute import Tensors, trees
    threads = threads or _threads()
    d = Tensors(runtime=CRuntime(threads, contract), planner=trees.Planner(enabled=False))
    T = d.Tensor
    if workload == "c2":
        c, h, w = 128, 56, 56
        full_n = 64
        n = 1
        while True:
            x = T.randomNormal([n, c, h, w], seed=0).doCache()
            bias = (T.randomNormal([c], seed=1) * T.fill(0.1, [c])).reshape([1, 1, 1, c]).doCache()
            y = T.max(x.permute([0, 2, 3, 1]) + bias.broadcast([n, h, w, c]), T.fill(0.0, [n, h, w, c]))
            s = y.translate([0, 0, 1, 0]).split(3).reduce(lambda a, b: a + b)
            s.flatArray()  # compile and warm up
            t0 = time.perf_counter()
            reps = 0
            while True:
                s.flatArray()
                reps += 1
                dt = time.perf_counter() - t0
                if dt > budget_s / 4 or reps >= 50:
                    break
            per = dt / reps
            if per * 4 > budget_s / 4 or n >= full_n:
                break
            n = min(full_n, n * 4)
        nbytes = 4 * (n * c * h * w + c + n * h * w)
        return {"gbs": nbytes / per / 1e9, "ms_per_step": per * 1e3 * full_n / n, "threads": threads,
                "sample": "x[%d,128,56,56] (%d of 64 images), %d reps; reference kernel structure: "
                          "permute+bias+max materialised NHWC, then translate+128-term channel sum"
                          % (n, n, reps),
                "config": {"workload": "view-heavy fused op (reference CPU path, OpenCL C on host cores)",
                           "x": [n, c, h, w]}}
    if workload == "c1":
        nm = 1024
        two, one = T.fill(2.0, [nm, nm]), T.fill(1.0, [nm, nm])
        abc = [(T.random([nm, nm], seed=s) * two - one).doCache() for s in (0, 1, 2)]
        e = T.tanh(abc[0] * abc[1] + abc[2]).sum()
        e.flatArray()
        t0 = time.perf_counter()
        reps = 0
        while True:
            e.flatArray()
            reps += 1
            dt = time.perf_counter() - t0
            if dt > budget_s / 2 or reps >= 100:
                break
        per = dt / reps
        nbytes = 4 * 3 * nm * nm + 4
        return {"gbs": nbytes / per / 1e9, "ms_per_step": per * 1e3, "threads": threads,
                "sample": "full workload, %d reps; tanh kernel materialised, then the one-work-item "
                          "16-lane sequential sum" % reps,
                "config": {"workload": "fused elementwise+sum (reference CPU path, OpenCL C on host cores)"}}
    raise ValueError(workload)


def time_expression(make, nbytes: int, budget_s: float = 15.0, threads=None):
    """GB/s of the reference's CPU path evaluating ``make(T)`` (a tensor built with
    the given Tensor companion, fusion off: the reference's kernel structure)."""
    root = os.path.dirname(HERE)
    sys.path.insert(0, os.path.join(root, "compute.scala_gb300"))
    from compute import Tensors, trees
    threads = threads or _threads()
    d = Tensors(runtime=CRuntime(threads), planner=trees.Planner(enabled=False))
    t = make(d.Tensor)
    t.flatArray()  # compile and warm up
    t0 = time.perf_counter()
    reps = 0
    while True:
        t.flatArray()
        reps += 1
        dt = time.perf_counter() - t0
        if dt > budget_s / 2 or reps >= 100:
            break
    per = dt / reps
    return {"gbs": nbytes / per / 1e9, "ms_per_step": per * 1e3, "threads": threads, "reps": reps}


def time_programs(make_programs, budget_s: float = 15.0, threads=None, max_programs: int = 64):
    """GB/s of the reference's CPU path over a sample of independent programs:
    ``make_programs(T)`` returns (tensor, inputs) pairs built with the given
    Tensor companion; each program is its own kernel, as in the reference
    (Tensors.scala:1331-1381).  The first ``max_programs`` are compiled and
    warmed up, then evaluated in turn until the budget is spent."""
    root = os.path.dirname(HERE)
    sys.path.insert(0, os.path.join(root, "compute.scala_gb300"))
    from compute import Tensors, trees
    threads = threads or _threads()
    d = Tensors(runtime=CRuntime(threads), planner=trees.Planner(enabled=False))
    progs = make_programs(d.Tensor)[:max_programs]
    nbytes = 0
    for t, inputs in progs:
        t.flatArray()  # compile and warm up
        nbytes += 4 * int(np.prod(t.shape)) * (len(inputs) + 1)
    t0 = time.perf_counter()
    rounds = 0
    while True:
        for t, _ in progs:
            t.flatArray()
        rounds += 1
        dt = time.perf_counter() - t0
        if dt > budget_s / 2 or rounds >= 20:
            break
    per = dt / rounds
    return {"gbs": nbytes / per / 1e9, "ms_per_round": per * 1e3, "threads": threads,
            "sample": "the first %d programs (%.0f MB per round), %d rounds; one reference kernel per program"
                      % (len(progs), nbytes / 1e6, rounds)}


FOLD_GEMM_C = r"""
/* The reference's matmul semantics (TensorsSpec.scala:468-485): each output is
 * the left fold over k of separately rounded float products, in k order.
 * Rows are spread over OpenMP threads; the j loop vectorises. */
void cc_fold_gemm(const float *restrict A, const float *restrict B, float *restrict C, int m, int n, int k) {
  #pragma omp parallel for schedule(static)
  for (int i = 0; i < m; ++i) {
    float *restrict c = C + (long)i * n;
    const float *restrict a = A + (long)i * k;
    for (int j = 0; j < n; ++j) c[j] = a[0] * B[j];
    for (int kk = 1; kk < k; ++kk) {
      const float av = a[kk];
      const float *restrict b = B + (long)kk * n;
      for (int j = 0; j < n; ++j) c[j] = c[j] + av * b[j];
    }
  }
}
"""


def time_contraction(shape, budget_s: float = 15.0, threads=None):
    """TFLOP/s of the reference's contraction semantics on the host cores, on a row sample.

    The reference itself would materialise the I*J*K product (256 GiB at these
    shapes); this times the same arithmetic without that, so it is an upper
    bound for the reference's CPU path.
    """
    m, k, n = shape
    threads = threads or _threads()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    lib = _compile(FOLD_GEMM_C, "foldgemm")
    lib.cc_fold_gemm.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 3
    lib.cc_fold_gemm.restype = None
    b = rng.random_normal(k * n, 0x40000001).reshape(k, n)
    rows = max(threads, 1)
    while True:
        a = rng.random_normal(rows * k, 0x40000000).reshape(rows, k)
        c = np.empty((rows, n), dtype=np.float32)
        t0 = time.perf_counter()
        lib.cc_fold_gemm(a.ctypes.data, b.ctypes.data, c.ctypes.data, rows, n, k)
        dt = time.perf_counter() - t0
        if dt > budget_s / 4 or rows >= m:
            break
        rows = min(m, rows * 4)
    tflops = 2.0 * rows * n * k / dt / 1e12
    return {"tflops": tflops, "ms_per_step": dt * 1e3 * m / rows, "threads": threads,
            "sample": "%d of %d rows of A[%d,%d] x B[%d,%d]; sequential-k FP32 fold, OpenMP over rows" % (rows, m, m, k, k, n),
            "config": {"workload": "contraction (reference fold semantics on host cores)", "shape": [m, k, n]}}

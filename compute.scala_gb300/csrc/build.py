"""Builds libcomputecuda.so in-tree (compute.scala_gb300/compute/libcomputecuda.so).

Host translation units compile with g++, device ones with nvcc for sm_103a
only; they compile in parallel and link with nvcc (static cudart, dynamic
NVRTC).  Driver API functions are resolved at run time through the CUDA
runtime, so the library loads on hosts without a GPU driver.  No cmake: the
same script runs on the x86 container and the aarch64 GPU hosts.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.normpath(os.path.join(HERE, "..", "compute"))
BUILD = os.path.normpath(os.path.join(HERE, "..", "_build"))
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SOURCES = ["runtime.cpp", "codegen.cpp", "tuning.cpp"]
DEVICE_SOURCES = ["kernels.cu", "noalloc.cu", "gemm.cu", "gemm_tc.cu", "mlp.cu"]
LIB_NAME = "libcomputecuda.so"


def cuda_home() -> str:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env and os.path.isdir(env):
        return env
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _embed(src: str, dst: str) -> None:
    """Turns a .cuh file into a C++ string-literal fragment (the NVRTC prelude)."""
    with open(src) as f:
        text = f.read()
    text = text.replace("#pragma once\n", "")
    chunks = [text[i:i + 8000] for i in range(0, len(text), 8000)] or [""]
    body = "\n".join('R"CCPRELUDE(%s)CCPRELUDE"' % c for c in chunks)
    if os.path.exists(dst):
        with open(dst) as f:
            if f.read() == body:
                return
    with open(dst, "w") as f:
        f.write(body)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = shutil.which("nvcc") or nvcc
    os.makedirs(BUILD, exist_ok=True)
    inc = os.path.join(BUILD, "device_common.inc")
    _embed(os.path.join(HERE, "device_common.cuh"), inc)
    headers = [os.path.join(HERE, h) for h in os.listdir(HERE) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "..", "include", "compute_cuda.h"))
    headers.append(inc)
    cuda_inc = os.path.join(home, "include")
    jobs = []
    objs = []
    for s in HOST_SOURCES:
        src = os.path.join(HERE, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function",
                         "-I", cuda_inc, "-I", BUILD, "-c", src, "-o", obj])
    for s in DEVICE_SOURCES:
        src = os.path.join(HERE, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", BUILD, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    lib = os.path.join(PKG, LIB_NAME)
    libdirs = []
    for d in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        p = os.path.join(home, d)
        if os.path.isdir(p):
            libdirs.append(p)
    if _stale(lib, objs):
        cmd = [nvcc, ARCH, "-shared", "-o", lib] + objs
        for d in libdirs:
            cmd += ["-L", d]
        cmd += ["-lnvrtc"]
        for d in libdirs:
            cmd += ["-Xlinker", "-rpath=" + d]
        _run(cmd)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

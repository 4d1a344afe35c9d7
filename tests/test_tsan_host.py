"""Race check of the C++ host runtime: the runtime's host sources built with
ThreadSanitizer, driven from 8 threads through the GPU-free entry points
(code generation in every read form, the NVRTC compile, error reporting),
report no data race.  (compute-sanitizer, for device code, is not available
here; the GPU paths' concurrency is covered by tests/test_threads_gpu.py.)"""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "compute.scala_gb300", "csrc")
BUILD = os.path.join(ROOT, "compute.scala_gb300", "_build")
OUT = os.path.join(BUILD, "tsan")

DRIVER = r"""
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include "compute_cuda.h"

static const char *kIr[] = {
  "ccir 1 ew\no 2 2 3\np 2 2 3 00000000\nx 0 3 1 0 0 0 1 0\np 2 2 3 00000000\nx 2 3 1 0 0 0 1 0\nb mul 1 3\nr 4\n",
  "ccir 1 sum\no 2 2 3\np 2 2 3 00000000\nx 0 3 1 0 0 0 1 0\nu tanh 1\nr 2\n",
};

int main() {
  std::vector<std::thread> ts;
  std::vector<int> fails(8, 0);
  for (int t = 0; t < 8; ++t)
    ts.emplace_back([t, &fails] {
      for (int rep = 0; rep < 20; ++rep) {
        const char *ir = kIr[(t + rep) % 2];
        const char *opts = rep % 3 == 0 ? "vl=1 points=2" : (rep % 3 == 1 ? "vl=0" : nullptr);
        size_t need = 0;
        if (cc_codegen_with(ir, strlen(ir), opts, nullptr, 0, &need) != CC_OK) ++fails[t];
        std::string buf(need, '\0');
        if (cc_codegen_with(ir, strlen(ir), opts, &buf[0], need, &need) != CC_OK) ++fails[t];
        if (cc_codegen("bad", 3, nullptr, 0, &need) == CC_OK) ++fails[t];
        char msg[128];
        cc_last_error(msg, sizeof msg);
        if (rep % 10 == 0 && cc_compile_check(ir, strlen(ir), 10, 3, 0) != CC_OK) ++fails[t];
      }
    });
  for (auto &th : ts) th.join();
  int failures = 0;
  for (int f : fails) failures += f;
  std::printf("failures %d\n", failures);
  return failures != 0;
}
"""


def test_host_runtime_has_no_data_race():
    gxx = shutil.which("g++")
    cuda = "/usr/local/cuda"
    device_objs = [os.path.join(BUILD, s + ".o") for s in ("kernels.cu", "noalloc.cu", "gemm.cu", "gemm_tc.cu", "mlp.cu")]
    if gxx is None or not all(os.path.exists(o) for o in device_objs):
        pytest.skip("needs g++ and the built device objects")
    os.makedirs(OUT, exist_ok=True)
    flags = ["-std=c++17", "-O1", "-g", "-fsanitize=thread", "-fPIC"]
    objs = []
    procs = []
    for s in ("runtime", "codegen", "tuning"):
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        procs.append(subprocess.Popen([gxx] + flags + ["-I", os.path.join(cuda, "include"), "-I", BUILD, "-c",
                                                        os.path.join(CSRC, s + ".cpp"), "-o", obj]))
    main_cpp = os.path.join(OUT, "main.cpp")
    with open(main_cpp, "w") as f:
        f.write(DRIVER)
    main_o = os.path.join(OUT, "main.o")
    procs.append(subprocess.Popen([gxx] + flags + ["-I", os.path.join(ROOT, "include"), "-c", main_cpp, "-o", main_o]))
    for p in procs:
        assert p.wait() == 0
    exe = os.path.join(OUT, "tsan_check")
    link = subprocess.run([gxx, "-fsanitize=thread", "-o", exe, main_o] + objs + device_objs +
                          ["-L", os.path.join(cuda, "lib64"), "-lcudart_static", "-lnvrtc", "-ldl", "-lpthread", "-lrt",
                           "-Wl,-rpath=" + os.path.join(cuda, "lib64")], capture_output=True, text=True)
    if link.returncode != 0:
        pytest.skip("ThreadSanitizer link unavailable: " + link.stderr[-300:])
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=0 report_signal_unsafe=0")
    run = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
    assert "WARNING: ThreadSanitizer" not in run.stderr, run.stderr[-3000:]
    assert run.returncode == 0 and "failures 0" in run.stdout, (run.stdout, run.stderr[-1000:])

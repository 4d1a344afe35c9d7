"""Python face of the native runtime: buffers, programs, launches and events.

Every method is one or two calls of the C ABI (include/compute_cuda.h); there
is no host-side compute and no fallback.  ``Tensors`` drives it the way the
reference's ``Tensors`` drives its OpenCL layer (allocateBuffer,
createProgramWithSource/build, Kernel.enqueue, toHostBuffer).
"""

from __future__ import annotations

import ctypes
from typing import Dict, Sequence

import numpy as np

from . import _native
from ._native import c_handle, call


class DeviceBuffer:
    """A reference-counted device buffer from the pool (OpenCL.scala:633-717)."""

    __slots__ = ("handle", "nbytes")

    def __init__(self, handle: int, nbytes: int):
        self.handle = handle
        self.nbytes = nbytes

    def retain(self):
        call("cc_buf_retain", c_handle(self.handle))

    def release(self):
        call("cc_buf_release", c_handle(self.handle))

    def device_ptr(self) -> int:
        p = ctypes.c_uint64()
        call("cc_buf_device_ptr", c_handle(self.handle), ctypes.byref(p))
        return p.value


class Program:
    __slots__ = ("handle", "kind", "n_inputs", "out_elems", "tuple_len", "text")

    def __init__(self, handle, kind, n_inputs, out_elems, tuple_len, text):
        self.handle = handle
        self.kind = kind
        self.n_inputs = n_inputs
        self.out_elems = out_elems
        self.tuple_len = tuple_len
        self.text = text

    def source(self) -> str:
        need = ctypes.c_size_t()
        call("cc_program_source", c_handle(self.handle), None, 0, ctypes.byref(need))
        buf = ctypes.create_string_buffer(need.value)
        call("cc_program_source", c_handle(self.handle), buf, need.value, ctypes.byref(need))
        return buf.value.decode()


class NativeRuntime:
    def __init__(self, device: int = 0, flags: int = 0):
        self.lib = _native.load()
        call("cc_init", int(device), int(flags))
        self._programs: Dict[str, Program] = {}

    # -- device
    def device_info(self):
        sm, ma, mi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        mem = ctypes.c_size_t()
        call("cc_device_info", ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi), ctypes.byref(mem))
        return {"sm_count": sm.value, "cc": (ma.value, mi.value), "total_mem": mem.value}

    def stream(self) -> int:
        s = ctypes.c_uint64()
        call("cc_get_stream", ctypes.byref(s))
        return s.value

    def synchronize(self):
        call("cc_synchronize")

    def config_set(self, key: str, value: int):
        """Sets a runtime tuning knob; programs are compiled again under the new setting."""
        call("cc_config_set", key.encode(), ctypes.c_int64(int(value)))
        self._programs.clear()

    def config_get(self, key: str) -> int:
        v = ctypes.c_int64()
        call("cc_config_get", key.encode(), ctypes.byref(v))
        return v.value

    # -- buffers
    def alloc(self, nbytes: int) -> DeviceBuffer:
        h = c_handle()
        call("cc_buf_alloc", ctypes.c_size_t(int(nbytes)), ctypes.byref(h))
        return DeviceBuffer(h.value, int(nbytes))

    def upload(self, buf: DeviceBuffer, array: np.ndarray, offset: int = 0):
        a = np.ascontiguousarray(array)
        call("cc_buf_upload", c_handle(buf.handle), ctypes.c_size_t(offset), a.ctypes.data_as(ctypes.c_void_p),
             ctypes.c_size_t(a.nbytes))

    def download(self, buf: DeviceBuffer, count: int, dtype=np.float32, offset: int = 0) -> np.ndarray:
        out = np.empty(int(count), dtype=dtype)
        call("cc_buf_download", c_handle(buf.handle), ctypes.c_size_t(offset), out.ctypes.data_as(ctypes.c_void_p),
             ctypes.c_size_t(out.nbytes))
        return out

    def pool_stats(self):
        a, b = ctypes.c_size_t(), ctypes.c_size_t()
        c, d = ctypes.c_uint64(), ctypes.c_uint64()
        call("cc_pool_stats", ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d))
        return {"in_use": a.value, "cached": b.value, "allocs": c.value, "reuses": d.value}

    def pool_trim(self):
        """Frees the pool's cached blocks (cudaFree)."""
        call("cc_pool_trim")

    def pool_set_limit(self, nbytes: int):
        call("cc_pool_set_limit", ctypes.c_size_t(int(nbytes)))

    # -- programs
    def program(self, text: str) -> Program:
        p = self._programs.get(text)
        if p is not None:
            return p
        raw = text.encode()
        h = c_handle()
        call("cc_program_get", raw, ctypes.c_size_t(len(raw)), ctypes.byref(h))
        kind, n_in, tl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        out_elems = ctypes.c_int64()
        call("cc_program_info", h, ctypes.byref(kind), ctypes.byref(n_in), ctypes.byref(out_elems), ctypes.byref(tl))
        p = Program(h.value, kind.value, n_in.value, out_elems.value, tl.value, text)
        self._programs[text] = p
        return p

    def cache_stats(self):
        h, m, e = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        call("cc_program_cache_stats", ctypes.byref(h), ctypes.byref(m), ctypes.byref(e))
        return {"hits": h.value, "misses": m.value, "entries": e.value}

    def launch(self, prog: Program, inputs: Sequence[DeviceBuffer], out: DeviceBuffer):
        n = len(inputs)
        arr = (c_handle * max(1, n))(*[b.handle for b in inputs])
        call("cc_launch", c_handle(prog.handle), arr, n, c_handle(out.handle))

    def launch_ptrs(self, prog: Program, input_ptrs: Sequence[int], out_ptr: int, stream: int = 0):
        n = len(input_ptrs)
        arr = (ctypes.c_uint64 * max(1, n))(*input_ptrs)
        call("cc_launch_ptrs", c_handle(prog.handle), arr, n, ctypes.c_uint64(out_ptr), ctypes.c_uint64(stream))

    # -- the asynchronous DAG (a pool of streams ordered by event wait lists)
    @staticmethod
    def _wait_list(wait):
        wait = list(wait or ())
        return (c_handle * max(1, len(wait)))(*wait), len(wait)

    def launch_ev(self, prog: Program, inputs: Sequence[DeviceBuffer], out: DeviceBuffer, wait=()) -> int:
        """Kernel.enqueue with waitingEvents: returns the event of this launch."""
        n = len(inputs)
        arr = (c_handle * max(1, n))(*[b.handle for b in inputs])
        w, nw = self._wait_list(wait)
        ev = c_handle()
        call("cc_launch_ev", c_handle(prog.handle), arr, n, c_handle(out.handle), w, nw, ctypes.byref(ev))
        return ev.value

    def upload_ev(self, buf: DeviceBuffer, host_ptr: int, nbytes: int, offset: int = 0, wait=()) -> int:
        w, nw = self._wait_list(wait)
        ev = c_handle()
        call("cc_buf_upload_ev", c_handle(buf.handle), ctypes.c_size_t(offset), ctypes.c_void_p(host_ptr),
             ctypes.c_size_t(nbytes), w, nw, ctypes.byref(ev))
        return ev.value

    def download_ev(self, buf: DeviceBuffer, host_ptr: int, nbytes: int, offset: int = 0, wait=()) -> int:
        w, nw = self._wait_list(wait)
        ev = c_handle()
        call("cc_buf_download_ev", c_handle(buf.handle), ctypes.c_size_t(offset), ctypes.c_void_p(host_ptr),
             ctypes.c_size_t(nbytes), w, nw, ctypes.byref(ev))
        return ev.value

    def stream_wait(self, events):
        w, nw = self._wait_list(events)
        call("cc_stream_wait_events", w, nw)

    def event_query(self, ev: int) -> bool:
        done = ctypes.c_int()
        call("cc_event_query", c_handle(ev), ctypes.byref(done))
        return bool(done.value)

    # -- fixed kernels
    def random(self, buf: DeviceBuffer, n: int, seed: int, normal: bool):
        call("cc_random", c_handle(buf.handle), ctypes.c_size_t(int(n)), ctypes.c_uint32(seed & 0xFFFFFFFF),
             1 if normal else 0)

    def reduce_sum_ptr(self, in_ptr: int, n: int, out_ptr: int, stream: int = 0):
        call("cc_reduce_sum_f32", ctypes.c_uint64(in_ptr), ctypes.c_size_t(int(n)), ctypes.c_uint64(out_ptr),
             ctypes.c_uint64(stream))

    GEMM_EXACT, GEMM_FP32, GEMM_BF16X6 = 0, 1, 2

    def gemm_ptr(self, a_ptr: int, b_ptr: int, c_ptr: int, m: int, n: int, k: int, mode: int,
                 lda: int = None, ldb: int = None, ldc: int = None, stream: int = 0):
        call("cc_gemm_f32", ctypes.c_uint64(a_ptr), ctypes.c_uint64(b_ptr), ctypes.c_uint64(c_ptr), int(m), int(n),
             int(k), ctypes.c_int64(k if lda is None else lda), ctypes.c_int64(n if ldb is None else ldb),
             ctypes.c_int64(n if ldc is None else ldc), int(mode), ctypes.c_uint64(stream))

    def tuner_choice(self, prog: Program) -> int:
        """The launch configuration the tuner chose for a program (-1: none yet)."""
        v = ctypes.c_int()
        call("cc_tuner_choice", c_handle(prog.handle), ctypes.byref(v))
        return v.value

    def device_errors(self) -> int:
        v = ctypes.c_int()
        call("cc_device_errors", ctypes.byref(v))
        return v.value

    PROBE_TIMEOUT = 90  # CC_DEVICE_ERR_PROBE_TIMEOUT

    def probe_bounded_wait(self, limit_ns: int, flag_value: int):
        """Enqueues a device wait on a word that is set (flag_value != 0) or never set."""
        call("cc_probe_bounded_wait", ctypes.c_uint64(int(limit_ns)), int(flag_value))

    # -- batches (many independent contiguous elementwise programs)
    BATCH_PERSISTENT, BATCH_PER_PROGRAM, BATCH_GRAPH = 0, 1, 2

    def batch_create(self, texts: Sequence[str]) -> int:
        raws = [t.encode() for t in texts]
        arr = (ctypes.c_char_p * len(raws))(*raws)
        lens = (ctypes.c_size_t * len(raws))(*[len(r) for r in raws])
        h = c_handle()
        call("cc_batch_create", arr, lens, len(raws), ctypes.byref(h))
        return h.value

    def batch_info(self, batch: int):
        """(programs, distinct structures, registers per thread, resident blocks per SM) of a batch."""
        n, k, r, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call("cc_batch_info", c_handle(batch), ctypes.byref(n), ctypes.byref(k), ctypes.byref(r), ctypes.byref(b))
        return n.value, k.value, r.value, b.value

    def batch_bind(self, batch: int, ptrs: Sequence[int]):
        arr = (ctypes.c_uint64 * len(ptrs))(*ptrs)
        call("cc_batch_bind", c_handle(batch), arr, ctypes.c_size_t(len(ptrs)))

    def batch_run(self, batch: int, mode: int = 0, stream: int = 0):
        call("cc_batch_run", c_handle(batch), int(mode), ctypes.c_uint64(stream))

    def batch_run_ev(self, batch: int, mode: int = 0, wait=()) -> int:
        w, nw = self._wait_list(wait)
        ev = c_handle()
        call("cc_batch_run_ev", c_handle(batch), int(mode), w, nw, ctypes.byref(ev))
        return ev.value

    def batch_upload_ev(self, batch: int, host_ptrs: Sequence[int], wait=()) -> int:
        """Every bound input from pinned host memory (per program, its inputs in order)."""
        arr = (ctypes.c_void_p * max(1, len(host_ptrs)))(*host_ptrs)
        w, nw = self._wait_list(wait)
        ev = c_handle()
        call("cc_batch_upload_ev", c_handle(batch), arr, ctypes.c_size_t(len(host_ptrs)), w, nw, ctypes.byref(ev))
        return ev.value

    def batch_download_ev(self, batch: int, host_ptrs: Sequence[int], wait=()) -> int:
        """Every program's output into pinned host memory."""
        arr = (ctypes.c_void_p * max(1, len(host_ptrs)))(*host_ptrs)
        w, nw = self._wait_list(wait)
        ev = c_handle()
        call("cc_batch_download_ev", c_handle(batch), arr, ctypes.c_size_t(len(host_ptrs)), w, nw, ctypes.byref(ev))
        return ev.value

    def batch_release(self, batch: int):
        call("cc_batch_release", c_handle(batch))

    # -- events
    def event(self) -> int:
        h = c_handle()
        call("cc_event_record", ctypes.byref(h))
        return h.value

    def event_wait(self, ev: int, timeout_ns: int = 10 ** 10):
        call("cc_event_wait", c_handle(ev), ctypes.c_uint64(timeout_ns))

    def event_elapsed_ms(self, start: int, end: int) -> float:
        ms = ctypes.c_float()
        call("cc_event_elapsed", c_handle(start), c_handle(end), ctypes.byref(ms))
        return ms.value

    def event_release(self, ev: int):
        call("cc_event_release", c_handle(ev))


def codegen(ir_text: str, options: str = None) -> str:
    """The CUDA C the runtime generates for an IR text (no GPU needed); options
    as "key=value" words (block, lookahead, ring, unroll, min_blocks, asm)."""
    raw = ir_text.encode()
    opts = options.encode() if options else None
    need = ctypes.c_size_t()
    call("cc_codegen_with", raw, ctypes.c_size_t(len(raw)), opts, None, 0, ctypes.byref(need))
    buf = ctypes.create_string_buffer(need.value)
    call("cc_codegen_with", raw, ctypes.c_size_t(len(raw)), opts, buf, need.value, ctypes.byref(need))
    return buf.value.decode()


def batch_compile_check(texts, cc=(10, 3)):
    """NVRTC-compiles the batch module of these programs (no GPU needed); returns (structures, seconds)."""
    raws = [t.encode() for t in texts]
    arr = (ctypes.c_char_p * len(raws))(*raws)
    lens = (ctypes.c_size_t * len(raws))(*[len(r) for r in raws])
    k, secs = ctypes.c_int(), ctypes.c_double()
    call("cc_batch_compile_check", arr, lens, len(raws), int(cc[0]), int(cc[1]), ctypes.byref(k), ctypes.byref(secs))
    return k.value, secs.value


def compile_check(ir_text: str, cc=(10, 3), flags: int = 0, options: str = None) -> None:
    """NVRTC-compiles the generated CUDA C for sm_<cc>a (no GPU needed); raises BuildProgramFailure."""
    raw = ir_text.encode()
    call("cc_compile_check_with", raw, ctypes.c_size_t(len(raw)), int(cc[0]), int(cc[1]), ctypes.c_uint32(flags),
         options.encode() if options else None)

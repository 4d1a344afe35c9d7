"""ctypes binding of the C ABI in include/compute_cuda.h (libcomputecuda.so).

The library is built in-tree next to this file.  Every call is checked: a
non-zero status raises the exception type the reference's
``OpenCL.Exceptions.fromErrorCode`` gives the same OpenCL error code
(OpenCL/src/main/scala/com/thoughtworks/compute/OpenCL.scala:251-303).
"""

from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcomputecuda.so")

c_handle = ctypes.c_uint64
c_size = ctypes.c_size_t


class ComputeError(Exception):
    code = 0


class IllegalArgumentException(ComputeError, ValueError):
    pass


class IllegalStateException(ComputeError, RuntimeError):
    pass


class DeviceNotFound(IllegalStateException):
    pass


class MemObjectAllocationFailure(IllegalStateException):
    pass


class OutOfResources(IllegalStateException):
    pass


class BuildProgramFailure(IllegalStateException):
    pass


class InvalidValue(IllegalArgumentException):
    pass


class InvalidMemObject(IllegalArgumentException):
    pass


class InvalidProgram(IllegalArgumentException):
    pass


class InvalidKernelArgs(IllegalArgumentException):
    pass


class InvalidEvent(IllegalArgumentException):
    pass


class InvalidOperation(IllegalArgumentException):
    pass


class WaitTimeout(IllegalStateException):
    pass


class NotInitialized(IllegalStateException):
    pass


class CudaError(IllegalStateException):
    pass


class DeviceReportedError(IllegalStateException):
    pass


_ERRORS = {
    -1: DeviceNotFound,
    -4: MemObjectAllocationFailure,
    -5: OutOfResources,
    -11: BuildProgramFailure,
    -30: InvalidValue,
    -38: InvalidMemObject,
    -44: InvalidProgram,
    -52: InvalidKernelArgs,
    -58: InvalidEvent,
    -59: InvalidOperation,
    -1001: WaitTimeout,
    -1002: NotInitialized,
    -1003: CudaError,
    -1004: DeviceReportedError,
}

# name -> (restype-is-status, argtypes)
_SIGNATURES = {
    "cc_init": [ctypes.c_int, ctypes.c_uint32],
    "cc_shutdown": [],
    "cc_last_error": [ctypes.c_char_p, c_size],
    "cc_device_info": [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                       ctypes.POINTER(c_size)],
    "cc_get_stream": [ctypes.POINTER(ctypes.c_uint64)],
    "cc_set_stream": [ctypes.c_uint64],
    "cc_synchronize": [],
    "cc_config_set": [ctypes.c_char_p, ctypes.c_int64],
    "cc_config_get": [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)],
    "cc_buf_alloc": [c_size, ctypes.POINTER(c_handle)],
    "cc_buf_retain": [c_handle],
    "cc_buf_release": [c_handle],
    "cc_buf_size": [c_handle, ctypes.POINTER(c_size)],
    "cc_buf_device_ptr": [c_handle, ctypes.POINTER(ctypes.c_uint64)],
    "cc_buf_upload": [c_handle, c_size, ctypes.c_void_p, c_size],
    "cc_buf_upload_async": [c_handle, c_size, ctypes.c_void_p, c_size],
    "cc_buf_download": [c_handle, c_size, ctypes.c_void_p, c_size],
    "cc_buf_download_async": [c_handle, c_size, ctypes.c_void_p, c_size],
    "cc_host_alloc": [c_size, ctypes.POINTER(ctypes.c_void_p)],
    "cc_host_free": [ctypes.c_void_p],
    "cc_pool_stats": [ctypes.POINTER(c_size), ctypes.POINTER(c_size), ctypes.POINTER(ctypes.c_uint64),
                      ctypes.POINTER(ctypes.c_uint64)],
    "cc_pool_set_limit": [c_size],
    "cc_pool_trim": [],
    "cc_program_get": [ctypes.c_char_p, c_size, ctypes.POINTER(c_handle)],
    "cc_program_info": [c_handle, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                        ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int)],
    "cc_program_source": [c_handle, ctypes.c_char_p, c_size, ctypes.POINTER(c_size)],
    "cc_program_cache_stats": [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                               ctypes.POINTER(ctypes.c_uint64)],
    "cc_codegen": [ctypes.c_char_p, c_size, ctypes.c_char_p, c_size, ctypes.POINTER(c_size)],
    "cc_compile_check": [ctypes.c_char_p, c_size, ctypes.c_int, ctypes.c_int, ctypes.c_uint32],
    "cc_launch": [c_handle, ctypes.POINTER(c_handle), ctypes.c_int, c_handle],
    "cc_launch_ptrs": [c_handle, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64],
    "cc_launch_ev": [c_handle, ctypes.POINTER(c_handle), ctypes.c_int, c_handle, ctypes.POINTER(c_handle), ctypes.c_int,
                     ctypes.POINTER(c_handle)],
    "cc_buf_upload_ev": [c_handle, c_size, ctypes.c_void_p, c_size, ctypes.POINTER(c_handle), ctypes.c_int,
                         ctypes.POINTER(c_handle)],
    "cc_buf_download_ev": [c_handle, c_size, ctypes.c_void_p, c_size, ctypes.POINTER(c_handle), ctypes.c_int,
                           ctypes.POINTER(c_handle)],
    "cc_stream_wait_events": [ctypes.POINTER(c_handle), ctypes.c_int],
    "cc_reduce_sum_f32": [ctypes.c_uint64, c_size, ctypes.c_uint64, ctypes.c_uint64],
    "cc_reduce_sum_f32_noalloc": [ctypes.c_uint64, c_size, ctypes.c_uint64, ctypes.c_uint64],
    "cc_random": [c_handle, c_size, ctypes.c_uint32, ctypes.c_int],
    "cc_gemm_f32": [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                    ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_uint64],
    "cc_device_errors": [ctypes.POINTER(ctypes.c_int)],
    "cc_probe_bounded_wait": [ctypes.c_uint64, ctypes.c_int],
    "cc_batch_create": [ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(c_size), ctypes.c_int, ctypes.POINTER(c_handle)],
    "cc_codegen_with": [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t,
                        ctypes.POINTER(ctypes.c_size_t)],
    "cc_compile_check_with": [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                              ctypes.c_char_p],
    "cc_tune_config": [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                       ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    "cc_program_features": [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)],
    "cc_tuner_choice": [c_handle, ctypes.POINTER(ctypes.c_int)],
    "cc_tuner_set_model": [c_handle, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
    "cc_tune_create": [ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_size_t), ctypes.c_int,
                       ctypes.POINTER(c_handle)],
    "cc_tune_info": [c_handle, ctypes.POINTER(ctypes.c_int)],
    "cc_tune_launch": [c_handle, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t, ctypes.c_int,
                       ctypes.c_uint64],
    "cc_tune_time": [c_handle, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t,
                     ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                     ctypes.POINTER(ctypes.c_float)],
    "cc_tune_release": [c_handle],
    "cc_tune_compile_check": [ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_size_t), ctypes.c_int,
                              ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)],
    "cc_mlp_create": [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(c_handle)],
    "cc_mlp_info": [c_handle, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_int)],
    "cc_mlp_set_params": [c_handle, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t],
    "cc_mlp_get_params": [c_handle, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t],
    "cc_mlp_forward": [c_handle, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64],
    "cc_mlp_gradients": [c_handle, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                         ctypes.POINTER(ctypes.c_float)],
    "cc_mlp_train_step": [c_handle, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_float)],
    "cc_mlp_release": [c_handle],
    "cc_batch_info": [c_handle, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                      ctypes.POINTER(ctypes.c_int)],
    "cc_batch_bind": [c_handle, ctypes.POINTER(ctypes.c_uint64), c_size],
    "cc_batch_run": [c_handle, ctypes.c_int, ctypes.c_uint64],
    "cc_batch_run_ev": [c_handle, ctypes.c_int, ctypes.POINTER(c_handle), ctypes.c_int, ctypes.POINTER(c_handle)],
    "cc_batch_upload_ev": [c_handle, ctypes.POINTER(ctypes.c_void_p), c_size, ctypes.POINTER(c_handle), ctypes.c_int,
                           ctypes.POINTER(c_handle)],
    "cc_batch_download_ev": [c_handle, ctypes.POINTER(ctypes.c_void_p), c_size, ctypes.POINTER(c_handle),
                             ctypes.c_int, ctypes.POINTER(c_handle)],
    "cc_batch_release": [c_handle],
    "cc_batch_compile_check": [ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(c_size), ctypes.c_int, ctypes.c_int,
                               ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)],
    "cc_event_record": [ctypes.POINTER(c_handle)],
    "cc_event_query": [c_handle, ctypes.POINTER(ctypes.c_int)],
    "cc_event_wait": [c_handle, ctypes.c_uint64],
    "cc_event_elapsed": [c_handle, c_handle, ctypes.POINTER(ctypes.c_float)],
    "cc_event_release": [c_handle],
}

_lib = None
_lock = threading.Lock()


def load():
    """Loads libcomputecuda.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError("libcomputecuda.so is not built (run __graft_entry__.build())")
            lib = ctypes.CDLL(LIB_PATH)
            for name, argtypes in _SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = argtypes
                fn.restype = ctypes.c_int
            _lib = lib
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1 << 16)
    load().cc_last_error(buf, len(buf))
    return buf.value.decode("utf-8", "replace")


def check(status: int, what: str = "") -> None:
    if status == 0:
        return
    cls = _ERRORS.get(status, CudaError)
    err = cls("%s%s (status %d)" % ((what + ": ") if what else "", last_error(), status))
    err.code = status
    raise err


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)

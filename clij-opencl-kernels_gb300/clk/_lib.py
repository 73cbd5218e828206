"""ctypes binding of include/clk.h (libclk_gb300.so, built in-tree).

There is no fallback: if the library was not built, importing the binding
raises, naming the build command.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "_build" / "libclk_gb300.so"

# clk_status
OK, UNKNOWN_KERNEL, BAD_ARG, UNSUPPORTED_DTYPE, OOM, LAUNCH_FAILED, TIMEOUT, NO_DEVICE, BUSY, CANCELLED = range(10)
STATUS_NAMES = ["CLK_OK", "CLK_UNKNOWN_KERNEL", "CLK_BAD_ARG", "CLK_UNSUPPORTED_DTYPE", "CLK_OOM",
                "CLK_LAUNCH_FAILED", "CLK_TIMEOUT", "CLK_NO_DEVICE", "CLK_BUSY", "CLK_CANCELLED"]
# clk_dtype
U8, I8, U16, I16, F32 = range(5)
# clk_arg_kind
ARG_IMAGE, ARG_INT, ARG_FLOAT = range(3)


class clk_image(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("dtype", C.c_int32), ("ndim", C.c_int32),
                ("width", C.c_int64), ("height", C.c_int64), ("depth", C.c_int64)]


class clk_arg(C.Structure):
    _fields_ = [("name", C.c_char_p), ("kind", C.c_int32), ("i", C.c_int32), ("f", C.c_float),
                ("image", clk_image)]


class clk_define(C.Structure):
    _fields_ = [("name", C.c_char_p), ("value", C.c_char_p)]


class clk_op(C.Structure):
    _fields_ = [("kernel", C.c_char_p), ("kind", C.c_int32), ("N", C.c_int32 * 3), ("s", C.c_float * 3),
                ("iterations", C.c_int32)]


OP_SEPARABLE, OP_KERNEL, OP_MORPHOLOGY = range(3)


class clk_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("bytes_in_use", C.c_int64), ("bytes_peak", C.c_int64), ("inflight", C.c_int32),
                ("queued", C.c_int32), ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("voxel_steps", C.c_double), ("busy_s", C.c_double), ("cancelled", C.c_uint64)]


class ClkError(RuntimeError):
    """A non-OK clk_status; .status holds the code."""

    def __init__(self, status: int, message: str):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {message}")
        self.status = status


EXPORTS = ["clk_execute", "clk_separable", "clk_separable_noalloc", "clk_morphology", "clk_batch_create",
           "clk_batch_run", "clk_batch_run_plain", "clk_batch_run_per_kernel", "clk_batch_launches", "clk_batch_destroy", "clk_server_create",
           "clk_server_submit", "clk_server_wait", "clk_server_cancel", "clk_server_drain", "clk_server_get_stats",
           "clk_server_destroy", "clk_supported", "clk_last_error_string", "clk_version",
           "clk_kernel_count", "clk_kernel_name", "clk_launch_count", "clk_host_image_pointer"]

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with "
                          f"`python clij-opencl-kernels_gb300/build.py` (or __graft_entry__.build())")
    lib = C.CDLL(str(LIB_PATH))
    lib.clk_execute.argtypes = [C.c_char_p, C.POINTER(clk_arg), C.c_size_t, C.POINTER(C.c_size_t),
                                C.POINTER(clk_define), C.c_size_t, C.c_void_p]
    lib.clk_execute.restype = C.c_int
    lib.clk_separable.argtypes = [C.c_char_p, C.POINTER(clk_image), C.POINTER(clk_image), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_float), C.POINTER(clk_define), C.c_size_t, C.c_void_p]
    lib.clk_separable.restype = C.c_int
    lib.clk_morphology.argtypes = [C.c_char_p, C.POINTER(clk_image), C.POINTER(clk_image), C.c_int32,
                                   C.POINTER(clk_define), C.c_size_t, C.c_void_p]
    lib.clk_morphology.restype = C.c_int
    lib.clk_batch_create.argtypes = [C.POINTER(clk_op), C.c_int32, C.POINTER(clk_image), C.POINTER(clk_image),
                                     C.c_int32, C.POINTER(clk_define), C.c_size_t, C.c_void_p,
                                     C.POINTER(C.c_void_p)]
    lib.clk_batch_create.restype = C.c_int
    lib.clk_batch_run.argtypes = [C.c_void_p, C.c_void_p]
    lib.clk_batch_run.restype = C.c_int
    lib.clk_batch_run_plain.argtypes = [C.c_void_p, C.c_void_p]
    lib.clk_batch_run_plain.restype = C.c_int
    lib.clk_batch_run_per_kernel.argtypes = [C.c_void_p, C.c_void_p]
    lib.clk_batch_run_per_kernel.restype = C.c_int
    lib.clk_batch_launches.argtypes = [C.c_void_p]
    lib.clk_batch_launches.restype = C.c_int32
    lib.clk_batch_destroy.argtypes = [C.c_void_p]
    lib.clk_batch_destroy.restype = None
    lib.clk_server_create.argtypes = [C.c_int32, C.c_int64, C.POINTER(C.c_void_p)]
    lib.clk_server_create.restype = C.c_int
    lib.clk_server_submit.argtypes = [C.c_void_p, C.POINTER(clk_op), C.c_int32, C.POINTER(clk_image),
                                      C.POINTER(clk_image), C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]
    lib.clk_server_submit.restype = C.c_int
    lib.clk_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_int32, C.POINTER(C.c_double)]
    lib.clk_server_wait.restype = C.c_int
    lib.clk_server_drain.argtypes = [C.c_void_p, C.c_int32]
    lib.clk_server_drain.restype = C.c_int
    lib.clk_server_cancel.argtypes = [C.c_void_p, C.c_uint64]
    lib.clk_server_cancel.restype = C.c_int
    lib.clk_server_get_stats.argtypes = [C.c_void_p, C.POINTER(clk_server_stats)]
    lib.clk_server_get_stats.restype = C.c_int
    lib.clk_server_destroy.argtypes = [C.c_void_p]
    lib.clk_server_destroy.restype = None
    lib.clk_supported.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32]
    lib.clk_supported.restype = C.c_int
    lib.clk_last_error_string.restype = C.c_char_p
    lib.clk_version.restype = C.c_char_p
    lib.clk_kernel_count.restype = C.c_int
    lib.clk_kernel_name.argtypes = [C.c_int]
    lib.clk_kernel_name.restype = C.c_char_p
    lib.clk_launch_count.restype = C.c_uint64
    lib.clk_host_image_pointer.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    lib.clk_host_image_pointer.restype = C.c_int
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        msg = load().clk_last_error_string().decode(errors="replace")
        raise ClkError(status, msg)

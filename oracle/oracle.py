"""ctypes front end of the oracle.  TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
never by the product path.  Two libraries:

  port  oracle/_build/libclk_oracle.so  -- oracle/clk_oracle.cpp, this
        project's restatement of the reference kernels (+ FP64 oracle);
  ref   oracle/_ref/libclkref.so        -- the reference's own .cl kernels
        compiled as C++ by oracle/build_ref.py (absent where the reference
        checkout was never available).

Arrays are numpy, C-ordered with shape (depth, height, width) for 3-D and
(height, width) for 2-D, i.e. x fastest as in the reference's buffers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libclk_oracle.so"
REF_LIB = HERE / "_ref" / "libclkref.so"

DTYPES = [np.uint8, np.int8, np.uint16, np.int16, np.float32]
FLAG_RTE = 1
FLAG_SOBEL_NARROW = 2

KERNELS = [
    "gaussian_blur_separable_2d", "gaussian_blur_separable_3d",
    "mean_separable_2d", "mean_separable_3d",
    "minimum_separable_2d", "minimum_separable_3d",
    "maximum_separable_2d", "maximum_separable_3d",
    "median_box_2d", "median_box_3d", "median_sphere_2d", "median_sphere_3d",
    "erode_box_2d", "erode_box_3d", "erode_sphere_2d", "erode_sphere_3d",
    "dilate_box_2d", "dilate_box_3d", "dilate_sphere_2d", "dilate_sphere_3d",
    "sobel_2d", "sobel_3d",
    "minimum_sphere_2d", "minimum_sphere_3d", "maximum_sphere_2d", "maximum_sphere_3d",
    "mean_sphere_2d", "mean_sphere_3d",
    "minimum_slice_by_slice_sphere_3d", "maximum_slice_by_slice_sphere_3d", "mean_slice_by_slice_sphere_3d",
    "median_slice_by_slice_box_3d", "median_slice_by_slice_sphere_3d",
    "erode_box_slice_by_slice_3d", "erode_sphere_slice_by_slice_3d",
    "dilate_box_slice_by_slice_3d", "dilate_sphere_slice_by_slice_3d",
    "greater_constant_2d", "greater_constant_3d", "copy_2d", "copy_3d",
    "gradient_x_2d", "gradient_y_2d", "gradient_x_3d", "gradient_y_3d", "gradient_z_3d",
    "laplace_box_2d", "laplace_box_3d", "laplace_diamond_2d", "laplace_diamond_3d",
    "convolve_2d", "convolve_3d",
]


def dtype_code(dt) -> int:
    dt = np.dtype(dt)
    for i, t in enumerate(DTYPES):
        if np.dtype(t) == dt:
            return i
    raise TypeError(f"unsupported pixel type {dt}")


def build_port(cxx: str = "g++") -> Path:
    src = HERE / "clk_oracle.cpp"
    PORT_LIB.parent.mkdir(exist_ok=True)
    if not PORT_LIB.exists() or PORT_LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run([cxx, "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                        "-std=c++17", "-shared", str(src), "-o", str(PORT_LIB)], check=True)
    return PORT_LIB


_port = None
_ref = None


def port() -> C.CDLL:
    global _port
    if _port is None:
        build_port()
        lib = C.CDLL(str(PORT_LIB))
        i3 = C.POINTER(C.c_int)
        lib.clko_execute.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, i3, C.c_void_p, i3, i3,
                                     i3, C.POINTER(C.c_float), C.c_int, C.c_int]
        lib.clko_separable.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, i3, C.c_int,
                                       i3, C.POINTER(C.c_float), C.c_int, C.c_int]
        lib.clko_fp64.argtypes = [C.c_char_p, C.c_int, C.c_void_p, i3, C.c_int, i3, C.POINTER(C.c_float),
                                  C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        lib.clko_median_offsets.argtypes = [C.c_int] * 5 + [i3, C.c_int]
        _port = lib
    return _port


class _RefCall(C.Structure):
    _fields_ = [("src", C.c_void_p), ("sw", C.c_int), ("sh", C.c_int), ("sd", C.c_int),
                ("dst", C.c_void_p), ("dw", C.c_int), ("dh", C.c_int), ("dd", C.c_int),
                ("gx", C.c_int), ("gy", C.c_int), ("gz", C.c_int),
                ("ia", C.c_int * 4), ("fa", C.c_float * 4), ("nthreads", C.c_int),
                ("kimg", C.c_void_p), ("kw", C.c_int), ("kh", C.c_int), ("kd", C.c_int)]


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            from . import build_ref  # noqa: F401  (package-relative use)
        _ref = C.CDLL(str(REF_LIB))
        for k in KERNELS:
            getattr(_ref, f"clkref_{k}").argtypes = [C.c_int, C.c_int, C.POINTER(_RefCall)]
    return _ref


def _xyz(a: np.ndarray):
    if a.ndim == 2:
        return [a.shape[1], a.shape[0], 1]
    return [a.shape[2], a.shape[1], a.shape[0]]


def _ia(v):
    v = list(v) + [0] * (4 - len(v))
    return (C.c_int * 4)(*v)


def _fa(v):
    v = list(v) + [0.0] * (4 - len(v))
    return (C.c_float * 4)(*v)


def execute(kernel: str, src: np.ndarray, dst_dtype, ints=(), floats=(), global_range=None,
            flags: int = 0, impl: str = "port", nthreads: int = 0, dst: np.ndarray | None = None,
            kernel_image: np.ndarray | None = None) -> np.ndarray:
    """One launch of `kernel` on the CPU; returns dst (fresh zeros unless given).
    kernel_image: the float32 kernel of convolve_{2d,3d}."""
    src = np.ascontiguousarray(src)
    if kernel.startswith("convolve"):
        return _convolve(kernel, src, dst_dtype, kernel_image, global_range, flags, impl, nthreads, dst)
    if dst is None:
        dst = np.zeros(src.shape, dtype=dst_dtype)
    sx, dx = _xyz(src), _xyz(dst)
    g = list(global_range) if global_range is not None else dx
    sdt, ddt = dtype_code(src.dtype), dtype_code(dst.dtype)
    if impl == "ref":
        call = _RefCall(src.ctypes.data, *sx, dst.ctypes.data, *dx, *g, _ia(ints), _fa(floats), nthreads)
        rc = getattr(ref(), f"clkref_{kernel}")(sdt, ddt, C.byref(call))
    else:
        i3 = lambda v: (C.c_int * 3)(*v)  # noqa: E731
        rc = port().clko_execute(kernel.encode(), sdt, ddt, src.ctypes.data, i3(sx), dst.ctypes.data, i3(dx),
                                 i3(g), _ia(ints), _fa(floats), flags, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle {impl} {kernel} failed ({rc})")
    return dst


def separable(kernel: str, src: np.ndarray, dst_dtype, N, s=(0.0, 0.0, 0.0), flags: int = 0,
              impl: str = "port", nthreads: int = 0) -> np.ndarray:
    """Whole separable filter X->Y(->Z) with dst-typed temporaries."""
    src = np.ascontiguousarray(src)
    ndim = src.ndim
    N = list(N) + [1] * (3 - len(N))
    s = list(s) + [0.0] * (3 - len(s))
    if impl == "ref":
        # the orchestration is the host's: three launches of the ref kernel
        cur = src
        for d in range(ndim):
            skip = N[d] <= 1 or (kernel.startswith("gaussian") and not s[d] > 0)
            if skip:
                out = _copy_convert(cur, dst_dtype, flags)
            else:
                out = execute(kernel, cur, dst_dtype, ints=(d, N[d]), floats=(s[d],), impl="ref",
                              nthreads=nthreads)
            cur = out
        return cur
    dst = np.zeros(src.shape, dtype=dst_dtype)
    i3 = lambda v: (C.c_int * 3)(*v)  # noqa: E731
    rc = port().clko_separable(kernel.encode(), dtype_code(src.dtype), dtype_code(dst.dtype), src.ctypes.data,
                               dst.ctypes.data, i3(_xyz(src)), ndim, i3(N), (C.c_float * 3)(*s), flags, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle separable {kernel} failed ({rc})")
    return dst


def _copy_convert(src: np.ndarray, dst_dtype, flags: int) -> np.ndarray:
    """copy_3d_x.cl semantics in numpy: float, then saturate + truncate."""
    dst_dtype = np.dtype(dst_dtype)
    v = src.astype(np.float32)
    if dst_dtype == np.float32:
        return v.copy()
    info = np.iinfo(dst_dtype)
    v = np.nan_to_num(v.astype(np.float64), nan=0.0)
    v = np.clip(v, info.min, info.max)
    v = np.rint(v) if flags & FLAG_RTE else np.trunc(v)
    return v.astype(dst_dtype)


def fp64(kernel: str, src: np.ndarray, N=(1, 1, 1), s=(0.0, 0.0, 0.0), flags: int = 0, nthreads: int = 0):
    """FP64 oracle: returns (value, scale) as float64 arrays of src's shape."""
    src = np.ascontiguousarray(src)
    N = list(N) + [1] * (3 - len(N))
    s = list(s) + [0.0] * (3 - len(s))
    out = np.zeros(src.shape, np.float64)
    scale = np.zeros(src.shape, np.float64)
    i3 = lambda v: (C.c_int * 3)(*v)  # noqa: E731
    rc = port().clko_fp64(kernel.encode(), dtype_code(src.dtype), src.ctypes.data, i3(_xyz(src)), src.ndim, i3(N),
                          (C.c_float * 3)(*s), flags, out.ctypes.data, scale.ctypes.data, nthreads)
    if rc != 0:
        raise RuntimeError(f"fp64 oracle {kernel} failed ({rc})")
    return out, scale


def median_offsets(sphere: bool, ndim: int, Nx: int, Ny: int, Nz: int = 1) -> np.ndarray:
    buf = (C.c_int * (3 * 4096))()
    n = port().clko_median_offsets(int(sphere), ndim, Nx, Ny, Nz, buf, 4096)
    return np.array(buf[:3 * min(n, 4096)], dtype=np.int32).reshape(-1, 3)


def nthreads_default() -> int:
    return os.cpu_count() or 1


def _convolve(kernel, src, dst_dtype, kimg, global_range, flags, impl, nthreads, dst):
    if kimg is None:
        raise ValueError("convolve needs kernel_image")
    kimg = np.ascontiguousarray(kimg, dtype=np.float32)
    if dst is None:
        dst = np.zeros(src.shape, dtype=dst_dtype)
    sx, dx, kx = _xyz(src), _xyz(dst), _xyz(kimg)
    g = list(global_range) if global_range is not None else dx
    sdt, ddt = dtype_code(src.dtype), dtype_code(dst.dtype)
    if impl == "ref":
        call = _RefCall(src.ctypes.data, *sx, dst.ctypes.data, *dx, *g, _ia(()), _fa(()), nthreads,
                        kimg.ctypes.data, *kx)
        rc = getattr(ref(), f"clkref_{kernel}")(sdt, ddt, C.byref(call))
    else:
        i3 = lambda v: (C.c_int * 3)(*v)  # noqa: E731
        lib = port()
        lib.clko_convolve.argtypes = [C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int), C.c_void_p,
                                      C.POINTER(C.c_int), C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.c_int, C.c_int]
        rc = lib.clko_convolve(sdt, ddt, src.ctypes.data, i3(sx), kimg.ctypes.data, i3(kx), dst.ctypes.data,
                               i3(dx), i3(g), flags, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle {impl} {kernel} failed ({rc})")
    return dst

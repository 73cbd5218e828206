"""Python mirror of the reference's call surface, over the C ABI.

Two levels, as in the reference's ecosystem:

* ``execute(kernel_name, params, global_range)`` -- the drop-in for one .cl
  kernel launch: the kernel's name and its named parameters (``src``/``dst``
  images, ``dim``/``N``/``s``/``Nx``/``Ny``/``Nz`` scalars), bound by name.
  This is how CLIc / clij-clearcl enqueue e.g. ``gaussian_blur_separable_3d``
  (kernels/gaussian_blur_separable_3d_x.cl:6-12).
* Orchestrator functions in pyclesperanto's vocabulary (``gaussian_blur``,
  ``mean_box``, ``minimum_box``, ``maximum_box``, ``median_box``,
  ``median_sphere``, ``erode_box`` ... ``sobel``) that pick the kernel, the
  per-axis N and run the separable passes.

Images are CUDA tensors (torch is only the device-memory container here),
C-contiguous, shape (depth, height, width) or (height, width): x fastest,
exactly the reference's buffer layout.  A pinned host tensor is accepted too
(zero-copy: the kernel stores its output straight into host memory over the
host link, which fuses the pull of the result into the filter).  Pixel types: uint8, int8, uint16,
int16, float32.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Mapping

import torch

from . import _lib as L

_DT = {torch.uint8: L.U8, torch.int8: L.I8, torch.uint16: L.U16, torch.int16: L.I16, torch.float32: L.F32}
_TORCH = {v: k for k, v in _DT.items()}


def dtype_code(dt: torch.dtype) -> int:
    try:
        return _DT[dt]
    except KeyError:
        raise L.ClkError(L.UNSUPPORTED_DTYPE, f"pixel type {dt} is not one of {list(_DT)}") from None


def torch_dtype(code: int) -> torch.dtype:
    return _TORCH[code]


def host_image_pointer(t: torch.Tensor) -> int:
    """The address under which kernels reach a pinned host tensor
    (clk_host_image_pointer); BAD_ARG for pageable memory."""
    lib = L.load()
    out = C.c_void_p()
    L.check(lib.clk_host_image_pointer(C.c_void_p(t.data_ptr()), C.byref(out)))
    return int(out.value)


def image_of(t: torch.Tensor) -> L.clk_image:
    """A CUDA tensor, or a pinned host tensor (zero-copy: the kernel reads or
    writes host memory over the host link; meant for outputs)."""
    if not isinstance(t, torch.Tensor):
        raise L.ClkError(L.BAD_ARG, "images must be CUDA tensors or pinned host tensors")
    if not t.is_contiguous():
        raise L.ClkError(L.BAD_ARG, "images must be C-contiguous (x fastest)")
    if t.dim() not in (2, 3):
        raise L.ClkError(L.BAD_ARG, f"images are 2-D or 3-D, got shape {tuple(t.shape)}")
    if t.is_cuda:
        ptr = t.data_ptr()
    elif t.device.type == "cpu" and t.is_pinned():
        ptr = host_image_pointer(t)
    else:
        raise L.ClkError(L.BAD_ARG, "images must be CUDA tensors or pinned host tensors (pin_memory())")
    if t.dim() == 2:
        return L.clk_image(ptr, dtype_code(t.dtype), 2, t.shape[1], t.shape[0], 1)
    if t.dim() == 3:
        return L.clk_image(ptr, dtype_code(t.dtype), 3, t.shape[2], t.shape[1], t.shape[0])
    raise L.ClkError(L.BAD_ARG, f"images are 2-D or 3-D, got shape {tuple(t.shape)}")


def _defines(defines: Mapping[str, object] | None):
    if not defines:
        return None, 0, []
    keep = [(str(k).encode(), str(v).encode()) for k, v in defines.items()]
    arr = (L.clk_define * len(keep))(*[L.clk_define(k, v) for k, v in keep])
    return arr, len(keep), keep


def _stream(stream) -> int | None:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def execute(kernel_name: str, params: Mapping[str, object], global_range=None,
            defines: Mapping[str, object] | None = None, stream=None) -> None:
    """Launch one reference kernel by name with named parameters.

    params maps parameter names to CUDA tensors (images), ints or floats.
    global_range: (x, y[, z]) work size; default the dst extent.
    """
    lib = L.load()
    args, keep = [], []
    for name, v in params.items():
        nb = name.encode()
        keep.append(nb)
        if isinstance(v, torch.Tensor):
            args.append(L.clk_arg(nb, L.ARG_IMAGE, 0, 0.0, image_of(v)))
        elif isinstance(v, bool) or not isinstance(v, (int, float)):
            raise L.ClkError(L.BAD_ARG, f"parameter {name!r}: unsupported value {v!r}")
        elif isinstance(v, int):
            args.append(L.clk_arg(nb, L.ARG_INT, int(v), 0.0, L.clk_image()))
        else:
            args.append(L.clk_arg(nb, L.ARG_FLOAT, 0, float(v), L.clk_image()))
    arr = (L.clk_arg * len(args))(*args)
    g = None
    if global_range is not None:
        gr = list(global_range) + [1] * (3 - len(global_range))
        g = (C.c_size_t * 3)(*gr)
    darr, nd, _k = _defines(defines)
    L.check(lib.clk_execute(kernel_name.encode(), arr, len(args), g, darr, nd, _stream(stream)))


def separable(kernel_name: str, src: torch.Tensor, dst: torch.Tensor, N, s=(0.0, 0.0, 0.0),
              defines: Mapping[str, object] | None = None, stream=None) -> torch.Tensor:
    """The whole X->Y(->Z) separable filter (the orchestrator's driver)."""
    lib = L.load()
    n = list(N) + [1] * (3 - len(N))
    sg = [float(v) for v in s] + [0.0] * (3 - len(s))
    di, si = image_of(dst), image_of(src)
    darr, nd, _k = _defines(defines)
    L.check(lib.clk_separable(kernel_name.encode(), C.byref(di), C.byref(si), (C.c_int32 * 3)(*n),
                              (C.c_float * 3)(*sg), darr, nd, _stream(stream)))
    return dst


def supported(kernel_name: str, src_dtype: torch.dtype, dst_dtype: torch.dtype, ndim: int) -> bool:
    return bool(L.load().clk_supported(kernel_name.encode(), dtype_code(src_dtype), dtype_code(dst_dtype), ndim))


def kernel_names() -> list[str]:
    lib = L.load()
    return [lib.clk_kernel_name(i).decode() for i in range(lib.clk_kernel_count())]


def version() -> str:
    return L.load().clk_version().decode()


def launch_count() -> int:
    return int(L.load().clk_launch_count())


# ----------------------------------------------------------------- orchestrator

def sigma_to_n(sigma: float) -> int:
    """Window N of a Gaussian of standard deviation sigma: radius ceil(3 sigma)."""
    return 2 * int(math.ceil(3.0 * float(sigma))) + 1 if sigma > 0 else 1


def _out(src: torch.Tensor, dst, dtype=None) -> torch.Tensor:
    if dst is not None:
        return dst
    return torch.empty_like(src, dtype=dtype or src.dtype)


def _suffix(t: torch.Tensor) -> str:
    return "_2d" if t.dim() == 2 else "_3d"


def gaussian_blur(src, dst=None, sigma_x=0.0, sigma_y=0.0, sigma_z=0.0, stream=None, defines=None):
    dst = _out(src, dst, torch.float32)
    sig = (sigma_x, sigma_y, sigma_z)
    return separable("gaussian_blur_separable" + _suffix(src), src, dst, [sigma_to_n(v) for v in sig], sig,
                     defines, stream)


def _box(kernel, src, dst, rx, ry, rz, stream, defines):
    dst = _out(src, dst)
    r = (rx, ry, rz)
    return separable(kernel + _suffix(src), src, dst, [2 * int(v) + 1 for v in r], [float(v) for v in r],
                     defines, stream)


def mean_box(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _box("mean_separable", src, dst, radius_x, radius_y, radius_z, stream, defines)


def minimum_box(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _box("minimum_separable", src, dst, radius_x, radius_y, radius_z, stream, defines)


def maximum_box(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _box("maximum_separable", src, dst, radius_x, radius_y, radius_z, stream, defines)


def _median(kind, src, dst, rx, ry, rz, stream, defines):
    dst = _out(src, dst)
    p = {"dst": dst, "src": src, "Nx": 2 * int(rx) + 1, "Ny": 2 * int(ry) + 1}
    if src.dim() == 3:
        p["Nz"] = 2 * int(rz) + 1
    execute(kind + _suffix(src), p, defines=defines, stream=stream)
    return dst


def median_box(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _median("median_box", src, dst, radius_x, radius_y, radius_z, stream, defines)


def median_sphere(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _median("median_sphere", src, dst, radius_x, radius_y, radius_z, stream, defines)


def morphology(kernel_name: str, src: torch.Tensor, dst: torch.Tensor, iterations: int = 1,
               defines: Mapping[str, object] | None = None, stream=None) -> torch.Tensor:
    """`iterations` successive launches of an r=1 erode/dilate kernel (the
    kernels have no radius parameter, erode_sphere_3d_x.cl:3-6); byte images
    run two iterations fused per pass."""
    lib = L.load()
    di, si = image_of(dst), image_of(src)
    darr, nd, _k = _defines(defines)
    L.check(lib.clk_morphology(kernel_name.encode(), C.byref(di), C.byref(si), int(iterations), darr, nd,
                               _stream(stream)))
    return dst


def _morph(kind, src, dst, radius, stream, defines):
    """Radius r = r successive launches of the r=1 kernel."""
    dst = _out(src, dst)
    return morphology(kind + _suffix(src), src, dst, int(radius), defines, stream)


def erode_box(src, dst=None, radius=1, stream=None, defines=None):
    return _morph("erode_box", src, dst, radius, stream, defines)


def erode_sphere(src, dst=None, radius=1, stream=None, defines=None):
    return _morph("erode_sphere", src, dst, radius, stream, defines)


def dilate_box(src, dst=None, radius=1, stream=None, defines=None):
    return _morph("dilate_box", src, dst, radius, stream, defines)


def dilate_sphere(src, dst=None, radius=1, stream=None, defines=None):
    return _morph("dilate_sphere", src, dst, radius, stream, defines)


def sobel(src, dst=None, stream=None, defines=None):
    dst = _out(src, dst, torch.float32)
    execute("sobel" + _suffix(src), {"dst": dst, "src": src}, defines=defines, stream=stream)
    return dst


def _sphere(kind, src, dst, rx, ry, rz, stream, defines):
    dst = _out(src, dst)
    p = {"dst": dst, "src": src, "Nx": 2 * int(rx) + 1, "Ny": 2 * int(ry) + 1}
    if src.dim() == 3:
        p["Nz"] = 2 * int(rz) + 1
    execute(kind + _suffix(src), p, defines=defines, stream=stream)
    return dst


def minimum_sphere(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _sphere("minimum_sphere", src, dst, radius_x, radius_y, radius_z, stream, defines)


def maximum_sphere(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _sphere("maximum_sphere", src, dst, radius_x, radius_y, radius_z, stream, defines)


def mean_sphere(src, dst=None, radius_x=1, radius_y=1, radius_z=1, stream=None, defines=None):
    return _sphere("mean_sphere", src, dst, radius_x, radius_y, radius_z, stream, defines)


def greater_constant(src, dst=None, scalar=0.0, stream=None, defines=None):
    dst = _out(src, dst, torch.uint8)
    execute("greater_constant" + _suffix(src), {"src1": src, "scalar": float(scalar), "dst": dst},
            defines=defines, stream=stream)
    return dst


def copy(src, dst=None, stream=None, defines=None):
    dst = _out(src, dst)
    execute("copy" + _suffix(src), {"dst": dst, "src": src}, defines=defines, stream=stream)
    return dst


def gradient(src, dst=None, axis="x", stream=None, defines=None):
    dst = _out(src, dst, torch.float32)
    execute(f"gradient_{axis}" + _suffix(src), {"dst": dst, "src": src}, defines=defines, stream=stream)
    return dst


def laplace(src, dst=None, kind="box", stream=None, defines=None):
    dst = _out(src, dst, torch.float32)
    execute(f"laplace_{kind}" + _suffix(src), {"dst": dst, "src": src}, defines=defines, stream=stream)
    return dst


def convolve(src, kernel, dst=None, stream=None, defines=None):
    """src * a float kernel image (convolve_3d_x.cl)."""
    dst = _out(src, dst, torch.float32)
    execute("convolve" + _suffix(src), {"src": src, "kernelImage": kernel.float().contiguous(), "dst": dst},
            defines=defines, stream=stream)
    return dst


# ----------------------------------------------------------------- batch

def op_separable(kernel: str, N, s=(0.0, 0.0, 0.0)) -> dict:
    """A separable step: kernel base name without _2d/_3d, per-axis N and s."""
    return {"kernel": kernel, "kind": L.OP_SEPARABLE, "N": list(N), "s": list(s)}


def op_kernel(kernel: str, N=(1, 1, 1)) -> dict:
    """A one-launch step (median_box / median_sphere with Nx, Ny, Nz; sobel)."""
    return {"kernel": kernel, "kind": L.OP_KERNEL, "N": list(N)}


def op_morphology(kernel: str, iterations: int = 1) -> dict:
    """An erode/dilate step: the r=1 kernel applied `iterations` times."""
    return {"kernel": kernel, "kind": L.OP_MORPHOLOGY, "iterations": int(iterations)}


class Batch:
    """A pipeline of steps over many images (clk_batch_*): one persistent
    launch per step and pixel type over a tile work list, captured once as a
    CUDA graph; results equal per-image plain calls."""

    def __init__(self, ops, srcs, dsts, defines=None, stream=None):
        lib = L.load()
        if len(srcs) != len(dsts):
            raise L.ClkError(L.BAD_ARG, "srcs and dsts differ in length")
        self._keep = []
        arr = (L.clk_op * len(ops))()
        for k, o in enumerate(ops):
            name = o["kernel"].encode()
            self._keep.append(name)
            n = list(o.get("N", (1, 1, 1))) + [1] * (3 - len(o.get("N", ())))
            sg = [float(v) for v in o.get("s", (0.0, 0.0, 0.0))] + [0.0] * (3 - len(o.get("s", ())))
            arr[k] = L.clk_op(name, o["kind"], (C.c_int32 * 3)(*n[:3]), (C.c_float * 3)(*sg[:3]),
                              int(o.get("iterations", 1)))
        si = (L.clk_image * len(srcs))(*[image_of(t) for t in srcs])
        di = (L.clk_image * len(dsts))(*[image_of(t) for t in dsts])
        darr, nd, self._dk = _defines(defines)
        h = C.c_void_p()
        L.check(lib.clk_batch_create(arr, len(ops), si, di, len(srcs), darr, nd, _stream(stream), C.byref(h)))
        self._h = h
        self._tensors = (list(srcs), list(dsts))  # keep the buffers alive

    def run(self, stream=None):
        L.check(L.load().clk_batch_run(self._h, _stream(stream)))

    def run_plain(self, stream=None):
        L.check(L.load().clk_batch_run_plain(self._h, _stream(stream)))

    def run_per_kernel(self, stream=None):
        L.check(L.load().clk_batch_run_per_kernel(self._h, _stream(stream)))

    @property
    def launches(self) -> int:
        return int(L.load().clk_batch_launches(self._h))

    def close(self):
        if getattr(self, "_h", None):
            L.load().clk_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ops_array(ops, keep):
    arr = (L.clk_op * len(ops))()
    for k, o in enumerate(ops):
        name = o["kernel"].encode()
        keep.append(name)
        n = list(o.get("N", (1, 1, 1))) + [1] * (3 - len(o.get("N", ())))
        sg = [float(v) for v in o.get("s", (0.0, 0.0, 0.0))] + [0.0] * (3 - len(o.get("s", ())))
        arr[k] = L.clk_op(name, o["kind"], (C.c_int32 * 3)(*n[:3]), (C.c_float * 3)(*sg[:3]),
                          int(o.get("iterations", 1)))
    return arr


class Server:
    """The served form (clk_server_*): requests are admitted in arrival
    order as soon as a slot and HBM budget are free, run concurrently on
    their own streams, and report their latency."""

    def __init__(self, slots: int = 8, hbm_budget_bytes: int = 64 << 30):
        h = C.c_void_p()
        L.check(L.load().clk_server_create(int(slots), int(hbm_budget_bytes), C.byref(h)))
        self._h = h
        self._keep = {}

    def submit(self, ops, src: torch.Tensor, dst: torch.Tensor, host_in=None, host_out=None) -> int:
        keep = [src, dst, host_in, host_out]
        arr = _ops_array(ops, keep)
        si, di = image_of(src), image_of(dst)
        t = C.c_uint64()
        hin = host_in.data_ptr() if host_in is not None else None
        hout = host_out.data_ptr() if host_out is not None else None
        L.check(L.load().clk_server_submit(self._h, arr, len(ops), C.byref(si), C.byref(di), hin, hout,
                                           C.byref(t)))
        self._keep[t.value] = keep
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000) -> float:
        lat = C.c_double()
        st = L.load().clk_server_wait(self._h, ticket, int(timeout_ms), C.byref(lat))
        if st != L.TIMEOUT:
            self._keep.pop(ticket, None)
        L.check(st)
        return lat.value

    def cancel(self, ticket: int):
        """Cancel a queued request (CLK_BUSY once it runs on the device)."""
        L.check(L.load().clk_server_cancel(self._h, ticket))

    def drain(self, timeout_ms: int = 600000):
        L.check(L.load().clk_server_drain(self._h, int(timeout_ms)))

    def stats(self) -> dict:
        s = L.clk_server_stats()
        L.check(L.load().clk_server_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def close(self):
        if getattr(self, "_h", None):
            L.load().clk_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""The C ABI without a GPU: the library loads, exports what include/clk.h
declares, and its host-side validation returns the documented statuses
(argument binding by name, kinds, extents, ranges, defines)."""
import ctypes as C
import re

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def L():
    from clk import _lib
    _lib.load()
    return _lib


def declared_functions():
    text = (ROOT / "include" / "clk.h").read_text()
    return sorted(set(re.findall(r"^\S[^;(]*?\b(clk_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(L):
    lib = L.load()
    names = declared_functions()
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(L.EXPORTS) | set(names)


def test_registry_lists_the_22_reference_kernels(L):
    from oracle.oracle import KERNELS
    import clk
    assert sorted(clk.kernel_names()) == sorted(KERNELS)
    assert "sm_103a" in clk.version()


FAKE = 0x1000  # never dereferenced: every case below fails validation first


def img(dt=2, ndim=3, w=8, h=8, d=8, ptr=FAKE):
    from clk import _lib
    return _lib.clk_image(ptr, dt, ndim, w, h, d)


def run(L, name, args, global_range=None, defines=None):
    lib = L.load()
    arr = (L.clk_arg * len(args))(*args)
    g = (C.c_size_t * 3)(*global_range) if global_range else None
    if defines:
        darr = (L.clk_define * len(defines))(*[L.clk_define(k.encode(), v.encode()) for k, v in defines])
        nd = len(defines)
    else:
        darr, nd = None, 0
    st = lib.clk_execute(name.encode() if name else None, arr, len(args), g, darr, nd, None)
    return st, lib.clk_last_error_string().decode()


def a_img(L, name, im):
    return L.clk_arg(name.encode(), L.ARG_IMAGE, 0, 0.0, im)


def a_int(L, name, v):
    return L.clk_arg(name.encode(), L.ARG_INT, v, 0.0, L.clk_image())


def a_flt(L, name, v):
    return L.clk_arg(name.encode(), L.ARG_FLOAT, 0, v, L.clk_image())


def sep_args(L, **over):
    args = {"dst": a_img(L, "dst", img()), "src": a_img(L, "src", img()), "dim": a_int(L, "dim", 0),
            "N": a_int(L, "N", 5), "s": a_flt(L, "s", 1.0)}
    args.update(over)
    return [v for v in args.values() if v is not None]


def test_unknown_kernel(L):
    st, msg = run(L, "gaussian_blur_separable_4d", sep_args(L))
    assert st == L.UNKNOWN_KERNEL and "unknown kernel" in msg
    st, _ = run(L, None, sep_args(L))
    assert st == L.UNKNOWN_KERNEL


def test_missing_extra_duplicate_and_mistyped_arguments(L):
    st, msg = run(L, "gaussian_blur_separable_3d", sep_args(L, N=None))
    assert st == L.BAD_ARG and "missing parameter 'N'" in msg
    st, msg = run(L, "gaussian_blur_separable_3d", sep_args(L) + [a_int(L, "Nz", 3)])
    assert st == L.BAD_ARG and "no parameter named 'Nz'" in msg
    st, msg = run(L, "gaussian_blur_separable_3d", sep_args(L) + [a_int(L, "dim", 1)])
    assert st == L.BAD_ARG and "given twice" in msg
    st, msg = run(L, "gaussian_blur_separable_3d", sep_args(L, dim=a_flt(L, "dim", 0.0)))
    assert st == L.BAD_ARG and "wrong kind" in msg
    st, msg = run(L, "gaussian_blur_separable_3d", sep_args(L, src=a_int(L, "src", 3)))
    assert st == L.BAD_ARG


def test_arguments_bind_by_name_not_position(L):
    # erode takes (src, dst), sobel (dst, src): any order is accepted, and the
    # first failure is the 2d/3d mismatch, not a binding error
    for name in ("erode_box_3d", "sobel_3d"):
        st, msg = run(L, name, [a_img(L, "dst", img(ndim=2, d=1)), a_img(L, "src", img())])
        assert st == L.BAD_ARG and "expects a 3d image" in msg


def test_image_validation(L):
    st, msg = run(L, "sobel_3d", [a_img(L, "dst", img(dt=9)), a_img(L, "src", img())])
    assert st == L.UNSUPPORTED_DTYPE
    st, msg = run(L, "sobel_3d", [a_img(L, "dst", img(w=0)), a_img(L, "src", img())])
    assert st == L.BAD_ARG and "positive" in msg
    st, msg = run(L, "sobel_3d", [a_img(L, "dst", img(ptr=0)), a_img(L, "src", img())])
    assert st == L.BAD_ARG and "null" in msg
    st, msg = run(L, "sobel_2d", [a_img(L, "dst", img(ndim=2, d=4)), a_img(L, "src", img(ndim=2, d=1))])
    assert st == L.BAD_ARG


def test_global_range_must_fit_dst(L):
    st, msg = run(L, "sobel_3d", [a_img(L, "dst", img()), a_img(L, "src", img())], global_range=(9, 8, 8))
    assert st == L.BAD_ARG and "exceeds" in msg


def test_median_limits(L):
    med = lambda n: [a_img(L, "dst", img()), a_img(L, "src", img()), a_int(L, "Nx", n), a_int(L, "Ny", n),
                     a_int(L, "Nz", n)]  # noqa: E731
    st, msg = run(L, "median_box_3d", med(5), defines=[("MAX_ARRAY_SIZE", "100")])
    assert st == L.BAD_ARG and "MAX_ARRAY_SIZE" in msg
    st, msg = run(L, "median_box_3d", med(11))
    assert st == L.BAD_ARG and "exceeds" in msg
    st, msg = run(L, "median_box_3d", med(-1))
    assert st == L.BAD_ARG and "empty" in msg
    st, msg = run(L, "median_box_3d", [a_img(L, "dst", img(dt=4)), a_img(L, "src", img(dt=2)), a_int(L, "Nx", 3),
                                       a_int(L, "Ny", 3), a_int(L, "Nz", 3)])
    assert st == L.UNSUPPORTED_DTYPE


def test_define_validation(L):
    st, msg = run(L, "sobel_3d", [a_img(L, "dst", img()), a_img(L, "src", img())],
                  defines=[("CLK_CONVERT_ROUNDING", "banker")])
    assert st == L.BAD_ARG and "rtz or rte" in msg
    st, msg = run(L, "sobel_3d", [a_img(L, "dst", img()), a_img(L, "src", img())],
                  defines=[("MAX_ARRAY_SIZE", "x")])
    assert st == L.BAD_ARG


def test_gaussian_window_limit(L):
    st, msg = run(L, "gaussian_blur_separable_3d", sep_args(L, N=a_int(L, "N", 5001)))
    assert st == L.BAD_ARG and "taps" in msg


def test_no_device_is_reported_not_crashed(L):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    st, msg = run(L, "sobel_3d", [a_img(L, "dst", img()), a_img(L, "src", img())])
    assert st == L.NO_DEVICE


def test_supported(L):
    lib = L.load()
    assert lib.clk_supported(b"median_box_3d", 2, 2, 3) == 1
    assert lib.clk_supported(b"median_box_3d", 2, 4, 3) == 0
    assert lib.clk_supported(b"median_box_3d", 2, 2, 2) == 0
    assert lib.clk_supported(b"sobel_3d", 2, 4, 3) == 1
    assert lib.clk_supported(b"nope", 2, 4, 3) == 0


def test_host_image_pointer_validation(L):
    out = C.c_void_p()
    assert L.load().clk_host_image_pointer(None, C.byref(out)) == L.BAD_ARG
    import torch
    if not torch.cuda.is_available():
        buf = (C.c_char * 64)()
        assert L.load().clk_host_image_pointer(C.cast(buf, C.c_void_p), C.byref(out)) == L.NO_DEVICE


def test_pageable_host_tensors_are_rejected():
    import torch
    import clk
    from clk import _lib as Lm
    with pytest.raises(Lm.ClkError) as e:
        clk.image_of(torch.zeros(4, 5, 6, dtype=torch.uint16))
    assert e.value.status == Lm.BAD_ARG and "pinned" in str(e.value)

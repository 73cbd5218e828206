"""Pinned host tensors as images (zero-copy, clk_host_image_pointer): a filter
that stores its output straight into page-locked host memory gives the same
bytes as the same filter writing device memory, on every path the output can
take (fused separable, line passes with device temporaries, selection
networks, sobel, byte morphology including radii whose intermediate passes
run in the output image), and a pinned host source reads the same values."""
import numpy as np
import pytest

from conftest import random_image

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clk():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import clk as m
    m.load()
    return m


def both(clk, fn, src, dtype):
    import torch
    dev = torch.full(src.shape, 3, dtype=dtype, device="cuda")
    host = torch.full(src.shape, 5, dtype=dtype).pin_memory()
    fn(src, dev)
    fn(src, host)
    torch.cuda.synchronize()
    return dev.cpu(), host


CASES = [
    ("gaussian u16->f32", np.uint16, "float32",
     lambda clk: lambda s, d: clk.separable("gaussian_blur_separable_3d", s, d, (7, 7, 5), (1.5, 1.5, 1.0))),
    ("mean u16", np.uint16, "uint16",
     lambda clk: lambda s, d: clk.separable("mean_separable_3d", s, d, (11, 11, 5), (5.0, 5.0, 2.0))),
    ("maximum r15 (line passes)", np.uint16, "uint16",
     lambda clk: lambda s, d: clk.separable("maximum_separable_3d", s, d, (31, 31, 31), (15.0, 15.0, 15.0))),
    ("median_box r1", np.uint16, "uint16",
     lambda clk: lambda s, d: clk.execute("median_box_3d", {"src": s, "dst": d, "Nx": 3, "Ny": 3, "Nz": 3})),
    ("median_sphere r2", np.int16, "int16",
     lambda clk: lambda s, d: clk.execute("median_sphere_3d", {"src": s, "dst": d, "Nx": 5, "Ny": 5, "Nz": 5})),
    ("sobel u16->f32", np.uint16, "float32",
     lambda clk: lambda s, d: clk.execute("sobel_3d", {"src": s, "dst": d})),
    ("erode_sphere r2 u8", np.uint8, "uint8",
     lambda clk: lambda s, d: clk.morphology("erode_sphere_3d", s, d, 2)),
    ("dilate_box r3 u8 (intermediate in dst)", np.uint8, "uint8",
     lambda clk: lambda s, d: clk.morphology("dilate_box_3d", s, d, 3)),
]


@pytest.mark.parametrize("name,sdt,ddt,make", CASES, ids=[c[0] for c in CASES])
def test_output_into_pinned_host_memory(clk, name, sdt, ddt, make):
    import torch
    rng = np.random.default_rng(abs(hash(name)) % 2**32)
    a = random_image(rng, (21, 70, 96), sdt, binary=sdt == np.uint8)
    src = torch.from_numpy(a).cuda()
    dev, host = both(clk, make(clk), src, getattr(torch, ddt))
    assert torch.equal(dev, host)


def test_pinned_host_source(clk):
    import torch
    rng = np.random.default_rng(11)
    a = random_image(rng, (9, 40, 64), np.uint16)
    s_dev = torch.from_numpy(a).cuda()
    s_host = torch.from_numpy(a).pin_memory()
    d1 = torch.empty(a.shape, dtype=torch.uint16, device="cuda")
    d2 = torch.empty_like(d1)
    clk.execute("median_box_3d", {"src": s_dev, "dst": d1, "Nx": 3, "Ny": 3, "Nz": 3})
    clk.execute("median_box_3d", {"src": s_host, "dst": d2, "Nx": 3, "Ny": 3, "Nz": 3})
    torch.cuda.synchronize()
    assert torch.equal(d1, d2)


def test_device_and_pageable_pointers_are_not_host_images(clk):
    import ctypes as C
    import torch
    from clk import _lib as L
    out = C.c_void_p()
    d = torch.zeros(64, dtype=torch.uint8, device="cuda")
    assert L.load().clk_host_image_pointer(C.c_void_p(d.data_ptr()), C.byref(out)) == L.BAD_ARG
    buf = (C.c_char * 4096)()
    assert L.load().clk_host_image_pointer(C.cast(buf, C.c_void_p), C.byref(out)) == L.BAD_ARG
    with pytest.raises(L.ClkError):
        clk.execute("sobel_3d", {"src": torch.zeros(4, 8, 8, dtype=torch.uint16, device="cuda"),
                                 "dst": torch.zeros(4, 8, 8, dtype=torch.float32)})

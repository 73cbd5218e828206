"""clk_separable_noalloc, called through the C ABI, against clk_separable.

The entry point serves callers that cannot let the library allocate device
memory (a host that owns the memory budget, a loop that must not stall or
hit out-of-memory midway): its two temporaries live in a fixed device array
instead of the stream-ordered allocator.  This test calls it twice in a row
on the same inputs (the array keeps the previous call's contents) and
compares both results with clk_separable's: bit-exact for integer outputs,
within the 1e-5 relative tolerance of the float tests for float outputs.
It also checks that a filter too large for the fixed array is refused.
The file is named to run last so that a failure here leaves every other
test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from clk import _lib as L
    from clk.api import image_of
    lib = L.load()
    lib.clk_separable_noalloc.argtypes = [C.c_char_p, C.POINTER(L.clk_image), C.POINTER(L.clk_image),
                                          C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(L.clk_define),
                                          C.c_size_t, C.c_void_p]
    lib.clk_separable_noalloc.restype = C.c_int
    return torch, L, lib, image_of


def call(env, fn, kernel, dst, src, N, s):
    torch, L, lib, image_of = env
    di, si = image_of(dst), image_of(src)
    st = getattr(lib, fn)(kernel.encode(), C.byref(di), C.byref(si), (C.c_int32 * 3)(*N), (C.c_float * 3)(*s),
                          None, 0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return st, lib.clk_last_error_string().decode()


CASES = [
    ("mean_separable_3d", np.uint16, np.uint16, (11, 11, 5), (5.0, 5.0, 2.0)),
    ("maximum_separable_3d", np.uint8, np.uint8, (7, 3, 5), (3.0, 1.0, 2.0)),
    ("gaussian_blur_separable_3d", np.uint16, np.float32, (13, 13, 7), (2.0, 2.0, 1.0)),
    ("gaussian_blur_separable_2d", np.float32, np.float32, (9, 5, 1), (1.5, 0.8, 0.0)),
]


@pytest.mark.parametrize("kernel,sdt,ddt,N,s", CASES)
def test_noalloc_matches_separable_twice(env, kernel, sdt, ddt, N, s):
    torch = env[0]
    rng = np.random.default_rng(41)
    shape = (96, 130) if kernel.endswith("2d") else (24, 64, 130)
    if np.dtype(sdt) == np.float32:
        a = rng.uniform(0.0, 1000.0, size=shape).astype(np.float32)
    else:
        a = rng.integers(0, np.iinfo(sdt).max + 1, size=shape).astype(sdt)
    src = torch.from_numpy(a).cuda()
    tdt = {np.dtype(np.uint8): torch.uint8, np.dtype(np.uint16): torch.uint16,
           np.dtype(np.float32): torch.float32}[np.dtype(ddt)]
    ref = torch.empty(shape, dtype=tdt, device="cuda")
    st, msg = call(env, "clk_separable", kernel, ref, src, N, s)
    assert st == 0, msg
    want = ref.cpu().numpy()
    for attempt in range(2):
        out = torch.full(shape, 3, dtype=tdt, device="cuda")
        st, msg = call(env, "clk_separable_noalloc", kernel, out, src, N, s)
        assert st == 0, msg
        got = out.cpu().numpy()
        if np.dtype(ddt) == np.float32:
            tol = REL_TOL * np.maximum(np.abs(want.astype(np.float64)), 1.0)
            assert (np.abs(got.astype(np.float64) - want) <= tol).all(), (kernel, attempt)
        else:
            assert np.array_equal(got, want), (kernel, attempt)


def test_noalloc_refuses_more_than_its_scratch(env):
    torch = env[0]
    # 16 Mi float voxels = 64 MiB per temporary, above the 32 MiB limit
    src = torch.zeros((16, 1024, 1024), dtype=torch.float32, device="cuda")
    dst = torch.empty_like(src)
    st, msg = call(env, "clk_separable_noalloc", "mean_separable_3d", dst, src, (3, 3, 3), (1.0, 1.0, 1.0))
    assert st == env[1].BAD_ARG and "scratch limit" in msg

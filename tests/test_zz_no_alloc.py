"""clk_separable_noalloc, called through the C ABI.

The entry point serves callers that cannot let the library allocate memory
(a host that owns the memory budget, a loop that must not stall or hit
out-of-memory midway).  It runs the fused kernel where one applies (no
temporaries) and otherwise the passes with their two temporaries in a fixed
device array instead of the stream-ordered allocator.

Each case calls it twice in a row on the same inputs (the array keeps the
previous call's contents) and compares both results with clk_separable's
and with the oracle: bit-exact for integer outputs, within the 1e-5 relative
tolerance of the float tests for float outputs.  The cases cover both forms
(fused: same pixel type, small radii; pass by pass: a uint8 -> uint16 pair
and radii above the fused limit).  A second test checks the defining
property: the driver's default memory pool (the one the stream-ordered
allocator draws from) records no use during the calls, while a clk_separable
call on the same pass-by-pass case does.  A third checks that a filter too
large for the fixed array is refused.

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
    for fn in ("clk_separable", "clk_separable_noalloc"):
        getattr(lib, fn).argtypes = [C.c_char_p, C.POINTER(L.clk_image), C.POINTER(L.clk_image),
                                     C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(L.clk_define),
                                     C.c_size_t, C.c_void_p]
        getattr(lib, fn).restype = C.c_int
    return torch, L, lib, image_of


def call(env, fn, kernel, dst, src, N, s):
    torch, L, lib, image_of = env
    di, si = image_of(dst), image_of(src)
    st = getattr(lib, fn)(kernel.encode(), C.byref(di), C.byref(si), (C.c_int32 * 3)(*N), (C.c_float * 3)(*s),
                          None, 0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return st, lib.clk_last_error_string().decode()


# (kernel, src type, dst type, N, s, form the call takes)
CASES = [
    ("mean_separable_3d", np.uint16, np.uint16, (11, 11, 5), (5.0, 5.0, 2.0), "fused"),
    ("maximum_separable_3d", np.uint8, np.uint8, (7, 3, 5), (3.0, 1.0, 2.0), "fused"),
    ("gaussian_blur_separable_3d", np.uint16, np.float32, (13, 13, 7), (2.0, 2.0, 1.0), "fused"),
    ("gaussian_blur_separable_2d", np.float32, np.float32, (9, 5, 1), (1.5, 0.8, 0.0), "fused"),
    ("mean_separable_3d", np.uint8, np.uint16, (5, 5, 3), (2.0, 2.0, 1.0), "passes"),
    ("maximum_separable_3d", np.float32, np.float32, (31, 31, 3), (15.0, 15.0, 1.0), "passes"),
    ("gaussian_blur_separable_3d", np.int16, np.float32, (41, 41, 9), (6.5, 6.5, 1.5), "passes"),
]


def source(sdt, shape, seed=41):
    rng = np.random.default_rng(seed)
    if np.dtype(sdt) == np.float32:
        return rng.uniform(-500.0, 1000.0, size=shape).astype(np.float32)
    info = np.iinfo(sdt)
    return rng.integers(info.min, int(info.max) + 1, size=shape).astype(sdt)


def tdtype(torch, dt):
    return {np.dtype(np.uint8): torch.uint8, np.dtype(np.uint16): torch.uint16, np.dtype(np.int16): torch.int16,
            np.dtype(np.float32): torch.float32}[np.dtype(dt)]


@pytest.mark.parametrize("kernel,sdt,ddt,N,s,form", CASES)
def test_noalloc_matches_separable_and_oracle_twice(env, oracle, kernel, sdt, ddt, N, s, form):
    torch = env[0]
    shape = (96, 130) if kernel.endswith("2d") else (24, 64, 130)
    a = source(sdt, shape)
    src = torch.from_numpy(a).cuda()
    ref = torch.empty(shape, dtype=tdtype(torch, ddt), device="cuda")
    st, msg = call(env, "clk_separable", kernel, ref, src, N, s)
    assert st == 0, msg
    want = ref.cpu().numpy()
    if np.dtype(ddt) == np.float32 and kernel.startswith("gaussian"):
        val, scale = oracle.fp64(kernel, a, N, s)
    else:
        val = oracle.separable(kernel, a, ddt, N, s)
        assert want.tobytes() == val.tobytes(), kernel
    for attempt in range(2):
        out = torch.full(shape, 3, dtype=tdtype(torch, ddt), device="cuda")
        st, msg = call(env, "clk_separable_noalloc", kernel, out, src, N, s)
        assert st == 0, msg
        assert msg == "", msg  # a successful call leaves no message behind
        got = out.cpu().numpy()
        # the same kernels as clk_separable: identical results
        assert got.tobytes() == want.tobytes(), (kernel, attempt)
        if np.dtype(ddt) == np.float32 and kernel.startswith("gaussian"):
            err = np.abs(got.astype(np.float64) - val)
            assert (err <= REL_TOL * np.maximum(np.abs(val), scale)).all(), (kernel, attempt)


class DefaultPool:
    """The driver's default memory pool of device 0 (the pool
    cudaMallocAsync draws from), through the driver API."""
    USED_MEM_HIGH = 8

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        dev = C.c_int()
        assert self.cu.cuDeviceGet(C.byref(dev), 0) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, C.byref(zero)) == 0

    def high(self):
        v = C.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, self.USED_MEM_HIGH, C.byref(v)) == 0
        return v.value


def test_noalloc_draws_nothing_from_the_pool(env):
    torch = env[0]
    kernel, sdt, ddt, N, s, _ = CASES[4]  # the pass-by-pass form: needs two temporaries
    shape = (24, 64, 130)
    src = torch.from_numpy(source(sdt, shape)).cuda()
    out = torch.empty(shape, dtype=tdtype(torch, ddt), device="cuda")
    st, msg = call(env, "clk_separable_noalloc", kernel, out, src, N, s)  # first call: address lookup
    assert st == 0, msg
    pool = DefaultPool()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    pool.reset_high()
    for _ in range(2):
        st, msg = call(env, "clk_separable_noalloc", kernel, out, src, N, s)
        assert st == 0, msg
    assert pool.high() == 0, "clk_separable_noalloc drew memory from the default pool"
    assert torch.cuda.mem_get_info()[0] == free0
    # control: clk_separable takes its temporaries from that pool
    pool.reset_high()
    st, msg = call(env, "clk_separable", kernel, out, src, N, s)
    assert st == 0, msg
    assert pool.high() >= out.numel() * out.element_size()


def test_noalloc_refuses_more_than_its_scratch(env):
    torch = env[0]
    # 16 Mi voxels of an int16 -> float pair whose radius needs the passes:
    # 64 MiB per temporary, above the 32 MiB limit
    src = torch.zeros((16, 1024, 1024), dtype=torch.int16, device="cuda")
    dst = torch.empty(src.shape, dtype=torch.float32, device="cuda")
    st, msg = call(env, "clk_separable_noalloc", "gaussian_blur_separable_3d", dst, src, (41, 41, 3),
                   (6.5, 6.5, 0.5))
    assert st == env[1].BAD_ARG and "scratch limit" in msg

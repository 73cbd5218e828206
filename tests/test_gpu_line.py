"""GPU parity of the line passes (clk_line.cu): separable filters whose
radius is beyond the fused register-window kernels run as one launch per
axis with dst-typed temporaries.  Integer min/max/mean and float min/max are
bit-exact against the oracle (NaN positions included); the Gaussian to
float is within the FP64 tolerance."""
import numpy as np
import pytest

from conftest import random_image

pytestmark = pytest.mark.gpu
REL_TOL = 1e-5


@pytest.fixture(scope="module")
def clk():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import clk as m
    m.load()
    return m


def run(clk, kernel, a, ddt, N, s):
    import torch
    from clk.api import torch_dtype
    from oracle.oracle import dtype_code
    d = torch.empty(a.shape, dtype=torch_dtype(dtype_code(ddt)), device="cuda")
    clk.separable(kernel, torch.from_numpy(a).cuda(), d, N, s)
    torch.cuda.synchronize()
    return d.cpu().numpy()


SHAPES = ((9, 40, 70), (3, 17, 129), (40, 5, 8))
RADII = ((13, 13, 13), (20, 3, 0), (0, 17, 2), (30, 30, 15), (2, 2, 40))


@pytest.mark.parametrize("kernel", ["minimum_separable_3d", "maximum_separable_3d", "mean_separable_3d"])
@pytest.mark.parametrize("dt", [np.uint16, np.int16, np.uint8, np.int8])
def test_integer_large_radii(clk, oracle, kernel, dt):
    rng = np.random.default_rng(71)
    for shp in SHAPES:
        a = random_image(rng, shp, dt)
        for r in RADII:
            N = tuple(2 * v + 1 for v in r)
            want = oracle.separable(kernel, a, dt, N, tuple(float(v) for v in r))
            got = run(clk, kernel, a, dt, N, tuple(float(v) for v in r))
            assert np.array_equal(got, want), (kernel, shp, np.dtype(dt), N)


@pytest.mark.parametrize("kernel", ["minimum_separable_3d", "maximum_separable_3d"])
def test_float_minmax_large_radii_with_nan(clk, oracle, kernel):
    rng = np.random.default_rng(72)
    for shp in SHAPES:
        a = random_image(rng, shp, np.float32)
        a.flat[rng.integers(0, a.size, 5)] = np.nan
        b = a.copy()  # dense NaNs, signed zeros and infinities: which one survives is the loop order's
        b[rng.random(shp) < 0.05] = np.nan
        b[rng.random(shp) < 0.1] = 0.0
        b[rng.random(shp) < 0.1] = -0.0
        b[rng.random(shp) < 0.02] = np.inf
        b[rng.random(shp) < 0.02] = -np.inf
        for img in (a, b):
            for r in RADII:
                N = tuple(2 * v + 1 for v in r)
                want = oracle.separable(kernel, img, np.float32, N, tuple(float(v) for v in r))
                got = run(clk, kernel, img, np.float32, N, tuple(float(v) for v in r))
                assert got.tobytes() == want.tobytes(), (kernel, shp, N)


@pytest.mark.parametrize("kernel", ["minimum_separable_3d", "maximum_separable_3d"])
def test_float_minmax_long_lines(clk, oracle, kernel):
    # float min/max along lines of 1024 voxels or more take 16 outputs per
    # thread: partial last tiles along x and y, dense NaNs and signed zeros
    rng = np.random.default_rng(76)
    for shp in ((2, 5, 1100), (2, 1030, 6)):
        a = random_image(rng, shp, np.float32)
        a[rng.random(shp) < 0.05] = np.nan
        a[rng.random(shp) < 0.1] = 0.0
        a[rng.random(shp) < 0.1] = -0.0
        for r in ((15, 15, 1), (8, 9, 0), (40, 12, 1)):
            N = tuple(2 * v + 1 for v in r)
            want = oracle.separable(kernel, a, np.float32, N, tuple(float(v) for v in r))
            got = run(clk, kernel, a, np.float32, N, tuple(float(v) for v in r))
            assert got.tobytes() == want.tobytes(), (kernel, shp, N)


@pytest.mark.parametrize("dt", [np.uint16, np.int8, np.float32])
def test_gaussian_large_sigma(clk, oracle, dt):
    rng = np.random.default_rng(73)
    for shp in SHAPES:
        a = random_image(rng, shp, dt)
        for s in ((5.0, 5.0, 5.0), (10.0, 10.0, 5.0), (7.0, 0.0, 2.0), (1.0, 1.0, 13.0)):
            N = tuple(2 * int(np.ceil(3 * v)) + 1 if v > 0 else 1 for v in s)
            val, scale = oracle.fp64("gaussian_blur_separable_3d", a, N, s)
            got = run(clk, "gaussian_blur_separable_3d", a, np.float32, N, s)
            err = np.abs(got.astype(np.float64) - val)
            assert (err <= REL_TOL * np.maximum(np.abs(val), scale)).all(), (shp, np.dtype(dt), s)


def test_gaussian_long_lines(clk, oracle):
    # lines of 256 voxels or more take 16 outputs per thread (tiles of 128
    # lines): partial last tiles along each axis in turn, one with a single
    # live group
    rng = np.random.default_rng(75)
    for shp in ((2, 9, 1100), (2, 1030, 12), (1030, 3, 8), (400, 2, 8), (2, 272, 6)):
        a = random_image(rng, shp, np.float32)
        for s in ((10.0, 10.0, 5.0), (5.0, 5.0, 5.0)):
            N = tuple(2 * int(np.ceil(3 * v)) + 1 for v in s)
            val, scale = oracle.fp64("gaussian_blur_separable_3d", a, N, s)
            got = run(clk, "gaussian_blur_separable_3d", a, np.float32, N, s)
            err = np.abs(got.astype(np.float64) - val)
            assert (err <= REL_TOL * np.maximum(np.abs(val), scale)).all(), (shp, s)


def test_2d_large_radii(clk, oracle):
    rng = np.random.default_rng(74)
    a = random_image(rng, (50, 300), np.uint16)
    for kernel in ("minimum_separable_2d", "maximum_separable_2d", "mean_separable_2d"):
        want = oracle.separable(kernel, a, np.uint16, (61, 31), (30.0, 15.0))
        assert np.array_equal(run(clk, kernel, a, np.uint16, (61, 31), (30.0, 15.0)), want), kernel
    val, scale = oracle.fp64("gaussian_blur_separable_2d", a, (61, 61), (10.0, 10.0))
    got = run(clk, "gaussian_blur_separable_2d", a, np.float32, (61, 61), (10.0, 10.0))
    assert (np.abs(got.astype(np.float64) - val) <= REL_TOL * np.maximum(np.abs(val), scale)).all()

"""GPU parity of the fused separable kernels over the radii and layouts they
specialise on: isotropic XY radii 1..8 (integer min/max/mean, bit-exact)
and 1..12 (Gaussian to float, within the FP64 tolerance), even and odd
widths, thin stacks, 2-D images, skipped axes."""
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


def run(clk, kernel, a, ddt, N, s, defines=None):
    import torch
    from clk.api import torch_dtype
    from oracle.oracle import dtype_code
    d = torch.empty(a.shape, dtype=torch_dtype(dtype_code(ddt)), device="cuda")
    clk.separable(kernel, torch.from_numpy(a).cuda(), d, N, s, defines=defines)
    torch.cuda.synchronize()
    return d.cpu().numpy()


def close(got, val, scale):
    err = np.abs(got.astype(np.float64) - val)
    return (err <= REL_TOL * np.maximum(np.abs(val), scale)).all()


@pytest.mark.parametrize("kernel", ["minimum_separable_3d", "maximum_separable_3d", "mean_separable_3d"])
@pytest.mark.parametrize("dt", [np.uint16, np.int16, np.uint8, np.int8])
def test_integer_isotropic_radii(clk, oracle, kernel, dt):
    rng = np.random.default_rng(31)
    # widths that are multiples of 16 take the vector staging (8/16-byte
    # loads, clamped vectors at the tile borders); the others the scalar one
    for shp in ((19, 70, 130), (3, 33, 64), (1, 40, 66), (40, 8, 10), (6, 29, 67), (2, 9, 1), (5, 37, 96),
                (4, 20, 16), (3, 70, 208)):
        a = random_image(rng, shp, dt)
        for R in range(1, 9):
            for rz in (0, 1, R):
                N = (2 * R + 1, 2 * R + 1, 2 * rz + 1)
                want = oracle.separable(kernel, a, dt, N, (R, R, rz))
                got = run(clk, kernel, a, dt, N, (R, R, rz))
                assert np.array_equal(got, want), (kernel, shp, np.dtype(dt), N)


@pytest.mark.parametrize("dt", [np.uint16, np.int16, np.uint8, np.float32])
def test_gaussian_to_float_isotropic(clk, oracle, dt):
    rng = np.random.default_rng(32)
    for shp in ((17, 70, 130), (2, 35, 64), (5, 23, 45), (6, 40, 96), (3, 19, 16), (4, 45, 144)):
        a = random_image(rng, shp, dt)
        for R in (1, 3, 6, 9, 12):
            sig = R / 3.0
            for sz in (0.0, 0.7, 1.5):
                N = (2 * R + 1, 2 * R + 1, 2 * int(np.ceil(3 * sz)) + 1 if sz > 0 else 1)
                s = (sig, sig, sz)
                val, scale = oracle.fp64("gaussian_blur_separable_3d", a, N, s)
                got = run(clk, "gaussian_blur_separable_3d", a, np.float32, N, s)
                assert close(got, val, scale), (shp, np.dtype(dt), N, s)


@pytest.mark.parametrize("kernel", ["minimum_separable_3d", "maximum_separable_3d"])
def test_float_min_max_reference_order(clk, oracle, kernel):
    # float pixels with NaNs and signed zeros: the reference's loop (start at
    # the centre, res = min(res, x) in tap order) decides which NaN / zero
    # survives; compared bit for bit
    rng = np.random.default_rng(36)
    for shp in ((9, 70, 130), (3, 33, 64), (5, 37, 96), (1, 40, 66)):
        a = (rng.standard_normal(shp) * 100).astype(np.float32)
        a[rng.random(shp) < 0.02] = np.nan
        a[rng.random(shp) < 0.05] = 0.0
        a[rng.random(shp) < 0.05] = -0.0
        a[rng.random(shp) < 0.01] = np.inf
        a[rng.random(shp) < 0.01] = -np.inf
        for R in (1, 2, 4, 5, 8):
            for rz in (0, 1, 3):
                N = (2 * R + 1, 2 * R + 1, 2 * rz + 1)
                want = oracle.separable(kernel, a, np.float32, N, (R, R, rz))
                got = run(clk, kernel, a, np.float32, N, (R, R, rz))
                assert got.tobytes() == want.tobytes(), (kernel, shp, N)


@pytest.mark.parametrize("dt", [np.uint16, np.int16, np.uint8, np.int8])
def test_gaussian_to_integer_bit_exact(clk, oracle, dt):
    # integer outputs: the reference's tap order, separately rounded products
    # and sums, IEEE division and a conversion after every pass, bit for bit
    rng = np.random.default_rng(35)
    for shp in ((9, 70, 130), (3, 33, 64), (1, 40, 66), (5, 37, 96), (4, 20, 16)):
        a = random_image(rng, shp, dt)
        for R in range(1, 9):
            for sz, cz in ((0.0, 0), (0.8, 1), (1.5, 3)):
                sig = R / 3.0 + 0.1
                N = (2 * R + 1, 2 * R + 1, 2 * cz + 1)
                s = (sig, sig, sz)
                want = oracle.separable("gaussian_blur_separable_3d", a, dt, N, s)
                got = run(clk, "gaussian_blur_separable_3d", a, dt, N, s)
                assert np.array_equal(got, want), (shp, np.dtype(dt), N, s)
    # the round-half-even conversion policy, every pass
    a = random_image(rng, (6, 40, 64), dt)
    for R in (2, 6):
        N, s = (2 * R + 1, 2 * R + 1, 5), (R / 2.0, R / 2.0, 1.0)
        want = oracle.separable("gaussian_blur_separable_3d", a, dt, N, s, flags=oracle.FLAG_RTE)
        got = run(clk, "gaussian_blur_separable_3d", a, dt, N, s, defines={"CLK_CONVERT_ROUNDING": "rte"})
        assert np.array_equal(got, want), ("rte", np.dtype(dt), N)


def test_2d_and_config_shapes(clk, oracle):
    rng = np.random.default_rng(33)
    a2 = random_image(rng, (96, 130), np.uint16)
    for kernel in ("minimum_separable_2d", "maximum_separable_2d", "mean_separable_2d"):
        want = oracle.separable(kernel, a2, np.uint16, (9, 9), (4, 4))
        assert np.array_equal(run(clk, kernel, a2, np.uint16, (9, 9), (4, 4)), want)
    val, scale = oracle.fp64("gaussian_blur_separable_2d", a2, (13, 13), (2.0, 2.0))
    assert close(run(clk, "gaussian_blur_separable_2d", a2, np.float32, (13, 13), (2.0, 2.0)), val, scale)
    # the headline configurations on a thin slab of the same shape family
    a = random_image(rng, (12, 64, 256), np.uint16)
    for kernel in ("mean_separable_3d", "minimum_separable_3d", "maximum_separable_3d"):
        want = oracle.separable(kernel, a, np.uint16, (11, 11, 5), (5, 5, 2))
        assert np.array_equal(run(clk, kernel, a, np.uint16, (11, 11, 5), (5, 5, 2)), want), kernel
    val, scale = oracle.fp64("gaussian_blur_separable_3d", a, (19, 19, 11), (3.0, 3.0, 1.5))
    assert close(run(clk, "gaussian_blur_separable_3d", a, np.float32, (19, 19, 11), (3.0, 3.0, 1.5)), val, scale)


def test_ragged_tile_grid(clk, oracle):
    # 15 x 17 tiles whose last column and row are partial (904 = 14 x 64 + 8,
    # 520 = 16 x 32 + 8), aligned rows (vector staging), 48 planes
    rng = np.random.default_rng(34)
    for dt in (np.uint16, np.uint8):
        a = random_image(rng, (48, 520, 904), dt)
        for kernel in ("minimum_separable_3d", "maximum_separable_3d", "mean_separable_3d"):
            want = oracle.separable(kernel, a, dt, (11, 11, 5), (5, 5, 2))
            assert np.array_equal(run(clk, kernel, a, dt, (11, 11, 5), (5, 5, 2)), want), (kernel, np.dtype(dt))
    a = random_image(rng, (48, 520, 904), np.uint16)
    for N, s in (((19, 19, 11), (3.0, 3.0, 1.5)), ((7, 7, 5), (1.0, 1.0, 0.6))):
        val, scale = oracle.fp64("gaussian_blur_separable_3d", a, N, s)
        assert close(run(clk, "gaussian_blur_separable_3d", a, np.float32, N, s), val, scale), N


@pytest.mark.parametrize("kernel", ["minimum_separable_3d", "maximum_separable_3d", "mean_separable_3d"])
def test_register_ring_kernels_every_z_radius(clk, oracle, kernel):
    # 16-bit pixels with x extents a multiple of 8 take the register-ring
    # kernels for Z radii 0..3 (every XY radius 1..8): tiny and one-plane
    # stacks, one-row images, tile-ragged extents, extremes of the pixel
    # range (signed and unsigned), against the oracle bit for bit
    rng = np.random.default_rng(41)
    for dt in (np.uint16, np.int16):
        for shp in ((7, 45, 72), (2, 3, 8), (1, 33, 64), (9, 1, 136), (5, 70, 200)):
            a = random_image(rng, shp, dt)
            info = np.iinfo(dt)
            a.flat[:: 97] = info.max
            a.flat[5:: 89] = info.min
            for R in range(1, 9):
                for rz in range(0, 4):
                    N = (2 * R + 1, 2 * R + 1, 2 * rz + 1)
                    want = oracle.separable(kernel, a, dt, N, (R, R, rz))
                    got = run(clk, kernel, a, dt, N, (R, R, rz))
                    assert np.array_equal(got, want), (kernel, shp, np.dtype(dt), N)


def test_register_ring_gaussian_every_z_radius(clk, oracle):
    # u16 -> f32 Gaussians on the register-ring kernel: XY radius 1..12, Z
    # radius 0..6, within the stated tolerance of the FP64 oracle
    rng = np.random.default_rng(42)
    for shp in ((14, 45, 72), (1, 33, 64), (3, 2, 16), (20, 70, 200)):
        a = random_image(rng, shp, np.uint16)
        for R in (1, 2, 4, 7, 10, 12):
            for cz in range(0, 7):
                N = (2 * R + 1, 2 * R + 1, 2 * cz + 1)
                s = (R / 3.0, R / 3.0, cz / 3.0 if cz else 0.0)
                val, scale = oracle.fp64("gaussian_blur_separable_3d", a, N, s)
                got = run(clk, "gaussian_blur_separable_3d", a, np.float32, N, s)
                assert close(got, val, scale), (shp, N, s)

"""GPU parity of the network medians (3x3x3 box, radius-2 sphere, 2-D 3x3)
against the oracle's insertion-sort restatement, bit-exact, for every
integer pixel type, with odd and tiny extents and the generic fallbacks
(odd width, float pixels, other radii)."""
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


def run(clk, kernel, a, params):
    import torch
    src = torch.from_numpy(a).cuda()
    dst = torch.empty_like(src)
    p = {"src": src, "dst": dst}
    p.update(params)
    clk.execute(kernel, p)
    torch.cuda.synchronize()
    return dst.cpu().numpy()


CASES = [("median_box_3d", {"Nx": 3, "Ny": 3, "Nz": 3}), ("median_sphere_3d", {"Nx": 5, "Ny": 5, "Nz": 5})]


@pytest.mark.parametrize("kernel,params", CASES)
@pytest.mark.parametrize("dt", [np.uint16, np.int16, np.uint8, np.int8, np.float32])
def test_network_median_3d(clk, oracle, kernel, params, dt):
    rng = np.random.default_rng(23)
    # widths of whole 16-byte vectors (the staged kernels: 8 pixels of 16 bits, 4 floats) with
    # partial tiles and both x borders, and widths that take the unstaged kernels
    for shp in ((21, 37, 130), (1, 5, 64), (2, 1, 2), (7, 64, 2), (33, 16, 66), (9, 13, 67), (4, 6, 1), (3, 5, 3),
                (21, 37, 132), (5, 9, 36), (11, 40, 96), (6, 19, 8)):
        for lo, hi in ((None, None), (0, 3)):  # full range, and many ties
            a = random_image(rng, shp, dt)
            if lo is not None:
                a = rng.integers(lo, hi, size=shp).astype(dt)
            want = oracle.execute(kernel, a, dt, list(params.values()))
            got = run(clk, kernel, a, params)
            assert np.array_equal(got, want), (kernel, shp, np.dtype(dt))


@pytest.mark.parametrize("dt", [np.uint16, np.int16, np.uint8, np.int8])
def test_network_median_2d(clk, oracle, dt):
    rng = np.random.default_rng(24)
    for shp in ((37, 130), (1, 64), (5, 2), (31, 67), (7, 1)):
        a = random_image(rng, shp, dt)
        want = oracle.execute("median_box_2d", a, dt, [3, 3])
        assert np.array_equal(run(clk, "median_box_2d", a, {"Nx": 3, "Ny": 3}), want)


def test_fallbacks_stay_exact(clk, oracle):
    rng = np.random.default_rng(25)
    cases = [((9, 13, 31), np.uint16, "median_box_3d", {"Nx": 3, "Ny": 3, "Nz": 3}),  # odd width
             ((9, 13, 32), np.float32, "median_sphere_3d", {"Nx": 5, "Ny": 5, "Nz": 5}),  # float pixels
             ((9, 13, 32), np.uint16, "median_box_3d", {"Nx": 5, "Ny": 3, "Nz": 3}),  # other window
             ((9, 13, 32), np.uint16, "median_sphere_3d", {"Nx": 3, "Ny": 3, "Nz": 3})]
    for shp, dt, kernel, params in cases:
        a = random_image(rng, shp, dt)
        want = oracle.execute(kernel, a, dt, list(params.values()))
        assert run(clk, kernel, a, params).tobytes() == want.tobytes(), (kernel, np.dtype(dt))

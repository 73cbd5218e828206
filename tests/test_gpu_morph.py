"""GPU parity of the morphology paths: the byte-tile kernel (r=1) and the
fused two-iteration kernel (radius 2), against the oracle applied
iteration by iteration, bit-exact; including extents that are not a multiple
of the tile, one-plane stacks, and non-byte pixel types (generic path)."""
import numpy as np
import pytest

from conftest import random_image

pytestmark = pytest.mark.gpu

MORPH = ["erode_sphere_3d", "dilate_sphere_3d", "erode_box_3d", "dilate_box_3d",
         "erode_sphere_slice_by_slice_3d", "dilate_sphere_slice_by_slice_3d",
         "erode_box_slice_by_slice_3d", "dilate_box_slice_by_slice_3d"]


@pytest.fixture(scope="module")
def clk():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import clk as m
    m.load()
    return m


def run(clk, kernel, a, ddt, iterations):
    import torch
    from clk.api import torch_dtype
    from oracle.oracle import dtype_code
    src = torch.from_numpy(a).cuda()
    dst = torch.full(a.shape, 7, dtype=torch_dtype(dtype_code(ddt)), device="cuda")
    clk.morphology(kernel, src, dst, iterations)
    torch.cuda.synchronize()
    return dst.cpu().numpy()


def oracle_iter(oracle, kernel, a, ddt, iterations):
    cur = a
    for _ in range(iterations):
        cur = oracle.execute(kernel, cur, ddt)
    if iterations == 0:
        cur = oracle.separable("maximum_separable_3d" if a.ndim == 3 else "maximum_separable_2d", a, ddt,
                               (1, 1, 1))
    return cur


@pytest.mark.parametrize("kernel", MORPH)
@pytest.mark.parametrize("density", [0.5, 0.93])
def test_byte_tiles_match_oracle(clk, oracle, kernel, density):
    rng = np.random.default_rng(17)
    # also: two-plane stacks, and deep thin stacks whose z-chunks (CTAs)
    # start and end inside the stack
    for shp in ((37, 70, 160), (5, 33, 48), (1, 9, 16), (40, 1, 32), (3, 64, 512), (2, 40, 64), (70, 40, 32),
                (100, 20, 16)):
        a = random_image(rng, shp, np.uint8, binary=True, density=density)
        for it in (1, 2, 3, 4):
            got = run(clk, kernel, a, np.uint8, it)
            want = oracle_iter(oracle, kernel, a, np.uint8, it)
            assert np.array_equal(got, want), (kernel, shp, it)


@pytest.mark.parametrize("kernel", MORPH)
def test_other_types_and_widths_fall_back_exactly(clk, oracle, kernel):
    rng = np.random.default_rng(18)
    cases = [((6, 11, 21), np.uint8, np.uint8), ((6, 12, 32), np.uint16, np.uint16), ((6, 12, 32), np.float32,
             np.float32), ((6, 12, 32), np.int8, np.uint8), ((6, 12, 32), np.uint8, np.float32)]
    for shp, sdt, ddt in cases:
        a = random_image(rng, shp, sdt, binary=True, density=0.8)
        for it in (0, 1, 2, 3):
            got = run(clk, kernel, a, ddt, it)
            want = oracle_iter(oracle, kernel, a, ddt, it)
            assert got.tobytes() == want.tobytes(), (kernel, shp, np.dtype(sdt), it)


def test_2d_morphology(clk, oracle):
    rng = np.random.default_rng(19)
    for kernel in ("erode_sphere_2d", "dilate_sphere_2d", "erode_box_2d", "dilate_box_2d"):
        a = random_image(rng, (45, 64), np.uint8, binary=True, density=0.7)
        for it in (1, 2):
            assert np.array_equal(run(clk, kernel, a, np.uint8, it), oracle_iter(oracle, kernel, a, np.uint8, it))


@pytest.mark.parametrize("kernel", MORPH[:4])
def test_bit_words_any_nonzero_byte(clk, oracle, kernel):
    # Rows of whole 32-voxel words take the bit-word kernels: every nonzero
    # byte value counts as set (signed and unsigned pixels), borders clamp,
    # one and two iterations per pass (and chains of them), results bit for
    # bit the oracle's.
    rng = np.random.default_rng(77)
    for shp in ((9, 37, 96), (4, 70, 256), (33, 5, 64), (2, 2, 32)):
        for sdt in (np.uint8, np.int8):
            a = rng.integers(0, 256, size=shp).astype(np.uint8)
            a[rng.random(shp) < 0.3] = 0
            a = a.view(sdt)
            for it in (1, 2, 3):
                got = run(clk, kernel, a, np.uint8, it)
                want = oracle_iter(oracle, kernel, a, np.uint8, it)
                assert np.array_equal(got, want), (kernel, shp, np.dtype(sdt), it)

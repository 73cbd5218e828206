"""GPU parity: the CUDA library, called through the C ABI, against the oracle
on the same seeded inputs.

Bar: integer outputs and the exact operations (min/max, median, erode/dilate)
bit-exact; float outputs of gaussian/mean/sobel bit-exact in the reference's
evaluation order (define CLK_EXACT_ORDER=1), and on the default fast path
within |gpu - fp64| <= 1e-5 * max(|fp64|, scale), where fp64 is the FP64
oracle and scale the per-voxel magnitude of the summed terms (the filter
applied to |src|; for sobel the norm of the per-component sums of |terms|).
"""
import numpy as np
import pytest

import golden_cases
from conftest import DTYPES, random_image

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
EXACT = {"CLK_EXACT_ORDER": "1"}


@pytest.fixture(scope="module")
def clk():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import clk as m
    m.load()
    return m


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def empty(shape, dt):
    import torch
    from clk.api import torch_dtype
    from oracle.oracle import dtype_code
    return torch.empty(shape, dtype=torch_dtype(dtype_code(dt)), device="cuda")


def assert_fp64_close(got, val, scale, what):
    got = got.astype(np.float64)
    err = np.abs(got - val)
    tol = REL_TOL * np.maximum(np.abs(val), scale)
    bad = err > tol
    assert not bad.any(), f"{what}: {bad.sum()} voxels off, worst {np.max(err / np.maximum(tol, 1e-300)):.3g} x tol"


def run_execute(clk, kernel, a, ddt, params, defines=None, global_range=None):
    d = empty(a.shape, ddt)
    d.zero_()
    p = {("src1" if kernel.startswith("greater_constant") else "src"): dev(a), "dst": d}
    p.update(params)
    clk.execute(kernel, p, global_range=global_range, defines=defines)
    return host(d)


def _params(kernel):
    is2 = kernel.endswith("2d")
    if "slice_by_slice" in kernel and not kernel.startswith(("erode", "dilate")):
        return [{"Nx": 3, "Ny": 3}, {"Nx": 5, "Ny": 5}, {"Nx": 7, "Ny": 3}]
    if "_sphere_" in kernel and kernel.startswith(("minimum", "maximum", "mean")):
        return ([{"Nx": 3, "Ny": 3}, {"Nx": 5, "Ny": 5}, {"Nx": 5, "Ny": 1}] if is2 else
                [{"Nx": 3, "Ny": 3, "Nz": 3}, {"Nx": 5, "Ny": 5, "Nz": 5}, {"Nx": 3, "Ny": 5, "Nz": 1}])
    if kernel.startswith("greater_constant"):
        return [{"scalar": 400.0}, {"scalar": -3.5}]
    if kernel.startswith(("gaussian", "mean", "minimum", "maximum")):
        dims = (0, 1) if is2 else (0, 1, 2)
        return [{"dim": d, "N": N, "s": s} for d in dims for N, s in ((5, 1.5), (4, 0.7), (1, 1.0), (13, 3.0))]
    if kernel.startswith("median"):
        return ([{"Nx": 3, "Ny": 3}, {"Nx": 5, "Ny": 5}, {"Nx": 5, "Ny": 1}] if is2 else
                [{"Nx": 3, "Ny": 3, "Nz": 3}, {"Nx": 5, "Ny": 5, "Nz": 5}, {"Nx": 3, "Ny": 5, "Nz": 1}])
    return [{}]


KERNELS = [k for k in __import__("oracle.oracle", fromlist=["KERNELS"]).KERNELS if not k.startswith("convolve")]


@pytest.mark.parametrize("kernel", KERNELS)
def test_execute_matches_oracle_every_dtype_pair(clk, oracle, kernel):
    rng = np.random.default_rng(abs(hash(kernel)) % 2**32)
    is2 = kernel.endswith("2d")
    morph = kernel.startswith(("erode", "dilate"))
    # widths that are multiples of 16 take the vectorised fast paths
    for shp in (((17, 33), (1, 7), (9, 16)) if is2 else ((9, 17, 33), (1, 5, 6), (4, 1, 1), (3, 9, 16))):
        for sdt in DTYPES:
            for ddt in DTYPES:
                if kernel.startswith("median") and sdt != ddt:
                    continue
                if kernel == "minimum_sphere_2d" and sdt == np.float32 and ddt != np.float32:
                    continue  # rejected: the kernel's C cast of an out-of-range float is undefined
                a = random_image(rng, shp, sdt, binary=morph)
                for p in _params(kernel):
                    ints, floats = golden_cases.split_params(p)
                    want = oracle.execute(kernel, a, ddt, ints, floats)
                    got = run_execute(clk, kernel, a, ddt, p, defines=EXACT)
                    assert got.tobytes() == want.tobytes(), (kernel, shp, np.dtype(sdt), np.dtype(ddt), p)


@pytest.mark.parametrize("kernel", ["convolve_2d", "convolve_3d"])
def test_convolve_matches_oracle(clk, oracle, kernel):
    rng = np.random.default_rng(82)
    is2 = kernel.endswith("2d")
    kshapes = ((3, 3), (5, 3), (4, 4), (1, 1)) if is2 else ((3, 3, 3), (5, 3, 1), (4, 2, 3), (1, 1, 1))
    for shp in (((17, 33), (1, 7)) if is2 else ((9, 17, 33), (1, 5, 6))):
        for sdt in DTYPES:
            for ddt in DTYPES:
                a = random_image(rng, shp, sdt)
                for ks in kshapes:
                    k = rng.standard_normal(ks).astype(np.float32)
                    want = oracle.execute(kernel, a, ddt, kernel_image=k)
                    got = run_execute(clk, kernel, a, ddt, {"kernelImage": dev(k)})
                    assert got.tobytes() == want.tobytes(), (kernel, shp, np.dtype(sdt), np.dtype(ddt), ks)


@pytest.mark.parametrize("kernel", ["sobel_2d", "sobel_3d"])
def test_sobel_fast_path_within_fp64_tolerance(clk, oracle, kernel):
    rng = np.random.default_rng(3)
    # 3-D: widths that are whole 16-byte vectors take the staged tiles, the
    # others the per-thread loads; thin stacks and ragged tile edges too
    shapes = [(64, 96)] if kernel == "sobel_2d" else [(20, 37, 70), (20, 37, 64), (3, 19, 128), (2, 70, 48)]
    for shp in shapes:
        for sdt in DTYPES:
            a = random_image(rng, shp, sdt)
            got = run_execute(clk, kernel, a, np.float32, {})
            val, scale = oracle.fp64(kernel, a)
            assert_fp64_close(got, val, scale, f"{kernel} {shp} {np.dtype(sdt)}")
            # integer outputs stay bit-exact on the fast path
            if np.dtype(sdt) != np.float32:
                got16 = run_execute(clk, kernel, a, np.uint16, {})
                assert got16.tobytes() == oracle.execute(kernel, a, np.uint16).tobytes()


def test_sobel3d_unsigned_wrap_counts_with_zero_pixels(clk, oracle):
    # unsigned pixels: every negative-coefficient tap with a nonzero pixel
    # adds 2^32; zero pixels (masks, sparse stacks, zero borders) change the
    # counts per output, and a wrong count moves a result by ~8%
    rng = np.random.default_rng(6)
    for shp in ((21, 37, 64), (9, 50, 128), (5, 33, 70)):
        for sdt in (np.uint16, np.uint8):
            for density in (0.05, 0.5, 0.95):
                a = random_image(rng, shp, sdt, binary=True, density=density)
                got = run_execute(clk, "sobel_3d", a, np.float32, {})
                val, scale = oracle.fp64("sobel_3d", a)
                assert_fp64_close(got, val, scale, f"sobel_3d {shp} {np.dtype(sdt)} density {density}")
            b = np.zeros(shp, sdt)  # a zero border around nonzero content
            b[1:-1, 2:-2, 3:-3] = random_image(rng, (shp[0] - 2, shp[1] - 4, shp[2] - 6), sdt)
            got = run_execute(clk, "sobel_3d", b, np.float32, {})
            val, scale = oracle.fp64("sobel_3d", b)
            assert_fp64_close(got, val, scale, f"sobel_3d {shp} {np.dtype(sdt)} zero border")


@pytest.mark.parametrize("kernel", ["laplace_diamond_2d", "laplace_box_2d", "laplace_diamond_3d", "laplace_box_3d"])
def test_laplace_row_path(clk, oracle, kernel):
    # widths that are whole 8-pixel vectors take the row kernels (integer
    # pixels; laplace_box_3d for signed ones), bit-exact; thin stacks, one
    # row, one plane, every pixel-type pair into float and into the source type
    rng = np.random.default_rng(7)
    shapes = [(33, 64), (1, 8), (7, 40)] if kernel.endswith("2d") else [(5, 33, 64), (1, 9, 16), (4, 1, 8), (6, 20, 96)]
    for shp in shapes:
        for sdt in DTYPES:
            a = random_image(rng, shp, sdt)
            for ddt in (np.float32, sdt):
                got = run_execute(clk, kernel, a, ddt, {})
                want = oracle.execute(kernel, a, ddt)
                assert got.tobytes() == want.tobytes(), (kernel, shp, np.dtype(sdt), np.dtype(ddt))


def test_partial_global_range_writes_only_that_box(clk, oracle):
    rng = np.random.default_rng(5)
    a = random_image(rng, (6, 10, 12), np.uint16)
    got = run_execute(clk, "maximum_separable_3d", a, np.uint16, {"dim": 1, "N": 5, "s": 0.0},
                      global_range=(7, 4, 3))
    want = np.zeros_like(a)
    full = oracle.execute("maximum_separable_3d", a, np.uint16, (1, 5), (0.0,))
    want[:3, :4, :7] = full[:3, :4, :7]
    assert np.array_equal(got, want)


def test_golden_fixtures_on_gpu(clk):
    """Every reference output in tests/golden, reproduced through the C ABI
    (reference evaluation order)."""
    n = 0
    for c, a, want in golden_cases.load():
        dt = golden_cases.NP[c["dst"]]
        if c["kind"] == "convolve":
            got = run_execute(clk, c["kernel"], a, dt, {"kernelImage": dev(c["kernel_image"])}, defines=EXACT)
        elif c["kind"] == "execute":
            got = run_execute(clk, c["kernel"], a, dt, c["params"], defines=EXACT)
        else:
            d = empty(a.shape, dt)
            clk.separable(c["kernel"], dev(a), d, c["params"]["N"], c["params"]["s"], defines=EXACT)
            got = host(d)
        assert got.tobytes() == want.tobytes(), c
        n += 1
    assert n > 800


SEP = ["gaussian_blur_separable_3d", "mean_separable_3d", "minimum_separable_3d", "maximum_separable_3d",
       "gaussian_blur_separable_2d", "mean_separable_2d", "minimum_separable_2d", "maximum_separable_2d"]


@pytest.mark.parametrize("kernel", SEP)
def test_separable_matches_oracle(clk, oracle, kernel):
    """Whole filter through clk_separable (the fused path where it applies):
    integer and min/max outputs bit-exact, float gaussian/mean within the
    FP64 tolerance."""
    rng = np.random.default_rng(11)
    shp = (70, 131) if kernel.endswith("2d") else (23, 45, 131)
    exact_op = kernel.startswith(("minimum", "maximum"))
    for sdt, ddt in ((np.uint16, np.uint16), (np.uint16, np.float32), (np.uint8, np.uint8),
                     (np.float32, np.float32), (np.int16, np.int16), (np.uint8, np.float32),
                     (np.float32, np.uint16), (np.int8, np.int8)):
        a = random_image(rng, shp, sdt)
        for N, s in (((7, 5, 3), (1.0, 0.8, 0.5)), ((1, 11, 5), (0.0, 1.7, 1.0)), ((19, 19, 11), (3.0, 3.0, 1.5))):
            d = empty(a.shape, ddt)
            clk.separable(kernel, dev(a), d, N, s)
            got = host(d)
            if np.dtype(ddt) != np.float32 or exact_op:
                want = oracle.separable(kernel, a, ddt, N, s)
                assert got.tobytes() == want.tobytes(), (kernel, np.dtype(sdt), np.dtype(ddt), N, s)
            else:
                val, scale = oracle.fp64(kernel, a, N, s)
                assert_fp64_close(got, val, scale, f"{kernel} {np.dtype(sdt)} N={N}")


def test_convert_rte_policy(clk, oracle):
    rng = np.random.default_rng(12)
    a = random_image(rng, (8, 16, 24), np.uint16)
    for kernel, p in (("mean_separable_3d", {"dim": 0, "N": 4, "s": 0.0}),
                      ("gaussian_blur_separable_3d", {"dim": 2, "N": 5, "s": 1.0})):
        ints, floats = golden_cases.split_params(p)
        want = oracle.execute(kernel, a, np.uint8, ints, floats, flags=oracle.FLAG_RTE)
        got = run_execute(clk, kernel, a, np.uint8, p, defines={"CLK_CONVERT_ROUNDING": "rte"})
        assert got.tobytes() == want.tobytes()


def test_sobel3d_narrow_read_policy(clk, oracle):
    rng = np.random.default_rng(13)
    a = random_image(rng, (8, 16, 24), np.uint16)
    want = oracle.execute("sobel_3d", a, np.float32, flags=oracle.FLAG_SOBEL_NARROW)
    got = run_execute(clk, "sobel_3d", a, np.float32, {}, defines={"CLK_SOBEL3D_READ": "narrow", **EXACT})
    assert got.tobytes() == want.tobytes()
    val, scale = oracle.fp64("sobel_3d", a, flags=oracle.FLAG_SOBEL_NARROW)
    got = run_execute(clk, "sobel_3d", a, np.float32, {}, defines={"CLK_SOBEL3D_READ": "narrow"})
    assert_fp64_close(got, val, scale, "sobel_3d narrow")


def test_errors_surface_as_exceptions(clk):
    import torch
    a = torch.zeros((4, 4, 4), dtype=torch.uint16, device="cuda")
    with pytest.raises(clk.ClkError) as e:
        clk.execute("median_box_3d", {"src": a, "dst": a, "Nx": 3, "Ny": 3})
    assert "missing parameter 'Nz'" in str(e.value)
    with pytest.raises(clk.ClkError):
        clk.execute("no_such_kernel", {"src": a, "dst": a})

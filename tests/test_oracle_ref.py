"""The oracle restatement against the reference's own kernels.

oracle/_ref is kernels/*.cl compiled as C++ (oracle/build_ref.py); it exists
where the reference checkout was available.  Every kernel, every pixel-type
pair, degenerate extents and parameters: bytes must be identical.
"""
import numpy as np
import pytest

from conftest import DTYPES, random_image

KERNELS = None


def _kernels():
    from oracle import oracle as O
    return O.KERNELS


def _cases(k):
    is2 = k.endswith("2d")
    if "slice_by_slice" in k and not k.startswith(("erode", "dilate")):
        return [((3, 3), ()), ((5, 5), ()), ((5, 3), ()), ((1, 7), ())]
    if "_sphere_" in k and k.startswith(("minimum", "maximum", "mean")):
        return [((3, 3), ()), ((5, 5), ()), ((5, 3), ()), ((1, 7), ())] if is2 else \
            [((3, 3, 3), ()), ((5, 5, 5), ()), ((3, 5, 1), ()), ((7, 3, 5), ()), ((1, 1, 9), ())]
    if k.startswith("greater_constant"):
        return [((), (400.0,)), ((), (-3.5,)), ((), (0.0,))]
    if k.startswith(("gaussian", "mean", "minimum", "maximum")):
        dims = (0, 1) if is2 else (0, 1, 2)
        return [((d, N), (s,)) for d in dims for N, s in ((5, 1.5), (7, 2.0), (4, 0.7), (1, 1.0), (0, 1.0),
                                                            (-1, 1.0), (9, 0.0))]
    if k.startswith("median"):
        return [((3, 3), ()), ((5, 5), ()), ((5, 3), ()), ((1, 7), ())] if is2 else \
            [((3, 3, 3), ()), ((5, 5, 5), ()), ((3, 5, 1), ()), ((7, 3, 5), ()), ((1, 1, 9), ())]
    return [((), ())]


def _ref_or_skip(O):
    if not O.ref_available():
        pytest.skip("oracle/_ref not built (reference checkout absent)")


@pytest.mark.parametrize("kernel", [k for k in __import__("oracle.oracle", fromlist=["KERNELS"]).KERNELS
                                    if not k.startswith("convolve")])
def test_port_matches_reference(oracle, kernel):
    O = oracle
    _ref_or_skip(O)
    rng = np.random.default_rng(abs(hash(kernel)) % 2**32)
    is2 = kernel.endswith("2d")
    shapes = ((9, 11), (1, 5), (4, 1)) if is2 else ((7, 9, 11), (1, 4, 5), (3, 1, 1))
    morph = kernel.startswith(("erode", "dilate"))
    n = 0
    for shp in shapes:
        for sdt in DTYPES:
            for ddt in DTYPES:
                if kernel.startswith("median") and sdt != ddt:
                    continue
                if kernel == "minimum_sphere_2d" and sdt == np.float32 and ddt != np.float32:
                    continue  # C cast of an out-of-range float: undefined in the kernel
                a = random_image(rng, shp, sdt, binary=morph)
                for ia, fa in _cases(kernel):
                    if kernel == "median_slice_by_slice_sphere_3d" and min(ia) <= 2:
                        continue  # no FLT_MIN guard there: empty neighbourhood (rejected by the library)
                    r = O.execute(kernel, a, ddt, ia, fa, impl="ref")
                    p = O.execute(kernel, a, ddt, ia, fa, impl="port")
                    assert r.tobytes() == p.tobytes(), (kernel, shp, np.dtype(sdt), np.dtype(ddt), ia, fa)
                    n += 1
    assert n > 0


@pytest.mark.parametrize("kernel", ["gaussian_blur_separable_3d", "mean_separable_3d", "minimum_separable_3d",
                                    "maximum_separable_3d", "gaussian_blur_separable_2d", "mean_separable_2d"])
def test_separable_orchestration_matches_reference(oracle, kernel):
    """Whole X->Y(->Z) filter: the port's driver vs three reference launches."""
    O = oracle
    _ref_or_skip(O)
    rng = np.random.default_rng(7)
    shp = (9, 13) if kernel.endswith("2d") else (6, 9, 13)
    for sdt, ddt in ((np.uint16, np.uint16), (np.uint16, np.float32), (np.uint8, np.uint8), (np.float32, np.float32),
                     (np.float32, np.uint8), (np.int16, np.int16)):
        a = random_image(rng, shp, sdt)
        for N, s in (((5, 7, 3), (1.0, 2.0, 0.5)), ((1, 5, 5), (0.0, 1.5, 1.5)), ((9, 1, 3), (2.0, 0.0, 0.0))):
            r = O.separable(kernel, a, ddt, N, s, impl="ref")
            p = O.separable(kernel, a, ddt, N, s, impl="port")
            assert r.tobytes() == p.tobytes(), (kernel, np.dtype(sdt), np.dtype(ddt), N, s)


@pytest.mark.parametrize("kernel", ["convolve_2d", "convolve_3d"])
def test_convolve_port_matches_reference(oracle, kernel):
    """convolve takes a float kernel image: odd, even and unit extents."""
    O = oracle
    _ref_or_skip(O)
    rng = np.random.default_rng(81)
    is2 = kernel.endswith("2d")
    shapes = ((9, 11), (1, 5)) if is2 else ((7, 9, 11), (1, 4, 5))
    kshapes = ((3, 3), (5, 3), (4, 4), (1, 1)) if is2 else ((3, 3, 3), (5, 3, 1), (4, 2, 3), (1, 1, 1))
    for shp in shapes:
        for sdt in DTYPES:
            for ddt in DTYPES:
                a = random_image(rng, shp, sdt)
                for ks in kshapes:
                    k = rng.standard_normal(ks).astype(np.float32)
                    r = O.execute(kernel, a, ddt, impl="ref", kernel_image=k)
                    p = O.execute(kernel, a, ddt, impl="port", kernel_image=k)
                    assert r.tobytes() == p.tobytes(), (kernel, shp, np.dtype(sdt), np.dtype(ddt), ks)

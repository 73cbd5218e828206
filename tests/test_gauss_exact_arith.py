"""The arithmetic the Gaussian to integer pixels keeps on the fast path
(clk_sep2_gaussx.cu): per pass, the taps h(v) = exp(v^2 / (-2 s^2)) in
order v = -c..c, float products and sums each rounded on their own, the
float sum of the taps as divisor (IEEE division), conversion to the dst
type (truncating, saturating) after every pass.  Restated here in numpy
float32 and checked bit for bit against the oracle's whole separable filter
(no GPU)."""
import numpy as np
import pytest

from conftest import random_image

f32 = np.float32


def taps(N, s):
    c = (N - 1) // 2
    n = f32(f32(-2.0 * f32(s)) * f32(s))
    hs, h = f32(0), []
    for v in range(-c, c + 1):
        q = f32(f32(v * v) / n)
        hv = f32(np.exp(np.float64(q)))  # the correctly rounded float of exp
        h.append(hv)
        hs = f32(hs + hv)
    return c, h, hs


def one_pass(x, axis, N, s, dt):
    c, h, hs = taps(N, s)
    xp = np.moveaxis(x.astype(f32), axis, -1)
    L = xp.shape[-1]
    at = lambda k: xp[..., np.clip(np.arange(L) + k, 0, L - 1)]  # noqa: E731  clamp to edge
    acc = (h[0] * at(-c)).astype(f32)
    for v in range(1, 2 * c + 1):
        acc = (acc + (h[v] * at(v - c)).astype(f32)).astype(f32)
    q = (acc / hs).astype(f32)
    info = np.iinfo(dt)
    q = np.trunc(np.clip(q, info.min, info.max)).astype(dt)
    return np.moveaxis(q, -1, axis)


@pytest.mark.parametrize("dt", [np.uint16, np.int16, np.uint8, np.int8])
def test_integer_gaussian_arithmetic_matches_oracle(oracle, dt):
    rng = np.random.default_rng(91)
    a = random_image(rng, (6, 23, 37), dt)
    for N, s in (((3, 3, 1), (0.43, 0.43, 0.0)), ((13, 13, 7), (2.0, 2.0, 1.0)), ((5, 9, 5), (1.0, 1.7, 0.8))):
        x = a
        for axis, (n, sg) in zip((2, 1, 0), zip(N, s)):
            if n > 1 and sg > 0:
                x = one_pass(x, axis, n, sg, dt)
        want = oracle.separable("gaussian_blur_separable_3d", a, dt, N, s)
        assert np.array_equal(x, want), (np.dtype(dt), N, s)

"""The fast sobel_3d kernel's algebra, checked on the CPU.

clk_sobel.cu evaluates the 3x3x4 window of sobel_3d_x.cl:44-52 through
per-plane row sums and differences and per-output z combinations, and adds
K * 2^32 per component for unsigned reads (negative coefficients times uint
pixels wrap).  Here the same decomposition is written in numpy and compared
with the window summed tap by tap using the coefficients the kernel reads
(flat array layout, the out-of-range tap = 0), the terms wrapped as uint32.
"""
import numpy as np


def coef(comp, m, n, k):
    h, hp = (1, 2, 1), (1, 0, -1)
    flat = 9 * m + 3 * n + k
    if flat >= 27:
        return 0
    mm, nn, kk = flat // 9, (flat // 3) % 3, flat % 3
    return (hp[mm] * h[nn] * h[kk], h[mm] * hp[nn] * h[kk], h[mm] * h[nn] * hp[kk])[comp]


def direct(v, x, y, z, wrap):
    out = []
    for comp in range(3):
        s = 0
        for m in range(3):
            for n in range(3):
                for k in range(4):
                    c = coef(comp, m, n, k)
                    val = int(v[z + k - 1, y + n - 1, x + m - 1])
                    s += ((c * val) & 0xFFFFFFFF) if wrap else c * val
        out.append(s)
    return out


def decomposed(v, x, y, z, wrap):
    def plane(p):
        P = v[p].astype(np.int64)
        sx = lambda r: P[r, x - 1] + 2 * P[r, x] + P[r, x + 1]  # noqa: E731
        dx = lambda r: P[r, x - 1] - P[r, x + 1]  # noqa: E731
        rm, rc, rp = y - 1, y, y + 1
        q = 2 * P[rp, x - 1] + P[rp, x]
        return dict(A=dx(rm) + 2 * dx(rc) + dx(rp), B=sx(rm) - sx(rp), C=sx(rm) + 2 * sx(rc) + sx(rp),
                    Ex=2 * dx(rm) + dx(rc) - P[rp, x], Ey=q - sx(rc), Ez=2 * sx(rm) + sx(rc) + q)
    a, b, c, e = plane(z - 1), plane(z), plane(z + 1), plane(z + 2)
    sx = a["A"] + 2 * b["A"] + c["A"] + e["Ex"]
    sy = a["B"] + 2 * b["B"] + c["B"] + e["Ey"]
    sz = a["C"] - c["C"] + e["Ez"]
    if wrap:
        nz = lambda dx_, dy_, dz_: int(v[z + dz_, y + dy_, x + dx_] != 0)  # noqa: E731
        kx = sum(nz(1, d, dz) for dz in (-1, 0, 1) for d in (-1, 0, 1)) + nz(0, 1, 2) + nz(1, -1, 2) + nz(1, 0, 2)
        ky = sum(nz(d, 1, dz) for dz in (-1, 0, 1) for d in (-1, 0, 1)) + nz(-1, 0, 2) + nz(0, 0, 2) + nz(1, 0, 2)
        kz = sum(nz(dx_, dy_, 1) for dx_ in (-1, 0, 1) for dy_ in (-1, 0, 1))
        sx, sy, sz = sx + kx * 2**32, sy + ky * 2**32, sz + kz * 2**32
    return [int(sx), int(sy), int(sz)]


def test_decomposition_matches_tap_by_tap_sum():
    rng = np.random.default_rng(3)
    for wrap in (True, False):
        for trial in range(300):
            v = rng.integers(0, 65536, size=(5, 3, 3 + 2)).astype(np.int64)
            if trial % 3 == 0:
                v[rng.random(v.shape) < 0.3] = 0  # zero pixels change the wrap counts
            assert decomposed(v, 2, 1, 1, wrap) == direct(v, 2, 1, 1, wrap)


def test_wrap_counts_without_zero_pixels():
    """12, 12, 9 negative-coefficient taps per component when no pixel is 0."""
    neg = [sum(1 for m in range(3) for n in range(3) for k in range(4) if coef(c, m, n, k) < 0) for c in range(3)]
    assert neg == [12, 12, 9]
